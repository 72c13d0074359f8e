// Launch interface between the host context (capi.cu) and the kernel
// translation units (lb_fp64.cu, lb_fp32.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hlbg {

struct StepArgs;

// Launch variants of the stream-and-collide kernel (FP32 / FP16 forms; FP64 has one):
// 0 default shape, 1: 128x8, 2: 256x4, 3: 512x2 threads x resident CTAs per SM,
// 4: one CTA per block, staged by bulk copies; 5, 6, 7: the fluid-list launch;
// 8: persistent, pipelined block staging (FP32 / FP16).
constexpr int kSCVariants = 9;

struct PostArgs {
  void* f_new;
  int64_t stride;
  const int32_t* slot;
  const int8_t* dir;
  const float* q;
  int64_t count;
  float fp16_scale, fp16_inv_scale;
};

struct InitArgs {
  void* f0;
  void* f1;
  int64_t stride, nslot;
  const uint32_t* site_code;
  const uint8_t* block_bulk;
  double value[19];
  float fp16_scale, fp16_inv_scale;
};

struct FieldArgs {
  void* f0;
  void* f1;
  int64_t stride;
  const int32_t* ref2slot;
  int64_t first, count;
  const double* rho;  // [count]
  const double* u;    // [count*3]
  float fp16_scale, fp16_inv_scale;
};

struct GatherArgs {
  const void* f;
  void* f_out;
  int64_t stride;
  const int32_t* ref2slot;
  int64_t first, count;
  double* aos;  // [count*19]
  double* rho;  // [count]
  double* u;    // [count*3]
  float fp16_scale, fp16_inv_scale;
};

struct MonitorArgs {
  const void* f_cur;
  const void* f_prev;
  int64_t stride, nslot;
  const uint32_t* site_code;
  const uint8_t* block_bulk;
  double* part_mass;
  double* part_max;
  double* part_min;
  unsigned long long* part_bad;
  float fp16_scale, fp16_inv_scale;
};

// Steady-state detection after every step (StabilityTester with its convergence
// check, Code/lb/StabilityTester.h:91-183): the last stage of the fused monitor's
// reduction counts checks and records the first check whose max |u_new - u_old|
// is within the threshold (tol * U_ref), and the first unstable one.
struct SteadyArgs {
  const double* threshold;  // tol * U_ref
  double* last_du;          // max |du| of the latest check
  long long* counters;      // [checks done, first converged check or -1, first unstable check or -1]
};

// f_cur <- (f_cur + f_prev) / 2 on every fluid slot
struct AverageArgs {
  void* f_cur;
  const void* f_prev;
  int64_t nslot;
  const uint32_t* site_code;
  const uint8_t* block_bulk;
  float fp16_scale, fp16_inv_scale;
};

// Wall shear stress magnitude per site in contiguous order (DBL_MAX where the
// site has no wall link), for the state in f.
struct WssArgs {
  const void* f;
  const int32_t* ref2slot;
  const uint32_t* site_code;
  const uint8_t* block_bulk;
  const uint32_t* b_wall;
  const float* b_normal;  // [nrec * 3]
  double stress_param;
  int64_t count;
  double* out;
  float fp16_inv_scale;
};

// Mass flux through each iolet: per listed site (a site with links to that
// iolet) its momentum along the iolet's inward normal.
struct FluxArgs {
  const void* f;
  const int32_t* slot;  // [count]
  const int32_t* gi;    // [count] inlets first, then outlets
  const IoletDev* iolets;
  int64_t count;
  double* out;  // [count]
  float fp16_inv_scale;
};

#define HLBG_DECLARE(P)                                                              \
  void launch_stream_collide_##P(const StepArgs& a, const int32_t* bxyz, cudaStream_t st,  \
                                 int variant);                                           \
  void launch_iolet_links_##P(const StepArgs& a, const int32_t* rec, const int32_t* rec_slot, \
                              int64_t n, const int32_t* bxyz, cudaStream_t st);          \
  void launch_post_step_##P(const PostArgs& p, cudaStream_t st);                     \
  void launch_init_uniform_##P(const InitArgs& ia, cudaStream_t st);                 \
  void launch_init_field_##P(const FieldArgs& fa, cudaStream_t st);                  \
  void launch_gather_##P(const GatherArgs& ga, cudaStream_t st);                     \
  void launch_scatter_##P(const GatherArgs& ga, cudaStream_t st);                    \
  void launch_macro_##P(const GatherArgs& ga, cudaStream_t st);                      \
  void launch_monitor_##P(const MonitorArgs& ma, int grid, cudaStream_t st);          \
  /* load the monitor kernels now (with lazy module loading they load on first use) */ \
  cudaError_t preload_monitor_##P();                                                 \
  int64_t monitored_grid_##P(int64_t nslot, int variant, int64_t n_warps);                                   \
  void launch_mon_reduce_##P(const double* part, int64_t nparts, double* part2, int64_t n2,    \
                             int32_t* mon_state, double* result, const SteadyArgs& sa,        \
                             int steady, cudaStream_t st);                                     \
  void launch_average_##P(const AverageArgs& aa, cudaStream_t st);                    \
  void launch_halo_copy_##P(void* f, const int64_t* off, int64_t n, int64_t limit, void* buf, \
                            int unpack, int32_t* err, cudaStream_t st);                  \
  void launch_wss_##P(const WssArgs& wa, cudaStream_t st);                                \
  void launch_flux_##P(const FluxArgs& fa, cudaStream_t st);

HLBG_DECLARE(0)
HLBG_DECLARE(1)
HLBG_DECLARE(2)

}  // namespace hlbg
