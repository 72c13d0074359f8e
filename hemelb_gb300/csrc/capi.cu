// Host side of the C ABI: context, single-device site layout, launches.
//
// The layout builder replaces the reference's Domain construction
// (Code/geometry/Domain.cc:69-505: ProcessReadSites, PopulateWithReadData,
// InitialiseNeighbourLookup) for one GPU: non-empty 8^3 blocks are put in Morton
// order (the octree leaf order of Code/geometry/LookupTree.h:23-41), every block
// keeps all 512 slots so neighbours are found by arithmetic plus a 27-entry
// neighbour-block table, and only sites next to a wall or iolet carry a record.
// The reference's contiguous site numbering (collision type, then block, then
// in-block order) is kept as a permutation for the FieldData-layout accessors.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hemelb_gb300.h"
#include "lb_device.cuh"
#include "lb_launch.h"

using namespace hlbg;

namespace {
constexpr double kPI = 3.14159265358979323846264338327950288;  // Code/constants.h:18
constexpr int64_t kStageSites = 1 << 22;
constexpr int kStepBatch = 1024;

const int HCX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int HCY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int HCZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
const int HINV[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

// Fluid list order within a block: its sites in slot order (HLBG_LIST_SPLIT=0);
// its bulk sites first and then its boundary sites (1), which keeps most warps on
// the bulk push path but leaves gaps in each warp's slots; or whole 8-site rows,
// those without a boundary site first (2).  Measured on the vascular forest: 1 is
// +4% to +9% for FP16 storage (instruction-bound) and -7% for FP32 deviations
// (bandwidth-bound); 2 is +/-0 for FP32 and +8% for FP16.  The default (-1) is 1
// for FP16 and 0 otherwise.
#ifndef HLBG_LIST_SPLIT
#define HLBG_LIST_SPLIT -1
#endif

// Device block order (HLBG_BLOCK_SORT): 0 z-columns in 2-D Morton order of (x, y);
// 1 3-D Morton order; 2 z-columns along a 2-D Hilbert curve of (x, y).
#ifndef HLBG_BLOCK_SORT
#define HLBG_BLOCK_SORT 0
#endif

// Index of (x, y) along a 2-D Hilbert curve over an n x n grid (n a power of two):
// the standard rotate-and-reflect walk from the top quadrant down.
uint64_t hilbert2(uint32_t n, uint32_t x, uint32_t y) {
  uint64_t d = 0;
  for (uint32_t s = n / 2; s > 0; s /= 2) {
    const uint32_t rx = (x & s) ? 1u : 0u, ry = (y & s) ? 1u : 0u;
    d += (uint64_t)s * s * ((3u * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {  // reflect (only the bits below s matter from here on)
        x = n - 1 - x;
        y = n - 1 - y;
      }
      const uint32_t t = x;
      x = y;
      y = t;
    }
  }
  return d;
}

uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  uint64_t m = 0;
  for (int k = 0; k < 16; ++k) {
    m |= (uint64_t)((x >> k) & 1u) << (3 * k + 2);
    m |= (uint64_t)((y >> k) & 1u) << (3 * k + 1);
    m |= (uint64_t)((z >> k) & 1u) << (3 * k);
  }
  return m;
}

int collision_type(uint32_t wall, int8_t site_type) {
  // SiteData::GetCollisionType (Code/geometry/SiteDataBare.cc:102-145) mapped to
  // the range index of Domain::ProcessReadSites (Code/geometry/Domain.cc:188-207)
  if (wall == 0) return site_type == HLBG_SITE_INLET ? 2 : (site_type == HLBG_SITE_OUTLET ? 3 : 0);
  return site_type == HLBG_SITE_INLET ? 4 : (site_type == HLBG_SITE_OUTLET ? 5 : 1);
}

double dot3(const double* a, const double* b) {
  double s = 0.0;
  s = s + a[0] * b[0];
  s = s + a[1] * b[1];
  s = s + a[2] * b[2];
  return s;
}

template <class F>
void parallel_for(int64_t n, F&& f) {
  int nt = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (n < 4096) nt = 1;
  std::atomic<int64_t> next{0};
  auto work = [&]() {
    for (;;) {
      int64_t c = next.fetch_add(1024);
      if (c >= n) break;
      int64_t e = std::min(n, c + 1024);
      for (int64_t i = c; i < e; ++i) f(i);
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work);
  work();
  for (auto& t : th) t.join();
}
}  // namespace

struct hlbg_ctx {
  std::string err;
  hlbg_params params{};
  int prec = 0;
  size_t elem = 8;
  int64_t nb = 0, nslot = 0, nsites = 0, nrec = 0;
  int64_t type_count[6] = {0, 0, 0, 0, 0, 0};
  std::vector<int32_t> h_block_xyz;
  std::vector<int32_t> h_ref2slot;
  std::vector<hlbg_iolet> inlets, outlets;
  double min_density = 1.0;
  uint64_t t1 = 1;
  int cur = 0;
  double* noalloc_scratch = nullptr;  // device address of hlbg_reduce_noalloc's static array
  void* f[2] = {nullptr, nullptr};
  int32_t* d_block_nbr = nullptr;
  int32_t* d_block_xyz = nullptr;
  uint32_t* d_site_code = nullptr;
  int32_t* d_warp_block = nullptr;  // fluid-list launch (StepArgs::warp_block)
  uint16_t* d_lane_slot = nullptr;
  int64_t n_warps = 0;
  uint64_t* d_blk_fluid = nullptr;  // block-staged launch (StepArgs::blk_*)
  uint64_t* d_blk_bnd = nullptr;
  uint32_t* d_blk_run_off = nullptr;
  uint16_t* d_blk_runs = nullptr;
  uint64_t* d_pipe_desc = nullptr;  // pipelined launch: per block, its fluid-list warps and row span
  int32_t* d_stage_err = nullptr;
  std::vector<int32_t> h_flux_slot, h_flux_gi;  // sites with iolet links, their iolet
  int32_t* d_flux_slot = nullptr;
  int32_t* d_flux_gi = nullptr;
  double* d_flux = nullptr;
  uint16_t* d_slot2site = nullptr;  // packed blocks: local site of each slot
  uint16_t* d_site2slot = nullptr;  // packed blocks: slot of each local site
  std::vector<uint16_t> h_slot2site;
  uint8_t* d_block_bulk = nullptr;
  uint32_t* d_b_wall = nullptr;
  uint32_t* d_b_iolet = nullptr;
  int32_t* d_b_ioid = nullptr;
  int8_t* d_b_type = nullptr;
  float* d_b_cut = nullptr;
  uint64_t* d_b_links = nullptr;  // 3-bit link code per direction (see lb_device.cuh)
  float* d_b_normal = nullptr;      // wall normal per record
  double* d_wss = nullptr;          // wall shear stress output, allocated on first use
  int32_t* d_rec_slot = nullptr;  // slot of each record
  std::vector<int32_t> h_new_of_old;  // device block index of each input block
  std::vector<uint16_t> h_site2slot;  // in-block slot of each local site (built by hlbg_halo_offsets)
  int32_t* d_halo_err = nullptr;      // out-of-range offsets seen by the halo pack / unpack
  double* d_blk_omega = nullptr;      // optional per-block (omega+, omega-)
  // CUDA graphs of k steps, keyed by (k, parity of the current array)
  struct GraphKey {
    int n, cur, check;  // check: a steady-state check after every step
    bool operator<(const GraphKey& o) const {
      return n != o.n ? n < o.n : (cur != o.cur ? cur < o.cur : check < o.check);
    }
  };
  std::map<GraphKey, cudaGraphExec_t> graphs;
  int32_t* d_io_rec = nullptr;    // records with at least one iolet link
  int64_t n_io_rec = 0;
  int32_t* d_ref2slot = nullptr;
  int32_t* d_ps_slot = nullptr;
  int8_t* d_ps_dir = nullptr;
  float* d_ps_q = nullptr;
  int64_t n_ps = 0;
  // per-range post step uses records directly (host list built on demand)
  std::vector<int32_t> h_ps_slot;
  std::vector<int8_t> h_ps_dir;
  std::vector<float> h_ps_q;
  std::vector<int32_t> h_rec_slot;
  IoletDev* d_iolets = nullptr;
  int n_io = 0;
  double* d_io_tab = nullptr;   // [kStepBatch][2][n_io]: rho, umax
  double* h_io_tab = nullptr;   // pinned staging
  cudaEvent_t io_copied = nullptr;
  double* d_stage = nullptr;
  double* d_stage_rho = nullptr;
  double* d_stage_u = nullptr;
  int32_t* d_list = nullptr;
  int64_t list_cap = 0;
  double* d_part = nullptr;  // monitor partials
  unsigned long long* d_part_bad = nullptr;
  // steady-state detection: [threshold, last max |du|] and the SteadyArgs counters
  double* d_steady = nullptr;
  long long* d_steady_n = nullptr;
  long long* h_steady_n = nullptr;  // pinned copy of the counters
  // fused StabilityTester: per-slot velocity of the last monitored step, partials
  // of the two reduction stages, the recorded-velocity flag and the last result
  void* d_mon_u = nullptr;
  double* d_mon_part = nullptr;
  double* d_mon_part2 = nullptr;
  int32_t* d_mon_state = nullptr;
  double* d_mon_result = nullptr;
  double* h_mon_result = nullptr;  // pinned
  bool mon_recorded = false;       // host view: velocities of the current state recorded
  int32_t mon_interval = 1;        // hlbg_step_monitored checks the steps t with t % interval == 0
  int64_t mon_checked_t = -1;      // the step of the last check hlbg_step_monitored launched
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t dev_bytes = 0;
  float fp16_scale = 1024.f;
  int sc_variant = 0;  // chosen by hlbg_autotune
  bool initialised = false;
};

namespace {

int fail(hlbg_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, HLBG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dev_alloc(hlbg_ctx* ctx, T** p, size_t count) {
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, HLBG_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                        cudaGetErrorString(e));
  }
  ctx->dev_bytes += bytes;
  return HLBG_OK;
}

template <class T>
int upload(hlbg_ctx* ctx, T** p, const std::vector<T>& v) {
  int rc = dev_alloc(ctx, p, v.size());
  if (rc) return rc;
  if (!v.empty()) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return HLBG_OK;
}

void fill_args(hlbg_ctx* ctx, StepArgs& a) {
  std::memset(&a, 0, sizeof(a));
  a.f_old = ctx->f[ctx->cur];
  a.f_new = ctx->f[ctx->cur ^ 1];
  a.stride = ctx->nslot;
  a.nslot = ctx->nslot;
  a.block_nbr = ctx->d_block_nbr;
  a.slot2site = ctx->d_slot2site;
  a.site2slot = ctx->d_site2slot;
  a.warp_block = ctx->d_warp_block;
  a.blk_fluid = ctx->d_blk_fluid;
  a.blk_bnd = ctx->d_blk_bnd;
  a.blk_run_off = ctx->d_blk_run_off;
  a.blk_runs = ctx->d_blk_runs;
  a.pipe_desc = ctx->d_pipe_desc;
  a.n_blocks = ctx->nb;
  a.stage_err = ctx->d_stage_err;
  a.pipe_ctr = ctx->d_stage_err + 1;
  a.lane_slot = ctx->d_lane_slot;
  a.n_warps = ctx->n_warps;
  a.site_code = ctx->d_site_code;
  a.block_bulk = ctx->d_block_bulk;
  a.b_wall = ctx->d_b_wall;
  a.b_iolet = ctx->d_b_iolet;
  a.b_ioid = ctx->d_b_ioid;
  a.b_type = ctx->d_b_type;
  a.b_cut = ctx->d_b_cut;
  a.b_links = ctx->d_b_links;
  a.blk_omega = ctx->d_blk_omega;
  a.iolets = ctx->d_iolets;
  a.n_in = (int32_t)ctx->inlets.size();
  a.kernel = ctx->params.kernel;
  a.wall = ctx->params.wall;
  a.inlet_model = ctx->params.inlet;
  a.outlet_model = ctx->params.outlet;
  // LbmParameters::CalcDerivedParams (Code/lb/LbmParameters.h:34-39) and
  // TRT::Collide's second relaxation time (Code/lb/kernels/TRT.h:167-172)
  const double tau = ctx->params.tau;
  a.omega = -1.0 / tau;
  const double tau_minus = 0.5 + (3.0 / 16.0) / (tau - 0.5);
  a.omega_minus = -1.0 / tau_minus;
  a.omega_f = (float)a.omega;
  a.omega_minus_f = (float)a.omega_minus;
  a.fp16_scale = ctx->fp16_scale;
  a.fp16_inv_scale = 1.0f / ctx->fp16_scale;
}

double iolet_density(const hlbg_ctx* ctx, const hlbg_iolet& io, uint64_t t) {
  // InOutLetCosine::GetDensity (Code/lb/iolets/InOutLetCosine.cc:26-43);
  // velocity iolets report 1.0 (Code/lb/iolets/InOutLetVelocity.cc:23-26)
  if (io.model != HLBG_IOLET_COSINE) return 1.0;
  double w = 2.0 * kPI / io.period;
  double target = io.density_mean + io.density_amp * std::cos(w * (double)t + io.phase);
  if (t >= io.warmup_steps) return target;
  double interp = ((double)t) / ((double)io.warmup_steps);
  return interp * target + (1. - interp) * ctx->min_density;
}

double iolet_umax(const hlbg_iolet& io, uint64_t t) {
  // peak speed of InOutLetParabolicVelocity::GetVelocity at time t
  // (Code/lb/iolets/InOutLetParabolicVelocity.cc:35-40); the pulsatile model
  // scales it by (1 - cos(2 pi t / T)) / 2 first
  if (io.model == HLBG_IOLET_COSINE) return 0.0;
  double max = io.max_speed;
  if (io.model == HLBG_IOLET_PULSATILE)
    max = max * (0.5 * (1.0 - std::cos(2.0 * kPI * (double)t / io.vel_period)));
  if (t < io.warmup_steps) max *= (double)t / (double)io.warmup_steps;
  return max;
}

int launch_collide(hlbg_ctx* ctx, StepArgs& a, cudaStream_t st) {
  switch (ctx->prec) {
    case 0: launch_stream_collide_0(a, ctx->d_block_xyz, st, ctx->sc_variant); break;
    case 1: launch_stream_collide_1(a, ctx->d_block_xyz, st, ctx->sc_variant); break;
    default: launch_stream_collide_2(a, ctx->d_block_xyz, st, ctx->sc_variant); break;
  }
  CK(cudaGetLastError());
  // the all-slots kernel leaves iolet links to k_iolet_links; the list kernel does them itself
  if (!a.list && ctx->n_io_rec > 0) {
    switch (ctx->prec) {
      case 0: launch_iolet_links_0(a, ctx->d_io_rec, ctx->d_rec_slot, ctx->n_io_rec, ctx->d_block_xyz, st); break;
      case 1: launch_iolet_links_1(a, ctx->d_io_rec, ctx->d_rec_slot, ctx->n_io_rec, ctx->d_block_xyz, st); break;
      default: launch_iolet_links_2(a, ctx->d_io_rec, ctx->d_rec_slot, ctx->n_io_rec, ctx->d_block_xyz, st); break;
    }
    CK(cudaGetLastError());
  }
  return HLBG_OK;
}

int launch_post(hlbg_ctx* ctx, const PostArgs& p, cudaStream_t st) {
  switch (ctx->prec) {
    case 0: launch_post_step_0(p, st); break;
    case 1: launch_post_step_1(p, st); break;
    default: launch_post_step_2(p, st); break;
  }
  CK(cudaGetLastError());
  return HLBG_OK;
}

// Fill the iolet table for steps [t1, t1 + n) and copy it to the device.
int upload_iolet_table(hlbg_ctx* ctx, int n, cudaStream_t st) {
  if (ctx->n_io == 0) return HLBG_OK;
  CK(cudaEventSynchronize(ctx->io_copied));
  for (int k = 0; k < n; ++k) {
    uint64_t t1 = ctx->t1 + k;
    double* row = ctx->h_io_tab + (size_t)k * 2 * ctx->n_io;
    int j = 0;
    for (auto* v : {&ctx->inlets, &ctx->outlets})
      for (auto& io : *v) {
        // Nash: BoundaryValues::GetBoundaryDensity uses the 0-indexed step
        // (Code/lb/iolets/BoundaryValues.cc:162-165); Ladd: BoundaryValues::GetTimeStep
        // returns the 1-indexed step as unsigned int (BoundaryValues.h:67-70)
        row[j] = iolet_density(ctx, io, t1 - 1);
        row[ctx->n_io + j] = iolet_umax(io, (uint64_t)(unsigned int)t1);
        ++j;
      }
  }
  CK(cudaMemcpyAsync(ctx->d_io_tab, ctx->h_io_tab, sizeof(double) * 2 * ctx->n_io * n,
                     cudaMemcpyHostToDevice, st));
  CK(cudaEventRecord(ctx->io_copied, st));
  return HLBG_OK;
}

int ensure_list(hlbg_ctx* ctx, int64_t n) {
  if (ctx->list_cap >= n) return HLBG_OK;
  if (ctx->d_list) cudaFree(ctx->d_list);
  ctx->d_list = nullptr;
  ctx->list_cap = 0;
  int rc = dev_alloc(ctx, &ctx->d_list, (size_t)n);
  if (rc) return rc;
  ctx->list_cap = n;
  return HLBG_OK;
}

int ensure_stage(hlbg_ctx* ctx) {
  if (ctx->d_stage) return HLBG_OK;
  int rc = dev_alloc(ctx, &ctx->d_stage, (size_t)kStageSites * 19);
  if (!rc) rc = dev_alloc(ctx, &ctx->d_stage_rho, (size_t)kStageSites);
  if (!rc) rc = dev_alloc(ctx, &ctx->d_stage_u, (size_t)kStageSites * 3);
  return rc;
}

void fill_gather(hlbg_ctx* ctx, GatherArgs& g) {
  std::memset(&g, 0, sizeof(g));
  g.stride = ctx->nslot;
  g.ref2slot = ctx->d_ref2slot;
  g.fp16_scale = ctx->fp16_scale;
  g.fp16_inv_scale = 1.0f / ctx->fp16_scale;
}

int build_layout(hlbg_ctx* ctx, const hlbg_geometry* g) {
  const int64_t nb = g->n_blocks;
  const int NX = g->blocks[0], NY = g->blocks[1], NZ = g->blocks[2];
  if (nb <= 0 || NX <= 0 || NY <= 0 || NZ <= 0 || !g->block_coords || !g->fluid_mask)
    return fail(ctx, HLBG_ERR_INVAL, "geometry has no blocks");
  if ((int64_t)NX * NY * NZ > (1ll << 31)) return fail(ctx, HLBG_ERR_INVAL, "block grid too large");
  if (nb * 512 >= (1ll << 31)) return fail(ctx, HLBG_ERR_INVAL, "more than 2^31 slots");
  // Device block order: z-columns (2-D Morton order of (x, y), then z).  The two
  // writers of every z-shifted row of a push are z-adjacent blocks; running them
  // back to back lets their partial 32-byte sectors merge in L2.  The reference's
  // own numbering (3-D Morton order) is kept separately in ref_rank below.
  uint32_t hn = 1;  // Hilbert grid side: a power of two covering the block grid
  while (hn < (uint32_t)std::max(NX, NY)) hn *= 2;
  (void)hn;
  std::vector<std::pair<uint64_t, int64_t>> order((size_t)nb);
  std::vector<std::pair<uint64_t, int64_t>> ref_order((size_t)nb);
  for (int64_t b = 0; b < nb; ++b) {
    int32_t x = g->block_coords[3 * b], y = g->block_coords[3 * b + 1], z = g->block_coords[3 * b + 2];
    if (x < 0 || y < 0 || z < 0 || x >= NX || y >= NY || z >= NZ)
      return fail(ctx, HLBG_ERR_INVAL, "block coordinate outside the block grid");
#if HLBG_BLOCK_SORT == 1
    order[b] = {morton3(x, y, z), b};
#elif HLBG_BLOCK_SORT == 2
    order[b] = {(hilbert2(hn, x, y) << 16) | (uint64_t)z, b};
#else
    order[b] = {(morton3(x, y, 0) << 16) | (uint64_t)z, b};
#endif
    ref_order[b] = {morton3(x, y, z), b};
  }
  std::sort(order.begin(), order.end());
  std::sort(ref_order.begin(), ref_order.end());
  std::vector<int32_t> new_of_old((size_t)nb);
  std::vector<int32_t> grid((size_t)NX * NY * NZ, -1);
  ctx->h_block_xyz.resize((size_t)nb * 3);
  std::vector<uint64_t> mask((size_t)nb * 8);
  for (int64_t nbi = 0; nbi < nb; ++nbi) {
    int64_t ob = order[nbi].second;
    new_of_old[ob] = (int32_t)nbi;
    int32_t x = g->block_coords[3 * ob], y = g->block_coords[3 * ob + 1], z = g->block_coords[3 * ob + 2];
    size_t gi = ((size_t)x * NY + y) * NZ + z;
    if (grid[gi] >= 0) return fail(ctx, HLBG_ERR_INVAL, "duplicate block coordinates");
    grid[gi] = (int32_t)nbi;
    ctx->h_block_xyz[3 * nbi] = x;
    ctx->h_block_xyz[3 * nbi + 1] = y;
    ctx->h_block_xyz[3 * nbi + 2] = z;
    for (int w = 0; w < 8; ++w) mask[nbi * 8 + w] = g->fluid_mask[ob * 8 + w];
  }
  ctx->h_new_of_old = new_of_old;
  std::vector<int32_t> bnbr((size_t)nb * 27);
  parallel_for(nb, [&](int64_t b) {
    int32_t x = ctx->h_block_xyz[3 * b], y = ctx->h_block_xyz[3 * b + 1], z = ctx->h_block_xyz[3 * b + 2];
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          int xx = x + dx, yy = y + dy, zz = z + dz;
          int32_t v = -1;
          if (xx >= 0 && yy >= 0 && zz >= 0 && xx < NX && yy < NY && zz < NZ)
            v = grid[((size_t)xx * NY + yy) * NZ + zz];
          bnbr[b * 27 + (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1)] = v;
        }
  });
  const int64_t nslot = nb * 512;
  auto fluid = [&](int64_t s) { return (mask[(s >> 9) * 8 + ((s & 511) >> 6)] >> (s & 63)) & 1ull; };
  auto neighbour = [&](int64_t s, int d) -> int64_t {
    int l = (int)(s & 511);
    int x = (l >> 6) + HCX[d], y = ((l >> 3) & 7) + HCY[d], z = (l & 7) + HCZ[d];
    int ox = x >> 3, oy = y >> 3, oz = z >> 3;
    int32_t nbk = bnbr[(s >> 9) * 27 + (ox + 1) * 9 + (oy + 1) * 3 + (oz + 1)];
    if (nbk < 0) return -1;
    return (int64_t)nbk * 512 + (((x & 7) * 8 + (y & 7)) * 8 + (z & 7));
  };
  // records from the input (by new slot)
  std::vector<int32_t> rec_of_slot((size_t)nslot, -1);
  const int64_t nin = g->n_link_sites;
  for (int64_t r = 0; r < nin; ++r) {
    int64_t os = g->link_site[r];
    if (os < 0 || os >= nslot) return fail(ctx, HLBG_ERR_INVAL, "link site outside the blocks");
    int64_t s = (int64_t)new_of_old[os >> 9] * 512 + (os & 511);
    if (!fluid(s)) return fail(ctx, HLBG_ERR_INVAL, "link record for a solid site");
    if (rec_of_slot[s] >= 0) return fail(ctx, HLBG_ERR_INVAL, "duplicate link record");
    rec_of_slot[s] = (int32_t)r;
  }
  // fluid sites that have a non-fluid neighbour but no record get an empty one
  std::vector<uint8_t> needs((size_t)nslot, 0);
  parallel_for(nb, [&](int64_t b) {
    for (int l = 0; l < 512; ++l) {
      int64_t s = b * 512 + l;
      if (!fluid(s)) continue;
      bool edge = false;
      for (int d = 1; d < 19 && !edge; ++d) {
        int64_t n = neighbour(s, d);
        if (n < 0 || !fluid(n)) edge = true;
      }
      needs[s] = edge || rec_of_slot[s] >= 0;
    }
  });
  std::vector<uint32_t> code((size_t)nslot, 0);
  std::vector<uint32_t> rw, ri;
  std::vector<int32_t> rid;
  std::vector<int8_t> rtype, stype;
  std::vector<float> rcut;
  std::vector<float> rnorm;
  const bool want_cut = ctx->params.wall == HLBG_WALL_BFL;
  if (want_cut && !g->cut_distance && nin > 0)
    return fail(ctx, HLBG_ERR_INVAL, "BFL walls need cut distances");
  std::vector<int8_t> site_ctype((size_t)nslot, -1);
  for (int64_t s = 0; s < nslot; ++s) {
    if (!fluid(s)) continue;
    if (!needs[s]) {
      code[s] = 1;
      site_ctype[s] = 0;
      continue;
    }
    int64_t r = (int64_t)rw.size();
    code[s] = (uint32_t)(2 + r);
    ctx->h_rec_slot.push_back((int32_t)s);
    int32_t ir = rec_of_slot[s];
    uint32_t wm = 0, im = 0;
    int32_t io = -1;
    int8_t st = HLBG_SITE_FLUID;
    if (ir >= 0) {
      wm = g->wall_mask[ir];
      im = g->iolet_mask[ir];
      io = g->iolet_id[ir];
      st = g->site_type ? g->site_type[ir] : (int8_t)HLBG_SITE_FLUID;
    }
    int ct = collision_type(wm, st);
    if (im && ct < 2) return fail(ctx, HLBG_ERR_INVAL, "iolet links on a site of fluid type");
    if (ct >= 2 && im) {
      bool inl = (ct == 2 || ct == 4);
      int lim = (int)(inl ? ctx->inlets.size() : ctx->outlets.size());
      if (io < 0 || io >= lim) return fail(ctx, HLBG_ERR_INVAL, "iolet id out of range");
    }
    rw.push_back(wm);
    ri.push_back(im);
    rid.push_back(io);
    {  // wall normal: the geometry's, else the normalised sum of the wall-link vectors
      double n[3] = {0.0, 0.0, 0.0};
      if (ir >= 0 && g->wall_normal) {
        for (int c = 0; c < 3; ++c) n[c] = g->wall_normal[ir * 3 + c];
      } else {
        for (int d = 1; d < 19; ++d)
          if ((wm >> (d - 1)) & 1u) {
            n[0] += HCX[d];
            n[1] += HCY[d];
            n[2] += HCZ[d];
          }
        const double m = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (m > 0)
          for (auto& c : n) c /= m;
      }
      for (double c : n) rnorm.push_back((float)c);
    }
    rtype.push_back((int8_t)ct);
    site_ctype[s] = (int8_t)ct;
    if (want_cut)
      for (int k = 0; k < 18; ++k)
        rcut.push_back(ir >= 0 && g->cut_distance ? g->cut_distance[ir * 18 + k] : -1.0f);
  }
  ctx->nrec = (int64_t)rw.size();
  // Per-record link codes with StreamerTypeFactory's precedence (iolet delegate for
  // types 2-5, wall delegate for types 1, 4, 5, else bulk) resolved on the host.
  std::vector<uint64_t> rlinks((size_t)ctx->nrec, 0);
  parallel_for(ctx->nrec, [&](int64_t r) {
    const int64_t s = ctx->h_rec_slot[r];
    const int ct = rtype[r];
    const bool can_wall = (ct == 1 || ct == 4 || ct == 5), can_iolet = ct >= 2;
    uint64_t codes = 0;
    for (int d = 0; d < 19; ++d) {
      uint64_t c = HLBG_LC_PUSH;
      const bool wbit = d > 0 && ((rw[r] >> (d - 1)) & 1u);
      const bool ibit = d > 0 && ((ri[r] >> (d - 1)) & 1u);
      if (can_iolet && ibit) {
        c = HLBG_LC_IOLET;
      } else if (can_wall && wbit) {
        c = HLBG_LC_BOUNCE;
        if (ctx->params.wall == HLBG_WALL_BFL) {
          const int inv = HINV[d];
          const float q = rcut[r * 18 + d - 1];
          if (!(((rw[r] >> (inv - 1)) & 1u) || q < 0.5f)) c = HLBG_LC_BFL;
        }
      } else if (d > 0) {
        int64_t n = neighbour(s, d);
        if (n < 0 || !fluid(n)) c = HLBG_LC_SKIP;  // the rubbish site
      }
      codes |= c << (3 * d);
    }
    rlinks[r] = codes;
  });
  std::vector<uint8_t> bulk((size_t)nb, 0);
  for (int64_t b = 0; b < nb; ++b) {
    bool all = true;
    for (int l = 0; l < 512 && all; ++l) all = code[b * 512 + l] == 1;
    bulk[b] = all;
  }
  // contiguous site ids (Domain::PopulateWithReadData order)
  int64_t cnt[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t s = 0; s < nslot; ++s)
    if (site_ctype[s] >= 0) cnt[site_ctype[s]]++;
  int64_t off[6];
  off[0] = 0;
  for (int t = 1; t < 6; ++t) off[t] = off[t - 1] + cnt[t - 1];
  ctx->nsites = off[5] + cnt[5];
  if (ctx->nsites == 0) return fail(ctx, HLBG_ERR_INVAL, "geometry has no fluid sites");
  for (int t = 0; t < 6; ++t) ctx->type_count[t] = cnt[t];
  ctx->h_ref2slot.assign((size_t)ctx->nsites, 0);
  for (int64_t rb = 0; rb < nb; ++rb) {
    const int64_t b = new_of_old[ref_order[rb].second];
    for (int l = 0; l < 512; ++l) {
      const int64_t s = b * 512 + l;
      if (site_ctype[s] >= 0) ctx->h_ref2slot[off[site_ctype[s]]++] = (int32_t)s;
    }
  }
  // BFL PostStep links
  if (want_cut) {
    for (int64_t r = 0; r < ctx->nrec; ++r) {
      int ct = rtype[r];
      if (!(ct == 1 || ct == 4 || ct == 5)) continue;
      for (int d = 1; d < 19; ++d) {
        if (!((rw[r] >> (d - 1)) & 1u)) continue;
        int inv = HINV[d];
        float q = rcut[r * 18 + d - 1];
        if (((rw[r] >> (inv - 1)) & 1u) || !(q < 0.5f)) continue;
        ctx->h_ps_slot.push_back(ctx->h_rec_slot[r]);
        ctx->h_ps_dir.push_back((int8_t)d);
        ctx->h_ps_q.push_back(q);
      }
    }
  }
  ctx->n_ps = (int64_t)ctx->h_ps_slot.size();
  ctx->nb = nb;
  ctx->nslot = nslot;
  // Packed builds (HLBG_PACK) pack the partly fluid blocks whose fluid sites fill
  // less than HLBG_PACK_FILL % of the z-rows they touch: their fluid sites take
  // slots 0 .. nf-1 in site order and their solid sites the rest.
  // Everything above was built with slot = local site index; map it now (every
  // block: the in-block order of slot_in_block, packed blocks their own).
  std::vector<uint16_t> site2slot((size_t)nslot), slot2site((size_t)nslot);
  std::vector<uint8_t> packed((size_t)nb, 0);
  parallel_for(nb, [&](int64_t b) {
    int nf = 0, rows = 0;
    for (int w = 0; w < 8; ++w) {
      nf += __builtin_popcountll(mask[b * 8 + w]);
      for (int k = 0; k < 8; ++k) rows += ((mask[b * 8 + w] >> (8 * k)) & 0xffull) != 0;
    }
    // only blocks whose fluid fills less than HLBG_PACK_FILL % of the z-rows
    // (sectors) it touches
    packed[b] = HLBG_PACK && nf < 512 && nf * 100 < HLBG_PACK_FILL * 8 * rows;
    if (!packed[b]) {  // the fixed in-block order of slot_in_block
      for (int l = 0; l < 512; ++l) {
        const int j = slot_of_local(l);
        site2slot[b * 512 + l] = (uint16_t)j;
        slot2site[b * 512 + j] = (uint16_t)l;
      }
      return;
    }
    int j = 0;
    for (int want = 1; want >= 0; --want)  // fluid sites first, then solid ones
      for (int l = 0; l < 512; ++l) {
        if ((fluid(b * 512 + l) != 0) != (want == 1)) continue;
        site2slot[b * 512 + l] = (uint16_t)j;
        slot2site[b * 512 + j] = (uint16_t)l;
        ++j;
      }
  });
  auto slot_of = [&](int64_t site) { return (site & ~(int64_t)511) | site2slot[site]; };
  {
    std::vector<uint32_t> pc((size_t)nslot, 0);
    for (int64_t t = 0; t < nslot; ++t) pc[slot_of(t)] = code[t];
    code.swap(pc);
  }
  for (auto& v : ctx->h_rec_slot) v = (int32_t)slot_of(v);
  // sites with links to an iolet, for hlbg_iolet_flux (record order)
  for (size_t r = 0; r < rtype.size(); ++r) {
    const int t = rtype[r];
    if (t < 2 || t > 5 || rid[r] < 0) continue;
    const bool inlet = (t == 2 || t == 4);
    ctx->h_flux_slot.push_back(ctx->h_rec_slot[r]);
    ctx->h_flux_gi.push_back(inlet ? rid[r] : (int32_t)ctx->inlets.size() + rid[r]);
  }
  for (auto& v : ctx->h_ref2slot) v = (int32_t)slot_of(v);
  for (auto& v : ctx->h_ps_slot) v = (int32_t)slot_of(v);
  for (auto& e : bnbr)
    if (e >= 0 && packed[e]) e |= kPackedBit;
  ctx->h_slot2site = slot2site;
  // device copies
  int rc;
  {
    // Fluid list: per block, its fluid slots in warps of 32 (the last padded with
    // idle lanes), then its solid slots that share an 8-slot sector with a fluid
    // slot, in zero-fill warps.
    std::vector<int32_t> wb;
    std::vector<uint16_t> ls;
    std::vector<uint16_t> tmp;
    auto flush = [&](int64_t b, bool zero) {
      for (size_t k = 0; k < tmp.size(); k += 32) {
        wb.push_back(zero ? (int32_t)((uint32_t)b | 0x80000000u) : (int32_t)b);
        for (size_t t = k; t < k + 32; ++t) ls.push_back(t < tmp.size() ? tmp[t] : (uint16_t)0xffff);
      }
      tmp.clear();
    };
    const int split = HLBG_LIST_SPLIT < 0 ? (ctx->prec == HLBG_FP16 ? 1 : 0) : HLBG_LIST_SPLIT;
    // pipelined launch, per block: its first list warp (bits 0-31), the span of
    // rows from its first fluid row to its last (32-37: first, 38-44: end), its
    // fluid warps (45-50) and zero-fill warps (51-56)
    std::vector<uint64_t> desc((size_t)nb, 0);
    for (int64_t b = 0; b < nb; ++b) {
      const uint64_t first = wb.size();
      int row0 = 64, rowe = 0;
      for (int row = 0; row < 64; ++row)
        for (int t = 0; t < 8; ++t)
          if (code[b * 512 + row * 8 + t]) {
            row0 = std::min(row0, row);
            rowe = row + 1;
          }
      if (rowe == 0) row0 = 0;
      if (split == 1) {
        // bulk sites first, then the boundary sites, so that most warps take the
        // bulk push path and only the warps holding boundary sites the mixed one
        for (int j = 0; j < 512; ++j)
          if (code[b * 512 + j] == 1) tmp.push_back((uint16_t)j);
        for (int j = 0; j < 512; ++j)
          if (code[b * 512 + j] >= 2) tmp.push_back((uint16_t)(j | kListBoundary));
      } else if (split == 2) {
        // whole 8-site rows (32-byte sectors in FP32): rows without a boundary site
        // first, then the others, so warps stay sector-aligned
        for (int pass = 0; pass < 2; ++pass)
          for (int row = 0; row < 64; ++row) {
            bool bnd = false;
            for (int t = 0; t < 8; ++t) bnd |= code[b * 512 + row * 8 + t] >= 2;
            if (bnd != (pass == 1)) continue;
            for (int t = 0; t < 8; ++t) {
              const uint32_t c = code[b * 512 + row * 8 + t];
              if (c) tmp.push_back((uint16_t)((row * 8 + t) | (c >= 2 ? kListBoundary : 0u)));
            }
          }
      } else {
        for (int j = 0; j < 512; ++j)
          if (code[b * 512 + j]) tmp.push_back((uint16_t)(j | (code[b * 512 + j] >= 2 ? kListBoundary : 0u)));
      }
      flush(b, false);
      const uint64_t nfw = wb.size() - first;
      for (int sec = 0; sec < 64; ++sec) {
        bool any = false;
        for (int t = 0; t < 8; ++t) any |= code[b * 512 + sec * 8 + t] != 0;
        if (!any) continue;
        for (int t = 0; t < 8; ++t)
          if (!code[b * 512 + sec * 8 + t]) tmp.push_back((uint16_t)(sec * 8 + t));
      }
      flush(b, true);
      const uint64_t nzw = wb.size() - first - nfw;
      desc[b] = first | ((uint64_t)row0 << 32) | ((uint64_t)rowe << 38) | (nfw << 45) | (nzw << 51);
    }
    ctx->n_warps = (int64_t)wb.size();
    if ((rc = upload(ctx, &ctx->d_warp_block, wb))) return rc;
    if ((rc = upload(ctx, &ctx->d_lane_slot, ls))) return rc;
    if (!HLBG_PACK && !HLBG_BLOCK_ORDER && ctx->n_warps < (int64_t)1 << 32 &&
        (rc = upload(ctx, &ctx->d_pipe_desc, desc)))
      return rc;
  }
  if (!HLBG_PACK && !HLBG_BLOCK_ORDER) {
    // block-staged launch: fluid / boundary bitmaps per block (slot order) and the
    // runs of consecutive rows that hold fluid
    std::vector<uint64_t> bf((size_t)nb * 8, 0), bb((size_t)nb * 8, 0);
    std::vector<uint32_t> roff((size_t)nb + 1, 0);
    std::vector<uint16_t> runs;
    for (int64_t b = 0; b < nb; ++b) {
      roff[b] = (uint32_t)runs.size();
      for (int j = 0; j < 512; ++j) {
        const uint32_t c = code[b * 512 + j];
        if (c) bf[b * 8 + (j >> 6)] |= 1ull << (j & 63);
        if (c >= 2) bb[b * 8 + (j >> 6)] |= 1ull << (j & 63);
      }
      int row = 0;
      while (row < 64) {
        if (((bf[b * 8 + (row >> 3)] >> ((row & 7) * 8)) & 0xffull) == 0) {
          ++row;
          continue;
        }
        int end = row + 1;
        while (end < 64 && ((bf[b * 8 + (end >> 3)] >> ((end & 7) * 8)) & 0xffull) != 0) ++end;
        runs.push_back((uint16_t)(row | ((end - row) << 6)));
        row = end;
      }
    }
    roff[nb] = (uint32_t)runs.size();
    if ((rc = upload(ctx, &ctx->d_blk_fluid, bf))) return rc;
    if ((rc = upload(ctx, &ctx->d_blk_bnd, bb))) return rc;
    if ((rc = upload(ctx, &ctx->d_blk_run_off, roff))) return rc;
    if ((rc = upload(ctx, &ctx->d_blk_runs, runs))) return rc;
  }
  // [0]: the staged launches' error flag; [1]: the pipelined launch's block counter
  if ((rc = dev_alloc(ctx, &ctx->d_stage_err, 2))) return rc;
  CK(cudaMemset(ctx->d_stage_err, 0, 2 * sizeof(int32_t)));
  if ((rc = upload(ctx, &ctx->d_block_nbr, bnbr))) return rc;
  if (HLBG_PACK) {  // the kernels read the tables only in packed builds
    if ((rc = upload(ctx, &ctx->d_slot2site, slot2site))) return rc;
    if ((rc = upload(ctx, &ctx->d_site2slot, site2slot))) return rc;
  }
  if ((rc = upload(ctx, &ctx->d_block_xyz, ctx->h_block_xyz))) return rc;
  if ((rc = upload(ctx, &ctx->d_site_code, code))) return rc;
  if ((rc = upload(ctx, &ctx->d_block_bulk, bulk))) return rc;
  if ((rc = upload(ctx, &ctx->d_b_wall, rw))) return rc;
  if ((rc = upload(ctx, &ctx->d_b_iolet, ri))) return rc;
  if ((rc = upload(ctx, &ctx->d_b_ioid, rid))) return rc;
  if ((rc = upload(ctx, &ctx->d_flux_slot, ctx->h_flux_slot))) return rc;
  if ((rc = upload(ctx, &ctx->d_flux_gi, ctx->h_flux_gi))) return rc;
  if ((rc = upload(ctx, &ctx->d_b_type, rtype))) return rc;
  if (want_cut && (rc = upload(ctx, &ctx->d_b_cut, rcut))) return rc;
  if ((rc = upload(ctx, &ctx->d_b_links, rlinks))) return rc;
  if ((rc = upload(ctx, &ctx->d_b_normal, rnorm))) return rc;
  if ((rc = upload(ctx, &ctx->d_rec_slot, ctx->h_rec_slot))) return rc;
  {
    std::vector<int32_t> io_rec;
    for (int64_t r = 0; r < ctx->nrec; ++r)
      for (int d = 1; d < 19; ++d)
        if (((rlinks[r] >> (3 * d)) & 7u) == HLBG_LC_IOLET) {
          io_rec.push_back((int32_t)r);
          break;
        }
    ctx->n_io_rec = (int64_t)io_rec.size();
    if ((rc = upload(ctx, &ctx->d_io_rec, io_rec))) return rc;
  }
  if ((rc = upload(ctx, &ctx->d_ref2slot, ctx->h_ref2slot))) return rc;
  if ((rc = upload(ctx, &ctx->d_ps_slot, ctx->h_ps_slot))) return rc;
  if ((rc = upload(ctx, &ctx->d_ps_dir, ctx->h_ps_dir))) return rc;
  if ((rc = upload(ctx, &ctx->d_ps_q, ctx->h_ps_q))) return rc;
  return HLBG_OK;
}

constexpr int64_t kMonStage2 = 1024;
constexpr int kMonFields = 7;  // partials: mass, max |du|, min f, unstable, min rho, max rho, max |u|
constexpr int kMonResult = 8;  // the same plus the valid flag

// Buffers of the fused StabilityTester, allocated on first use.
int mon_prepare(hlbg_ctx* ctx) {
  if (ctx->d_mon_u) return HLBG_OK;
  const size_t es = ctx->prec == 0 ? sizeof(double) : sizeof(float);
  uint8_t* u = nullptr;
  int rc = dev_alloc(ctx, &u, 3 * (size_t)ctx->nslot * es);
  if (rc) return rc;
  ctx->d_mon_u = u;
  // one partial per CTA of 128 or more threads, for every launch shape: all slots,
  // or the fluid list (whose padded warps can outnumber a block's 16)
  const int64_t max_ctas = (std::max(ctx->nslot, ctx->n_warps * 32) + 127) / 128;
  if ((rc = dev_alloc(ctx, &ctx->d_mon_part, kMonFields * (size_t)max_ctas))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->d_mon_part2, kMonFields * (size_t)kMonStage2))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->d_mon_state, 1))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->d_mon_result, kMonResult))) return rc;
  CK(cudaMemsetAsync(ctx->d_mon_result, 0, kMonResult * sizeof(double), ctx->stream));  // no check yet
  CK(cudaMallocHost((void**)&ctx->h_mon_result, kMonResult * sizeof(double)));
  CK(cudaMemsetAsync(ctx->d_mon_state, 0, sizeof(int32_t), ctx->stream));
  ctx->mon_recorded = false;
  return HLBG_OK;
}

// The distributions changed outside a monitored step: the recorded velocities no
// longer belong to the state, so the next monitored step only records.
int mon_invalidate(hlbg_ctx* ctx) {
  if (ctx->d_mon_state && ctx->mon_recorded) {
    CK(cudaMemsetAsync(ctx->d_mon_state, 0, sizeof(int32_t), ctx->stream));
    ctx->mon_recorded = false;
  }
  return HLBG_OK;
}

int64_t monitored_grid(const hlbg_ctx* ctx) {
  switch (ctx->prec) {
    case 0: return monitored_grid_0(ctx->nslot, ctx->sc_variant, ctx->n_warps);
    case 1: return monitored_grid_1(ctx->nslot, ctx->sc_variant, ctx->n_warps);
    default: return monitored_grid_2(ctx->nslot, ctx->sc_variant, ctx->n_warps);
  }
}

// Monitor fields of a step's arguments (the kernel then records velocities and
// writes one partial per CTA).
void mon_args(hlbg_ctx* ctx, StepArgs& a) {
  a.mon_u = ctx->d_mon_u;
  a.mon_part = ctx->d_mon_part;
  a.mon_nparts = monitored_grid(ctx);
  a.mon_state = ctx->d_mon_state;
}

// The two reduction stages after a monitored step (steady: count the check).
int mon_reduce(hlbg_ctx* ctx, const StepArgs& a, bool steady, cudaStream_t st) {
  const int64_t n2 = std::min<int64_t>(kMonStage2, a.mon_nparts);
  SteadyArgs sa{ctx->d_steady, ctx->d_steady ? ctx->d_steady + 1 : nullptr, ctx->d_steady_n};
  switch (ctx->prec) {
    case 0: launch_mon_reduce_0(a.mon_part, a.mon_nparts, ctx->d_mon_part2, n2, ctx->d_mon_state, ctx->d_mon_result, sa, steady, st); break;
    case 1: launch_mon_reduce_1(a.mon_part, a.mon_nparts, ctx->d_mon_part2, n2, ctx->d_mon_state, ctx->d_mon_result, sa, steady, st); break;
    default: launch_mon_reduce_2(a.mon_part, a.mon_nparts, ctx->d_mon_part2, n2, ctx->d_mon_state, ctx->d_mon_result, sa, steady, st); break;
  }
  CK(cudaGetLastError());
  return HLBG_OK;
}

int run_post(hlbg_ctx* ctx, cudaStream_t st, const int32_t* slot, const int8_t* dir, const float* q,
             int64_t count) {
  if (ctx->params.wall != HLBG_WALL_BFL || count == 0) return HLBG_OK;
  PostArgs p{};
  p.f_new = ctx->f[ctx->cur ^ 1];
  p.stride = ctx->nslot;
  p.slot = slot;
  p.dir = dir;
  p.q = q;
  p.count = count;
  p.fp16_scale = ctx->fp16_scale;
  p.fp16_inv_scale = 1.0f / ctx->fp16_scale;
  return launch_post(ctx, p, st);
}

}  // namespace

namespace {

// One replay of the graph of n steps (captured on first use per step count, array
// parity and check flag), after refreshing the pinned iolet table for its steps.
int graph_steps(hlbg_ctx* ctx, int n, bool check) {
  if (ctx->n_io) {
    CK(cudaEventSynchronize(ctx->io_copied));
    for (int k = 0; k < n; ++k) {
      uint64_t t1 = ctx->t1 + k;
      double* row = ctx->h_io_tab + (size_t)k * 2 * ctx->n_io;
      int j = 0;
      for (auto* v : {&ctx->inlets, &ctx->outlets})
        for (auto& io : *v) {
          row[j] = iolet_density(ctx, io, t1 - 1);
          row[ctx->n_io + j] = iolet_umax(io, (uint64_t)(unsigned int)t1);
          ++j;
        }
    }
  }
  if (!check) {
    int rc = mon_invalidate(ctx);
    if (rc) return rc;
  }
  hlbg_ctx::GraphKey key{n, ctx->cur, check ? 1 : 0};
  auto it = ctx->graphs.find(key);
  if (it == ctx->graphs.end()) {
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = HLBG_OK;
    if (ctx->n_io) {
      cudaError_t e = cudaMemcpyAsync(ctx->d_io_tab, ctx->h_io_tab, sizeof(double) * 2 * ctx->n_io * n,
                                      cudaMemcpyHostToDevice, ctx->stream);
      if (e != cudaSuccess) rc = fail(ctx, HLBG_ERR_CUDA, cudaGetErrorString(e));
    }
    const int cur0 = ctx->cur;
    StepArgs a;
    for (int k = 0; k < n && !rc; ++k) {
      fill_args(ctx, a);
      a.iolet_rho = ctx->d_io_tab + (size_t)k * 2 * ctx->n_io;
      a.iolet_umax = a.iolet_rho + ctx->n_io;
      if (check) mon_args(ctx, a);
      rc = launch_collide(ctx, a, ctx->stream);
      if (!rc) rc = run_post(ctx, ctx->stream, ctx->d_ps_slot, ctx->d_ps_dir, ctx->d_ps_q, ctx->n_ps);
      ctx->cur ^= 1;
      if (!rc && check) rc = mon_reduce(ctx, a, true, ctx->stream);
    }
    ctx->cur = cur0;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return fail(ctx, HLBG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(ctx, HLBG_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    it = ctx->graphs.emplace(key, exec).first;
  }
  CK(cudaGraphLaunch(it->second, ctx->stream));
  if (ctx->n_io) CK(cudaEventRecord(ctx->io_copied, ctx->stream));
  ctx->cur ^= (n & 1);
  if (check) ctx->mon_checked_t = (int64_t)(ctx->t1 + n - 1);
  ctx->t1 += n;
  if (check) ctx->mon_recorded = true;
  return HLBG_OK;
}

}  // namespace

namespace {

// Iolet parameters of a context: the models must match the streamers (Nash reads
// a density, Ladd a velocity), and the warm-up start density is the smallest iolet
// density (LBM::PrepareBoundaryObjects, Code/lb/lb.hpp:127-152).
int set_iolet_params(hlbg_ctx* ctx, const hlbg_iolet* inlets, int32_t n_inlets, const hlbg_iolet* outlets,
                     int32_t n_outlets) {
  const hlbg_params* p = &ctx->params;
  for (int32_t k = 0; k < n_inlets; ++k)
    if ((p->inlet == HLBG_IOLET_NASH) != (inlets[k].model == HLBG_IOLET_COSINE))
      return fail(ctx, HLBG_ERR_INVAL, "inlet model does not match the inlet streamer");
  for (int32_t k = 0; k < n_outlets; ++k)
    if ((p->outlet == HLBG_IOLET_NASH) != (outlets[k].model == HLBG_IOLET_COSINE))
      return fail(ctx, HLBG_ERR_INVAL, "outlet model does not match the outlet streamer");
  ctx->inlets.assign(inlets, inlets + n_inlets);
  ctx->outlets.assign(outlets, outlets + n_outlets);
  double mind = 1.7976931348623157e308;
  for (auto* v : {&ctx->inlets, &ctx->outlets})
    for (auto& io : *v) {
      double dm = io.model == HLBG_IOLET_COSINE ? io.density_mean - io.density_amp : 1.0;
      mind = std::min(mind, dm);
    }
  ctx->min_density = mind;
  return HLBG_OK;
}

// Device copy of the iolets' geometry: position, normal normalised
// (InOutLet::SetNormal) and rounded to float as the Nash link reads it, radius, model.
std::vector<IoletDev> iolet_table(const hlbg_ctx* ctx) {
  std::vector<IoletDev> iod;
  for (auto* v : {&ctx->inlets, &ctx->outlets})
    for (auto& io : *v) {
      IoletDev d{};
      double mag = std::sqrt(dot3(io.normal, io.normal));
      for (int k = 0; k < 3; ++k) {
        d.pos[k] = io.position[k];
        d.n[k] = io.normal[k] / mag;
        d.nf[k] = (double)(float)d.n[k];
      }
      d.radius = io.radius;
      d.model = io.model;
      iod.push_back(d);
    }
  return iod;
}

// A staged or pipelined CTA that gave up waiting for its staged rows leaves a flag.
int check_stage_err(hlbg_ctx* ctx) {
  int32_t e = 0;
  CK(cudaMemcpy(&e, ctx->d_stage_err, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) return fail(ctx, HLBG_ERR_TIMEOUT, "a staged update gave up waiting for its copies");
  return HLBG_OK;
}

}  // namespace

namespace {
int prepare_noalloc(hlbg_ctx* ctx);  // defined beside hlbg_reduce_noalloc
}  // namespace

extern "C" {

int hlbg_set_iolets(hlbg_ctx* ctx, const hlbg_iolet* inlets, int32_t n_inlets, const hlbg_iolet* outlets,
                    int32_t n_outlets) {
  if (!ctx || (n_inlets && !inlets) || (n_outlets && !outlets)) return HLBG_ERR_INVAL;
  if (n_inlets != (int32_t)ctx->inlets.size() || n_outlets != (int32_t)ctx->outlets.size())
    return fail(ctx, HLBG_ERR_INVAL, "the geometry's iolet counts cannot change");
  // the previous step's iolet values must have been copied before they change
  CK(cudaStreamSynchronize(ctx->stream));
  int rc = set_iolet_params(ctx, inlets, n_inlets, outlets, n_outlets);
  if (rc) return rc;
  const std::vector<IoletDev> iod = iolet_table(ctx);
  if (!iod.empty())
    CK(cudaMemcpy(ctx->d_iolets, iod.data(), iod.size() * sizeof(IoletDev), cudaMemcpyHostToDevice));
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);  // captured iolet values changed
  ctx->graphs.clear();
  return HLBG_OK;
}

const char* hlbg_version(void) { return "hemelb_gb300 0.1 (sm_103a, D3Q19)"; }

const char* hlbg_last_error(const hlbg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void hlbg_destroy(hlbg_ctx* ctx) {
  if (!ctx) return;
  void* ptrs[] = {ctx->f[0],        ctx->f[1],        ctx->d_block_nbr, ctx->d_block_xyz,
                  ctx->d_site_code, ctx->d_block_bulk, ctx->d_b_wall,   ctx->d_b_iolet,
                  ctx->d_b_ioid,    ctx->d_b_type,    ctx->d_b_cut,     ctx->d_ref2slot, ctx->d_b_links,
                  ctx->d_rec_slot,  ctx->d_io_rec,
                  ctx->d_ps_slot,   ctx->d_ps_dir,    ctx->d_ps_q,      ctx->d_iolets,
                  ctx->d_io_tab,    ctx->d_stage,     ctx->d_stage_rho, ctx->d_stage_u,
                  ctx->d_list,      ctx->d_part,      ctx->d_part_bad,  ctx->d_steady,
                  ctx->d_steady_n,  ctx->d_slot2site, ctx->d_site2slot, ctx->d_mon_u,
                  ctx->d_mon_part,  ctx->d_mon_part2, ctx->d_mon_state, ctx->d_mon_result,
                  ctx->d_warp_block, ctx->d_lane_slot, ctx->d_b_normal, ctx->d_wss,
                  ctx->d_blk_fluid, ctx->d_blk_bnd, ctx->d_blk_run_off, ctx->d_blk_runs, ctx->d_pipe_desc, ctx->d_stage_err,
                  ctx->d_flux_slot, ctx->d_flux_gi, ctx->d_flux, ctx->d_halo_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
  if (ctx->d_blk_omega) cudaFree(ctx->d_blk_omega);
  if (ctx->h_io_tab) cudaFreeHost(ctx->h_io_tab);
  if (ctx->h_steady_n) cudaFreeHost(ctx->h_steady_n);
  if (ctx->h_mon_result) cudaFreeHost(ctx->h_mon_result);
  if (ctx->io_copied) cudaEventDestroy(ctx->io_copied);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int hlbg_create(const hlbg_geometry* g, const hlbg_params* p, const hlbg_iolet* inlets,
                int32_t n_inlets, const hlbg_iolet* outlets, int32_t n_outlets, hlbg_ctx** out) {
  if (!out) return HLBG_ERR_INVAL;
  *out = nullptr;
  if (!g || !p) return HLBG_ERR_INVAL;
  hlbg_ctx* ctx = new (std::nothrow) hlbg_ctx();
  if (!ctx) return HLBG_ERR_OOM;
  *out = ctx;  // returned even on failure so hlbg_last_error can explain; caller destroys
  if (g->q != 19) return fail(ctx, HLBG_ERR_INVAL, "the device path implements D3Q19 only");
  if (g->block_size != 8) return fail(ctx, HLBG_ERR_INVAL, "block_size must be 8");
  if (p->kernel != HLBG_KERNEL_LBGK && p->kernel != HLBG_KERNEL_TRT)
    return fail(ctx, HLBG_ERR_INVAL, "unknown kernel");
  if (p->wall != HLBG_WALL_SBB && p->wall != HLBG_WALL_BFL) return fail(ctx, HLBG_ERR_INVAL, "unknown wall");
  if ((p->inlet != HLBG_IOLET_NASH && p->inlet != HLBG_IOLET_LADD) ||
      (p->outlet != HLBG_IOLET_NASH && p->outlet != HLBG_IOLET_LADD))
    return fail(ctx, HLBG_ERR_INVAL, "unknown iolet streamer");
  if (p->precision < HLBG_FP64 || p->precision > HLBG_FP16)
    return fail(ctx, HLBG_ERR_INVAL, "unknown precision");
  if (!(p->tau > 0.5)) return fail(ctx, HLBG_ERR_INVAL, "tau must exceed 0.5");
  if (n_inlets < 0 || n_outlets < 0 || (n_inlets && !inlets) || (n_outlets && !outlets))
    return fail(ctx, HLBG_ERR_INVAL, "bad iolet arrays");
  ctx->params = *p;
  ctx->prec = p->precision;
  ctx->elem = p->precision == HLBG_FP64 ? 8 : (p->precision == HLBG_FP32DEV ? 4 : 2);
  int rc = set_iolet_params(ctx, inlets, n_inlets, outlets, n_outlets);
  if (rc) return rc;
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&ctx->ev0));
  CK(cudaEventCreate(&ctx->ev1));
  CK(cudaEventCreateWithFlags(&ctx->io_copied, cudaEventDisableTiming));
  CK(cudaEventRecord(ctx->io_copied, ctx->stream));
  if ((rc = prepare_noalloc(ctx))) return rc;
  if ((rc = build_layout(ctx, g))) return rc;
  // iolet constants
  ctx->n_io = (int)(ctx->inlets.size() + ctx->outlets.size());
  if ((rc = upload(ctx, &ctx->d_iolets, iolet_table(ctx)))) return rc;
  if (ctx->n_io) {
    if ((rc = dev_alloc(ctx, &ctx->d_io_tab, (size_t)kStepBatch * 2 * ctx->n_io))) return rc;
    CK(cudaMallocHost((void**)&ctx->h_io_tab, sizeof(double) * kStepBatch * 2 * ctx->n_io));
  }
  // distributions
  for (int k = 0; k < 2; ++k) {
    size_t bytes = (size_t)19 * ctx->nslot * ctx->elem;
    cudaError_t e = cudaMalloc(&ctx->f[k], bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, HLBG_ERR_OOM, "distribution arrays: " + std::string(cudaGetErrorString(e)));
    }
    ctx->dev_bytes += bytes;
    CK(cudaMemsetAsync(ctx->f[k], 0, bytes, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return HLBG_OK;
}

int64_t hlbg_site_count(const hlbg_ctx* ctx) { return ctx ? ctx->nsites : 0; }
int64_t hlbg_slot_count(const hlbg_ctx* ctx) { return ctx ? ctx->nslot : 0; }
int32_t hlbg_launches_per_step(const hlbg_ctx* ctx) {
  if (!ctx) return 0;
  return 1 + (ctx->n_io_rec > 0 ? 1 : 0) + (ctx->params.wall == HLBG_WALL_BFL && ctx->n_ps > 0 ? 1 : 0);
}
size_t hlbg_device_bytes(const hlbg_ctx* ctx) { return ctx ? ctx->dev_bytes : 0; }

int hlbg_collision_counts(const hlbg_ctx* ctx, int64_t counts[6]) {
  if (!ctx || !counts) return HLBG_ERR_INVAL;
  for (int t = 0; t < 6; ++t) counts[t] = ctx->type_count[t];
  return HLBG_OK;
}

int hlbg_site_order(const hlbg_ctx* ctx, int64_t* ref_to_slot) {
  if (!ctx || !ref_to_slot) return HLBG_ERR_INVAL;
  for (int64_t i = 0; i < ctx->nsites; ++i) ref_to_slot[i] = ctx->h_ref2slot[i];
  return HLBG_OK;
}

int hlbg_site_coords(const hlbg_ctx* ctx, int32_t* xyz) {
  if (!ctx || !xyz) return HLBG_ERR_INVAL;
  for (int64_t i = 0; i < ctx->nsites; ++i) {
    const int64_t s = ctx->h_ref2slot[i], b = s >> 9;
    const int l = ctx->h_slot2site[s];
    xyz[3 * i] = ctx->h_block_xyz[3 * b] * 8 + (l >> 6);
    xyz[3 * i + 1] = ctx->h_block_xyz[3 * b + 1] * 8 + ((l >> 3) & 7);
    xyz[3 * i + 2] = ctx->h_block_xyz[3 * b + 2] * 8 + (l & 7);
  }
  return HLBG_OK;
}

int hlbg_init_equilibrium(hlbg_ctx* ctx, double density, double vx, double vy, double vz) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx) return HLBG_ERR_INVAL;
  if (!(density > 0.0)) return fail(ctx, HLBG_ERR_INVAL, "density must be positive");
  // EquilibriumInitialCondition::SetFs (Code/lb/InitialCondition.hpp:40-52):
  // feq(rho, rho*u) with Lattice::CalculateFeq's scalar order, for every site
  InitArgs ia{};
  ia.f0 = ctx->f[0];
  ia.f1 = ctx->f[1];
  ia.stride = ctx->nslot;
  ia.nslot = ctx->nslot;
  ia.site_code = ctx->d_site_code;
  ia.block_bulk = ctx->d_block_bulk;
  ia.fp16_scale = ctx->fp16_scale;
  ia.fp16_inv_scale = 1.0f / ctx->fp16_scale;
  const double mx = density * vx, my = density * vy, mz = density * vz;
  const double density_1 = 1. / density;
  const double m2 = mx * mx + my * my + mz * mz;
  for (int i = 0; i < 19; ++i) {
    const double mde = HCX[i] * mx + HCY[i] * my + HCZ[i] * mz;
    const double w = weight_d(i);
    const double feq = w * (density - (3. / 2.) * m2 * density_1 + (9. / 2.) * density_1 * mde * mde +
                            3. * mde);
    ia.value[i] = ctx->prec == 0 ? feq : feq - w;
  }
  switch (ctx->prec) {
    case 0: launch_init_uniform_0(ia, ctx->stream); break;
    case 1: launch_init_uniform_1(ia, ctx->stream); break;
    default: launch_init_uniform_2(ia, ctx->stream); break;
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->cur = 0;
  ctx->t1 = 1;
  ctx->initialised = true;
  return HLBG_OK;
}

int hlbg_init_equilibrium_field(hlbg_ctx* ctx, const double* rho, const double* u) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx || !rho || !u) return HLBG_ERR_INVAL;
  int rc = ensure_stage(ctx);
  if (rc) return rc;
  for (int64_t first = 0; first < ctx->nsites; first += kStageSites) {
    int64_t n = std::min<int64_t>(kStageSites, ctx->nsites - first);
    CK(cudaMemcpyAsync(ctx->d_stage_rho, rho + first, sizeof(double) * n, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_stage_u, u + 3 * first, sizeof(double) * 3 * n, cudaMemcpyHostToDevice,
                       ctx->stream));
    FieldArgs fa{};
    fa.f0 = ctx->f[0];
    fa.f1 = ctx->f[1];
    fa.stride = ctx->nslot;
    fa.ref2slot = ctx->d_ref2slot;
    fa.first = first;
    fa.count = n;
    fa.rho = ctx->d_stage_rho;
    fa.u = ctx->d_stage_u;
    fa.fp16_scale = ctx->fp16_scale;
    fa.fp16_inv_scale = 1.0f / ctx->fp16_scale;
    switch (ctx->prec) {
      case 0: launch_init_field_0(fa, ctx->stream); break;
      case 1: launch_init_field_1(fa, ctx->stream); break;
      default: launch_init_field_2(fa, ctx->stream); break;
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
  }
  ctx->cur = 0;
  ctx->t1 = 1;
  ctx->initialised = true;
  return HLBG_OK;
}

int hlbg_step(hlbg_ctx* ctx, int32_t nsteps, void* cuda_stream) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx || nsteps < 0) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  cudaStream_t st = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
  StepArgs a;
  for (int done = 0; done < nsteps;) {
    int n = std::min(kStepBatch, nsteps - done);
    int rc = upload_iolet_table(ctx, n, st);
    if (rc) return rc;
    for (int k = 0; k < n; ++k) {
      fill_args(ctx, a);
      a.iolet_rho = ctx->d_io_tab + (size_t)k * 2 * ctx->n_io;
      a.iolet_umax = a.iolet_rho + ctx->n_io;
      if ((rc = launch_collide(ctx, a, st))) return rc;
      if ((rc = run_post(ctx, st, ctx->d_ps_slot, ctx->d_ps_dir, ctx->d_ps_q, ctx->n_ps))) return rc;
      ctx->cur ^= 1;  // FieldData::SwapOldAndNew
      ctx->t1++;      // SimulationState::Increment
    }
    done += n;
  }
  return HLBG_OK;
}

int hlbg_set_block_tau(hlbg_ctx* ctx, const double* tau) {
  if (!ctx || !tau) return HLBG_ERR_INVAL;
  std::vector<double> w((size_t)ctx->nb * 2);
  for (int64_t ob = 0; ob < ctx->nb; ++ob) {
    const double t = tau[ob];
    if (!(t > 0.5)) return fail(ctx, HLBG_ERR_INVAL, "every tau must exceed 0.5");
    const int64_t b = ctx->h_new_of_old[ob];
    // LbmParameters::CalcDerivedParams and TRT's second rate, per block
    w[2 * b] = -1.0 / t;
    w[2 * b + 1] = -1.0 / (0.5 + (3.0 / 16.0) / (t - 0.5));
  }
  if (!ctx->d_blk_omega) {
    int rc = dev_alloc(ctx, &ctx->d_blk_omega, w.size());
    if (rc) return rc;
  }
  CK(cudaMemcpy(ctx->d_blk_omega, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice));
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);  // captured args changed
  ctx->graphs.clear();
  return HLBG_OK;
}

int hlbg_step_graph(hlbg_ctx* ctx, int32_t nsteps) {
  // nsteps time steps as CUDA graph launches: the iolet-table copy and every
  // kernel of every step, captured once per (step count, array parity) and
  // replayed.  The host refreshes the pinned iolet table before each replay.
  if (!ctx || nsteps < 0) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  for (int done = 0; done < nsteps;) {
    const int n = std::min(kStepBatch, nsteps - done);
    int rc = graph_steps(ctx, n, false);
    if (rc) return rc;
    done += n;
  }
  return HLBG_OK;
}

int hlbg_run_to_steady(hlbg_ctx* ctx, double tol, double u_ref, int64_t max_steps, int32_t check_batch,
                       int64_t* steps_to_steady, int64_t* steps_run, double* final_rel_du) {
  // Time steps until StabilityTester's convergence test holds: after every step,
  // max over sites |u_new - u_old| / U_ref <= tol (Code/lb/StabilityTester.h:91-183),
  // evaluated on the device by the fused monitor (the check of step k is made
  // while step k + 1 collides).  Steps run in CUDA graphs of check_batch steps;
  // the host reads the device counters after each batch, so between 1 and
  // check_batch steps run past the first converged one.
  if (!ctx || !(tol > 0.0) || !(u_ref > 0.0) || max_steps < 1 || check_batch < 1 ||
      check_batch > kStepBatch)
    return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  int rc0 = mon_prepare(ctx);
  if (rc0) return rc0;
  // every call starts by recording velocities: its first check is its first step
  CK(cudaMemsetAsync(ctx->d_mon_state, 0, sizeof(int32_t), ctx->stream));
  if (!ctx->d_steady) {
    int rc = dev_alloc(ctx, &ctx->d_steady, 2);
    if (!rc) rc = dev_alloc(ctx, &ctx->d_steady_n, 3);
    if (rc) return rc;
    CK(cudaMallocHost((void**)&ctx->h_steady_n, 3 * sizeof(long long)));
  }
  const double hv[2] = {tol * u_ref, -1.0};
  const long long hn[3] = {0, -1, -1};
  CK(cudaMemcpyAsync(ctx->d_steady, hv, sizeof(hv), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_steady_n, hn, sizeof(hn), cudaMemcpyHostToDevice, ctx->stream));
  int64_t run = 0;
  int status = HLBG_ERR_TIMEOUT;
  while (run < max_steps) {
    const int n = (int)std::min<int64_t>(check_batch, max_steps - run);
    int rc = graph_steps(ctx, n, true);
    if (rc) return rc;
    run += n;
    CK(cudaMemcpyAsync(ctx->h_steady_n, ctx->d_steady_n, 3 * sizeof(long long), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_steady_n[2] >= 0) {
      status = HLBG_ERR_UNSTABLE;
      break;
    }
    if (ctx->h_steady_n[1] >= 0) {
      status = HLBG_OK;
      break;
    }
  }
  double last = 0.0;
  CK(cudaMemcpy(&last, ctx->d_steady + 1, sizeof(double), cudaMemcpyDeviceToHost));
  if (steps_to_steady) *steps_to_steady = status == HLBG_OK ? ctx->h_steady_n[1] : -1;
  if (steps_run) *steps_run = run;
  if (final_rel_du) *final_rel_du = last / u_ref;
  if (status == HLBG_ERR_UNSTABLE) return fail(ctx, status, "unstable: a distribution is not positive");
  if (status == HLBG_ERR_TIMEOUT) return fail(ctx, status, "not converged within max_steps");
  return HLBG_OK;
}

int hlbg_set_monitor_interval(hlbg_ctx* ctx, int32_t interval) {
  if (!ctx || interval < 1) return HLBG_ERR_INVAL;
  ctx->mon_interval = interval;
  return HLBG_OK;
}

int hlbg_step_monitored(hlbg_ctx* ctx, int32_t nsteps, hlbg_stats* out) {
  // nsteps time steps with the StabilityTester fused into the update.  With the
  // check interval K (hlbg_set_monitor_interval, default 1), step t checks when
  // t % K == 0 -- comparing the velocities of the state it collides with those the
  // step before recorded -- the step before a check records only, and the others
  // run the plain update.  The stats are those of the last check made.
  if (!ctx || nsteps < 1 || !out) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  int rc = mon_prepare(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->stream;
  const uint64_t K = (uint64_t)ctx->mon_interval;
  StepArgs a;
  for (int done = 0; done < nsteps;) {
    const int n = std::min(kStepBatch, nsteps - done);
    if ((rc = upload_iolet_table(ctx, n, st))) return rc;
    for (int k = 0; k < n; ++k) {
      const uint64_t t = ctx->t1;
      const bool check = t % K == 0;
      const bool record = !check && (t + 1) % K == 0;
      fill_args(ctx, a);
      a.iolet_rho = ctx->d_io_tab + (size_t)k * 2 * ctx->n_io;
      a.iolet_umax = a.iolet_rho + ctx->n_io;
      if (check || record) mon_args(ctx, a);
      // a record-only step compares nothing: the velocities on record are older
      if (record) CK(cudaMemsetAsync(ctx->d_mon_state, 0, sizeof(int32_t), st));
      if ((rc = launch_collide(ctx, a, st))) return rc;
      if ((rc = run_post(ctx, st, ctx->d_ps_slot, ctx->d_ps_dir, ctx->d_ps_q, ctx->n_ps))) return rc;
      ctx->cur ^= 1;
      ctx->t1++;
      if (check) {
        if ((rc = mon_reduce(ctx, a, false, st))) return rc;
        ctx->mon_checked_t = (int64_t)t;
      } else if (record) {
        // the next step's check is valid (any nonzero word marks the record present)
        CK(cudaMemsetAsync(ctx->d_mon_state, 1, sizeof(int32_t), st));
      }
      ctx->mon_recorded = check || record;
    }
    done += n;
  }
  CK(cudaMemcpyAsync(ctx->h_mon_result, ctx->d_mon_result, kMonResult * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const double* r = ctx->h_mon_result;
  const bool valid = r[4] != 0.0;
  out->mass = valid ? r[0] : 0.0;
  out->max_du = valid ? r[1] : 0.0;
  out->min_f = valid ? r[2] : 0.0;
  out->unstable_sites = valid ? (int64_t)r[3] : 0;
  out->time_step = valid ? ctx->mon_checked_t : -1;
  return valid && r[3] > 0.0 ? HLBG_ERR_UNSTABLE : HLBG_OK;
}

}  // extern "C"

// ---- XTR distribution checkpoints (doc/dev/file-formats/extraction.md, version 5) ----
namespace {

struct XdrOut {
  std::vector<uint8_t> b;
  void u32(uint32_t v) {
    for (int k = 3; k >= 0; --k) b.push_back((uint8_t)(v >> (8 * k)));
  }
  void u64(uint64_t v) {
    for (int k = 7; k >= 0; --k) b.push_back((uint8_t)(v >> (8 * k)));
  }
  void f64(double d) {
    uint64_t v;
    std::memcpy(&v, &d, 8);
    u64(v);
  }
  void str(const std::string& t) {  // XDR string: length, bytes, zero padding to 4
    u32((uint32_t)t.size());
    b.insert(b.end(), t.begin(), t.end());
    while (b.size() % 4) b.push_back(0);
  }
};

struct XdrIn {
  const uint8_t* p;
  size_t n, at = 0;
  bool ok = true;
  uint64_t get(int bytes) {
    if (at + bytes > n) {
      ok = false;
      return 0;
    }
    uint64_t v = 0;
    for (int k = 0; k < bytes; ++k) v = (v << 8) | p[at++];
    return v;
  }
  uint32_t u32() { return (uint32_t)get(4); }
  uint64_t u64() { return get(8); }
  double f64() {
    const uint64_t v = get(8);
    double d;
    std::memcpy(&d, &v, 8);
    return d;
  }
  std::string str() {
    const uint32_t len = u32();
    if (!ok || at + len > n) {
      ok = false;
      return std::string();
    }
    std::string t((const char*)p + at, len);
    at += (len + 3) / 4 * 4;
    return t;
  }
};

constexpr uint32_t kHemeLbMagic = 0x686c6221u, kXtrMagic = 0x78747204u, kXtrVersion = 5u;
constexpr uint32_t kOffMagic = 0x6f666604u, kOffVersion = 1u, kTypeDouble = 1u;
const char* const kDistField = "distributions";

// Main header (60 bytes) and the one field header of a distribution checkpoint
// (LocalPropertyOutput::PrepareHeader, Code/extraction/LocalPropertyOutput.cc).
std::vector<uint8_t> checkpoint_header(uint64_t nsites, double voxel, const double origin[3]) {
  XdrOut field;
  field.str(kDistField);
  field.u32(19);           // values per site
  field.u32(kTypeDouble);  // full precision
  field.u32(0);            // no offsets
  XdrOut h;
  h.u32(kHemeLbMagic);
  h.u32(kXtrMagic);
  h.u32(kXtrVersion);
  h.f64(voxel);
  for (int c = 0; c < 3; ++c) h.f64(origin ? origin[c] : 0.0);
  h.u64(nsites);
  h.u32(1);
  h.u32((uint32_t)field.b.size());
  h.b.insert(h.b.end(), field.b.begin(), field.b.end());
  return h.b;
}

std::string offset_path(const std::string& xtr) {  // io::formats::offset::ExtractionToOffset
  const size_t dot = xtr.rfind('.');
  return dot == std::string::npos ? std::string() : xtr.substr(0, dot) + ".off";
}

}  // namespace

extern "C" {

int hlbg_write_checkpoint(hlbg_ctx* ctx, const char* path, uint64_t timestep, double voxel_size,
                          const double origin[3], int32_t append) {
  // One timestep record: the step number, then per site in contiguous order its
  // grid position and its 19 distributions of the current state (the reference's
  // GetFOld), as LocalPropertyOutput::Write does for a "distributions" field.
  // The record is encoded and written in chunks of sites.
  if (!ctx || !path) return HLBG_ERR_INVAL;
  const std::string opath = offset_path(path);
  if (opath.empty()) return fail(ctx, HLBG_ERR_INVAL, "checkpoint path needs an extension");
  const int64_t n = ctx->nsites;
  std::vector<double> f((size_t)n * 19);
  std::vector<int32_t> xyz((size_t)n * 3);
  int rc = hlbg_get_f(ctx, f.data(), 0);
  if (!rc) rc = hlbg_site_coords(ctx, xyz.data());
  if (rc) return rc;
  const std::vector<uint8_t> head = checkpoint_header((uint64_t)n, voxel_size, origin);
  const uint64_t rec_len = 8 + (uint64_t)n * (12 + 19 * 8);
  FILE* fp = nullptr;
  if (append && (fp = std::fopen(path, "rb"))) {  // append to a file of the same geometry
    std::vector<uint8_t> old(head.size());
    const bool same = std::fread(old.data(), 1, old.size(), fp) == old.size() &&
                      std::memcmp(old.data() + 48, head.data() + 48, head.size() - 48) == 0;
    // hlbg_read_checkpoint finds a timestep by binary search over the records, so
    // they must stay in increasing timestep order: compare with the last record's.
    long long fsize = -1;
    uint64_t last_ts = 0;
    bool has_last = false, whole = false;
    if (same && std::fseek(fp, 0, SEEK_END) == 0 && (fsize = (long long)std::ftell(fp)) >= 0) {
      const long long body = fsize - (long long)head.size();
      whole = body >= 0 && body % (long long)rec_len == 0;
      if (whole && body > 0) {
        uint8_t b8[8];
        has_last = std::fseek(fp, (long)(fsize - (long long)rec_len), SEEK_SET) == 0 &&
                   std::fread(b8, 1, 8, fp) == 8;
        XdrIn t{b8, 8};
        last_ts = has_last ? t.u64() : 0;
        whole = has_last;
      }
    }
    std::fclose(fp);
    if (!same) return fail(ctx, HLBG_ERR_INVAL, "checkpoint file holds another geometry");
    if (!whole) return fail(ctx, HLBG_ERR_INVAL, "checkpoint length is not a whole number of timesteps");
    if (has_last && timestep <= last_ts)
      return fail(ctx, HLBG_ERR_INVAL,
                  "checkpoint timestep " + std::to_string(timestep) + " does not follow the file's last, " +
                      std::to_string(last_ts));
    fp = std::fopen(path, "ab");
    if (!fp) return fail(ctx, HLBG_ERR_INVAL, "cannot open checkpoint file");
  } else {
    append = 0;
    fp = std::fopen(path, "wb");
    if (!fp) return fail(ctx, HLBG_ERR_INVAL, "cannot create checkpoint file");
  }
  bool ok = append || std::fwrite(head.data(), 1, head.size(), fp) == head.size();
  XdrOut rec;
  rec.u64(timestep);
  constexpr int64_t kChunk = 1 << 16;  // sites per write
  for (int64_t i0 = 0; ok && i0 < n; i0 += kChunk) {
    const int64_t i1 = std::min(n, i0 + kChunk);
    rec.b.reserve(rec.b.size() + (size_t)(i1 - i0) * (12 + 19 * 8));
    for (int64_t i = i0; i < i1; ++i) {
      for (int c = 0; c < 3; ++c) rec.u32((uint32_t)xyz[3 * i + c]);
      for (int d = 0; d < 19; ++d) rec.f64(f[(size_t)i * 19 + d]);
    }
    ok = std::fwrite(rec.b.data(), 1, rec.b.size(), fp) == rec.b.size();
    rec.b.clear();
  }
  if (n == 0 && ok) ok = std::fwrite(rec.b.data(), 1, rec.b.size(), fp) == rec.b.size();
  ok = (std::fclose(fp) == 0) && ok;
  if (ok && !append) {
    // offset file: one rank, its chunk of the first timestep (LocalPropertyOutput::WriteOffsetFile)
    XdrOut off;
    off.u32(kHemeLbMagic);
    off.u32(kOffMagic);
    off.u32(kOffVersion);
    off.u32(1);  // int32 rank count
    off.u64(head.size());
    off.u64(head.size() + rec_len);
    FILE* fo = std::fopen(opath.c_str(), "wb");
    ok = fo && std::fwrite(off.b.data(), 1, off.b.size(), fo) == off.b.size();
    if (fo) ok = (std::fclose(fo) == 0) && ok;
  }
  return ok ? HLBG_OK : fail(ctx, HLBG_ERR_INVAL, "checkpoint write failed");
}

int hlbg_read_checkpoint(hlbg_ctx* ctx, const char* path, int64_t timestep, uint64_t* found) {
  // LocalDistributionInput::LoadDistribution (Code/extraction/LocalDistributionInput.cc:
  // 56-251): the header checks, the record of the requested timestep (the last one
  // if timestep < 0), each site's grid position against this geometry's contiguous
  // order, and the distributions into both time levels.  Only the header, the
  // records' timesteps and the chosen record are read.
  if (!ctx || !path) return HLBG_ERR_INVAL;
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return fail(ctx, HLBG_ERR_INVAL, "cannot open checkpoint file");
  struct Closer {
    FILE* f;
    ~Closer() { std::fclose(f); }
  } closer{fp};
  std::fseek(fp, 0, SEEK_END);
  const long long fsize = (long long)std::ftell(fp);
  std::fseek(fp, 0, SEEK_SET);
  std::vector<uint8_t> hb((size_t)std::min<long long>(std::max<long long>(fsize, 0), 4096));
  if (std::fread(hb.data(), 1, hb.size(), fp) != hb.size()) return fail(ctx, HLBG_ERR_INVAL, "checkpoint read failed");
  XdrIn in{hb.data(), hb.size()};
  if (in.u32() != kHemeLbMagic || in.u32() != kXtrMagic) return fail(ctx, HLBG_ERR_INVAL, "not an extraction file");
  if (in.u32() != kXtrVersion) return fail(ctx, HLBG_ERR_INVAL, "extraction version is not 5");
  for (int k = 0; k < 4; ++k) in.f64();  // voxel size, origin
  const uint64_t nsites = in.u64();
  const uint32_t nfields = in.u32(), fhl = in.u32();
  const size_t field_start = in.at;
  const std::string name = in.str();
  const uint32_t nelem = in.u32(), type = in.u32(), noff = in.u32();
  if (!in.ok || nfields != 1 || name != kDistField || nelem != 19 || type != kTypeDouble || noff != 0 ||
      in.at - field_start != fhl)
    return fail(ctx, HLBG_ERR_INVAL, "not a D3Q19 distribution checkpoint");
  if ((int64_t)nsites != ctx->nsites) return fail(ctx, HLBG_ERR_INVAL, "checkpoint site count differs");
  const long long head = (long long)in.at, rec = 8 + (long long)nsites * (12 + 19 * 8);
  if (fsize <= head || (fsize - head) % rec)
    return fail(ctx, HLBG_ERR_INVAL, "checkpoint length is not a whole number of timesteps");
  const long long nt = (fsize - head) / rec;
  bool io_ok = true;
  auto ts_at = [&](long long k) {
    uint8_t b8[8];
    if (std::fseek(fp, (long)(head + k * rec), SEEK_SET) != 0 || std::fread(b8, 1, 8, fp) != 8) io_ok = false;
    XdrIn t{b8, 8};
    return t.u64();
  };
  long long k = nt - 1;
  if (timestep >= 0) {  // the timesteps are increasing: binary search
    long long lo = 0, len = nt;
    while (len) {
      const long long half = len / 2, m = lo + half;
      if (ts_at(m) < (uint64_t)timestep) {
        lo = m + 1;
        len -= half + 1;
      } else {
        len = half;
      }
    }
    if (lo >= nt || ts_at(lo) != (uint64_t)timestep)
      return fail(ctx, HLBG_ERR_INVAL, io_ok ? "timestep not found in checkpoint file" : "checkpoint read failed");
    k = lo;
  }
  const uint64_t ts = ts_at(k);
  if (!io_ok) return fail(ctx, HLBG_ERR_INVAL, "checkpoint read failed");
  std::vector<int32_t> xyz((size_t)nsites * 3);
  int rc = hlbg_site_coords(ctx, xyz.data());
  if (rc) return rc;
  std::vector<double> f((size_t)nsites * 19);
  constexpr uint64_t kChunk = 1 << 16;  // sites per read
  std::vector<uint8_t> buf;
  for (uint64_t i0 = 0; i0 < nsites; i0 += kChunk) {  // the file position follows the timestep
    const uint64_t i1 = std::min<uint64_t>(nsites, i0 + kChunk);
    buf.resize((size_t)(i1 - i0) * (12 + 19 * 8));
    if (std::fread(buf.data(), 1, buf.size(), fp) != buf.size()) return fail(ctx, HLBG_ERR_INVAL, "truncated checkpoint");
    XdrIn d{buf.data(), buf.size()};
    for (uint64_t i = i0; i < i1; ++i) {
      for (int c = 0; c < 3; ++c)
        if ((int32_t)d.u32() != xyz[3 * i + c])
          return fail(ctx, HLBG_ERR_INVAL, "site " + std::to_string(i) + " of the checkpoint is not this geometry's");
      for (int q = 0; q < 19; ++q) f[i * 19 + q] = d.f64();
    }
  }
  if ((rc = hlbg_put_f(ctx, f.data(), 0)) || (rc = hlbg_put_f(ctx, f.data(), 1))) return rc;
  if (found) *found = ts;
  return HLBG_OK;
}

int hlbg_wall_shear_stress(hlbg_ctx* ctx, double* out) {
  if (!ctx || !out) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  if (!ctx->d_wss) {
    int rc = dev_alloc(ctx, &ctx->d_wss, (size_t)ctx->nsites);
    if (rc) return rc;
  }
  WssArgs wa{};
  wa.f = ctx->f[ctx->cur];
  wa.ref2slot = ctx->d_ref2slot;
  wa.site_code = ctx->d_site_code;
  wa.block_bulk = ctx->d_block_bulk;
  wa.b_wall = ctx->d_b_wall;
  wa.b_normal = ctx->d_b_normal;
  // LbmParameters::CalcDerivedParams (Code/lb/LbmParameters.h:37)
  wa.stress_param = (1.0 - 1.0 / (2.0 * ctx->params.tau)) / std::sqrt(2.0);
  wa.count = ctx->nsites;
  wa.out = ctx->d_wss;
  wa.fp16_inv_scale = 1.0f / ctx->fp16_scale;
  switch (ctx->prec) {
    case 0: launch_wss_0(wa, ctx->stream); break;
    case 1: launch_wss_1(wa, ctx->stream); break;
    default: launch_wss_2(wa, ctx->stream); break;
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, ctx->d_wss, sizeof(double) * ctx->nsites, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return HLBG_OK;
}

int hlbg_iolet_flux(hlbg_ctx* ctx, double* out, int32_t n) {
  if (!ctx || (!out && n > 0)) return HLBG_ERR_INVAL;
  const int32_t nio = (int32_t)(ctx->inlets.size() + ctx->outlets.size());
  if (n != nio) return fail(ctx, HLBG_ERR_INVAL, "flux array must hold one value per inlet and outlet");
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  const int64_t m = (int64_t)ctx->h_flux_slot.size();
  std::vector<double> per(m);
  if (m > 0) {
    if (!ctx->d_flux) {
      int rc = dev_alloc(ctx, &ctx->d_flux, (size_t)m);
      if (rc) return rc;
    }
    FluxArgs fa{};
    fa.f = ctx->f[ctx->cur];
    fa.slot = ctx->d_flux_slot;
    fa.gi = ctx->d_flux_gi;
    fa.iolets = ctx->d_iolets;
    fa.count = m;
    fa.out = ctx->d_flux;
    fa.fp16_inv_scale = 1.0f / ctx->fp16_scale;
    switch (ctx->prec) {
      case 0: launch_flux_0(fa, ctx->stream); break;
      case 1: launch_flux_1(fa, ctx->stream); break;
      default: launch_flux_2(fa, ctx->stream); break;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(per.data(), ctx->d_flux, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  for (int32_t k = 0; k < n; ++k) out[k] = 0.0;
  for (int64_t i = 0; i < m; ++i) out[ctx->h_flux_gi[i]] += per[i];  // fixed order
  return HLBG_OK;
}

int hlbg_incompressibility(hlbg_ctx* ctx, hlbg_incomp* out) {
  if (!ctx || !out) return HLBG_ERR_INVAL;
  if (!ctx->d_mon_result) return fail(ctx, HLBG_ERR_STATE, "no monitored step yet");
  CK(cudaMemcpyAsync(ctx->h_mon_result, ctx->d_mon_result, kMonResult * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const double* r = ctx->h_mon_result;
  const bool valid = r[4] != 0.0;
  out->min_density = valid ? r[5] : 0.0;
  out->max_density = valid ? r[6] : 0.0;
  out->max_velocity = valid ? r[7] : 0.0;
  // IncompressibilityChecker::GetMaxRelativeDensityDifference, REFERENCE_DENSITY = 1
  out->max_relative_density_difference = valid ? r[6] - r[5] : 0.0;
  out->time_step = valid ? ctx->mon_checked_t : -1;
  return HLBG_OK;
}

int hlbg_average_time_levels(hlbg_ctx* ctx) {
  if (!ctx) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  {
    int rc = mon_invalidate(ctx);
    if (rc) return rc;
  }
  AverageArgs aa{};
  aa.f_cur = ctx->f[ctx->cur];
  aa.f_prev = ctx->f[ctx->cur ^ 1];
  aa.nslot = ctx->nslot;
  aa.site_code = ctx->d_site_code;
  aa.block_bulk = ctx->d_block_bulk;
  aa.fp16_scale = ctx->fp16_scale;
  aa.fp16_inv_scale = 1.0f / ctx->fp16_scale;
  switch (ctx->prec) {
    case 0: launch_average_0(aa, ctx->stream); break;
    case 1: launch_average_1(aa, ctx->stream); break;
    default: launch_average_2(aa, ctx->stream); break;
  }
  CK(cudaGetLastError());
  return HLBG_OK;
}

int hlbg_autotune(hlbg_ctx* ctx, int32_t steps_per_trial, int32_t* chosen, float* best_ms) {
  // Time every launch variant of the stream-and-collide kernel on this context for
  // steps_per_trial steps (after one untimed step each) and keep the fastest.
  // Stepping advances the state, exactly as hlbg_step would.
  if (!ctx || steps_per_trial < 1) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  int best = ctx->sc_variant;
  float best_t = 1e30f;
  static const int kFp64Variants[2] = {0, 5};
  for (int k = 0; k < (ctx->prec == 0 ? 2 : kSCVariants); ++k) {
    const int v = ctx->prec == 0 ? kFp64Variants[k] : k;
    ctx->sc_variant = v;
    int rc = hlbg_step(ctx, 1, nullptr);
    if (rc) return rc;
    float ms = 0.f;
    if ((rc = hlbg_time_steps(ctx, steps_per_trial, &ms))) return rc;
    if (ms < best_t) {
      best_t = ms;
      best = v;
    }
  }
  ctx->sc_variant = best;
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
  ctx->graphs.clear();
  if (chosen) *chosen = best;
  if (best_ms) *best_ms = best_t / steps_per_trial;
  return HLBG_OK;
}

int hlbg_set_launch_variant(hlbg_ctx* ctx, int32_t variant) {
  if (!ctx || variant < 0 || variant >= kSCVariants) return HLBG_ERR_INVAL;
  ctx->sc_variant = variant;
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);  // captured launches changed
  ctx->graphs.clear();
  return HLBG_OK;
}

int hlbg_sync(hlbg_ctx* ctx) {
  if (!ctx) return HLBG_ERR_INVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  return check_stage_err(ctx);
}

int hlbg_stream_and_collide_range(hlbg_ctx* ctx, int64_t first, int64_t count) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx || first < 0 || count < 0 || first + count > ctx->nsites) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  if (count == 0) return HLBG_OK;
  int rc = ensure_list(ctx, count);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->d_list, ctx->d_ref2slot + first, sizeof(int32_t) * count,
                     cudaMemcpyDeviceToDevice, ctx->stream));
  if ((rc = upload_iolet_table(ctx, 1, ctx->stream))) return rc;
  StepArgs a;
  fill_args(ctx, a);
  a.iolet_rho = ctx->d_io_tab;
  a.iolet_umax = ctx->d_io_tab + ctx->n_io;
  a.list = ctx->d_list;
  a.list_count = count;
  if ((rc = launch_collide(ctx, a, ctx->stream))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return HLBG_OK;
}

int hlbg_post_step_range(hlbg_ctx* ctx, int64_t first, int64_t count) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx || first < 0 || count < 0 || first + count > ctx->nsites) return HLBG_ERR_INVAL;
  if (ctx->params.wall != HLBG_WALL_BFL || count == 0 || ctx->n_ps == 0) return HLBG_OK;
  // the PostStep links whose site lies in the contiguous-id range
  std::vector<uint8_t> in((size_t)ctx->nslot, 0);
  for (int64_t i = first; i < first + count; ++i) in[ctx->h_ref2slot[i]] = 1;
  std::vector<int32_t> sl;
  std::vector<int8_t> dr;
  std::vector<float> qq;
  for (int64_t k = 0; k < ctx->n_ps; ++k)
    if (in[ctx->h_ps_slot[k]]) {
      sl.push_back(ctx->h_ps_slot[k]);
      dr.push_back(ctx->h_ps_dir[k]);
      qq.push_back(ctx->h_ps_q[k]);
    }
  if (sl.empty()) return HLBG_OK;
  int32_t* ds = nullptr;
  int8_t* dd = nullptr;
  float* dq = nullptr;
  int rc = HLBG_OK;
  if (!rc) rc = upload(ctx, &ds, sl);
  if (!rc) rc = upload(ctx, &dd, dr);
  if (!rc) rc = upload(ctx, &dq, qq);
  if (!rc) rc = run_post(ctx, ctx->stream, ds, dd, dq, (int64_t)sl.size());
  cudaStreamSynchronize(ctx->stream);
  size_t freed = sl.size() * (sizeof(int32_t) + sizeof(int8_t) + sizeof(float));
  if (ds) cudaFree(ds);
  if (dd) cudaFree(dd);
  if (dq) cudaFree(dq);
  ctx->dev_bytes -= std::min(ctx->dev_bytes, freed);
  return rc;
}

int hlbg_swap(hlbg_ctx* ctx) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx) return HLBG_ERR_INVAL;
  ctx->cur ^= 1;
  ctx->t1++;
  return HLBG_OK;
}

int hlbg_set_time_step(hlbg_ctx* ctx, uint64_t t1) {
  if (!ctx || t1 < 1) return HLBG_ERR_INVAL;
  ctx->t1 = t1;
  return HLBG_OK;
}

static int gather_common(hlbg_ctx* ctx, double* out, int32_t which, bool to_host) {
  if (!ctx || !out || (which != 0 && which != 1)) return HLBG_ERR_INVAL;
  int rc = ensure_stage(ctx);
  if (rc) return rc;
  GatherArgs ga;
  fill_gather(ctx, ga);
  ga.f = ctx->f[ctx->cur ^ which];
  for (int64_t first = 0; first < ctx->nsites; first += kStageSites) {
    int64_t n = std::min<int64_t>(kStageSites, ctx->nsites - first);
    ga.first = first;
    ga.count = n;
    ga.aos = to_host ? ctx->d_stage : out + first * 19;
    switch (ctx->prec) {
      case 0: launch_gather_0(ga, ctx->stream); break;
      case 1: launch_gather_1(ga, ctx->stream); break;
      default: launch_gather_2(ga, ctx->stream); break;
    }
    CK(cudaGetLastError());
    if (to_host) {
      CK(cudaMemcpyAsync(out + first * 19, ctx->d_stage, sizeof(double) * 19 * n,
                         cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return HLBG_OK;
}

static int scatter_common(hlbg_ctx* ctx, const double* in, int32_t which, bool from_host) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx || !in || (which != 0 && which != 1)) return HLBG_ERR_INVAL;
  int rc = ensure_stage(ctx);
  if (rc) return rc;
  GatherArgs ga;
  fill_gather(ctx, ga);
  ga.f_out = ctx->f[ctx->cur ^ which];
  for (int64_t first = 0; first < ctx->nsites; first += kStageSites) {
    int64_t n = std::min<int64_t>(kStageSites, ctx->nsites - first);
    ga.first = first;
    ga.count = n;
    if (from_host) {
      CK(cudaMemcpyAsync(ctx->d_stage, in + first * 19, sizeof(double) * 19 * n,
                         cudaMemcpyHostToDevice, ctx->stream));
      ga.aos = ctx->d_stage;
    } else {
      ga.aos = const_cast<double*>(in) + first * 19;
    }
    switch (ctx->prec) {
      case 0: launch_scatter_0(ga, ctx->stream); break;
      case 1: launch_scatter_1(ga, ctx->stream); break;
      default: launch_scatter_2(ga, ctx->stream); break;
    }
    CK(cudaGetLastError());
    if (from_host) CK(cudaStreamSynchronize(ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->initialised = true;
  return HLBG_OK;
}

int hlbg_get_f(hlbg_ctx* ctx, double* host, int32_t which) { return gather_common(ctx, host, which, true); }
int hlbg_put_f(hlbg_ctx* ctx, const double* host, int32_t which) {
  return scatter_common(ctx, host, which, true);
}
int hlbg_get_f_device(hlbg_ctx* ctx, double* dev, int32_t which) {
  return gather_common(ctx, dev, which, false);
}
int hlbg_put_f_device(hlbg_ctx* ctx, const double* dev, int32_t which) {
  return scatter_common(ctx, dev, which, false);
}

int hlbg_get_macro(hlbg_ctx* ctx, double* rho, double* u) {
  if (!ctx || !rho || !u) return HLBG_ERR_INVAL;
  int rc = ensure_stage(ctx);
  if (rc) return rc;
  GatherArgs ga;
  fill_gather(ctx, ga);
  ga.f = ctx->f[ctx->cur];
  for (int64_t first = 0; first < ctx->nsites; first += kStageSites) {
    int64_t n = std::min<int64_t>(kStageSites, ctx->nsites - first);
    ga.first = first;
    ga.count = n;
    ga.rho = ctx->d_stage_rho;
    ga.u = ctx->d_stage_u;
    switch (ctx->prec) {
      case 0: launch_macro_0(ga, ctx->stream); break;
      case 1: launch_macro_1(ga, ctx->stream); break;
      default: launch_macro_2(ga, ctx->stream); break;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rho + first, ctx->d_stage_rho, sizeof(double) * n, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaMemcpyAsync(u + 3 * first, ctx->d_stage_u, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return HLBG_OK;
}

int hlbg_reduce(hlbg_ctx* ctx, hlbg_stats* out) {
  if (!ctx || !out) return HLBG_ERR_INVAL;
  const int64_t nparts = (ctx->nslot + 255) / 256;
  if (!ctx->d_part) {
    int rc = dev_alloc(ctx, &ctx->d_part, (size_t)nparts * 3);
    if (!rc) rc = dev_alloc(ctx, &ctx->d_part_bad, (size_t)nparts);
    if (rc) return rc;
  }
  MonitorArgs ma{};
  ma.f_cur = ctx->f[ctx->cur];
  ma.f_prev = ctx->f[ctx->cur ^ 1];
  ma.stride = ctx->nslot;
  ma.nslot = ctx->nslot;
  ma.site_code = ctx->d_site_code;
  ma.block_bulk = ctx->d_block_bulk;
  ma.part_mass = ctx->d_part;
  ma.part_max = ctx->d_part + nparts;
  ma.part_min = ctx->d_part + 2 * nparts;
  ma.part_bad = ctx->d_part_bad;
  ma.fp16_scale = ctx->fp16_scale;
  ma.fp16_inv_scale = 1.0f / ctx->fp16_scale;
  switch (ctx->prec) {
    case 0: launch_monitor_0(ma, 0, ctx->stream); break;
    case 1: launch_monitor_1(ma, 0, ctx->stream); break;
    default: launch_monitor_2(ma, 0, ctx->stream); break;
  }
  CK(cudaGetLastError());
  double res[3];
  unsigned long long bad = 0;
  for (int k = 0; k < 3; ++k)
    CK(cudaMemcpyAsync(&res[k], ctx->d_part + k * nparts, sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
  CK(cudaMemcpyAsync(&bad, ctx->d_part_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  out->mass = res[0];
  out->max_du = res[1];
  out->min_f = res[2];
  out->unstable_sites = (int64_t)bad;
  out->time_step = (int64_t)ctx->t1;
  return bad ? HLBG_ERR_UNSTABLE : HLBG_OK;
}

}  // extern "C"

// ---- allocation-free StabilityTester reduction --------------------------------
// Scratch of hlbg_reduce_noalloc: the per-CTA partials of k_monitor (mass, max|du|,
// min f, unstable count) for at most kNoAllocParts reduction blocks, laid out as
// four consecutive runs of kNoAllocParts values (2 MiB).  The array belongs to this
// translation unit's device module: the module, and with it the array, is placed on
// a GPU when the module loads there -- at library load with eager module loading,
// or with lazy loading (CUDA_MODULE_LOADING=LAZY, the default since CUDA 12.2) on
// the first use of the module on that device.  It then stays until the process
// exits or the device is reset.  Host code must not use the symbol as a pointer:
// the device address comes from cudaGetSymbolAddress.
static constexpr int64_t kNoAllocParts = HLBG_NOALLOC_MAX_SLOTS / 256;
static __device__ __align__(256) double g_reduce_scratch[4 * kNoAllocParts];

namespace {
// Run by hlbg_create with the context's device current.  Looking up the array's
// address is this module's first use on the device, so under lazy loading the
// 2 MiB are placed here, at context creation, not inside a later
// hlbg_reduce_noalloc call; loading the monitor kernels now keeps their lazy
// load out of that call as well.  The address is kept per context: a context
// does not outlive a reset of its device, and a context created after a reset
// looks the array up again.
int prepare_noalloc(hlbg_ctx* ctx) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_reduce_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return fail(ctx, HLBG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  }
  ctx->noalloc_scratch = static_cast<double*>(p);
  e = ctx->prec == 0 ? preload_monitor_0() : (ctx->prec == 1 ? preload_monitor_1() : preload_monitor_2());
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, HLBG_ERR_CUDA, std::string("monitor kernels: ") + cudaGetErrorString(e));
  }
  return HLBG_OK;
}
}  // namespace

extern "C" {

int hlbg_reduce_noalloc(hlbg_ctx* ctx, hlbg_stats* out) {
  if (!ctx || !out) return HLBG_ERR_INVAL;
  const int64_t nparts = (ctx->nslot + 255) / 256;
  if (nparts > kNoAllocParts)
    return fail(ctx, HLBG_ERR_INVAL,
                "hlbg_reduce_noalloc: " + std::to_string(ctx->nslot) + " slots exceed its limit of " +
                    std::to_string(HLBG_NOALLOC_MAX_SLOTS) + " (use hlbg_reduce)");
  double* scratch = ctx->noalloc_scratch;
  if (!scratch) return fail(ctx, HLBG_ERR_INVAL, "hlbg_reduce_noalloc: context has no scratch address");
  // Every partial k_monitor reads is written earlier in the same call (one per
  // CTA, then the final pass into element 0 of each run), so nothing needs clearing.
  MonitorArgs ma{};
  ma.f_cur = ctx->f[ctx->cur];
  ma.f_prev = ctx->f[ctx->cur ^ 1];
  ma.stride = ctx->nslot;
  ma.nslot = ctx->nslot;
  ma.site_code = ctx->d_site_code;
  ma.block_bulk = ctx->d_block_bulk;
  ma.part_mass = scratch;
  ma.part_max = scratch + kNoAllocParts;
  ma.part_min = scratch + 2 * kNoAllocParts;
  ma.part_bad = reinterpret_cast<unsigned long long*>(scratch + 3 * kNoAllocParts);
  ma.fp16_scale = ctx->fp16_scale;
  ma.fp16_inv_scale = 1.0f / ctx->fp16_scale;
  switch (ctx->prec) {
    case 0: launch_monitor_0(ma, 0, ctx->stream); break;
    case 1: launch_monitor_1(ma, 0, ctx->stream); break;
    default: launch_monitor_2(ma, 0, ctx->stream); break;
  }
  CK(cudaGetLastError());
  double res[3];
  unsigned long long bad = 0;
  CK(cudaMemcpyAsync(&res[0], ma.part_mass, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&res[1], ma.part_max, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&res[2], ma.part_min, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&bad, ma.part_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  out->mass = res[0];
  out->max_du = res[1];
  out->min_f = res[2];
  out->unstable_sites = (int64_t)bad;
  out->time_step = (int64_t)ctx->t1;
  return bad ? HLBG_ERR_UNSTABLE : HLBG_OK;
}

int hlbg_iolet_density(const hlbg_ctx* ctx, int32_t is_outlet, int32_t index, uint64_t t,
                       double* density) {
  if (!ctx || !density) return HLBG_ERR_INVAL;
  const auto& v = is_outlet ? ctx->outlets : ctx->inlets;
  if (index < 0 || index >= (int32_t)v.size()) return HLBG_ERR_INVAL;
  *density = iolet_density(ctx, v[index], t);
  return HLBG_OK;
}

int hlbg_time_kernels(hlbg_ctx* ctx, int32_t nsteps, float* collide_ms, float* post_ms) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  // Same work as hlbg_step, with CUDA events recorded on the context stream
  // around every launch; returns the summed device time of each kernel kind.
  if (!ctx || !collide_ms || !post_ms || nsteps < 0) return HLBG_ERR_INVAL;
  if (!ctx->initialised) return fail(ctx, HLBG_ERR_STATE, "no initial condition set");
  std::vector<cudaEvent_t> ev((size_t)4 * std::max(nsteps, 1));
  for (auto& e : ev) CK(cudaEventCreate(&e));
  cudaStream_t st = ctx->stream;
  StepArgs a;
  int rc = HLBG_OK;
  for (int k = 0; k < nsteps && !rc; ++k) {
    if ((k % kStepBatch) == 0) rc = upload_iolet_table(ctx, std::min(kStepBatch, nsteps - k), st);
    if (rc) break;
    fill_args(ctx, a);
    a.iolet_rho = ctx->d_io_tab + (size_t)(k % kStepBatch) * 2 * ctx->n_io;
    a.iolet_umax = a.iolet_rho + ctx->n_io;
    cudaEventRecord(ev[4 * k], st);
    rc = launch_collide(ctx, a, st);
    cudaEventRecord(ev[4 * k + 1], st);
    if (!rc) rc = run_post(ctx, st, ctx->d_ps_slot, ctx->d_ps_dir, ctx->d_ps_q, ctx->n_ps);
    cudaEventRecord(ev[4 * k + 2], st);
    ctx->cur ^= 1;
    ctx->t1++;
  }
  cudaError_t e = cudaStreamSynchronize(st);
  float c = 0.f, p = 0.f;
  for (int k = 0; k < nsteps && e == cudaSuccess && !rc; ++k) {
    float x = 0.f, y = 0.f;
    cudaEventElapsedTime(&x, ev[4 * k], ev[4 * k + 1]);
    cudaEventElapsedTime(&y, ev[4 * k + 1], ev[4 * k + 2]);
    c += x;
    p += y;
  }
  for (auto& ee : ev) cudaEventDestroy(ee);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(ctx, HLBG_ERR_CUDA, cudaGetErrorString(e));
  *collide_ms = c;
  *post_ms = p;
  return check_stage_err(ctx);
}

int hlbg_time_steps(hlbg_ctx* ctx, int32_t nsteps, float* ms) {
  if (ctx) {  // the distributions change outside a monitored step
    const int rc_ = mon_invalidate(ctx);
    if (rc_) return rc_;
  }
  if (!ctx || !ms) return HLBG_ERR_INVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  int rc = hlbg_step(ctx, nsteps, nullptr);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  CK(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
  return check_stage_err(ctx);
}

}  // extern "C"

// ---- multi-rank exchange on the device ----------------------------------------
extern "C" {

int hlbg_halo_offsets(hlbg_ctx* ctx, const int32_t* block, const int8_t* direction, const int16_t* site,
                      int64_t n, int64_t* out) {
  if (!ctx || n < 0 || (n && (!block || !direction || !site || !out))) return HLBG_ERR_INVAL;
  if (ctx->h_site2slot.empty()) {  // invert the in-block order once
    ctx->h_site2slot.resize(ctx->h_slot2site.size());
    for (size_t s = 0; s < ctx->h_slot2site.size(); ++s)
      ctx->h_site2slot[(s & ~(size_t)511) | ctx->h_slot2site[s]] = (uint16_t)(s & 511);
  }
  const int64_t nin = (int64_t)ctx->h_new_of_old.size();
  for (int64_t i = 0; i < n; ++i) {
    if (block[i] < 0 || block[i] >= nin || direction[i] < 0 || direction[i] >= 19 || site[i] < 0 ||
        site[i] >= 512)
      return fail(ctx, HLBG_ERR_INVAL, "halo entry " + std::to_string(i) + " out of range");
    const int64_t b = ctx->h_new_of_old[block[i]];
    const int64_t slot = b * 512 + ctx->h_site2slot[(size_t)b * 512 + site[i]];
    out[i] = fidx(slot, direction[i]);
  }
  return HLBG_OK;
}

static int halo_copy(hlbg_ctx* ctx, const int64_t* offsets, int64_t n, void* buf, int unpack) {
  if (!ctx || n < 0 || (n && (!offsets || !buf))) return HLBG_ERR_INVAL;
  if (!ctx->d_halo_err) {
    int rc = dev_alloc(ctx, &ctx->d_halo_err, 1);
    if (rc) return rc;
    CK(cudaMemsetAsync(ctx->d_halo_err, 0, sizeof(int32_t), ctx->stream));
  }
  void* fnew = ctx->f[ctx->cur ^ 1];
  const int64_t limit = (int64_t)19 * ctx->nslot;
  switch (ctx->prec) {
    case 0: launch_halo_copy_0(fnew, offsets, n, limit, buf, unpack, ctx->d_halo_err, ctx->stream); break;
    case 1: launch_halo_copy_1(fnew, offsets, n, limit, buf, unpack, ctx->d_halo_err, ctx->stream); break;
    default: launch_halo_copy_2(fnew, offsets, n, limit, buf, unpack, ctx->d_halo_err, ctx->stream); break;
  }
  CK(cudaGetLastError());
  return HLBG_OK;
}

int hlbg_halo_pack_device(hlbg_ctx* ctx, const int64_t* offsets, int64_t n, void* buf) {
  return halo_copy(ctx, offsets, n, buf, 0);
}

int hlbg_halo_unpack_device(hlbg_ctx* ctx, const int64_t* offsets, int64_t n, const void* buf) {
  return halo_copy(ctx, offsets, n, const_cast<void*>(buf), 1);
}

int hlbg_halo_check(hlbg_ctx* ctx) {
  if (!ctx) return HLBG_ERR_INVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  if (!ctx->d_halo_err) return HLBG_OK;
  int32_t e = 0;
  CK(cudaMemcpy(&e, ctx->d_halo_err, sizeof(e), cudaMemcpyDeviceToHost));
  if (!e) return HLBG_OK;
  CK(cudaMemset(ctx->d_halo_err, 0, sizeof(int32_t)));
  return fail(ctx, HLBG_ERR_INVAL, "a halo pack or unpack was given an offset outside the distributions");
}

int hlbg_storage_bytes(const hlbg_ctx* ctx) { return ctx ? (int)ctx->elem : 0; }

}  // extern "C"

