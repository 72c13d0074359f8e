// Device kernels of the GB300 lattice-Boltzmann update (D3Q19).
//
// Layout in HBM (built by the host in capi.cu, build_layout):
//   * non-empty 8^3 blocks in z-column order (2-D Morton order of the block's
//     (x, y), then z); local site index l = (x * 8 + y) * 8 + z, the reference's
//     SiteTraverser order; slot = block * 512 + j;
//   * a block that is entirely fluid keeps j = l; in every other block the fluid
//     sites are packed into slots 0 .. nf-1 in site order and the solid sites
//     follow, so the distributions of a partly fluid block fill whole 32-byte
//     sectors; slot2site / site2slot translate for those blocks;
//   * distributions block-major structure-of-arrays: for block b, direction d and
//     slot j, f[(b * 19 + d) * 512 + j]; each block's 19 x 512 values are
//     contiguous, so a site's 19 loads share one base address; two copies
//     (old / new) swapped every step (FieldData::SwapOldAndNew);
//   * block_nbr[block * 27 + (dx+1)*9 + (dy+1)*3 + (dz+1)] = neighbouring block
//     index, with kPackedBit set when that block is packed, or -1;
//   * site_code[slot] = 0 solid, 1 bulk (all 18 links fluid-fluid, no wall or
//     iolet bit), 2 + r for boundary record r;
//   * boundary records (wall / iolet masks, iolet id, collision type, cut
//     distances) for the few percent of sites next to a wall or an iolet.
//
// One thread collides one site and pushes its 19 post-collision values to the
// neighbours' slots of f_new (BulkLink, Code/lb/streamers/BulkStreamer.h:142-150),
// or, for wall and iolet links, into its own slot of the inverse direction
// (SimpleBounceBack.h:245-254, BouzidiFirdaousLallemand.h:307-334,
// NashZerothOrderPressure.h:388-421, LaddIolet.h:465-502).  The link precedence is
// StreamerTypeFactory's (Code/lb/streamers/StreamerTypeFactory.h:65-79): iolet
// first, then wall, else bulk, with the iolet/wall delegates present only for the
// collision types that carry them.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

namespace hlbg {

constexpr int Q = 19;
constexpr int kSites = 512;

// Link codes of a boundary record, 3 bits per direction (bits 3d..3d+2).
#define HLBG_LC_PUSH 0ull  // stream to the neighbour (BulkLink)
#define HLBG_LC_SKIP 1ull       // neighbour not fluid: the reference writes the rubbish site
#define HLBG_LC_BOUNCE 2ull     // SimpleBounceBack, or BFL falling back to it
#define HLBG_LC_BFL 3ull        // BFL eq. 5b interpolation
#define HLBG_LC_IOLET 4ull      // Nash or Ladd iolet link

static __constant__ int c_cx[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static __constant__ int c_cy[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
static __constant__ int c_cz[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
static __constant__ int c_inv[Q] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

// Compile-time lattice tables for fully unrolled loops (constant-folded).
struct Lat {
  __host__ __device__ static constexpr int cx(int i) {
    constexpr int t[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
    return t[i];
  }
  __host__ __device__ static constexpr int cy(int i) {
    constexpr int t[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
    return t[i];
  }
  __host__ __device__ static constexpr int cz(int i) {
    constexpr int t[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
    return t[i];
  }
  __host__ __device__ static constexpr int inv(int i) { return i == 0 ? 0 : (i & 1 ? i + 1 : i - 1); }
};
// D3Q19 weights (Code/lb/lattices/D3Q19.h:39-47), as the same double expressions.
__host__ __device__ constexpr double weight_d(int i) {
  return i == 0 ? 1.0 / 3.0 : (i < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// Per-iolet constants on the device.
struct IoletDev {
  double pos[3];
  double n[3];   // normalised normal (InOutLet::SetNormal)
  double nf[3];  // the normal rounded to float, as double (GetNormal().as<float>())
  double radius;
  int32_t model;
  int32_t pad_;
};

// Flag of a block_nbr entry whose block has its fluid sites packed (slot != site).
constexpr int32_t kPackedBit = 1 << 30;
// Flag of a fluid-list entry whose site has a boundary record (site_code >= 2).
constexpr unsigned kListBoundary = 1u << 14;
// HLBG_PACK=1 builds the packed layout (fluid sites of partly fluid blocks in the
// first slots; with HLBG_PACK_FILL=p only the blocks whose fluid fills less than
// p % of the z-rows it touches).  It moves 5-12% fewer bytes but the packed code
// path of the pushes (a flag test and a conditional slot lookup each) costs more
// than that saves, whatever the share of packed blocks (measured on the vascular
// forest), so the default is off.
#ifndef HLBG_PACK
#define HLBG_PACK 0
#endif
#ifndef HLBG_PACK_FILL
#define HLBG_PACK_FILL 101
#endif

// Order of the 512 slots of a block.  HLBG_BLOCK_ORDER=0 (default): z-rows,
// slot = (x*8 + y)*8 + z, so a 32-byte sector of FP32 values is a 1x1x8 row.  1:
// the bits of the local (x, y, z) interleaved, z fastest, a sector being a 2x2x2
// cube (FP64: 1x2x2; FP16: 2x2x4).  Cubes cut by vessel walls are fewer (sectors
// touched per fluid site 1.06 instead of 1.14 on the vascular forest), but a cube
// on an x or y face of a block is then written by two blocks that the z-column
// launch order runs far apart, so its halves leave L2 separately: measured, the
// DRAM bytes did not drop and the update was 9% slower.  Rows only split across z
// faces, between blocks that run back to back.
#ifndef HLBG_BLOCK_ORDER
#define HLBG_BLOCK_ORDER 0
#endif
#if HLBG_PACK && HLBG_BLOCK_ORDER
#error "the packed layout is built on z-row blocks (HLBG_BLOCK_ORDER=0)"
#endif
// bits 0, 1, 2 of v to bits 0, 3, 6 and back
__host__ __device__ __forceinline__ int dilate3(int v) { return (v & 1) | ((v & 2) << 2) | ((v & 4) << 4); }
__host__ __device__ __forceinline__ int undilate3(int m) { return (m & 1) | ((m >> 2) & 2) | ((m >> 4) & 4); }
// Slot of the site at local coordinates (x, y, z), each 0..7, of an unpacked block.
__host__ __device__ __forceinline__ int slot_in_block(int x, int y, int z) {
#if HLBG_BLOCK_ORDER
  return (dilate3(x) << 2) | (dilate3(y) << 1) | dilate3(z);
#else
  return (x << 6) | (y << 3) | z;
#endif
}
// Local site index (x*8 + y)*8 + z of slot j of an unpacked block, and back.
__host__ __device__ __forceinline__ int local_of_slot(int j) {
#if HLBG_BLOCK_ORDER
  return (undilate3(j >> 2) << 6) | (undilate3(j >> 1) << 3) | undilate3(j);
#else
  return j;
#endif
}
__host__ __device__ __forceinline__ int slot_of_local(int l) { return slot_in_block(l >> 6, (l >> 3) & 7, l & 7); }

struct StepArgs {
  const void* f_old;
  void* f_new;
  int64_t stride;  // elements between directions (= slot count)
  int64_t nslot;
  const int32_t* block_nbr;
  const uint16_t* slot2site;  // [nslot] local site of each slot (packed blocks)
  const uint16_t* site2slot;  // [nslot] slot of each local site (packed blocks)
  // Fused StabilityTester (monitored steps only): each site's velocity at its last
  // update, u[(block * 3 + c) * 512 + slot] (double for FP64, float otherwise); the
  // per-CTA partials [mass | max |du| | min f | unstable] with stride mon_nparts;
  // mon_state 0 while no velocity has been recorded since the state was set.
  void* mon_u;
  double* mon_part;
  int64_t mon_nparts;
  const int32_t* mon_state;
  // Fluid-list launch: warp w works on block warp_block[w] & 0x7fffffff, lane k on
  // its slot lane_slot[32 w + k] & 511 (0xffff: idle; kListBoundary set for a site
  // with a boundary record); a negative warp_block marks a warp that only writes
  // zeros into the solid slots sharing a 32-byte sector with fluid.
  const int32_t* warp_block;
  const uint16_t* lane_slot;
  int64_t n_warps;
  // Block-staged launch: per block its fluid and boundary-site bitmaps (8 words,
  // bit j = slot j), and its runs of consecutive 8-slot rows that hold fluid
  // (blk_runs[blk_run_off[b] .. blk_run_off[b+1]), start row | length << 6);
  // stage_err is set when a CTA's wait for its staged rows gives up.
  const uint64_t* blk_fluid;
  const uint64_t* blk_bnd;
  const uint32_t* blk_run_off;
  const uint16_t* blk_runs;
  const uint64_t* pipe_desc;  // pipelined launch: per block, its list warps and row span
  int64_t n_blocks;
  int32_t* stage_err;
  int32_t* pipe_ctr;  // next block of the pipelined launch (zeroed before each launch)
  const uint32_t* site_code;
  const uint8_t* block_bulk;  // 1: all 512 slots are bulk sites
  const uint32_t* b_wall;
  const uint32_t* b_iolet;
  const int32_t* b_ioid;
  const int8_t* b_type;
  const float* b_cut;  // [nrec * 18] or null
  const uint64_t* b_links;  // [nrec] 3-bit link code per direction (HLBG_LC_*)
  const int32_t* list;  // optional slot list (per-range drop-in), null = all slots
  int64_t list_count;
  const IoletDev* iolets;     // [n_in + n_out]
  const double* iolet_rho;    // [n_in + n_out] ghost density for this step (Nash)
  const double* iolet_umax;   // [n_in + n_out] peak speed for this step (Ladd)
  int32_t n_in;
  int32_t kernel;   // 0 LBGK, 1 TRT
  int32_t wall;     // 0 SBB, 1 BFL
  int32_t inlet_model, outlet_model;
  double omega, omega_minus;
  float omega_f, omega_minus_f;
  const double* blk_omega;  // optional [n_blocks * 2]: (omega+, omega-) per block (ensembles)
  float fp16_scale, fp16_inv_scale;
};

// ---- storage forms ---------------------------------------------------------
// FP64: f itself.  FP32DEV / FP16: g = f - w_d (FP16 scaled by fp16_scale).
template <int P>
struct Store;
template <>
struct Store<0> {
  using S = double;
  static __device__ __forceinline__ double load(const S* p, int64_t i, const StepArgs&) {
    return __ldg(p + i);
  }
  static __device__ __forceinline__ void store(S* p, int64_t i, double v, const StepArgs&) {
    p[i] = v;
  }
};
// Distributions of the old array are read exactly once per step.  The streaming
// hint (ld.global.cs, HLBG_STREAM_LOADS=1) was meant to keep them from displacing
// the partially written sectors of the new array in L2, but on the 187M-site
// forest it measured 6% slower than the read-only path (25.3 vs 26.9 GLUPS), so
// plain __ldg is the default.
#ifndef HLBG_STREAM_LOADS
#define HLBG_STREAM_LOADS 0
#endif
// HLBG_STREAM_STORES=1: cache-streaming stores (st.global.cs) for the new array.
#ifndef HLBG_STREAM_STORES
#define HLBG_STREAM_STORES 0
#endif
template <>
struct Store<1> {
  using S = float;
  static __device__ __forceinline__ float load(const S* p, int64_t i, const StepArgs&) {
#if HLBG_STREAM_LOADS
    return __ldcs(p + i);
#else
    return __ldg(p + i);
#endif
  }
  static __device__ __forceinline__ void store(S* p, int64_t i, float v, const StepArgs&) {
#if HLBG_STREAM_STORES
    __stcs(p + i, v);
#else
    p[i] = v;
#endif
  }
};
template <>
struct Store<2> {
  using S = __half;
  static __device__ __forceinline__ float load(const S* p, int64_t i, const StepArgs& a) {
#if HLBG_STREAM_LOADS
    return __half2float(__ldcs(p + i)) * a.fp16_inv_scale;
#else
    return __half2float(__ldg(p + i)) * a.fp16_inv_scale;
#endif
  }
  static __device__ __forceinline__ void store(S* p, int64_t i, float v, const StepArgs& a) {
    p[i] = __float2half_rn(v * a.fp16_scale);
  }
};

// Element index of (slot s, direction d) in the block-major layout.
__host__ __device__ __forceinline__ int64_t fidx(int64_t s, int d) {
  return ((s >> 9) * Q + d) * kSites + (s & (kSites - 1));
}

__device__ __forceinline__ int bit(uint32_t m, int d) { return d ? (int)((m >> (d - 1)) & 1u) : 0; }


// ---- FP64 collide in the reference's scalar evaluation order ---------------
// Lattice::CalculateDensityAndMomentum (Code/lb/lattices/Lattice.h:181-191),
// CalculateFeq (:332-355), LBGK::Collide (Code/lb/kernels/LBGK.h:56-63) and TRT
// (Code/lb/kernels/TRT.h:160-188).  This translation unit is compiled with
// --fmad=false so each operation rounds on its own.
__device__ __forceinline__ void feq64(double rho, double mx, double my, double mz, double* feq) {
  const double density_1 = 1. / rho;
  const double m2 = mx * mx + my * my + mz * mz;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const double mde = Lat::cx(i) * mx + Lat::cy(i) * my + Lat::cz(i) * mz;
    feq[i] = weight_d(i) * (rho - (3. / 2.) * m2 * density_1 + (9. / 2.) * density_1 * mde * mde +
                            3. * mde);
  }
}

__device__ __forceinline__ double feq64_one(double rho, double mx, double my, double mz, int i) {
  const double density_1 = 1. / rho;
  const double m2 = mx * mx + my * my + mz * mz;
  const double mde = c_cx[i] * mx + c_cy[i] * my + c_cz[i] * mz;
  return weight_d(i) * (rho - (3. / 2.) * m2 * density_1 + (9. / 2.) * density_1 * mde * mde +
                        3. * mde);
}

__device__ __forceinline__ void collide64(const StepArgs& a, const double* f, double& rho,
                                          double& mx, double& my, double& mz, double* fpost,
                                          double omega, double omega_minus) {
  double r = 0.0, x = 0.0, y = 0.0, z = 0.0;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    r += f[i];
    x += (double)Lat::cx(i) * f[i];
    y += (double)Lat::cy(i) * f[i];
    z += (double)Lat::cz(i) * f[i];
  }
  rho = r;
  mx = x;
  my = y;
  mz = z;
  double feq[Q];
  feq64(rho, mx, my, mz, feq);
  if (a.kernel == 0) {
#pragma unroll
    for (int i = 0; i < Q; ++i) fpost[i] = f[i] + (f[i] - feq[i]) * omega;
  } else {
    fpost[0] = f[0] + omega * (f[0] - feq[0]);
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
      const int ib = i + 1;
      const double ni = f[i] - feq[i], nb = f[ib] - feq[ib];
      const double sym = 0.5 * omega * (ni + nb);
      const double asym = 0.5 * omega_minus * (ni - nb);
      fpost[i] = f[i] + sym + asym;
      fpost[ib] = f[ib] + sym - asym;
    }
  }
}

// ---- FP32 collide on deviations g = f - w ----------------------------------
// Same model (compressible D3Q19 equilibrium, LBGK or TRT); sums are formed on
// the deviations so that FP32 keeps the small departures from rest.
__device__ __forceinline__ float weight_f(int i) {
  return i == 0 ? (float)(1.0 / 3.0) : (i < 7 ? (float)(1.0 / 18.0) : (float)(1.0 / 36.0));
}

__device__ __forceinline__ void moments_dev(const float* g, float& dr, float& mx, float& my,
                                            float& mz) {
  // pairwise grouping by direction families keeps FP32 rounding small
  dr = g[0] + ((g[1] + g[2]) + (g[3] + g[4]) + (g[5] + g[6])) +
       (((g[7] + g[8]) + (g[9] + g[10])) + ((g[11] + g[12]) + (g[13] + g[14])) +
        ((g[15] + g[16]) + (g[17] + g[18])));
  mx = (g[1] - g[2]) + ((g[7] - g[8]) + (g[9] - g[10])) + ((g[11] - g[12]) + (g[13] - g[14]));
  my = (g[3] - g[4]) + ((g[7] - g[8]) - (g[9] - g[10])) + ((g[15] - g[16]) + (g[17] - g[18]));
  mz = (g[5] - g[6]) + ((g[11] - g[12]) - (g[13] - g[14])) + ((g[15] - g[16]) - (g[17] - g[18]));
}

__device__ __forceinline__ float geq_dev(float dr, float inv_rho, float m2x15, float mx, float my,
                                         float mz, int i) {
  const float mde = Lat::cx(i) * mx + Lat::cy(i) * my + Lat::cz(i) * mz;
  return weight_f(i) * ((dr - m2x15 * inv_rho) + mde * (3.f + 4.5f * inv_rho * mde));
}

// Collide on opposite-direction pairs (i, i+1): with e = f_eq - w split into its
// even part w (A + 4.5 (c.m)^2 / rho) and odd part 3 w (c.m), the symmetric and
// antisymmetric non-equilibrium parts relax with omega+ and omega- (TRT,
// Code/lb/kernels/TRT.h:160-188); LBGK is the case omega- = omega+.
__device__ __forceinline__ void collide_dev(const StepArgs& a, const float* g, float& dr, float& mx,
                                            float& my, float& mz, float* gpost, float wp_in,
                                            float wm_in) {
  moments_dev(g, dr, mx, my, mz);
  const float inv_rho = 1.f / (1.f + dr);
  const float A = dr - 1.5f * (mx * mx + my * my + mz * mz) * inv_rho;
  const float c45 = 4.5f * inv_rho;
  const float wp = wp_in;
  const float wm = a.kernel == 0 ? wp_in : wm_in;
  gpost[0] = g[0] + wp * (g[0] - weight_f(0) * A);
#pragma unroll
  for (int i = 1; i < Q; i += 2) {
    const float mde = Lat::cx(i) * mx + Lat::cy(i) * my + Lat::cz(i) * mz;
    const float w = weight_f(i);
    const float e_sym = w * fmaf(c45 * mde, mde, A);
    const float e_asym = (3.f * w) * mde;
    const float sym = fmaf(0.5f, g[i] + g[i + 1], -e_sym);
    const float asym = fmaf(0.5f, g[i] - g[i + 1], -e_asym);
    const float t = wp * sym, u = wm * asym;
    gpost[i] = g[i] + t + u;
    gpost[i + 1] = g[i + 1] + t - u;
  }
}

// Relaxation rates of block b: per block for ensembles, else the context's.
__device__ __forceinline__ void block_rates(const StepArgs& a, int64_t b, double& wp, double& wm) {
  if (a.blk_omega) {
    wp = __ldg(a.blk_omega + 2 * b);
    wm = __ldg(a.blk_omega + 2 * b + 1);
  } else {
    wp = a.omega;
    wm = a.omega_minus;
  }
}

template <int P, class T>
__device__ __forceinline__ void collide_any(const StepArgs& a, int64_t b, const T* f, T& m0, T& mx,
                                            T& my, T& mz, T* fpost) {
  double wp, wm;
  block_rates(a, b, wp, wm);
  if constexpr (P == 0)
    collide64(a, f, m0, mx, my, mz, fpost, wp, wm);
  else
    collide_dev(a, f, m0, mx, my, mz, fpost, a.blk_omega ? (float)wp : a.omega_f,
                a.blk_omega ? (float)wm : a.omega_minus_f);
}

// ---- boundary link values ---------------------------------------------------
// FP64 form: exact reference arithmetic.
__device__ __forceinline__ double dot3d(double ax, double ay, double az, double bx, double by,
                                       double bz) {
  double s = 0.0;  // std::inner_product from RES{0}
  s = s + ax * bx;
  s = s + ay * by;
  s = s + az * bz;
  return s;
}

// NashZerothOrderPressureLink::StreamLink (NashZerothOrderPressure.h:388-421)
__device__ __forceinline__ double nash64(const IoletDev& io, double ghost_rho, double rho, double mx,
                                         double my, double mz, int unstreamed) {
  const double component = dot3d(mx, my, mz, io.nf[0], io.nf[1], io.nf[2]) / rho;
  const double gx = io.nf[0] * component * ghost_rho;
  const double gy = io.nf[1] * component * ghost_rho;
  const double gz = io.nf[2] * component * ghost_rho;
  return feq64_one(ghost_rho, gx, gy, gz, unstreamed);
}

// InOutLetParabolicVelocity::GetVelocity (InOutLetParabolicVelocity.cc:23-43) at the
// link midpoint with the step's peak speed, then LaddIoletLink's correction
// (LaddIolet.h:481-501).
__device__ __forceinline__ double ladd_correction64(const IoletDev& io, double umax, double rho,
                                                    int l_x, int l_y, int l_z, int d) {
  const double hx = (double)l_x + 0.5 * c_cx[d];
  const double hy = (double)l_y + 0.5 * c_cy[d];
  const double hz = (double)l_z + 0.5 * c_cz[d];
  const double dx = hx - io.pos[0], dy = hy - io.pos[1], dz = hz - io.pos[2];
  const double z = dot3d(dx, dy, dz, io.n[0], io.n[1], io.n[2]);
  const double rSq = (dot3d(dx, dy, dz, dx, dy, dz) - z * z) / (io.radius * io.radius);
  const double s = umax * (1. - rSq);
  double wx = io.n[0] * s, wy = io.n[1] * s, wz = io.n[2] * s;
  wx *= rho;
  wy *= rho;
  wz *= rho;
  const double dd = dot3d(wx, wy, wz, (double)c_cx[d], (double)c_cy[d], (double)c_cz[d]);
  return 2. * weight_d(d) * dd / (1.0 / 3.0);
}

// The same correction in FP32 for the FP32 / FP16 forms (their link arithmetic is
// FP32 throughout; only the iolet bookkeeping and the reductions stay FP64).
__device__ __forceinline__ float ladd_correction32(const IoletDev& io, float umax, float rho, int l_x, int l_y,
                                                   int l_z, int d) {
  const float n0 = (float)io.n[0], n1 = (float)io.n[1], n2 = (float)io.n[2];
  const float dx = ((float)l_x + 0.5f * (float)c_cx[d]) - (float)io.pos[0];
  const float dy = ((float)l_y + 0.5f * (float)c_cy[d]) - (float)io.pos[1];
  const float dz = ((float)l_z + 0.5f * (float)c_cz[d]) - (float)io.pos[2];
  const float z = dx * n0 + dy * n1 + dz * n2;
  const float rSq = (dx * dx + dy * dy + dz * dz - z * z) / (float)(io.radius * io.radius);
  const float s = umax * (1.f - rSq) * rho;
  const float dd = (n0 * (float)c_cx[d] + n1 * (float)c_cy[d] + n2 * (float)c_cz[d]) * s;
  return 6.f * weight_f(d) * dd;  // 2 w (c . u rho) / c_s^2
}

}  // namespace hlbg
