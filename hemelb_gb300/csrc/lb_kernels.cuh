// Kernel templates, instantiated per storage form in lb_fp64.cu (FP64, built
// with --fmad=false) and lb_fp32.cu (FP32 / FP16 deviation forms).
#pragma once

#include "lb_device.cuh"
#include "lb_launch.h"

#include <algorithm>
#include <atomic>
#include <type_traits>

// Launch shape of the stream-and-collide kernel (threads per CTA must divide 512;
// minimum resident CTAs per SM for the FP32 / FP16 forms and for FP64).
#ifndef HLBG_SC_THREADS
#define HLBG_SC_THREADS 128
#endif
#ifndef HLBG_SC_MINB
#define HLBG_SC_MINB 10
#endif
#ifndef HLBG_SC_MINB64
#define HLBG_SC_MINB64 2
#endif

namespace hlbg {

template <int P>
struct Calc {
  using T = float;
};
template <>
struct Calc<0> {
  using T = double;
};

// ---------------------------------------------------------------------------
// Value an iolet link writes into the site's own inverse-direction slot:
// Nash (NashZerothOrderPressure.h:388-421) or Ladd (LaddIolet.h:465-502).  Out of
// line with scalar arguments: iolet links are a fraction of a percent of links.
// m0 is the density (FP64 form) or the density deviation (FP32 / FP16 forms).
// ---------------------------------------------------------------------------
template <int P>
__device__ __noinline__ typename Calc<P>::T iolet_link_value(
    const StepArgs& a, int gi, int model, int d, typename Calc<P>::T fpost_d,
    typename Calc<P>::T m0, typename Calc<P>::T mx, typename Calc<P>::T my,
    typename Calc<P>::T mz, int gx, int gy, int gz) {
  using T = typename Calc<P>::T;
  const int un = c_inv[d];
  const IoletDev& io = a.iolets[gi];
  if (model == 0) {
    if constexpr (P == 0) {
      return nash64(io, a.iolet_rho[gi], m0, mx, my, mz, un);
    } else {
      const double grho = a.iolet_rho[gi];
      const float gdr = (float)(grho - 1.0);
      const float grho_f = (float)grho;
      const float rho = 1.f + m0;
      const float comp = (mx * (float)io.nf[0] + my * (float)io.nf[1] + mz * (float)io.nf[2]) / rho;
      const float gxv = (float)io.nf[0] * comp * grho_f;
      const float gyv = (float)io.nf[1] * comp * grho_f;
      const float gzv = (float)io.nf[2] * comp * grho_f;
      const float inv_g = 1.f / grho_f;
      const float mde = c_cx[un] * gxv + c_cy[un] * gyv + c_cz[un] * gzv;
      return weight_f(un) *
             ((gdr - 1.5f * (gxv * gxv + gyv * gyv + gzv * gzv) * inv_g) + mde * (3.f + 4.5f * inv_g * mde));
    }
  }
  if constexpr (P == 0) {
    return fpost_d - ladd_correction64(io, a.iolet_umax[gi], m0, gx, gy, gz, d);
  } else {
    return fpost_d - ladd_correction32(io, (float)a.iolet_umax[gi], 1.f + m0, gx, gy, gz, d);
  }
}

// Entry k of the 27-block table around a site's block (neighbour block index,
// kPackedBit when that block is packed, -1 when absent): served by shuffle from
// lanes 0..26 in the all-slots kernel, from the global table in the list kernel.
struct ShflBase {
  int32_t reg;
  __device__ __forceinline__ int32_t operator()(int k) const { return __shfl_sync(0xffffffffu, reg, k); }
};
struct GlobalBase {
  const int32_t* tab;
  __device__ __forceinline__ int32_t operator()(int k) const { return __ldg(tab + k); }
};

// Slot of the slot-in-block tl (slot_in_block of the target's local coordinates;
// in packed builds its local site index) in the block of table entry e (e >= 0).
__device__ __forceinline__ int64_t target_slot(const StepArgs& a, int32_t e, int tl) {
#if HLBG_PACK
  const int64_t nb = e & ~kPackedBit;
  const int ts = (e & kPackedBit) ? (int)__ldg(a.site2slot + (nb << 9) + tl) : tl;
  return (nb << 9) + ts;
#else
  return ((int64_t)e << 9) + tl;
#endif
}
// Element offset of direction D of slot-in-block tl in the block of entry e (e >= 0).
__device__ __forceinline__ int64_t target_off(const StepArgs& a, int32_t e, int D, int tl) {
#if HLBG_PACK
  const int32_t nb = e & ~kPackedBit;
  const int ts = (e & kPackedBit) ? (int)__ldg(a.site2slot + ((int64_t)nb << 9) + tl) : tl;
  return (int64_t)nb * (Q * kSites) + (D * kSites + ts);
#else
  return (int64_t)e * (Q * kSites) + (D * kSites + tl);
#endif
}
// Local site index of slot s (its block's packed flag in `packed`).
__device__ __forceinline__ int site_of_slot(const StepArgs& a, int64_t s, bool packed) {
#if HLBG_PACK
  return packed ? (int)__ldg(a.slot2site + s) : (int)(s & (kSites - 1));
#else
  return local_of_slot((int)(s & (kSites - 1)));
#endif
}

// HLBG_PUSH_FENCE=1: keep each push's lookup and store together (no hoisting of
// the next direction's loads above this store).
#ifndef HLBG_PUSH_FENCE
#define HLBG_PUSH_FENCE 0
#endif
__device__ __forceinline__ void push_fence() {
#if HLBG_PUSH_FENCE
  asm volatile("" ::: "memory");
#endif
}

// Per-link dispatch of a site next to a wall or an iolet, unrolled over the 19
// directions (StreamerTypeFactory.h:65-79: iolet first, then wall, else bulk).
template <int P, int D>
struct BoundaryAll {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S* fn, const StepArgs& a, const B& base, int64_t s,
                                             int x, int y, int z, uint32_t wm, uint32_t im,
                                             int type, int ioid, int64_t r, const T* fpost, T m0,
                                             T mx, T my, T mz, const int32_t* block_xyz) {
    constexpr int inv = Lat::inv(D);
    const int64_t own = fidx(s, 0) - (int64_t)(s & (kSites - 1));  // this block's element base
    const int l = (int)(s & (kSites - 1));  // this site's slot in its block
    constexpr int db = D > 0 ? D - 1 : 0, ib = inv > 0 ? inv - 1 : 0;  // bit of D, of its inverse
    if (D > 0 && type >= 2 && ((im >> db) & 1u)) {
      const bool is_inlet = (type == 2 || type == 4);
      const int gi = is_inlet ? ioid : a.n_in + ioid;
      const int model = is_inlet ? a.inlet_model : a.outlet_model;
      const int64_t b = s >> 9;
      const T v = iolet_link_value<P>(a, gi, model, D, fpost[D], m0, mx, my, mz,
                                      block_xyz[3 * b] * 8 + x, block_xyz[3 * b + 1] * 8 + y,
                                      block_xyz[3 * b + 2] * 8 + z);
      Store<P>::store(fn + own, inv * kSites + l, v, a);
    } else if (D > 0 && (type == 1 || type == 4 || type == 5) && ((wm >> db) & 1u)) {
      T v = fpost[D];
      if (a.wall == 1) {
        const T q = (T)a.b_cut[r * (Q - 1) + D - 1];
        if (!(((wm >> ib) & 1u) || q < (T)0.5))
          v = (fpost[D] + ((T)2.0 * q - (T)1) * fpost[inv]) / ((T)2.0 * q);
      }
      Store<P>::store(fn + own, inv * kSites + l, v, a);
    } else {
      constexpr int cx = Lat::cx(D), cy = Lat::cy(D), cz = Lat::cz(D);
      const int xx = x + cx, yy = y + cy, zz = z + cz;
      const int k = 13 + 9 * (xx >> 3) + 3 * (yy >> 3) + (zz >> 3);
      const int tl = slot_in_block(xx & 7, yy & 7, zz & 7);
      const int32_t e = base(k);
      if (e >= 0) {
        const int64_t ns = target_slot(a, e, tl);
        const uint32_t nc = a.block_bulk[ns >> 9] ? 1u : a.site_code[ns];
        if (nc != 0) Store<P>::store(fn, fidx(ns, D), fpost[D], a);
      }
    }
    BoundaryAll<P, D + 1>::run(fn, a, base, s, x, y, z, wm, im, type, ioid, r, fpost, m0, mx, my, mz,
                               block_xyz);
  }
};
template <int P>
struct BoundaryAll<P, Q> {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S*, const StepArgs&, const B&, int64_t, int, int, int,
                                             uint32_t, uint32_t, int, int, int64_t, const T*, T, T, T,
                                             T, const int32_t*) {}
};

// Push of a bulk site's post-collision value along direction D (compile-time):
// neighbour block from the 27-entry table, local index by wrap-around arithmetic.
template <int P, int D>
struct PushAll {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S* fn, const StepArgs& a, const B& base, int x, int y,
                                             int z, const T* fpost) {
    constexpr int cx = Lat::cx(D), cy = Lat::cy(D), cz = Lat::cz(D);
    const int xx = x + cx, yy = y + cy, zz = z + cz;
    const int k = 13 + 9 * (xx >> 3) + 3 * (yy >> 3) + (zz >> 3);
    const int tl = slot_in_block(xx & 7, yy & 7, zz & 7);
    Store<P>::store(fn, target_off(a, base(k), D, tl), fpost[D], a);
    PushAll<P, D + 1>::run(fn, a, base, x, y, z, fpost);
  }
};
template <int P>
struct PushAll<P, Q> {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S*, const StepArgs&, const B&, int, int, int, const T*) {}
};

// Pushes of the all-slots kernel: every lane takes part in the shuffles, only
// bulk sites store.
template <int P, int D>
struct PushBulk {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S* fn, const StepArgs& a, const B& base, int x, int y,
                                             int z, bool store, const T* fpost) {
    constexpr int cx = Lat::cx(D), cy = Lat::cy(D), cz = Lat::cz(D);
    const int xx = x + cx, yy = y + cy, zz = z + cz;
    const int k = 13 + 9 * (xx >> 3) + 3 * (yy >> 3) + (zz >> 3);
    const int tl = slot_in_block(xx & 7, yy & 7, zz & 7);
    const int32_t e = base(k);  // every lane shuffles
    if (store) Store<P>::store(fn, target_off(a, e, D, tl), fpost[D], a);
    push_fence();
    PushBulk<P, D + 1>::run(fn, a, base, x, y, z, store, fpost);
  }
};
template <int P>
struct PushBulk<P, Q> {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S*, const StepArgs&, const B&, int, int, int, bool,
                                             const T*) {}
};

// Pushes of a warp that holds at least one boundary site.  Every lane computes
// the bulk target (shuffles stay converged); a boundary lane then redirects the
// link by its precomputed code: skip (the reference's rubbish site), bounce-back
// into its own inverse slot, BFL eq. 5b, or an iolet value.
template <int P, int D>
struct PushMixed {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S* fn, const StepArgs& a, const B& base, int x, int y,
                                             int z, int j, int64_t own, bool active, bool row_fluid,
                                             uint64_t links,
                                             int64_t r, int type, int ioid, const T* fpost, T m0,
                                             T mx, T my, T mz, int64_t b,
                                             const int32_t* __restrict__ block_xyz) {
    constexpr int cx = Lat::cx(D), cy = Lat::cy(D), cz = Lat::cz(D);
    constexpr int inv = Lat::inv(D);
    const int xx = x + cx, yy = y + cy, zz = z + cz;
    const int k = 13 + 9 * (xx >> 3) + 3 * (yy >> 3) + (zz >> 3);
    const int tl = slot_in_block(xx & 7, yy & 7, zz & 7);
    const int32_t e = base(k);  // every lane shuffles
    const unsigned lc = (unsigned)((links >> (3 * D)) & 7u);
    int64_t off = 0;
    T v = fpost[D];
    bool st = true;
    if (!active) {
      // A solid slot is never written by a push nor ever read; a zero there completes
      // the 32-byte sector of slots it shares with fluid slots (sectors without any
      // receive no write at all and stay untouched).
      off = own + D * kSites + j;
      v = (T)0;
      st = row_fluid;
    } else if (lc == HLBG_LC_PUSH) {
      off = target_off(a, e, D, tl);
    } else {
      if (lc == HLBG_LC_SKIP) {
        st = false;
      } else {
        off = own + inv * kSites + j;
        if (lc == HLBG_LC_BFL) {
          const T q = (T)a.b_cut[r * (Q - 1) + D - 1];
          v = (fpost[D] + ((T)2.0 * q - (T)1) * fpost[inv]) / ((T)2.0 * q);
        }
        if (lc == HLBG_LC_IOLET) st = false;  // written by k_iolet_links
      }
    }
    if (st) Store<P>::store(fn, off, v, a);
    push_fence();
    PushMixed<P, D + 1>::run(fn, a, base, x, y, z, j, own, active, row_fluid, links, r, type, ioid,
                             fpost, m0, mx, my, mz, b, block_xyz);
  }
};
template <int P>
struct PushMixed<P, Q> {
  template <class S, class T, class B>
  static __device__ __forceinline__ void run(S*, const StepArgs&, const B&, int, int, int, int,
                                             int64_t, bool, bool, uint64_t, int64_t, int, int,
                                             const T*, T, T, T, T, int64_t, const int32_t*) {}
};

// StabilityTester::PostSendToParent (Code/lb/StabilityTester.h:91-149) and
// ComputeRelativeDifference (:160-183) plus total mass: one slot per thread, one
// partial per CTA, reduced by k_monitor_final in a fixed order (deterministic).
// The fused monitor also tracks IncompressibilityChecker's quantities
// (Code/lb/IncompressibilityChecker.hpp:157-199): smallest and largest density and
// largest velocity magnitude over the sites.
struct MonAcc {
  double mass, maxdu, minf;
  unsigned long long bad;
  double rmin, rmax, umax;
};

__device__ __forceinline__ MonAcc mon_neutral() {
  return MonAcc{0.0, 0.0, 1.0e300, 0ull, 1.0e300, -1.0e300, 0.0};
}

__device__ __forceinline__ void mon_combine(MonAcc& a, const MonAcc& b) {
  a.mass += b.mass;
  if (!(b.maxdu <= a.maxdu)) a.maxdu = b.maxdu;  // NaN-propagating max
  a.minf = fmin(a.minf, b.minf);
  a.bad += b.bad;
  a.rmin = fmin(a.rmin, b.rmin);
  a.rmax = fmax(a.rmax, b.rmax);
  if (!(b.umax <= a.umax)) a.umax = b.umax;
}

__device__ __forceinline__ MonAcc mon_shfl(const MonAcc& v, int off) {
  MonAcc o;
  o.mass = __shfl_down_sync(0xffffffffu, v.mass, off);
  o.maxdu = __shfl_down_sync(0xffffffffu, v.maxdu, off);
  o.minf = __shfl_down_sync(0xffffffffu, v.minf, off);
  o.bad = __shfl_down_sync(0xffffffffu, v.bad, off);
  o.rmin = __shfl_down_sync(0xffffffffu, v.rmin, off);
  o.rmax = __shfl_down_sync(0xffffffffu, v.rmax, off);
  o.umax = __shfl_down_sync(0xffffffffu, v.umax, off);
  return o;
}

// CTA-wide reduction (up to 1024 threads) in a fixed order; result valid in thread 0.
__device__ __forceinline__ MonAcc mon_block(MonAcc v) {
  __shared__ MonAcc sh[32];
  for (int off = 16; off > 0; off >>= 1) mon_combine(v, mon_shfl(v, off));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sh[lane] : mon_neutral();
    for (int off = 16; off > 0; off >>= 1) mon_combine(v, mon_shfl(v, off));
  }
  return v;
}

// The FP32 forms accumulate their monitor values in FP32 and integers up to the
// CTA's partial (min / max are exact in any precision; the mass is a count plus
// the sum of the density deviations, which are small); only the second reduction
// stage works in FP64: GB300's FP64 rate would otherwise make every monitored CTA
// an FP64 workload.
struct MonAccF {
  float dm, maxdu, minf, dmin, dmax, umax;  // dm: sum of rho - 1; dmin/dmax: of rho - 1;
  unsigned count, bad;                      // maxdu, umax: squared (see mon_site)
};
__device__ __forceinline__ MonAccF mon_neutral_f() {
  return MonAccF{0.f, 0.f, 1.0e30f, 1.0e30f, -1.0e30f, 0.f, 0u, 0u};
}
__device__ __forceinline__ void mon_combine_f(MonAccF& a, const MonAccF& b) {
  a.dm += b.dm;
  if (!(b.maxdu <= a.maxdu)) a.maxdu = b.maxdu;
  a.minf = fminf(a.minf, b.minf);
  a.dmin = fminf(a.dmin, b.dmin);
  a.dmax = fmaxf(a.dmax, b.dmax);
  if (!(b.umax <= a.umax)) a.umax = b.umax;
  a.count += b.count;
  a.bad += b.bad;
}
// CTA-wide, in FP32 and integers throughout (a fixed order); valid in thread 0.
__device__ __forceinline__ MonAccF mon_shfl_f(const MonAccF& v, int off) {
  MonAccF o;
  o.dm = __shfl_down_sync(0xffffffffu, v.dm, off);
  o.maxdu = __shfl_down_sync(0xffffffffu, v.maxdu, off);
  o.minf = __shfl_down_sync(0xffffffffu, v.minf, off);
  o.dmin = __shfl_down_sync(0xffffffffu, v.dmin, off);
  o.dmax = __shfl_down_sync(0xffffffffu, v.dmax, off);
  o.umax = __shfl_down_sync(0xffffffffu, v.umax, off);
  o.count = __shfl_down_sync(0xffffffffu, v.count, off);
  o.bad = __shfl_down_sync(0xffffffffu, v.bad, off);
  return o;
}
__device__ __forceinline__ MonAccF mon_block_f(MonAccF v) {
  __shared__ MonAccF sh[32];
  for (int off = 16; off > 0; off >>= 1) mon_combine_f(v, mon_shfl_f(v, off));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) mon_combine_f(v, sh[k]);
  }
  return v;
}

// The velocity recorded at a site's last update, loaded before the site's
// distributions are used so that its latency overlaps theirs.
template <int P>
struct MonOld {
  using U = typename std::conditional<P == 0, double, float>::type;
  U x = 0, y = 0, z = 0;
  __device__ __forceinline__ void load(const StepArgs& a, int64_t s, bool want) {
    if (!want) return;
    const int64_t ui = (s >> 9) * (3 * kSites) + (s & (kSites - 1));
    const U* u = static_cast<const U*>(a.mon_u);
    x = u[ui];
    y = u[ui + kSites];
    z = u[ui + 2 * kSites];
  }
};

// Fused StabilityTester for one fluid site of a monitored step
// (Code/lb/StabilityTester.h:91-183): the velocity of the state being collided,
// m / rho with the moments of the collision (the reference's
// CalculateDensityAndMomentum), against the one recorded when this site was last
// updated; f > 0 over all directions; the density for the mass.  The new velocity
// is recorded for the next step.
template <int P>
__device__ __forceinline__ void mon_site(const StepArgs& a, int64_t s, const double* f, double m0, double mx,
                                         double my, double mz, MonAcc& acc, bool check, const MonOld<P>& uo) {
  // FP64 form: the reference's arithmetic (m / rho, |du| by inner product)
  const int64_t ui = (s >> 9) * (3 * kSites) + (s & (kSites - 1));
  double* u = static_cast<double*>(a.mon_u);
  const double ux = mx / m0, uy = my / m0, uz = mz / m0;
  if (check) {
    const double dx = ux - uo.x, dy = uy - uo.y, dz = uz - uo.z;
    const double du = sqrt(dot3d(dx, dy, dz, dx, dy, dz));
    if (!(du <= acc.maxdu)) acc.maxdu = du;
    acc.mass += m0;
    acc.rmin = fmin(acc.rmin, m0);
    acc.rmax = fmax(acc.rmax, m0);
    const double um = sqrt(dot3d(ux, uy, uz, ux, uy, uz));
    if (!(um <= acc.umax)) acc.umax = um;
    bool bad = false;
    double mn = f[0];
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      bad |= !(f[d] > 0.0);
      mn = fmin(mn, f[d]);
    }
    acc.minf = fmin(acc.minf, mn);
    acc.bad += bad ? 1ull : 0ull;
  }
  u[ui] = ux;
  u[ui + kSites] = uy;
  u[ui + 2 * kSites] = uz;
}

template <int P>
__device__ __forceinline__ void mon_site(const StepArgs& a, int64_t s, const float* f, float m0, float mx,
                                         float my, float mz, MonAccF& acc, bool check, const MonOld<P>& uo) {
  // deviation forms: m0 = rho - 1
  const int64_t ui = (s >> 9) * (3 * kSites) + (s & (kSites - 1));
  float* u = static_cast<float*>(a.mon_u);
  const float ir = 1.f / (1.f + m0);
  const float ux = mx * ir, uy = my * ir, uz = mz * ir;
  if (check) {
    // |du| and |u| are kept squared until the CTA's partial is written (the square
    // root is monotonic, so the maximum is the same)
    const float dx = ux - uo.x, dy = uy - uo.y, dz = uz - uo.z;
    const float du2 = dx * dx + dy * dy + dz * dz;
    if (!(du2 <= acc.maxdu)) acc.maxdu = du2;
    acc.dm += m0;
    acc.dmin = fminf(acc.dmin, m0);
    acc.dmax = fmaxf(acc.dmax, m0);
    const float um2 = ux * ux + uy * uy + uz * uz;
    if (!(um2 <= acc.umax)) acc.umax = um2;
    float mn = 1.0e30f;
#pragma unroll
    for (int d = 0; d < Q; ++d) mn = fminf(mn, f[d] + weight_f(d));
    // some f <= 0, or a NaN among them (which fminf skips but the density sum keeps)
    const bool bad = !(mn > 0.f) || m0 != m0;
    acc.minf = fminf(acc.minf, mn);
    acc.bad += bad ? 1u : 0u;
    acc.count += 1u;
  }
  u[ui] = ux;
  u[ui + kSites] = uy;
  u[ui + 2 * kSites] = uz;
}

template <int P>
using MonAccT = typename std::conditional<P == 0, MonAcc, MonAccF>::type;
template <int P>
__device__ __forceinline__ MonAccT<P> mon_neutral_t() {
  if constexpr (P == 0) return mon_neutral(); else return mon_neutral_f();
}
// One CTA's monitor partial: FP64 form as 7 doubles [mass | max |du| | min f |
// unstable | min rho | max rho | max |u|], stride mon_nparts; FP32 forms as 8
// 32-bit words [sum (rho-1) | max |du| | min f | min (rho-1) | max (rho-1) | max |u|
// | count | unstable] in the same buffer, converted to FP64 by the second stage.
template <int P>
__device__ __forceinline__ void mon_write_partial(const StepArgs& a, const MonAccT<P>& acc) {
  const int64_t n = a.mon_nparts;
  if constexpr (P == 0) {
    const MonAcc r = mon_block(acc);
    if (threadIdx.x == 0) {
      a.mon_part[blockIdx.x] = r.mass;
      a.mon_part[n + blockIdx.x] = r.maxdu;
      a.mon_part[2 * n + blockIdx.x] = r.minf;
      a.mon_part[3 * n + blockIdx.x] = (double)r.bad;
      a.mon_part[4 * n + blockIdx.x] = r.rmin;
      a.mon_part[5 * n + blockIdx.x] = r.rmax;
      a.mon_part[6 * n + blockIdx.x] = r.umax;
    }
  } else {
    const MonAccF r = mon_block_f(acc);
    if (threadIdx.x == 0) {
      float* p = reinterpret_cast<float*>(a.mon_part);
      p[blockIdx.x] = r.dm;
      p[n + blockIdx.x] = sqrtf(r.maxdu);
      p[2 * n + blockIdx.x] = r.minf;
      p[3 * n + blockIdx.x] = r.dmin;
      p[4 * n + blockIdx.x] = r.dmax;
      p[5 * n + blockIdx.x] = sqrtf(r.umax);
      p[6 * n + blockIdx.x] = __uint_as_float(r.count);
      p[7 * n + blockIdx.x] = __uint_as_float(r.bad);
    }
  }
}

// ---------------------------------------------------------------------------
// One site: collide, then push along the 19 links.
// ---------------------------------------------------------------------------
template <int P, class B>
__device__ __forceinline__ void site_update(const StepArgs& a, const B& base,
                                            const int32_t* __restrict__ tab, int64_t s,
                                            uint32_t code, const int32_t* __restrict__ block_xyz) {
  using St = Store<P>;
  using S = typename St::S;
  using T = typename Calc<P>::T;
  const int j = (int)(s & (kSites - 1));
  const int64_t b = s >> 9;
  const int l = site_of_slot(a, s, (__ldg(tab + 13) & kPackedBit) != 0);
  const S* fo = static_cast<const S*>(a.f_old) + b * (Q * kSites) + j;
  S* fn = static_cast<S*>(a.f_new);
  T f[Q], fpost[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) f[i] = St::load(fo, i * kSites, a);
  T m0, mx, my, mz;
  collide_any<P>(a, b, f, m0, mx, my, mz, fpost);
  if (code == 1) {
    PushAll<P, 0>::run(fn, a, base, l >> 6, (l >> 3) & 7, l & 7, fpost);
    return;
  }
  const int64_t r = code - 2;
  BoundaryAll<P, 0>::run(fn, a, base, s, l >> 6, (l >> 3) & 7, l & 7, a.b_wall[r], a.b_iolet[r],
                         (int)a.b_type[r], a.b_ioid[r], r, fpost, m0, mx, my, mz, block_xyz);
}

// One warp's 32 slots of one block (a warp never spans two blocks).  Lanes 0..26
// hold the block's neighbour table and serve it to the bulk pushes by shuffle, so
// every lane of a warp with any fluid site stays converged through the pushes.
template <int P, bool MON>
__device__ __forceinline__ void collide_slot(const StepArgs& a, int64_t s,
                                             const int32_t* __restrict__ block_xyz, MonAccT<P>& acc,
                                             bool check) {
  using St = Store<P>;
  using S = typename St::S;
  using T = typename Calc<P>::T;
  const int64_t b = s >> 9;
  const int lane = threadIdx.x & 31;
  const int32_t* tab = a.block_nbr + b * 27;
  const int32_t tabreg = lane < 27 ? __ldg(tab + lane) : 0;
  const uint32_t code = a.block_bulk[b] ? 1u : a.site_code[s];
  const unsigned fluid_lanes = __ballot_sync(0xffffffffu, code != 0);
  if (fluid_lanes == 0) return;
  // lanes 8r..8r+7 hold eight consecutive slots (a 32-byte sector of each direction in FP32)
  const bool row_fluid = ((fluid_lanes >> (lane & ~7)) & 0xFFu) != 0;
  const int j = (int)(s & (kSites - 1));
  const bool packed = (__shfl_sync(0xffffffffu, tabreg, 13) & kPackedBit) != 0;
  const int l = site_of_slot(a, s, packed);
  const S* fo = static_cast<const S*>(a.f_old) + b * (Q * kSites) + j;
  S* fn = static_cast<S*>(a.f_new);
  MonOld<P> uo;
  if constexpr (MON) uo.load(a, s, check && code != 0);
  T f[Q], fpost[Q];
  if (code != 0) {
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = St::load(fo, i * kSites, a);
  } else {
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = (T)(P == 0 ? weight_d(i) : 0.0);
  }
  T m0, mx, my, mz;
  collide_any<P>(a, b, f, m0, mx, my, mz, fpost);
  if constexpr (MON) {
    if (code != 0) mon_site<P>(a, s, f, m0, mx, my, mz, acc, check, uo);
  }
  const int x = l >> 6, y = (l >> 3) & 7, z = l & 7;
  const bool bnd = code >= 2;
  if (__ballot_sync(0xffffffffu, bnd) == 0) {
    PushBulk<P, 0>::run(fn, a, ShflBase{tabreg}, x, y, z, code == 1, fpost);
  } else {
    const int64_t r = bnd ? (int64_t)code - 2 : 0;
    const uint64_t links = bnd ? a.b_links[r] : 0ull;
    const int type = bnd ? (int)a.b_type[r] : 0;
    const int ioid = bnd ? a.b_ioid[r] : 0;
    PushMixed<P, 0>::run(fn, a, ShflBase{tabreg}, x, y, z, j, b * (Q * kSites), code != 0, row_fluid,
                         links, r, type, ioid, fpost, m0, mx, my, mz, b, block_xyz);
  }
}

// One warp of the fluid list: 32 fluid sites of one block (or the zero-fill of its
// solid slots that share sectors with fluid), so no lane is spent on a solid slot.
// Collide one lane's site (code 0: an idle lane, computed on the rest state and
// stored nowhere) and push its post-collision values, on the warp's bulk path when
// no lane has a boundary record.  tabreg: the block's neighbour table in lanes
// 0..26.  Every lane of the warp must take part (shuffles, ballot).
template <int P, bool MON>
__device__ __forceinline__ void collide_and_push(const StepArgs& a, int64_t b, int j, int64_t s, int l,
                                                 uint32_t code, int32_t tabreg, typename Calc<P>::T* f,
                                                 const int32_t* __restrict__ block_xyz, MonAccT<P>& acc,
                                                 bool check, const MonOld<P>& uo) {
  using S = typename Store<P>::S;
  using T = typename Calc<P>::T;
  S* fn = static_cast<S*>(a.f_new);
  T fpost[Q];
  T m0, mx, my, mz;
  collide_any<P>(a, b, f, m0, mx, my, mz, fpost);
  if constexpr (MON) {
    if (code != 0) mon_site<P>(a, s, f, m0, mx, my, mz, acc, check, uo);
  }
  const int x = l >> 6, y = (l >> 3) & 7, z = l & 7;
  const bool bnd = code >= 2;
  if (__ballot_sync(0xffffffffu, bnd) == 0) {
    PushBulk<P, 0>::run(fn, a, ShflBase{tabreg}, x, y, z, code == 1, fpost);
  } else {
    const int64_t r = bnd ? (int64_t)code - 2 : 0;
    const uint64_t links = bnd ? a.b_links[r] : 0ull;
    const int type = bnd ? (int)a.b_type[r] : 0;
    const int ioid = bnd ? a.b_ioid[r] : 0;
    PushMixed<P, 0>::run(fn, a, ShflBase{tabreg}, x, y, z, j, b * (Q * kSites), code != 0, false, links,
                         r, type, ioid, fpost, m0, mx, my, mz, b, block_xyz);
  }
}

// The unit's list entries (block e, this lane's slot js) are loaded by the caller.
template <int P, bool MON>
__device__ __forceinline__ void collide_listed_unit(const StepArgs& a, int32_t e, unsigned js,
                                                    const int32_t* __restrict__ block_xyz, MonAccT<P>& acc,
                                                    bool check) {
  using St = Store<P>;
  using S = typename St::S;
  using T = typename Calc<P>::T;
  const int lane = threadIdx.x & 31;
  const int64_t b = e & 0x7fffffff;
  const bool on = js != 0xffffu;
  const int j = on ? (int)(js & (kSites - 1)) : 0;
  const int64_t s = b * kSites + j;
  S* fn = static_cast<S*>(a.f_new);
  if (e < 0) {  // zero-fill warp: complete the sectors its slots share with fluid
    if (on) {
#pragma unroll
      for (int d = 0; d < Q; ++d) St::store(fn, fidx(s, d), (T)0, a);
    }
    return;
  }
  const int32_t* tab = a.block_nbr + b * 27;
  const int32_t tabreg = lane < 27 ? __ldg(tab + lane) : 0;
  // every listed lane is a fluid site: its loads need not wait for its code, and
  // only the boundary sites (flagged in the list) read one
  const uint32_t code = on ? ((js & kListBoundary) ? a.site_code[s] : 1u) : 0u;
  const bool packed = (__shfl_sync(0xffffffffu, tabreg, 13) & kPackedBit) != 0;
  const int l = on ? site_of_slot(a, s, packed) : 0;
  const S* fo = static_cast<const S*>(a.f_old) + b * (Q * kSites) + j;
  MonOld<P> uo;
  if constexpr (MON) uo.load(a, s, check && on);
  T f[Q];
  if (on) {
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = St::load(fo, i * kSites, a);
  } else {
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = (T)(P == 0 ? weight_d(i) : 0.0);
  }
  collide_and_push<P, MON>(a, b, j, s, l, code, tabreg, f, block_xyz, acc, check, uo);
}

template <int P, bool MON>
__device__ __forceinline__ void collide_listed_warp(const StepArgs& a, int64_t w,
                                                    const int32_t* __restrict__ block_xyz, MonAccT<P>& acc,
                                                    bool check) {
  if (w >= a.n_warps) return;  // whole warp
  collide_listed_unit<P, MON>(a, __ldg(a.warp_block + w), __ldg(a.lane_slot + w * 32 + (threadIdx.x & 31)),
                              block_xyz, acc, check);
}

template <int P, int THREADS, int MINB, bool MON>
__global__ void __launch_bounds__(THREADS, MINB) k_stream_collide_listed(StepArgs a, const int32_t* block_xyz) {
  MonAccT<P> acc = mon_neutral_t<P>();
  bool check = false;
  if constexpr (MON) check = *a.mon_state != 0;
  collide_listed_warp<P, MON>(a, ((int64_t)blockIdx.x * THREADS + threadIdx.x) >> 5, block_xyz, acc, check);
  if constexpr (MON) mon_write_partial<P>(a, acc);
}

// ---------------------------------------------------------------------------
// Block-staged launch (FP32 / FP16 storage): one CTA per 8^3 block.  Its rows of
// the old distributions that hold fluid (whole 8-slot rows, every direction) come
// into shared memory by bulk asynchronous copies (cp.async.bulk, completion counted
// on an mbarrier), so a CTA has its whole block in flight at once and no lane waits
// on a list entry; the CTA then collides its fluid sites from shared memory in
// compacted warps (the k-th thread takes the k-th fluid site of the block), pushes
// as the other launches do, and zero-fills the solid slots of its fluid rows.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Position of the n-th (from 0) set bit of w (n < popc(w)), by halving.
__device__ __forceinline__ int select32(uint32_t w, int n) {
  int pos = 0, c;
  c = __popc(w & 0xffffu);
  if (n >= c) { n -= c; pos += 16; w >>= 16; }
  c = __popc(w & 0xffu);
  if (n >= c) { n -= c; pos += 8; w >>= 8; }
  c = __popc(w & 0xfu);
  if (n >= c) { n -= c; pos += 4; w >>= 4; }
  c = __popc(w & 0x3u);
  if (n >= c) { n -= c; pos += 2; w >>= 2; }
  if (n >= (int)(w & 1u)) pos += 1;
  return pos;
}

// Wait for phase `parity` of the mbarrier at shared address bar; false after
// kStageWaitLimit polls (each try_wait may suspend the thread for a while).
constexpr int64_t kStageWaitLimit = 1ll << 24;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int64_t it = 0; it < kStageWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <int P, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_stream_collide_block(StepArgs a, const int32_t* block_xyz) {
  static_assert(P != 0, "the staged block holds FP32 or FP16 values");
  using S = typename Store<P>::S;
  using T = typename Calc<P>::T;
  extern __shared__ __align__(128) unsigned char stage_raw[];
  S* stage = reinterpret_cast<S*>(stage_raw);  // [Q][kSites]
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t wfl[16], wbd[16], wpre[17];
  __shared__ uint32_t stage_bytes;
  const int64_t b = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31;
  const uint32_t bar = smem_u32(&mbar);
  const uint32_t r0 = __ldg(a.blk_run_off + b), r1 = __ldg(a.blk_run_off + b + 1);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    uint32_t bytes = 0;
    for (uint32_t r = r0; r < r1; ++r) bytes += (uint32_t)(__ldg(a.blk_runs + r) >> 6) * 8u * (uint32_t)sizeof(S);
    stage_bytes = bytes * Q;
  }
  if (tid < 16) {
    wfl[tid] = __ldg(reinterpret_cast<const uint32_t*>(a.blk_fluid + b * 8) + tid);
    wbd[tid] = __ldg(reinterpret_cast<const uint32_t*>(a.blk_bnd + b * 8) + tid);
  }
  __syncthreads();
  if (tid == 0)
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(stage_bytes)
                 : "memory");
  __syncthreads();
  // the copies: (run, direction) pairs over the threads; sizes and both addresses
  // are multiples of 16 bytes (rows of 8 values of 2 or 4 bytes)
  const uint32_t ncopy = (r1 - r0) * Q;
  const char* src0 = static_cast<const char*>(a.f_old) + (size_t)b * (Q * kSites) * sizeof(S);
  const uint32_t dst0 = smem_u32(stage);
  for (uint32_t k = tid; k < ncopy; k += THREADS) {
    const uint32_t run = __ldg(a.blk_runs + r0 + k / Q), d = k % Q;
    const uint32_t off = (d * kSites + (run & 63u) * 8u) * (uint32_t)sizeof(S);
    const uint32_t size = (run >> 6) * 8u * (uint32_t)sizeof(S);
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst0 + off),
        "l"(src0 + off), "r"(size), "r"(bar)
        : "memory");
  }
  const int32_t tabreg = lane < 27 ? __ldg(a.block_nbr + b * 27 + lane) : 0;
  if (tid == 0) {
    uint32_t acc = 0;
    for (int k = 0; k < 16; ++k) {
      wpre[k] = acc;
      acc += __popc(wfl[k]);
    }
    wpre[16] = acc;
  }
  const bool landed = mbar_wait(bar, 0);
  if (!__syncthreads_and(landed)) {  // every copy this CTA issued has to land before it may exit
    if (tid == 0) atomicExch(a.stage_err, 1);
    mbar_wait(bar, 0);
    return;
  }
  const int nf = (int)wpre[16];
  MonAccT<P> acc = mon_neutral_t<P>();  // unused: staged steps are not monitored
  const MonOld<P> uo;
  for (int base = tid & ~31; base < nf; base += THREADS) {  // warp-uniform trips
    const int t = base + lane;
    const bool on = t < nf;
    int j = 0;
    if (on) {
      int k = 0;  // the word holding the t-th fluid slot
#pragma unroll
      for (int h = 8; h > 0; h >>= 1)
        if ((int)wpre[k + h] <= t) k += h;
      j = k * 32 + select32(wfl[k], t - (int)wpre[k]);
    }
    const int64_t s = b * kSites + j;
    const bool bnd = on && ((wbd[j >> 5] >> (j & 31)) & 1u);
    const uint32_t code = on ? (bnd ? a.site_code[s] : 1u) : 0u;
    T f[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      if constexpr (P == 1)
        f[d] = on ? stage[d * kSites + j] : 0.f;
      else
        f[d] = on ? __half2float(stage[d * kSites + j]) * a.fp16_inv_scale : 0.f;
    }
    collide_and_push<P, false>(a, b, j, s, j, code, tabreg, f, block_xyz, acc, false, uo);
  }
  // solid slots of the rows that hold fluid: zeros complete their sectors
  S* fn = static_cast<S*>(a.f_new);
  for (int j = tid; j < kSites; j += THREADS) {
    const uint32_t w = wfl[j >> 5];
    if (((w >> (j & 24)) & 0xffu) != 0 && !((w >> (j & 31)) & 1u)) {
#pragma unroll
      for (int d = 0; d < Q; ++d) Store<P>::store(fn, fidx(b * kSites + j, d), (T)0, a);
    }
  }
}

template <int P, int THREADS, int MINB>
void launch_block_staged(const StepArgs& a, const int32_t* bxyz, cudaStream_t st) {
  constexpr size_t smem = (size_t)Q * kSites * sizeof(typename Store<P>::S);
  static bool carveout = false;  // as much shared memory as the SM has, once
  if (!carveout) {
    cudaFuncSetAttribute(k_stream_collide_block<P, THREADS, MINB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         100);
    carveout = true;
  }
  if (a.n_blocks > 0)
    k_stream_collide_block<P, THREADS, MINB><<<(unsigned)a.n_blocks, THREADS, smem, st>>>(a, bxyz);
}

// ---------------------------------------------------------------------------
// Pipelined launch (FP32 / FP16 storage): one persistent CTA per SM, a producer
// warp and NCW consumer warps around a ring of STAGES shared-memory buffers, each
// holding one 8^3 block: its rows of the old distributions from the first fluid
// row to the last (one bulk copy per direction) and its warps of the fluid list
// (the same lane entries the fluid-list launch reads).  The producer takes chunks
// of consecutive blocks of the z-column order from a global counter (the blocks
// in flight stay a narrow window of that order, as in a one-shot launch), reads
// their descriptors (pipe_desc: first list warp, row span, fluid and zero-fill
// warps) and stages each block up to STAGES - 1 blocks ahead of the consumers,
// so the copies in flight hold no registers and no warp waits on a list entry or
// a distribution in DRAM.  The consumers take the staged block's list warps
// round-robin (warp task t of the launch to consumer warp t mod NCW), collide and
// push exactly as a fluid-list warp does, zero-fill as its zero-fill warps do,
// and release the buffer.  Every wait is bounded; a CTA that gives up raises
// stage_err and lets its copies land before it exits.
// ---------------------------------------------------------------------------
// Blocks per fetch of the pipelined launch's counter.
#ifndef HLBG_PIPE_CHUNK
#define HLBG_PIPE_CHUNK 8
#endif
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Bytes of one ring buffer: the distributions of a whole block, then up to 32
// list warps (16 fluid + 16 zero-fill) of 32 uint16 entries.
template <int P>
struct PipeStage {
  static constexpr uint32_t kValues = (uint32_t)(Q * kSites * sizeof(typename Store<P>::S));
  static constexpr uint32_t kBytes = kValues + 32 * 32 * 2;
};

template <int P, int NCW, int STAGES>
__global__ void __launch_bounds__((NCW + 1) * 32, 1) k_stream_collide_pipe(StepArgs a, const int32_t* block_xyz) {
  static_assert(P != 0, "the staged block holds FP32 or FP16 values");
  using S = typename Store<P>::S;
  using T = typename Calc<P>::T;
  using PS = PipeStage<P>;
  extern __shared__ __align__(128) unsigned char pipe_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES];
  __shared__ int32_t st_block[STAGES];
  __shared__ uint32_t st_warps[STAGES];  // fluid warps | zero-fill warps << 8
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int k = 0; k < STAGES; ++k) {
      mbar_init(smem_u32(&full_bar[k]), 1);
      mbar_init(smem_u32(&empty_bar[k]), NCW);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (warp == 0) {
    // ---- producer ----
    constexpr int CH = HLBG_PIPE_CHUNK;
    int k = 0;
    bool ok = true;
    for (bool more = true; more && ok;) {
      int32_t c0 = 0;
      if (lane == 0) c0 = atomicAdd(a.pipe_ctr, CH);
      c0 = __shfl_sync(0xffffffffu, c0, 0);
      const int nch = c0 < a.n_blocks ? (a.n_blocks - c0 < CH ? (int)(a.n_blocks - c0) : CH) : 0;
      // the chunk's descriptors, one per lane
      const uint64_t mine = lane < nch ? __ldg(a.pipe_desc + c0 + lane) : 0ull;
      for (int i = 0; i < nch; ++i, ++k) {
        const int sb = k % STAGES;
        if (k >= STAGES && !mbar_wait(smem_u32(&empty_bar[sb]), ((k / STAGES) - 1) & 1)) {
          ok = false;
          break;
        }
        const uint64_t dsc = __shfl_sync(0xffffffffu, mine, i);
        const int64_t b = c0 + i;
        const uint32_t first = (uint32_t)dsc;
        const uint32_t row0 = (uint32_t)(dsc >> 32) & 63u, rowe = (uint32_t)(dsc >> 38) & 127u;
        const uint32_t nfw = (uint32_t)(dsc >> 45) & 63u, nzw = (uint32_t)(dsc >> 51) & 63u;
        const uint32_t span = (rowe - row0) * 8u * (uint32_t)sizeof(S);
        const uint32_t lbytes = (nfw + nzw) * 64u;
        if (lane == 0) {
          st_block[sb] = (int32_t)b;
          st_warps[sb] = nfw | (nzw << 8);
        }
        __syncwarp();
        const uint32_t bar = smem_u32(&full_bar[sb]);
        if (lane == 0)
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                       "r"(span * Q + lbytes)
                       : "memory");
        __syncwarp();
        // sizes and both addresses are multiples of 16 bytes (rows of 8 values of 2
        // or 4 bytes; list warps of 64 bytes)
        const uint32_t dst0 = smem_u32(pipe_raw) + (uint32_t)sb * PS::kBytes;
        if (lane < Q && span > 0) {
          const uint32_t off = ((uint32_t)lane * kSites + row0 * 8u) * (uint32_t)sizeof(S);
          bulk_copy(dst0 + off, static_cast<const char*>(a.f_old) + (size_t)b * Q * kSites * sizeof(S) + off, span,
                    bar);
        }
        if (lane == Q && lbytes > 0) bulk_copy(dst0 + PS::kValues, a.lane_slot + (size_t)first * 32, lbytes, bar);
      }
      if (ok && nch < CH) {  // the blocks are used up: the consumers stop at the next buffer
        const int sb = k % STAGES;
        if (k >= STAGES && !mbar_wait(smem_u32(&empty_bar[sb]), ((k / STAGES) - 1) & 1)) {
          ok = false;
        } else {
          if (lane == 0) {
            st_block[sb] = -1;
            mbar_arrive(smem_u32(&full_bar[sb]));
          }
          ++k;
        }
        more = false;
      }
    }
    if (!ok) {
      if (lane == 0) atomicExch(a.stage_err, 1);
      // every copy armed so far has to land before the CTA may exit
      for (int j = k - STAGES > 0 ? k - STAGES : 0; j < k; ++j) mbar_wait(smem_u32(&full_bar[j % STAGES]), (j / STAGES) & 1);
    }
    return;
  }
  // ---- consumers ----
  const int cw = warp - 1;
  MonAccT<P> acc = mon_neutral_t<P>();  // unused: pipelined steps are not monitored
  const MonOld<P> uo;
  S* fn = static_cast<S*>(a.f_new);
  int rot = 0;  // list warps of the earlier blocks, mod NCW
  for (int k = 0;; ++k) {
    const int sb = k % STAGES;
    if (!mbar_wait(smem_u32(&full_bar[sb]), (k / STAGES) & 1)) {
      if (lane == 0) atomicExch(a.stage_err, 1);
      return;
    }
    const int64_t b = st_block[sb];
    if (b < 0) return;
    const S* stage = reinterpret_cast<const S*>(pipe_raw + (size_t)sb * PS::kBytes);
    const uint16_t* list = reinterpret_cast<const uint16_t*>(pipe_raw + (size_t)sb * PS::kBytes + PS::kValues);
    const int nfw = (int)(st_warps[sb] & 0xffu), ntask = nfw + (int)(st_warps[sb] >> 8);
    const int first = ((cw - rot) % NCW + NCW) % NCW;
    const int32_t tabreg = lane < 27 && first < nfw ? __ldg(a.block_nbr + b * 27 + lane) : 0;
    for (int task = first; task < ntask; task += NCW) {  // warp-uniform trips
      const unsigned js = list[task * 32 + lane];
      const bool on = js != 0xffffu;
      const int j = on ? (int)(js & (kSites - 1)) : 0;
      const int64_t s = b * kSites + j;
      if (task >= nfw) {  // zero-fill warp: complete the sectors its slots share with fluid
        if (on) {
#pragma unroll
          for (int d = 0; d < Q; ++d) Store<P>::store(fn, fidx(s, d), (T)0, a);
        }
        continue;
      }
      const uint32_t code = on ? ((js & kListBoundary) ? a.site_code[s] : 1u) : 0u;
      T f[Q];
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        if constexpr (P == 1)
          f[d] = on ? stage[d * kSites + j] : 0.f;
        else
          f[d] = on ? __half2float(stage[d * kSites + j]) * a.fp16_inv_scale : 0.f;
      }
      collide_and_push<P, false>(a, b, j, s, j, code, tabreg, f, block_xyz, acc, false, uo);
    }
    rot = (rot + ntask) % NCW;
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_u32(&empty_bar[sb]));
  }
}

#ifndef HLBG_PIPE_NCW
#define HLBG_PIPE_NCW 31
#endif
#ifndef HLBG_PIPE_STAGES
#define HLBG_PIPE_STAGES 4
#endif

template <int P, int NCW, int STAGES>
void launch_pipe(const StepArgs& a, const int32_t* bxyz, cudaStream_t st) {
  constexpr size_t smem = (size_t)STAGES * PipeStage<P>::kBytes;
  static std::atomic<bool> configured[64];
  static int sms[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!configured[dev].load()) {  // per device: the attribute belongs to the current context
    cudaFuncSetAttribute(k_stream_collide_pipe<P, NCW, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    configured[dev].store(true);
  }
  if (a.n_blocks <= 0) return;
  cudaMemsetAsync(a.pipe_ctr, 0, sizeof(int32_t), st);
  const int64_t grid = std::min<int64_t>(sms[dev] > 0 ? sms[dev] : 1, a.n_blocks);
  k_stream_collide_pipe<P, NCW, STAGES><<<(unsigned)grid, (NCW + 1) * 32, smem, st>>>(a, bxyz);
}

// Resident CTAs per SM of the 128-thread fluid-list launch (variant 6) in plain steps.
#ifndef HLBG_LIST_MINB
#define HLBG_LIST_MINB 8
#endif

template <int P, int THREADS, int MINB, bool MON>
void launch_listed(const StepArgs& a, const int32_t* bxyz, cudaStream_t st) {
  const int64_t g = (a.n_warps * 32 + THREADS - 1) / THREADS;
  if (g) k_stream_collide_listed<P, THREADS, MINB, MON><<<(unsigned)g, THREADS, 0, st>>>(a, bxyz);
}

// Fluid-list shape of launch variant 7: 64-thread CTAs, 16 per SM (the 32
// resident warps of 128 x 8 in smaller CTAs).  Measured on the forest: FP16
// storage +1% over 128 x 8, FP32 deviations -0.5%; 32-thread CTAs -4%.
#ifndef HLBG_LISTED7_THREADS
#define HLBG_LISTED7_THREADS 64
#endif

// All slots, one thread per slot: THREADS threads per CTA with at least MINB CTAs
// resident per SM.  The shapes are the autotuner's candidates.
template <int P, int THREADS, int MINB, bool MON>
__global__ void __launch_bounds__(THREADS, MINB)
    k_stream_collide(StepArgs a, const int32_t* block_xyz) {
  MonAccT<P> acc = mon_neutral_t<P>();
  bool check = false;
  if constexpr (MON) check = *a.mon_state != 0;
  collide_slot<P, MON>(a, (int64_t)blockIdx.x * THREADS + threadIdx.x, block_xyz, acc, check);
  if constexpr (MON) mon_write_partial<P>(a, acc);
}

// Second stage of the fused StabilityTester's reduction: CTA c folds partials
// [c * per, (c + 1) * per) in a fixed order into out[c] (same layout, stride n_out).
// fp32 != 0: the partials are the FP32 forms' 32-bit words (mon_write_partial).
static __global__ void __launch_bounds__(256) k_mon_stage2(const double* __restrict__ in, int64_t n_in,
                                                           int64_t per, double* __restrict__ out,
                                                           int64_t n_out, int fp32) {
  MonAcc acc = mon_neutral();
  const int64_t lo = (int64_t)blockIdx.x * per, hi = lo + per < n_in ? lo + per : n_in;
  const float* inf = reinterpret_cast<const float*>(in);
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    if (fp32) {
      const unsigned count = __float_as_uint(inf[6 * n_in + i]);
      if (count == 0) continue;  // a CTA of idle lanes only
      mon_combine(acc, MonAcc{(double)count + (double)inf[i], (double)inf[n_in + i], (double)inf[2 * n_in + i],
                              (unsigned long long)__float_as_uint(inf[7 * n_in + i]), 1.0 + (double)inf[3 * n_in + i],
                              1.0 + (double)inf[4 * n_in + i], (double)inf[5 * n_in + i]});
    } else {
      mon_combine(acc, MonAcc{in[i], in[n_in + i], in[2 * n_in + i], (unsigned long long)in[3 * n_in + i],
                              in[4 * n_in + i], in[5 * n_in + i], in[6 * n_in + i]});
    }
  }
  __syncthreads();
  acc = mon_block(acc);
  if (threadIdx.x == 0) {
    out[blockIdx.x] = acc.mass;
    out[n_out + blockIdx.x] = acc.maxdu;
    out[2 * n_out + blockIdx.x] = acc.minf;
    out[3 * n_out + blockIdx.x] = (double)acc.bad;
    out[4 * n_out + blockIdx.x] = acc.rmin;
    out[5 * n_out + blockIdx.x] = acc.rmax;
    out[6 * n_out + blockIdx.x] = acc.umax;
  }
}

// Last stage: result = [mass, max |du|, min f, unstable, valid, min rho, max rho,
// max |u|]; valid is 0 for the
// first step after the state was set (it only recorded velocities).  With sa, a
// valid check is also counted for steady-state detection.
// Every step then marks the recorded velocities as present.
static __global__ void __launch_bounds__(256) k_mon_final(const double* __restrict__ part, int64_t n,
                                                          int32_t* mon_state, double* result,
                                                          SteadyArgs sa, int steady) {
  MonAcc acc = mon_neutral();
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    mon_combine(acc, MonAcc{part[i], part[n + i], part[2 * n + i], (unsigned long long)part[3 * n + i],
                            part[4 * n + i], part[5 * n + i], part[6 * n + i]});
  __syncthreads();
  acc = mon_block(acc);
  if (threadIdx.x == 0) {
    const int valid = *mon_state != 0;
    result[0] = acc.mass;
    result[1] = acc.maxdu;
    result[2] = acc.minf;
    result[3] = (double)acc.bad;
    result[4] = valid;
    result[5] = acc.rmin;
    result[6] = acc.rmax;
    result[7] = acc.umax;
    if (steady && valid) {
      const long long k = sa.counters[0] + 1;
      sa.counters[0] = k;
      *sa.last_du = acc.maxdu;
      if (acc.bad && sa.counters[2] < 0) sa.counters[2] = k;
      if (acc.maxdu <= *sa.threshold && sa.counters[1] < 0) sa.counters[1] = k;
    }
    *mon_state = 1;
  }
}

template <int P>
__global__ void __launch_bounds__(256) k_stream_collide_list(StepArgs a, const int32_t* block_xyz) {
  const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (i >= a.list_count) return;
  const int64_t s = a.list[i];
  const int64_t b = s >> 9;
  const uint32_t code = a.block_bulk[b] ? 1u : a.site_code[s];
  if (code == 0) return;
  const int32_t* tab = a.block_nbr + b * 27;
  site_update<P>(a, GlobalBase{tab}, tab, s, code, block_xyz);
}

// Iolet links (Nash / Ladd) of the sites listed in `rec`: the site's collision is
// recomputed from f_old with the same arithmetic as k_stream_collide, and each iolet
// link writes the site's own inverse-direction slot.  These slots have no other
// writer, so this launch and k_stream_collide may run in either order.
template <int P>
__global__ void __launch_bounds__(128) k_iolet_links(StepArgs a, const int32_t* __restrict__ rec,
                                                     const int32_t* __restrict__ rec_slot, int64_t n,
                                                     const int32_t* __restrict__ block_xyz) {
  using St = Store<P>;
  using S = typename St::S;
  using T = typename Calc<P>::T;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t r = rec[i];
  const int64_t s = rec_slot[r];
  const int64_t b = s >> 9;
  const int l = (int)(s & (kSites - 1));
  const S* fo = static_cast<const S*>(a.f_old) + b * (Q * kSites) + l;
  S* fn = static_cast<S*>(a.f_new) + b * (Q * kSites) + l;
  T f[Q], fpost[Q];
#pragma unroll
  for (int d = 0; d < Q; ++d) f[d] = St::load(fo, d * kSites, a);
  T m0, mx, my, mz;
  collide_any<P>(a, b, f, m0, mx, my, mz, fpost);
  const uint64_t links = a.b_links[r];
  const int type = a.b_type[r];
  const int ioid = a.b_ioid[r];
  const bool is_inlet = (type == 2 || type == 4);
  const int gi = is_inlet ? ioid : a.n_in + ioid;
  const int model = is_inlet ? a.inlet_model : a.outlet_model;
  const int ls = site_of_slot(a, s, (__ldg(a.block_nbr + b * 27 + 13) & kPackedBit) != 0);
  const int gx = block_xyz[3 * b] * 8 + (ls >> 6), gy = block_xyz[3 * b + 1] * 8 + ((ls >> 3) & 7),
            gz = block_xyz[3 * b + 2] * 8 + (ls & 7);
#pragma unroll 1
  for (int d = 1; d < Q; ++d) {
    if (((links >> (3 * d)) & 7u) != HLBG_LC_IOLET) continue;
    T fp = fpost[0];
#pragma unroll
    for (int e = 1; e < Q; ++e)
      if (e == d) fp = fpost[e];
    const T v = iolet_link_value<P>(a, gi, model, d, fp, m0, mx, my, mz, gx, gy, gz);
    St::store(fn, c_inv[d] * kSites, v, a);
  }
}

// BouzidiFirdaousLallemandLink::PostStepLink (BouzidiFirdaousLallemand.h:336-357)
// over the precomputed links with !HasWall(inverse) and q < 0.5.
template <int P>
__global__ void k_post_step(PostArgs p) {
  using St = Store<P>;
  using S = typename St::S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.count) return;
  StepArgs a{};
  a.fp16_scale = p.fp16_scale;
  a.fp16_inv_scale = p.fp16_inv_scale;
  S* fn = static_cast<S*>(p.f_new);
  const int64_t s = p.slot[i];
  const int d = p.dir[i];
  const int inv = c_inv[d];
  if constexpr (P == 0) {
    const double q = (double)p.q[i];
    const double vi = St::load(fn, fidx(s, inv), a);
    const double vd = St::load(fn, fidx(s, d), a);
    St::store(fn, fidx(s, inv), 2.0 * q * vi + (1.0 - 2.0 * q) * vd, a);
  } else {
    const float q = p.q[i];
    const float vi = St::load(fn, fidx(s, inv), a);
    const float vd = St::load(fn, fidx(s, d), a);
    St::store(fn, fidx(s, inv), 2.f * q * vi + (1.f - 2.f * q) * vd, a);
  }
}

// Uniform initial state: value[d] per direction into every fluid slot of both arrays.
template <int P>
__global__ void k_init_uniform(InitArgs ia) {
  using St = Store<P>;
  using S = typename St::S;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ia.nslot) return;
  const uint32_t code = ia.block_bulk[s >> 9] ? 1u : ia.site_code[s];
  if (code == 0) return;
  StepArgs a{};
  a.fp16_scale = ia.fp16_scale;
  a.fp16_inv_scale = ia.fp16_inv_scale;
  S* f0 = static_cast<S*>(ia.f0);
  S* f1 = static_cast<S*>(ia.f1);
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    if constexpr (P == 0) {
      St::store(f0, fidx(s, d), ia.value[d], a);
      St::store(f1, fidx(s, d), ia.value[d], a);
    } else {
      St::store(f0, fidx(s, d), (float)ia.value[d], a);
      St::store(f1, fidx(s, d), (float)ia.value[d], a);
    }
  }
}

// Per-site equilibrium from (rho, u) fields given in contiguous site order.
template <int P>
__global__ void k_init_field(FieldArgs fa) {
  using St = Store<P>;
  using S = typename St::S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= fa.count) return;
  const int64_t s = fa.ref2slot[fa.first + i];
  StepArgs a{};
  a.fp16_scale = fa.fp16_scale;
  a.fp16_inv_scale = fa.fp16_inv_scale;
  const double rho = fa.rho[i];
  const double mx = rho * fa.u[3 * i], my = rho * fa.u[3 * i + 1], mz = rho * fa.u[3 * i + 2];
  double feq[Q];
  feq64(rho, mx, my, mz, feq);
  S* f0 = static_cast<S*>(fa.f0);
  S* f1 = static_cast<S*>(fa.f1);
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    if constexpr (P == 0) {
      St::store(f0, fidx(s, d), feq[d], a);
      St::store(f1, fidx(s, d), feq[d], a);
    } else {
      const float v = (float)(feq[d] - weight_d(d));
      St::store(f0, fidx(s, d), v, a);
      St::store(f1, fidx(s, d), v, a);
    }
  }
}

// Gather f into AoS doubles in contiguous site order (FieldData layout).
template <int P>
__global__ void k_gather(GatherArgs ga) {
  using St = Store<P>;
  using S = typename St::S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ga.count) return;
  const int64_t s = ga.ref2slot[ga.first + i];
  StepArgs a{};
  a.fp16_scale = ga.fp16_scale;
  a.fp16_inv_scale = ga.fp16_inv_scale;
  const S* f = static_cast<const S*>(ga.f);
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    double v = (double)St::load(f, fidx(s, d), a);
    if constexpr (P != 0) v += weight_d(d);
    ga.aos[i * Q + d] = v;
  }
}

template <int P>
__global__ void k_scatter(GatherArgs ga) {
  using St = Store<P>;
  using S = typename St::S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ga.count) return;
  const int64_t s = ga.ref2slot[ga.first + i];
  StepArgs a{};
  a.fp16_scale = ga.fp16_scale;
  a.fp16_inv_scale = ga.fp16_inv_scale;
  S* f = static_cast<S*>(ga.f_out);
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    const double v = ga.aos[i * Q + d];
    if constexpr (P == 0)
      St::store(f, fidx(s, d), v, a);
    else
      St::store(f, fidx(s, d), (float)(v - weight_d(d)), a);
  }
}

// Density and velocity per site in contiguous order.
template <int P>
__global__ void k_macro(GatherArgs ga) {
  using St = Store<P>;
  using S = typename St::S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ga.count) return;
  const int64_t s = ga.ref2slot[ga.first + i];
  StepArgs a{};
  a.fp16_scale = ga.fp16_scale;
  a.fp16_inv_scale = ga.fp16_inv_scale;
  const S* f = static_cast<const S*>(ga.f);
  if constexpr (P == 0) {
    double r = 0.0, x = 0.0, y = 0.0, z = 0.0;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      const double v = St::load(f, fidx(s, d), a);
      r += v;
      x += (double)Lat::cx(d) * v;
      y += (double)Lat::cy(d) * v;
      z += (double)Lat::cz(d) * v;
    }
    ga.rho[i] = r;
    ga.u[3 * i] = x / r;
    ga.u[3 * i + 1] = y / r;
    ga.u[3 * i + 2] = z / r;
  } else {
    float g[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) g[d] = St::load(f, fidx(s, d), a);
    float dr, mx, my, mz;
    moments_dev(g, dr, mx, my, mz);
    const double rho = 1.0 + (double)dr;
    ga.rho[i] = rho;
    ga.u[3 * i] = (double)mx / rho;
    ga.u[3 * i + 1] = (double)my / rho;
    ga.u[3 * i + 2] = (double)mz / rho;
  }
}

template <int P>
__global__ void __launch_bounds__(256) k_monitor(MonitorArgs ma) {
  using St = Store<P>;
  using S = typename St::S;
  StepArgs a{};
  a.fp16_scale = ma.fp16_scale;
  a.fp16_inv_scale = ma.fp16_inv_scale;
  MonAcc acc = mon_neutral();
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t code = (s < ma.nslot) ? (ma.block_bulk[s >> 9] ? 1u : ma.site_code[s]) : 0u;
  if (code != 0) {
    const int64_t off = fidx(s, 0);
    const S* fc = static_cast<const S*>(ma.f_cur) + off;
    const S* fp = static_cast<const S*>(ma.f_prev) + off;
    bool bad = false;
    double rn, dx, dy, dz;
    if constexpr (P == 0) {
      // Lattice::CalculateDensityAndMomentum (scalar order) on fNew and fOld
      double xn = 0.0, yn = 0.0, zn = 0.0, ro = 0.0, xo = 0.0, yo = 0.0, zo = 0.0;
      rn = 0.0;
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        const double vn = St::load(fc, d * kSites, a);
        const double vo = St::load(fp, d * kSites, a);
        if (!(vn > 0.0)) bad = true;
        acc.minf = fmin(acc.minf, vn);
        rn += vn;
        xn += (double)Lat::cx(d) * vn;
        yn += (double)Lat::cy(d) * vn;
        zn += (double)Lat::cz(d) * vn;
        ro += vo;
        xo += (double)Lat::cx(d) * vo;
        yo += (double)Lat::cy(d) * vo;
        zo += (double)Lat::cz(d) * vo;
      }
      dx = xn / rn - xo / ro;
      dy = yn / rn - yo / ro;
      dz = zn / rn - zo / ro;
    } else {
      // deviation form: FP32 on g = f - w; only the mass accumulates in FP64
      float gn[Q], go[Q];
      float mn = 1.0e30f;
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        gn[d] = St::load(fc, d * kSites, a);
        go[d] = St::load(fp, d * kSites, a);
        const float fv = gn[d] + weight_f(d);
        if (!(fv > 0.f)) bad = true;
        mn = fminf(mn, fv);
      }
      acc.minf = (double)mn;
      float drn, mxn, myn, mzn, dro, mxo, myo, mzo;
      moments_dev(gn, drn, mxn, myn, mzn);
      moments_dev(go, dro, mxo, myo, mzo);
      rn = 1.0 + (double)drn;
      const float irn = 1.f / (1.f + drn), iro = 1.f / (1.f + dro);
      dx = (double)(mxn * irn - mxo * iro);
      dy = (double)(myn * irn - myo * iro);
      dz = (double)(mzn * irn - mzo * iro);
    }
    acc.bad = bad ? 1ull : 0ull;
    acc.mass = rn;
    acc.maxdu = sqrt(dot3d(dx, dy, dz, dx, dy, dz));
  }
  acc = mon_block(acc);
  if (threadIdx.x == 0) {
    ma.part_mass[blockIdx.x] = acc.mass;
    ma.part_max[blockIdx.x] = acc.maxdu;
    ma.part_min[blockIdx.x] = acc.minf;
    ma.part_bad[blockIdx.x] = acc.bad;
  }
}

// Reduce the per-CTA partials of k_monitor in a fixed order into element 0 of
// each partial array (one CTA of 256 threads; thread t folds partials t, t+256, ...).
static __global__ void __launch_bounds__(256) k_monitor_final(MonitorArgs ma, int64_t nparts) {
  MonAcc acc = mon_neutral();
  for (int64_t i = threadIdx.x; i < nparts; i += blockDim.x)
    mon_combine(acc, MonAcc{ma.part_mass[i], ma.part_max[i], ma.part_min[i], ma.part_bad[i], 1.0e300, -1.0e300,
                            0.0});
  __syncthreads();
  acc = mon_block(acc);
  if (threadIdx.x == 0) {
    ma.part_mass[0] = acc.mass;
    ma.part_max[0] = acc.maxdu;
    ma.part_min[0] = acc.minf;
    ma.part_bad[0] = acc.bad;
  }
}

// Lattice::CalculateWallShearStressMagnitude (Code/lb/lattices/Lattice.h:652-686)
// with CalculatePiTensor (:696-726) on f_neq = f - f_eq of the state, as
// Mass flux through the iolets: for every site with links to iolet gi, its
// momentum sum_d c_d f_d (the reference's CalculateDensityAndMomentum order) along
// the iolet's normalised inward normal, in FP64.  No reference counterpart: the
// host sums the per-site values of each iolet in list order.
template <int P>
__global__ void k_iolet_flux(FluxArgs fa) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= fa.count) return;
  const int64_t s = fa.slot[i];
  const int64_t off = fidx(s, 0);
  double mx = 0.0, my = 0.0, mz = 0.0;
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    double fd;
    if constexpr (P == 0) {
      fd = static_cast<const double*>(fa.f)[off + d * kSites];
    } else if constexpr (P == 1) {
      fd = (double)static_cast<const float*>(fa.f)[off + d * kSites] + weight_d(d);
    } else {
      fd = (double)(__half2float(static_cast<const __half*>(fa.f)[off + d * kSites]) * fa.fp16_inv_scale) +
           weight_d(d);
    }
    mx += (double)Lat::cx(d) * fd;
    my += (double)Lat::cy(d) * fd;
    mz += (double)Lat::cz(d) * fd;
  }
  const IoletDev& io = fa.iolets[fa.gi[i]];
  fa.out[i] = dot3d(mx, my, mz, io.n[0], io.n[1], io.n[2]);
}

// UpdateCachePostCollision fills wallShearStressMagnitudeCache
// (Code/lb/streamers/Common.h:35-52): FP64 and the reference's operation order.
template <int P>
__global__ void k_wss(WssArgs wa) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= wa.count) return;
  const int64_t s = wa.ref2slot[i];
  const uint32_t code = wa.block_bulk[s >> 9] ? 1u : wa.site_code[s];
  const uint32_t wm = code >= 2 ? wa.b_wall[code - 2] : 0u;
  if (wm == 0) {  // site.IsWall() is false: NO_VALUE
    wa.out[i] = 1.7976931348623157e308;
    return;
  }
  double f[Q];
  const int64_t off = fidx(s, 0);
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    if constexpr (P == 0) {
      f[d] = static_cast<const double*>(wa.f)[off + d * kSites];
    } else if constexpr (P == 1) {
      f[d] = (double)static_cast<const float*>(wa.f)[off + d * kSites] + weight_d(d);
    } else {
      f[d] = (double)(__half2float(static_cast<const __half*>(wa.f)[off + d * kSites]) * wa.fp16_inv_scale) +
             weight_d(d);
    }
  }
  double rho = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    rho += f[d];
    mx += (double)Lat::cx(d) * f[d];
    my += (double)Lat::cy(d) * f[d];
    mz += (double)Lat::cz(d) * f[d];
  }
  double feq[Q];
  feq64(rho, mx, my, mz, feq);
  double fneq[Q];
#pragma unroll
  for (int d = 0; d < Q; ++d) fneq[d] = f[d] - feq[d];
  double pi[3][3];
#pragma unroll
  for (int ii = 0; ii < 3; ++ii)
#pragma unroll
    for (int jj = 0; jj <= ii; ++jj) {
      double acc = 0.0;
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        const double ci = ii == 0 ? (double)Lat::cx(d) : (ii == 1 ? (double)Lat::cy(d) : (double)Lat::cz(d));
        const double cj = jj == 0 ? (double)Lat::cx(d) : (jj == 1 ? (double)Lat::cy(d) : (double)Lat::cz(d));
        acc += fneq[d] * ci * cj;
      }
      pi[ii][jj] = acc;
      pi[jj][ii] = acc;
    }
  const double nor[3] = {(double)wa.b_normal[3 * (code - 2)], (double)wa.b_normal[3 * (code - 2) + 1],
                         (double)wa.b_normal[3 * (code - 2) + 2]};
  const double temp = wa.stress_param * (-sqrt(2.0));
  double sq = 0.0, nrm = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double sv = 0.0;
#pragma unroll
    for (int b = 0; b < 3; ++b) sv += pi[a][b] * nor[b] * temp;
    sq += sv * sv;
    nrm += sv * nor[a];
  }
  wa.out[i] = sqrt(sq - nrm * nrm);
}

// Mean of the two time levels on every fluid slot (the arrays hold consecutive
// states right after a step): removes the period-two component of the state.
template <int P>
__global__ void __launch_bounds__(256) k_average(AverageArgs aa) {
  using St = Store<P>;
  using S = typename St::S;
  StepArgs a{};
  a.fp16_scale = aa.fp16_scale;
  a.fp16_inv_scale = aa.fp16_inv_scale;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t code = (s < aa.nslot) ? (aa.block_bulk[s >> 9] ? 1u : aa.site_code[s]) : 0u;
  if (code == 0) return;
  const int64_t off = fidx(s, 0);
  S* fc = static_cast<S*>(aa.f_cur) + off;
  const S* fp = static_cast<const S*>(aa.f_prev) + off;
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    const auto v = St::load(fc, d * kSites, a) + St::load(fp, d * kSites, a);
    St::store(fc, d * kSites, v * 0.5f, a);
  }
}

}  // namespace hlbg

namespace hlbg {
template <int P, int THREADS, int MINB, bool MON = false>
void launch_sc(const StepArgs& a, const int32_t* bxyz, cudaStream_t st) {
  const unsigned g = (unsigned)(a.nslot / THREADS);
  if (g) k_stream_collide<P, THREADS, MINB, MON><<<g, THREADS, 0, st>>>(a, bxyz);
}
}  // namespace hlbg

namespace hlbg {
// Multi-rank exchange: copy stored distributions (the storage element type, so the
// exchange is exact in every form) between the new-distribution array and a
// contiguous buffer, at element offsets from hlbg_halo_offsets.  An offset outside
// [0, limit) is skipped and flagged in *err (a bad list must not write elsewhere).
template <int P>
__global__ void k_halo_pack(const void* f, const int64_t* off, int64_t n, int64_t limit, void* buf,
                            int32_t* err) {
  using S = typename Store<P>::S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = off[i];
  if (o < 0 || o >= limit) {
    atomicOr(err, 1);
    return;
  }
  static_cast<S*>(buf)[i] = static_cast<const S*>(f)[o];
}

template <int P>
__global__ void k_halo_unpack(void* f, const int64_t* off, int64_t n, int64_t limit, const void* buf,
                              int32_t* err) {
  using S = typename Store<P>::S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = off[i];
  if (o < 0 || o >= limit) {
    atomicOr(err, 1);
    return;
  }
  static_cast<S*>(f)[o] = static_cast<const S*>(buf)[i];
}
}  // namespace hlbg

#define HLBG_INSTANTIATE(P)                                                                     \
  namespace hlbg {                                                                              \
  void launch_stream_collide_##P(const StepArgs& a, const int32_t* bxyz, cudaStream_t st,      \
                                 int variant) {                                                 \
    if (a.list) {                                                                               \
      unsigned g = (unsigned)((a.list_count + 255) / 256);                                      \
      if (g) k_stream_collide_list<P><<<g, 256, 0, st>>>(a, bxyz);                              \
      return;                                                                                   \
    }                                                                                           \
    /* monitored steps: the 10-CTA all-slots shape becomes 128 x 8, every fluid-list    */      \
    /* shape the 128 x 8 fluid list (one partial per 128-thread CTA)                     */      \
    if (a.mon_u && variant == 0) variant = 1;                                                   \
    if (a.mon_u && variant >= 4) variant = 6;                                                   \
    if (variant == 4) {                                                                         \
      if constexpr (P != 0) {                                                                   \
        if (a.blk_runs) {                                                                       \
          launch_block_staged<P, 256, 4>(a, bxyz, st);                                          \
          return;                                                                               \
        }                                                                                       \
      }                                                                                         \
      variant = 6; /* FP64, or a layout without the block tables */                             \
    }                                                                                           \
    if (variant == 8) {                                                                         \
      if constexpr (P != 0) {                                                                   \
        if (a.pipe_desc && !a.mon_u) {                                                          \
          launch_pipe<P, HLBG_PIPE_NCW, (P == 1 ? HLBG_PIPE_STAGES : 2 * HLBG_PIPE_STAGES)>(a, bxyz, st); \
          return;                                                                               \
        }                                                                                       \
      }                                                                                         \
      variant = 6; /* FP64, monitored steps, or a layout without the block tables */            \
    }                                                                                           \
    if (variant == 5) {                                                                         \
      launch_listed<P, 128, (P == 0 ? 2 : 9), false>(a, bxyz, st);                              \
      return;                                                                                   \
    }                                                                                           \
    if (variant == 7) {                                                                         \
      if (!a.mon_u) {                                                                           \
        launch_listed<P, HLBG_LISTED7_THREADS, (P == 0 ? 2 : 1024 / HLBG_LISTED7_THREADS),      \
                      false>(a, bxyz, st);                                                      \
        return;                                                                                 \
      }                                                                                         \
      variant = 6; /* monitored steps keep 128-thread CTAs (one partial per CTA) */             \
    }                                                                                           \
    if (variant == 6) {                                                                         \
      if (a.mon_u) launch_listed<P, 128, (P == 0 ? 2 : 8), true>(a, bxyz, st);                  \
      else launch_listed<P, 128, (P == 0 ? 2 : HLBG_LIST_MINB), false>(a, bxyz, st);            \
      return;                                                                                   \
    }                                                                                           \
    if (P == 0) variant = -1;                                                                   \
    if (a.mon_u) { /* one partial per CTA */                                                    \
      switch (variant) {                                                                        \
        case 2: launch_sc<P, 256, (P == 0 ? 2 : 4), true>(a, bxyz, st); break;                  \
        case 3: launch_sc<P, 512, (P == 0 ? 1 : 2), true>(a, bxyz, st); break;                  \
        case -1: launch_sc<P, 128, 2, true>(a, bxyz, st); break;                                \
        default: launch_sc<P, 128, (P == 0 ? 2 : 8), true>(a, bxyz, st); break;                 \
      }                                                                                         \
      return;                                                                                   \
    }                                                                                           \
    switch (variant) {                                                                          \
      case 1: launch_sc<P, 128, (P == 0 ? 2 : 8)>(a, bxyz, st); break;                          \
      case 2: launch_sc<P, 256, (P == 0 ? 2 : 4)>(a, bxyz, st); break;                          \
      case 3: launch_sc<P, 512, (P == 0 ? 1 : 2)>(a, bxyz, st); break;                          \
      case -1: launch_sc<P, 128, 2>(a, bxyz, st); break;                                        \
      default: launch_sc<P, HLBG_SC_THREADS, HLBG_SC_MINB>(a, bxyz, st); break;                 \
    }                                                                                           \
  }                                                                                             \
  int64_t monitored_grid_##P(int64_t nslot, int variant, int64_t n_warps) {                    \
    if (variant >= 4) return (n_warps * 32 + 127) / 128; /* monitored 4..8 run as 6 */          \
    if (P == 0) return nslot / 128;                                                             \
    switch (variant) {                                                                          \
      case 1: return nslot / 128;                                                               \
      case 2: return nslot / 256;                                                               \
      case 3: return nslot / 512;                                                               \
      default: return nslot / 128; /* monitored steps: the 128 x 8 shape */                     \
    }                                                                                           \
  }                                                                                             \
  void launch_mon_reduce_##P(const double* part, int64_t nparts, double* part2, int64_t n2,      \
                             int32_t* mon_state, double* result, const SteadyArgs& sa,          \
                             int steady, cudaStream_t st) {                                      \
    const int64_t per = (nparts + n2 - 1) / n2;                                                 \
    k_mon_stage2<<<(unsigned)n2, 256, 0, st>>>(part, nparts, per, part2, n2, P != 0);           \
    k_mon_final<<<1, 256, 0, st>>>(part2, n2, mon_state, result, sa, steady);                   \
  }                                                                                             \
  void launch_iolet_links_##P(const StepArgs& a, const int32_t* rec, const int32_t* rec_slot,    \
                              int64_t n, const int32_t* bxyz, cudaStream_t st) {                \
    unsigned g = (unsigned)((n + 127) / 128);                                                   \
    if (g) k_iolet_links<P><<<g, 128, 0, st>>>(a, rec, rec_slot, n, bxyz);                      \
  }                                                                                             \
  void launch_post_step_##P(const PostArgs& p, cudaStream_t st) {                               \
    unsigned g = (unsigned)((p.count + 255) / 256);                                             \
    if (g) k_post_step<P><<<g, 256, 0, st>>>(p);                                                \
  }                                                                                             \
  void launch_init_uniform_##P(const InitArgs& ia, cudaStream_t st) {                           \
    unsigned g = (unsigned)((ia.nslot + 255) / 256);                                            \
    if (g) k_init_uniform<P><<<g, 256, 0, st>>>(ia);                                            \
  }                                                                                             \
  void launch_init_field_##P(const FieldArgs& fa, cudaStream_t st) {                            \
    unsigned g = (unsigned)((fa.count + 255) / 256);                                            \
    if (g) k_init_field<P><<<g, 256, 0, st>>>(fa);                                              \
  }                                                                                             \
  void launch_gather_##P(const GatherArgs& ga, cudaStream_t st) {                               \
    unsigned g = (unsigned)((ga.count + 255) / 256);                                            \
    if (g) k_gather<P><<<g, 256, 0, st>>>(ga);                                                  \
  }                                                                                             \
  void launch_scatter_##P(const GatherArgs& ga, cudaStream_t st) {                              \
    unsigned g = (unsigned)((ga.count + 255) / 256);                                            \
    if (g) k_scatter<P><<<g, 256, 0, st>>>(ga);                                                 \
  }                                                                                             \
  void launch_macro_##P(const GatherArgs& ga, cudaStream_t st) {                                \
    unsigned g = (unsigned)((ga.count + 255) / 256);                                            \
    if (g) k_macro<P><<<g, 256, 0, st>>>(ga);                                                   \
  }                                                                                             \
  cudaError_t preload_monitor_##P() {                                                           \
    cudaFuncAttributes fa;                                                                      \
    cudaError_t e = cudaFuncGetAttributes(&fa, k_monitor<P>);                                   \
    return e != cudaSuccess ? e : cudaFuncGetAttributes(&fa, k_monitor_final);                  \
  }                                                                                             \
  void launch_monitor_##P(const MonitorArgs& ma, int grid, cudaStream_t st) {                   \
    (void)grid;                                                                                 \
    const int64_t nparts = (ma.nslot + 255) / 256;                                              \
    k_monitor<P><<<(unsigned)nparts, 256, 0, st>>>(ma);                                         \
    k_monitor_final<<<1, 256, 0, st>>>(ma, nparts);                                             \
  }                                                                                             \
  void launch_halo_copy_##P(void* f, const int64_t* off, int64_t n, int64_t limit, void* buf,     \
                            int unpack, int32_t* err, cudaStream_t st) {                        \
    unsigned g = (unsigned)((n + 255) / 256);                                                   \
    if (!g) return;                                                                             \
    if (unpack)                                                                                 \
      k_halo_unpack<P><<<g, 256, 0, st>>>(f, off, n, limit, buf, err);                          \
    else                                                                                        \
      k_halo_pack<P><<<g, 256, 0, st>>>(f, off, n, limit, buf, err);                            \
  }                                                                                             \
  void launch_wss_##P(const WssArgs& wa, cudaStream_t st) {                                     \
    unsigned g = (unsigned)((wa.count + 255) / 256);                                            \
    if (g) k_wss<P><<<g, 256, 0, st>>>(wa);                                                     \
  }                                                                                             \
  void launch_flux_##P(const FluxArgs& fa, cudaStream_t st) {                                   \
    unsigned g = (unsigned)((fa.count + 255) / 256);                                            \
    if (g) k_iolet_flux<P><<<g, 256, 0, st>>>(fa);                                              \
  }                                                                                             \
  void launch_average_##P(const AverageArgs& aa, cudaStream_t st) {                             \
    unsigned g = (unsigned)((aa.nslot + 255) / 256);                                            \
    if (g) k_average<P><<<g, 256, 0, st>>>(aa);                                                 \
  }                                                                                             \
  }
