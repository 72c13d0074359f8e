// Kernel templates, instantiated per storage form in lb_fp64.cu (FP64, built
// with --fmad=false) and lb_fp32.cu (FP32 / FP16 deviation forms).
#pragma once

#include "lb_device.cuh"
#include "lb_launch.h"

namespace hlbg {

// ---------------------------------------------------------------------------
// One site: collide, then push along the 19 links.
// ---------------------------------------------------------------------------
template <int P>
__device__ __forceinline__ void site_update(const StepArgs& a, const int32_t* nbr, int64_t s,
                                            uint32_t code, const int32_t* block_xyz) {
  using St = Store<P>;
  using S = typename St::S;
  const S* fo = static_cast<const S*>(a.f_old);
  S* fn = static_cast<S*>(a.f_new);
  const int l = (int)(s & (kSites - 1));
  if constexpr (P == 0) {
    double f[Q], fpost[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = St::load(fo, i * a.stride + s, a);
    double rho, mx, my, mz;
    collide64(a, f, rho, mx, my, mz, fpost);
    if (code == 1) {
#pragma unroll
      for (int i = 0; i < Q; ++i) St::store(fn, i * a.stride + nbr_slot(nbr, l, i), fpost[i], a);
      return;
    }
    const int64_t r = code - 2;
    const uint32_t wm = a.b_wall[r], im = a.b_iolet[r];
    const int type = a.b_type[r];
    const int ioid = a.b_ioid[r];
    const bool can_wall = (type == 1 || type == 4 || type == 5);
    const bool can_iolet = type >= 2;
    const bool is_inlet = (type == 2 || type == 4);
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      if (can_iolet && bit(im, d)) {
        const int gi = is_inlet ? ioid : a.n_in + ioid;
        const int model = is_inlet ? a.inlet_model : a.outlet_model;
        const int un = Lat::inv(d);
        double v;
        if (model == 0) {
          v = nash64(a.iolets[gi], a.iolet_rho[gi], rho, mx, my, mz, un);
        } else {
          const int64_t b = s >> 9;
          const int gx = block_xyz[3 * b] * 8 + (l >> 6);
          const int gy = block_xyz[3 * b + 1] * 8 + ((l >> 3) & 7);
          const int gz = block_xyz[3 * b + 2] * 8 + (l & 7);
          v = fpost[d] - ladd_correction64(a.iolets[gi], a.iolet_umax[gi], rho, gx, gy, gz, d);
        }
        St::store(fn, un * a.stride + s, v, a);
      } else if (can_wall && bit(wm, d)) {
        const int inv = Lat::inv(d);
        double v = fpost[d];
        if (a.wall == 1) {
          const double q = (double)a.b_cut[r * (Q - 1) + d - 1];
          if (!(bit(wm, inv) || q < 0.5)) v = (fpost[d] + (2.0 * q - 1) * fpost[inv]) / (2.0 * q);
        }
        St::store(fn, inv * a.stride + s, v, a);
      } else {
        const int64_t ns = nbr_slot(nbr, l, d);
        if (ns < 0) continue;
        const uint32_t nc = a.block_bulk[ns >> 9] ? 1u : a.site_code[ns];
        if (nc == 0) continue;  // rubbish site
        St::store(fn, d * a.stride + ns, fpost[d], a);
      }
    }
  } else {
    float g[Q], gpost[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) g[i] = St::load(fo, i * a.stride + s, a);
    float dr, mx, my, mz;
    collide_dev(a, g, dr, mx, my, mz, gpost);
    if (code == 1) {
#pragma unroll
      for (int i = 0; i < Q; ++i) St::store(fn, i * a.stride + nbr_slot(nbr, l, i), gpost[i], a);
      return;
    }
    const int64_t r = code - 2;
    const uint32_t wm = a.b_wall[r], im = a.b_iolet[r];
    const int type = a.b_type[r];
    const int ioid = a.b_ioid[r];
    const bool can_wall = (type == 1 || type == 4 || type == 5);
    const bool can_iolet = type >= 2;
    const bool is_inlet = (type == 2 || type == 4);
    const float rho = 1.f + dr;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      if (can_iolet && bit(im, d)) {
        const int gi = is_inlet ? ioid : a.n_in + ioid;
        const int model = is_inlet ? a.inlet_model : a.outlet_model;
        const int un = Lat::inv(d);
        float v;
        const IoletDev& io = a.iolets[gi];
        if (model == 0) {
          const double grho = a.iolet_rho[gi];
          const float gdr = (float)(grho - 1.0);
          const float grho_f = (float)grho;
          const float comp = (mx * (float)io.nf[0] + my * (float)io.nf[1] + mz * (float)io.nf[2]) / rho;
          const float gx = (float)io.nf[0] * comp * grho_f;
          const float gy = (float)io.nf[1] * comp * grho_f;
          const float gz = (float)io.nf[2] * comp * grho_f;
          const float inv_g = 1.f / grho_f;
          v = geq_dev(gdr, inv_g, 1.5f * (gx * gx + gy * gy + gz * gz), gx, gy, gz, un);
        } else {
          const int64_t b = s >> 9;
          const int gxx = block_xyz[3 * b] * 8 + (l >> 6);
          const int gyy = block_xyz[3 * b + 1] * 8 + ((l >> 3) & 7);
          const int gzz = block_xyz[3 * b + 2] * 8 + (l & 7);
          v = gpost[d] - (float)ladd_correction64(io, a.iolet_umax[gi], (double)rho, gxx, gyy, gzz, d);
        }
        St::store(fn, un * a.stride + s, v, a);
      } else if (can_wall && bit(wm, d)) {
        const int inv = Lat::inv(d);
        float v = gpost[d];
        if (a.wall == 1) {
          const float q = a.b_cut[r * (Q - 1) + d - 1];
          if (!(bit(wm, inv) || q < 0.5f)) v = (gpost[d] + (2.f * q - 1.f) * gpost[inv]) / (2.f * q);
        }
        St::store(fn, inv * a.stride + s, v, a);
      } else {
        const int64_t ns = nbr_slot(nbr, l, d);
        if (ns < 0) continue;
        const uint32_t nc = a.block_bulk[ns >> 9] ? 1u : a.site_code[ns];
        if (nc == 0) continue;
        St::store(fn, d * a.stride + ns, gpost[d], a);
      }
    }
  }
}

template <int P>
__global__ void __launch_bounds__(256) k_stream_collide(StepArgs a, const int32_t* block_xyz) {
  __shared__ int32_t sh_nbr[27];
  const int64_t s = (int64_t)blockIdx.x * 256 + threadIdx.x;
  const int64_t b = ((int64_t)blockIdx.x * 256) >> 9;
  if (threadIdx.x < 27) sh_nbr[threadIdx.x] = a.block_nbr[b * 27 + threadIdx.x];
  __syncthreads();
  if (s >= a.nslot) return;
  const uint32_t code = a.block_bulk[b] ? 1u : a.site_code[s];
  if (code == 0) return;
  site_update<P>(a, sh_nbr, s, code, block_xyz);
}

template <int P>
__global__ void __launch_bounds__(256) k_stream_collide_list(StepArgs a, const int32_t* block_xyz) {
  const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (i >= a.list_count) return;
  const int64_t s = a.list[i];
  const int64_t b = s >> 9;
  const uint32_t code = a.block_bulk[b] ? 1u : a.site_code[s];
  if (code == 0) return;
  site_update<P>(a, a.block_nbr + b * 27, s, code, block_xyz);
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
    const double vi = St::load(fn, inv * p.stride + s, a);
    const double vd = St::load(fn, d * p.stride + s, a);
    St::store(fn, inv * p.stride + s, 2.0 * q * vi + (1.0 - 2.0 * q) * vd, a);
  } else {
    const float q = p.q[i];
    const float vi = St::load(fn, inv * p.stride + s, a);
    const float vd = St::load(fn, d * p.stride + s, a);
    St::store(fn, inv * p.stride + s, 2.f * q * vi + (1.f - 2.f * q) * vd, a);
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
      St::store(f0, d * ia.stride + s, ia.value[d], a);
      St::store(f1, d * ia.stride + s, ia.value[d], a);
    } else {
      St::store(f0, d * ia.stride + s, (float)ia.value[d], a);
      St::store(f1, d * ia.stride + s, (float)ia.value[d], a);
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
      St::store(f0, d * fa.stride + s, feq[d], a);
      St::store(f1, d * fa.stride + s, feq[d], a);
    } else {
      const float v = (float)(feq[d] - weight_d(d));
      St::store(f0, d * fa.stride + s, v, a);
      St::store(f1, d * fa.stride + s, v, a);
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
    double v = (double)St::load(f, d * ga.stride + s, a);
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
      St::store(f, d * ga.stride + s, v, a);
    else
      St::store(f, d * ga.stride + s, (float)(v - weight_d(d)), a);
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
      const double v = St::load(f, d * ga.stride + s, a);
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
    for (int d = 0; d < Q; ++d) g[d] = St::load(f, d * ga.stride + s, a);
    float dr, mx, my, mz;
    moments_dev(g, dr, mx, my, mz);
    const double rho = 1.0 + (double)dr;
    ga.rho[i] = rho;
    ga.u[3 * i] = (double)mx / rho;
    ga.u[3 * i + 1] = (double)my / rho;
    ga.u[3 * i + 2] = (double)mz / rho;
  }
}

// StabilityTester::PostSendToParent (Code/lb/StabilityTester.h:91-149) and
// ComputeRelativeDifference (:160-183) over all fluid slots, plus total mass.
// Fixed grid, one partial per CTA: the host sums the partials in a fixed order.
template <int P>
__global__ void __launch_bounds__(256) k_monitor(MonitorArgs ma) {
  using St = Store<P>;
  using S = typename St::S;
  StepArgs a{};
  a.fp16_scale = ma.fp16_scale;
  a.fp16_inv_scale = ma.fp16_inv_scale;
  const S* fc = static_cast<const S*>(ma.f_cur);
  const S* fp = static_cast<const S*>(ma.f_prev);
  double mass = 0.0, maxdu = 0.0, minf = 1.0e300;
  unsigned long long unstable = 0;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ma.nslot;
       s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t code = ma.block_bulk[s >> 9] ? 1u : ma.site_code[s];
    if (code == 0) continue;
    double rn = 0.0, xn = 0.0, yn = 0.0, zn = 0.0, ro = 0.0, xo = 0.0, yo = 0.0, zo = 0.0;
    bool bad = false;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      double vn = (double)St::load(fc, d * ma.stride + s, a);
      double vo = (double)St::load(fp, d * ma.stride + s, a);
      if constexpr (P != 0) {
        vn += weight_d(d);
        vo += weight_d(d);
      }
      if (!(vn > 0.0)) bad = true;
      minf = fmin(minf, vn);
      rn += vn;
      xn += (double)Lat::cx(d) * vn;
      yn += (double)Lat::cy(d) * vn;
      zn += (double)Lat::cz(d) * vn;
      ro += vo;
      xo += (double)Lat::cx(d) * vo;
      yo += (double)Lat::cy(d) * vo;
      zo += (double)Lat::cz(d) * vo;
    }
    if (bad) unstable++;
    mass += rn;
    const double dx = xn / rn - xo / ro, dy = yn / rn - yo / ro, dz = zn / rn - zo / ro;
    const double du = sqrt(dot3d(dx, dy, dz, dx, dy, dz));
    if (!(du <= maxdu)) maxdu = du;  // NaN-propagating max
  }
  // block reduction
  __shared__ double sh_mass[256], sh_max[256], sh_min[256];
  __shared__ unsigned long long sh_bad[256];
  sh_mass[threadIdx.x] = mass;
  sh_max[threadIdx.x] = maxdu;
  sh_min[threadIdx.x] = minf;
  sh_bad[threadIdx.x] = unstable;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh_mass[threadIdx.x] += sh_mass[threadIdx.x + w];
      const double m2 = sh_max[threadIdx.x + w];
      if (!(m2 <= sh_max[threadIdx.x])) sh_max[threadIdx.x] = m2;
      sh_min[threadIdx.x] = fmin(sh_min[threadIdx.x], sh_min[threadIdx.x + w]);
      sh_bad[threadIdx.x] += sh_bad[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ma.part_mass[blockIdx.x] = sh_mass[0];
    ma.part_max[blockIdx.x] = sh_max[0];
    ma.part_min[blockIdx.x] = sh_min[0];
    ma.part_bad[blockIdx.x] = sh_bad[0];
  }
}

}  // namespace hlbg

#define HLBG_INSTANTIATE(P)                                                                     \
  namespace hlbg {                                                                              \
  void launch_stream_collide_##P(const StepArgs& a, const int32_t* bxyz, cudaStream_t st) {     \
    if (a.list) {                                                                               \
      unsigned g = (unsigned)((a.list_count + 255) / 256);                                      \
      if (g) k_stream_collide_list<P><<<g, 256, 0, st>>>(a, bxyz);                              \
    } else {                                                                                    \
      unsigned g = (unsigned)((a.nslot + 255) / 256);                                           \
      if (g) k_stream_collide<P><<<g, 256, 0, st>>>(a, bxyz);                                   \
    }                                                                                           \
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
  void launch_monitor_##P(const MonitorArgs& ma, int grid, cudaStream_t st) {                   \
    k_monitor<P><<<grid, 256, 0, st>>>(ma);                                                     \
  }                                                                                             \
  }
