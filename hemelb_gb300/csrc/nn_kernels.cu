// BF16 tensor-core kernels of the warm-start surrogate (a 3-D convolutional U-Net
// that predicts velocity and pressure from geometry features).
//
// Activations are channels-last (N, D, H, W, C) BF16; weights are
// [27 taps][C_out][C_in] BF16 (C_in fastest) with FP32 master copies; every
// product accumulates in FP32 on the tensor cores (mma.sync m16n8k16 .bf16).
// A 3x3x3 convolution is an implicit GEMM: rows = output voxels, columns = output
// channels, reduction = 27 * C_in (C_in a multiple of 16, so a 16-wide reduction
// chunk never straddles two taps).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "../../include/hemelb_gb300_nn.h"

namespace {

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

struct Vox {
  int n, z, y, x;
};
__device__ __forceinline__ Vox unflat(int64_t m, int D, int H, int W) {
  Vox v;
  v.x = (int)(m % W);
  m /= W;
  v.y = (int)(m % H);
  m /= H;
  v.z = (int)(m % D);
  v.n = (int)(m / D);
  return v;
}

// ---------------------------------------------------------------------------
// Convolution (stride 1, zero padding 1, or a 1x1x1 "taps == 1" convolution).
// out[m, co] = act( sum_{tap, ci} in[m + off(tap), ci] * w[tap][co][ci] + bias[co] )
// One warp: 16 output voxels x (8 * NT) output channels.  flip: use tap 26 - t
// (the data-gradient convolution runs the flipped, transposed kernel).
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(128) k_conv3d(const __nv_bfloat16* __restrict__ in, int Cin,
                                                 const __nv_bfloat16* __restrict__ w,
                                                 const float* __restrict__ bias,
                                                 __nv_bfloat16* __restrict__ out, float* __restrict__ out_f32,
                                                 int Cout, int N, int D, int H, int W, int taps,
                                                 int relu) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * 4) + (threadIdx.x >> 5);
  const int64_t M = (int64_t)N * D * H * W;
  const int64_t m0 = (int64_t)warp * 16;
  const int co0 = blockIdx.y * 8 * NT;
  if (m0 >= M) return;
  const int g = lane >> 2, t = lane & 3;
  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  // the two output voxels whose A rows this lane loads
  const int64_t ma = m0 + g, mb = m0 + g + 8;
  const Vox va = unflat(ma < M ? ma : 0, D, H, W), vb = unflat(mb < M ? mb : 0, D, H, W);
  const int chunks = Cin / 16;
  for (int tap = 0; tap < taps; ++tap) {
    int dz = 0, dy = 0, dx = 0;
    if (taps == 27) {
      dz = tap / 9 - 1;
      dy = (tap / 3) % 3 - 1;
      dx = tap % 3 - 1;
    }
    const int za = va.z + dz, ya = va.y + dy, xa = va.x + dx;
    const int zb = vb.z + dz, yb = vb.y + dy, xb = vb.x + dx;
    const bool oka = ma < M && za >= 0 && za < D && ya >= 0 && ya < H && xa >= 0 && xa < W;
    const bool okb = mb < M && zb >= 0 && zb < D && yb >= 0 && yb < H && xb >= 0 && xb < W;
    const __nv_bfloat16* pa = in + ((((int64_t)va.n * D + za) * H + ya) * W + xa) * Cin;
    const __nv_bfloat16* pb = in + ((((int64_t)vb.n * D + zb) * H + yb) * W + xb) * Cin;
    const __nv_bfloat16* wt = w + (int64_t)tap * Cout * Cin;
    for (int c = 0; c < chunks; ++c) {
      const int ci = c * 16 + t * 2;
      uint32_t a[4];
      a[0] = oka ? ld2(pa + ci) : 0u;
      a[1] = okb ? ld2(pb + ci) : 0u;
      a[2] = oka ? ld2(pa + ci + 8) : 0u;
      a[3] = okb ? ld2(pb + ci + 8) : 0u;
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int co = co0 + j * 8 + g;
        uint32_t b[2];
        if (co < Cout) {
          b[0] = ld2(wt + (int64_t)co * Cin + ci);
          b[1] = ld2(wt + (int64_t)co * Cin + ci + 8);
        } else {
          b[0] = b[1] = 0u;
        }
        mma_bf16(acc[j], a, b);
      }
    }
  }
  // epilogue: rows g and g+8, columns 2t and 2t+1 of each 8-wide tile
#pragma unroll
  for (int j = 0; j < NT; ++j) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t m = m0 + g + 8 * h;
      if (m >= M) continue;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int co = co0 + j * 8 + 2 * t + e;
        if (co >= Cout) continue;
        float v = acc[j][2 * h + e] + (bias ? bias[co] : 0.f);
        if (relu && v < 0.f) v = 0.f;
        out[m * Cout + co] = __float2bfloat16_rn(v);
        if (out_f32) out_f32[m * Cout + co] = v;
      }
    }
  }
}

// Weight gradient: dw[tap][co][ci] += sum_m dy[m, co] * x[m + off(tap), ci] over a
// slice of voxels; one warp = one (tap, 16 co, 8 ci) tile; FP32 atomics join slices.
__global__ void __launch_bounds__(128) k_conv3d_wgrad(const __nv_bfloat16* __restrict__ x, int Cin,
                                                       const __nv_bfloat16* __restrict__ dy, int Cout,
                                                       float* __restrict__ dw, int N, int D, int H,
                                                       int W, int taps, int64_t slice) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int tiles_co = (Cout + 15) / 16, tiles_ci = Cin / 8;
  const int64_t tile = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
  const int64_t ntile = (int64_t)taps * tiles_co * tiles_ci;
  if (tile >= ntile) return;
  const int tap = (int)(tile / (tiles_co * tiles_ci));
  const int co0 = (int)((tile / tiles_ci) % tiles_co) * 16;
  const int ci0 = (int)(tile % tiles_ci) * 8;
  int dz = 0, dy_ = 0, dx = 0;
  if (taps == 27) {
    dz = tap / 9 - 1;
    dy_ = (tap / 3) % 3 - 1;
    dx = tap % 3 - 1;
  }
  const int64_t M = (int64_t)N * D * H * W;
  const int64_t mbeg = (int64_t)blockIdx.y * slice, mend = mbeg + slice < M ? mbeg + slice : M;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
  for (int64_t m = mbeg; m < mend; m += 16) {
    // A (16 co x 16 m): rows co0+g / co0+g+8, columns m+2t, m+2t+1, m+2t+8, m+2t+9
    // B (16 m x 8 ci): rows m+2t, m+2t+1, m+2t+8, m+2t+9, column ci0+g
    uint32_t a[4], b[2];
    __nv_bfloat16 av[8], bv[4];
    const int64_t mm[4] = {m + 2 * t, m + 2 * t + 1, m + 2 * t + 8, m + 2 * t + 9};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool in_m = mm[k] < mend;
      const int coa = co0 + g, cob = co0 + g + 8;
      av[2 * k] = (in_m && coa < Cout) ? dy[mm[k] * Cout + coa] : zero;
      av[2 * k + 1] = (in_m && cob < Cout) ? dy[mm[k] * Cout + cob] : zero;
      __nv_bfloat16 xv = zero;
      if (in_m) {
        Vox v = unflat(mm[k], D, H, W);
        const int z = v.z + dz, y = v.y + dy_, xx = v.x + dx;
        if (z >= 0 && z < D && y >= 0 && y < H && xx >= 0 && xx < W)
          xv = x[((((int64_t)v.n * D + z) * H + y) * W + xx) * Cin + ci0 + g];
      }
      bv[k] = xv;
    }
    a[0] = pack2(av[0], av[2]);  // row g: m+2t, m+2t+1
    a[1] = pack2(av[1], av[3]);  // row g+8
    a[2] = pack2(av[4], av[6]);  // row g: m+2t+8, m+2t+9
    a[3] = pack2(av[5], av[7]);
    b[0] = pack2(bv[0], bv[1]);
    b[1] = pack2(bv[2], bv[3]);
    mma_bf16(acc, a, b);
  }
  // D rows = co (g, g+8), columns = ci (2t, 2t+1)
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int co = co0 + g + 8 * h, ci = ci0 + 2 * t + e;
      if (co < Cout) atomicAdd(dw + ((int64_t)tap * Cout + co) * Cin + ci, acc[2 * h + e]);
    }
}

// ---------------------------------------------------------------------------
// Weight gradient of a 3x3x3 convolution, tiled through shared memory.
// A CTA owns a (16 C_out) x (16 NCI C_in) block of dW for all 27 taps and runs
// over a range of 4x4x8 voxel bricks: per brick it stages dY (128 voxels x 16 co)
// and X on the brick plus a one-voxel halo (6x6x10 voxels x 16 NCI ci) with
// cp.async (zero fill outside the volume), then each of the 8 warps accumulates
// its taps (warp, warp + 8, warp + 16, warp + 24) as
//   dW[tap] += dY^T (16 co x 16 voxels) * X_shifted (16 voxels x 8 ci)
// on mma.sync with both operands read by ldmatrix.trans (rows of 16 bytes; the
// row pitches of 48/80 bytes put the 8 rows of one ldmatrix in distinct banks).
// The FP32 accumulators are added to dW once per CTA (red.global.add).
// ---------------------------------------------------------------------------
constexpr int kBZ = 4, kBY = 4, kBX = 8, kBV = kBZ * kBY * kBX;  // brick
constexpr int kHZ = kBZ + 2, kHY = kBY + 2, kHX = kBX + 2, kHV = kHZ * kHY * kHX;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool ok) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int sz = ok ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}
__device__ __forceinline__ void ldsm_x4_trans(uint32_t* r, const void* smem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}
__device__ __forceinline__ void red_add(float* p, float v) {
  asm volatile("red.global.add.f32 [%0], %1;\n" ::"l"(p), "f"(v) : "memory");
}

template <int NCI>
__global__ void __launch_bounds__(256) k_wgrad_brick(const __nv_bfloat16* __restrict__ x, int Cin,
                                                      const __nv_bfloat16* __restrict__ dy, int Cout,
                                                      float* __restrict__ dw, int D, int H, int W, int nbz,
                                                      int nby, int nbx, int64_t nbricks, int bricks_per_cta) {
  constexpr int CIB = 16 * NCI, XS = CIB + 8, DS = 16 + 8, NTILE = 2 * NCI;
  __shared__ __align__(16) __nv_bfloat16 Xs[kHV * XS];
  __shared__ __align__(16) __nv_bfloat16 Ds[kBV * DS];
  const int co0 = blockIdx.y * 16, ci0 = blockIdx.z * CIB;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = lane >> 3, rr = lane & 7;
  float acc[4][NTILE][4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int nt = 0; nt < NTILE; ++nt) acc[j][nt][0] = acc[j][nt][1] = acc[j][nt][2] = acc[j][nt][3] = 0.f;
  const int64_t b0 = (int64_t)blockIdx.x * bricks_per_cta;
  const int64_t b1 = b0 + bricks_per_cta < nbricks ? b0 + bricks_per_cta : nbricks;
  for (int64_t b = b0; b < b1; ++b) {
    const int bx = (int)(b % nbx);
    int64_t r = b / nbx;
    const int by = (int)(r % nby);
    r /= nby;
    const int bz = (int)(r % nbz);
    const int n = (int)(r / nbz);
    const int z0 = bz * kBZ, y0 = by * kBY, x0 = bx * kBX;
    for (int c = threadIdx.x; c < kBV * 2; c += 256) {
      const int v = c >> 1, part = c & 1;
      const int z = z0 + v / (kBY * kBX), y = y0 + (v / kBX) % kBY, xx = x0 + v % kBX;
      const bool ok = z < D && y < H && xx < W;
      const __nv_bfloat16* src = ok ? dy + ((((int64_t)n * D + z) * H + y) * W + xx) * Cout + co0 + part * 8 : dy;
      cp_async16(&Ds[v * DS + part * 8], src, ok);
    }
    for (int c = threadIdx.x; c < kHV * NTILE; c += 256) {
      const int h = c / NTILE, part = c % NTILE;
      const int z = z0 + h / (kHY * kHX) - 1, y = y0 + (h / kHX) % kHY - 1, xx = x0 + h % kHX - 1;
      const bool ok = z >= 0 && z < D && y >= 0 && y < H && xx >= 0 && xx < W;
      const __nv_bfloat16* src = ok ? x + ((((int64_t)n * D + z) * H + y) * W + xx) * Cin + ci0 + part * 8 : x;
      cp_async16(&Xs[h * XS + part * 8], src, ok);
    }
    cp_async_wait_all();
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < kBV / 16; ++s) {
      uint32_t a[4];
      ldsm_x4_trans(a, &Ds[(16 * s + rr + ((q >> 1) << 3)) * DS + (q & 1) * 8]);
      // the voxel whose X row this lane addresses for the B operand
      const int vb = 16 * s + rr + ((q & 1) << 3);
      const int vz = vb / (kBY * kBX), vy = (vb / kBX) % kBY, vx = vb % kBX;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int tap = warp + 8 * j;
        if (tap < 27) {
          const int h = ((vz + tap / 9) * kHY + (vy + (tap / 3) % 3)) * kHX + (vx + tap % 3);
#pragma unroll
          for (int nt = 0; nt < NTILE; nt += 2) {
            uint32_t bf[4];
            ldsm_x4_trans(bf, &Xs[h * XS + (nt + (q >> 1)) * 8]);
            mma_bf16(acc[j][nt], a, bf);
            mma_bf16(acc[j][nt + 1], a, bf + 2);
          }
        }
      }
    }
    __syncthreads();
  }
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int tap = warp + 8 * j;
    if (tap < 27) {
#pragma unroll
      for (int nt = 0; nt < NTILE; ++nt)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
          for (int e = 0; e < 2; ++e)
            red_add(dw + ((int64_t)tap * Cout + co0 + g + 8 * hh) * Cin + ci0 + nt * 8 + 2 * t + e,
                    acc[j][nt][2 * hh + e]);
    }
  }
}

// ---------------------------------------------------------------------------
// 3x3x3 convolution tiled through shared memory.  A CTA computes one 4x4x8 voxel
// brick (8 warps x 16 voxels) for 16 NCO output channels.  For each 16-channel
// slice of the input it stages X on the brick plus halo (6x6x10 voxels) with
// cp.async (zero fill outside the volume), and for each plane of 9 taps the
// weights W[tap][co][ci] of that slice; the warps then accumulate
//   out (16 voxels x 8 co) += X_shifted (16 voxels x 16 ci) * W[tap]^T (16 ci x 8 co)
// with A read by ldmatrix from the halo rows of the shifted voxels and B by
// ldmatrix from the weight rows.  Epilogue: bias, optional ReLU, BF16 (and FP32).
// ---------------------------------------------------------------------------
template <int NCO>
__global__ void __launch_bounds__(256) k_conv_brick(const __nv_bfloat16* __restrict__ in, int Cin,
                                                     const __nv_bfloat16* __restrict__ w,
                                                     const float* __restrict__ bias,
                                                     __nv_bfloat16* __restrict__ out, float* __restrict__ out_f32,
                                                     int Cout, int D, int H, int W, int nbz, int nby, int nbx,
                                                     int relu) {
  constexpr int COB = 16 * NCO, NTILE = 2 * NCO, XS = 24, WS = 24;
  __shared__ __align__(16) __nv_bfloat16 Xs[kHV * XS];
  __shared__ __align__(16) __nv_bfloat16 Ws[9 * COB * WS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = lane >> 3, rr = lane & 7;
  const int co0 = blockIdx.y * COB;
  int64_t r = blockIdx.x;
  const int bx = (int)(r % nbx);
  r /= nbx;
  const int by = (int)(r % nby);
  r /= nby;
  const int bz = (int)(r % nbz);
  const int n = (int)(r / nbz);
  const int z0 = bz * kBZ, y0 = by * kBY, x0 = bx * kBX;
  float acc[NTILE][4];
#pragma unroll
  for (int nt = 0; nt < NTILE; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
  // this lane's A row: voxel 16 warp + rr + 8 (q & 1) of the brick, channel half q >> 1
  const int va = 16 * warp + rr + ((q & 1) << 3);
  const int az = va / (kBY * kBX), ay = (va / kBX) % kBY, ax = va % kBX;
  for (int ci0 = 0; ci0 < Cin; ci0 += 16) {
    for (int c = threadIdx.x; c < kHV * 2; c += 256) {
      const int h = c >> 1, part = c & 1;
      const int z = z0 + h / (kHY * kHX) - 1, y = y0 + (h / kHX) % kHY - 1, xx = x0 + h % kHX - 1;
      const bool ok = z >= 0 && z < D && y >= 0 && y < H && xx >= 0 && xx < W;
      const __nv_bfloat16* src = ok ? in + ((((int64_t)n * D + z) * H + y) * W + xx) * Cin + ci0 + part * 8 : in;
      cp_async16(&Xs[h * XS + part * 8], src, ok);
    }
#pragma unroll 1
    for (int plane = 0; plane < 3; ++plane) {
      for (int c = threadIdx.x; c < 9 * COB * 2; c += 256) {
        const int row = c >> 1, part = c & 1;  // row = tap-in-plane * COB + co
        const int tp = row / COB, co = row % COB;
        const __nv_bfloat16* src = w + ((int64_t)(plane * 9 + tp) * Cout + co0 + co) * Cin + ci0 + part * 8;
        cp_async16(&Ws[row * WS + part * 8], src, true);
      }
      cp_async_wait_all();
      __syncthreads();
#pragma unroll
      for (int tp = 0; tp < 9; ++tp) {
        const int h = ((az + plane) * kHY + (ay + tp / 3)) * kHX + (ax + tp % 3);
        uint32_t a[4];
        {
          const unsigned sa = (unsigned)__cvta_generic_to_shared(&Xs[h * XS + (q >> 1) * 8]);
          asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                       : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
                       : "r"(sa));
        }
#pragma unroll
        for (int nt = 0; nt < NTILE; nt += 2) {
          uint32_t b[4];
          const unsigned sb =
              (unsigned)__cvta_generic_to_shared(&Ws[(tp * COB + (nt + (q >> 1)) * 8 + rr) * WS + (q & 1) * 8]);
          asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                       : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3])
                       : "r"(sb));
          mma_bf16(acc[nt], a, b);
          mma_bf16(acc[nt + 1], a, b + 2);
        }
      }
      __syncthreads();
    }
  }
  // epilogue: rows g and g + 8 of the warp's 16 voxels, columns 2t, 2t + 1 of each tile
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int v = 16 * warp + g + 8 * hh;
    const int z = z0 + v / (kBY * kBX), y = y0 + (v / kBX) % kBY, xx = x0 + v % kBX;
    if (z >= D || y >= H || xx >= W) continue;
    const int64_t m = (((int64_t)n * D + z) * H + y) * W + xx;
#pragma unroll
    for (int nt = 0; nt < NTILE; ++nt)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int co = co0 + nt * 8 + 2 * t + e;
        float vv = acc[nt][2 * hh + e] + (bias ? bias[co] : 0.f);
        if (relu && vv < 0.f) vv = 0.f;
        out[m * Cout + co] = __float2bfloat16_rn(vv);
        if (out_f32) out_f32[m * Cout + co] = vv;
      }
  }
}

// Flipped, transposed weights for the data-gradient convolution:
// wt[26 - tap][ci][co] = w[tap][co][ci]
__global__ void k_flip_transpose(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt,
                                 int Cout, int Cin, int taps) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)taps * Cout * Cin;
  if (i >= n) return;
  const int ci = (int)(i % Cin), co = (int)((i / Cin) % Cout), tap = (int)(i / ((int64_t)Cin * Cout));
  wt[((int64_t)(taps - 1 - tap) * Cin + ci) * Cout + co] = w[i];
}

// ReLU gradient in place: dy *= (y > 0)
__global__ void k_relu_bwd(__nv_bfloat16* __restrict__ dy, const __nv_bfloat16* __restrict__ y, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(__bfloat162float(y[i]) > 0.f)) dy[i] = __float2bfloat16_rn(0.f);
}

// Bias gradient: db[c] += sum_m dy[m, c]
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dy, float* __restrict__ db, int64_t M, int C) {
  const int c = blockIdx.y;
  float s = 0.f;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x)
    s += __bfloat162float(dy[m * C + c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(db + c, s);
}

// 2x average pooling (channels last) and its gradient
__global__ void k_pool2(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int N, int D,
                        int H, int W, int C) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int d = D / 2, h = H / 2, w = W / 2;
  const int64_t n = (int64_t)N * d * h * w * C;
  if (i >= n) return;
  const int c = (int)(i % C);
  Vox v = unflat(i / C, d, h, w);
  float s = 0.f;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int e = 0; e < 2; ++e)
        s += __bfloat162float(x[((((int64_t)v.n * D + 2 * v.z + a) * H + 2 * v.y + b) * W + 2 * v.x + e) * C + c]);
  y[i] = __float2bfloat16_rn(0.125f * s);
}
__global__ void k_pool2_bwd(const __nv_bfloat16* __restrict__ dy, __nv_bfloat16* __restrict__ dx, int N,
                            int D, int H, int W, int C) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)N * D * H * W * C;
  if (i >= n) return;
  const int c = (int)(i % C);
  Vox v = unflat(i / C, D, H, W);
  dx[i] = __float2bfloat16_rn(
      0.125f * __bfloat162float(dy[((((int64_t)v.n * (D / 2) + v.z / 2) * (H / 2) + v.y / 2) * (W / 2) + v.x / 2) * C + c]));
}
// nearest 2x upsampling and its gradient (sum over the 8 copies)
__global__ void k_up2(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int N, int D,
                      int H, int W, int C) {  // D, H, W: output (fine) sizes
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)N * D * H * W * C;
  if (i >= n) return;
  const int c = (int)(i % C);
  Vox v = unflat(i / C, D, H, W);
  y[i] = x[((((int64_t)v.n * (D / 2) + v.z / 2) * (H / 2) + v.y / 2) * (W / 2) + v.x / 2) * C + c];
}
__global__ void k_up2_bwd(const __nv_bfloat16* __restrict__ dy, __nv_bfloat16* __restrict__ dx, int N, int D,
                          int H, int W, int C) {  // D, H, W: coarse sizes
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)N * D * H * W * C;
  if (i >= n) return;
  const int c = (int)(i % C);
  Vox v = unflat(i / C, D, H, W);
  float s = 0.f;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int e = 0; e < 2; ++e)
        s += __bfloat162float(dy[((((int64_t)v.n * 2 * D + 2 * v.z + a) * 2 * H + 2 * v.y + b) * 2 * W + 2 * v.x + e) * C + c]);
  dx[i] = __float2bfloat16_rn(s);
}
// channel concatenation y = [a | b] and its split
__global__ void k_concat(const __nv_bfloat16* __restrict__ a, int Ca, const __nv_bfloat16* __restrict__ b,
                         int Cb, __nv_bfloat16* __restrict__ y, int64_t M) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int C = Ca + Cb;
  if (i >= M * C) return;
  const int64_t m = i / C;
  const int c = (int)(i % C);
  y[i] = c < Ca ? a[m * Ca + c] : b[m * Cb + (c - Ca)];
}
__global__ void k_split(const __nv_bfloat16* __restrict__ y, __nv_bfloat16* __restrict__ da, int Ca,
                        __nv_bfloat16* __restrict__ db, int Cb, int64_t M, int accumulate_b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int C = Ca + Cb;
  if (i >= M * C) return;
  const int64_t m = i / C;
  const int c = (int)(i % C);
  if (c < Ca) {
    da[m * Ca + c] = y[i];
  } else {
    const int64_t j = m * Cb + (c - Ca);
    db[j] = accumulate_b ? __float2bfloat16_rn(__bfloat162float(db[j]) + __bfloat162float(y[i])) : y[i];
  }
}
// in-place add: a += b
__global__ void k_add(__nv_bfloat16* __restrict__ a, const __nv_bfloat16* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = __float2bfloat16_rn(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}
// masked mean-squared error over voxels with mask > 0; returns loss sum in *loss
// and dy = 2 (pred - target) mask / count
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ target,
                      const float* __restrict__ mask, __nv_bfloat16* __restrict__ dpred, float* __restrict__ loss,
                      int64_t M, int C, float inv_count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < M * C) {
    const float mk = mask[i / C];
    const float d = (pred[i] - target[i]) * mk;
    l = d * d;
    dpred[i] = __float2bfloat16_rn(2.f * d * inv_count);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}
// Adam on FP32 master weights, refreshing the BF16 copy
__global__ void k_adam(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, int64_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16_rn(wi);
}
__global__ void k_f32_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

int check_launch() { return cudaGetLastError() == cudaSuccess ? 0 : 3; }

}  // namespace

extern "C" {

int hlbg_nn_conv3d(const void* in, int32_t cin, const void* w, const float* bias, void* out, float* out_f32,
                   int32_t cout, int32_t n, int32_t d, int32_t h, int32_t wd, int32_t taps, int32_t relu,
                   void* stream) {
  if (!in || !w || !out || cin <= 0 || cin % 16 || cout <= 0 || (taps != 27 && taps != 1)) return 1;
  const int64_t M = (int64_t)n * d * h * wd;
  cudaStream_t st = (cudaStream_t)stream;
  if (taps == 27 && cout % 16 == 0) {
    const int nbz = (d + kBZ - 1) / kBZ, nby = (h + kBY - 1) / kBY, nbx = (wd + kBX - 1) / kBX;
    const int64_t nbricks = (int64_t)n * nbz * nby * nbx;
    auto I = (const __nv_bfloat16*)in;
    auto Wt = (const __nv_bfloat16*)w;
    auto O = (__nv_bfloat16*)out;
    if (cout % 64 == 0) {
      dim3 grid((unsigned)nbricks, (unsigned)(cout / 64));
      k_conv_brick<4><<<grid, 256, 0, st>>>(I, cin, Wt, bias, O, out_f32, cout, d, h, wd, nbz, nby, nbx, relu);
    } else if (cout % 32 == 0) {
      dim3 grid((unsigned)nbricks, (unsigned)(cout / 32));
      k_conv_brick<2><<<grid, 256, 0, st>>>(I, cin, Wt, bias, O, out_f32, cout, d, h, wd, nbz, nby, nbx, relu);
    } else {
      dim3 grid((unsigned)nbricks, (unsigned)(cout / 16));
      k_conv_brick<1><<<grid, 256, 0, st>>>(I, cin, Wt, bias, O, out_f32, cout, d, h, wd, nbz, nby, nbx, relu);
    }
    return check_launch();
  }
  const int warps = (int)((M + 15) / 16);
  dim3 grid((unsigned)((warps + 3) / 4), 1);
  auto I = (const __nv_bfloat16*)in;
  auto Wt = (const __nv_bfloat16*)w;
  auto O = (__nv_bfloat16*)out;
  if (cout % 32 == 0) {
    grid.y = cout / 32;
    k_conv3d<4><<<grid, 128, 0, st>>>(I, cin, Wt, bias, O, out_f32, cout, n, d, h, wd, taps, relu);
  } else {
    grid.y = (cout + 7) / 8;
    k_conv3d<1><<<grid, 128, 0, st>>>(I, cin, Wt, bias, O, out_f32, cout, n, d, h, wd, taps, relu);
  }
  return check_launch();
}

int hlbg_nn_conv3d_wgrad(const void* x, int32_t cin, const void* dy, int32_t cout, float* dw, int32_t n,
                         int32_t d, int32_t h, int32_t wd, int32_t taps, void* stream) {
  if (!x || !dy || !dw || cin % 8 || cout <= 0) return 1;
  if (taps == 27 && cin % 16 == 0 && cout % 16 == 0) {
    const int nbz = (d + kBZ - 1) / kBZ, nby = (h + kBY - 1) / kBY, nbx = (wd + kBX - 1) / kBX;
    const int64_t nbricks = (int64_t)n * nbz * nby * nbx;
    const int nci = cin % 32 == 0 ? 2 : 1;
    const int gy = cout / 16, gz = cin / (16 * nci);
    // about four waves of 2 CTAs per SM over 152 SMs
    int64_t bpc = (nbricks * gy * gz + 1215) / 1216;
    if (bpc < 1) bpc = 1;
    dim3 grid((unsigned)((nbricks + bpc - 1) / bpc), (unsigned)gy, (unsigned)gz);
    auto X = (const __nv_bfloat16*)x;
    auto DY = (const __nv_bfloat16*)dy;
    if (nci == 2)
      k_wgrad_brick<2><<<grid, 256, 0, (cudaStream_t)stream>>>(X, cin, DY, cout, dw, d, h, wd, nbz, nby, nbx,
                                                                nbricks, (int)bpc);
    else
      k_wgrad_brick<1><<<grid, 256, 0, (cudaStream_t)stream>>>(X, cin, DY, cout, dw, d, h, wd, nbz, nby, nbx,
                                                                nbricks, (int)bpc);
    return check_launch();
  }
  const int64_t M = (int64_t)n * d * h * wd;
  const int64_t ntile = (int64_t)taps * ((cout + 15) / 16) * (cin / 8);
  const int64_t slice = 4096;
  dim3 grid((unsigned)((ntile + 3) / 4), (unsigned)((M + slice - 1) / slice));
  k_conv3d_wgrad<<<grid, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)x, cin, (const __nv_bfloat16*)dy,
                                                        cout, dw, n, d, h, wd, taps, slice);
  return check_launch();
}

int hlbg_nn_flip_transpose(const void* w, void* wt, int32_t cout, int32_t cin, int32_t taps, void* stream) {
  const int64_t n = (int64_t)taps * cout * cin;
  k_flip_transpose<<<blocks(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)w, (__nv_bfloat16*)wt,
                                                                  cout, cin, taps);
  return check_launch();
}

int hlbg_nn_relu_bwd(void* dy, const void* y, int64_t n, void* stream) {
  k_relu_bwd<<<blocks(n), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16*)dy, (const __nv_bfloat16*)y, n);
  return check_launch();
}

int hlbg_nn_bias_grad(const void* dy, float* db, int64_t m, int32_t c, void* stream) {
  dim3 grid((unsigned)std::min<int64_t>((m + 255) / 256, 512), (unsigned)c);
  k_bias_grad<<<grid, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)dy, db, m, c);
  return check_launch();
}

int hlbg_nn_pool2(const void* x, void* y, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, int32_t backward,
                  void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (!backward) {
    const int64_t cnt = (int64_t)n * (d / 2) * (h / 2) * (w / 2) * c;
    k_pool2<<<blocks(cnt), 256, 0, st>>>((const __nv_bfloat16*)x, (__nv_bfloat16*)y, n, d, h, w, c);
  } else {  // x = dy (coarse), y = dx (fine); d, h, w fine sizes
    const int64_t cnt = (int64_t)n * d * h * w * c;
    k_pool2_bwd<<<blocks(cnt), 256, 0, st>>>((const __nv_bfloat16*)x, (__nv_bfloat16*)y, n, d, h, w, c);
  }
  return check_launch();
}

int hlbg_nn_up2(const void* x, void* y, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, int32_t backward,
                void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t cnt = (int64_t)n * d * h * w * c;
  if (!backward)  // d, h, w fine sizes
    k_up2<<<blocks(cnt), 256, 0, st>>>((const __nv_bfloat16*)x, (__nv_bfloat16*)y, n, d, h, w, c);
  else  // x = dy (fine), y = dx (coarse); d, h, w coarse sizes
    k_up2_bwd<<<blocks(cnt), 256, 0, st>>>((const __nv_bfloat16*)x, (__nv_bfloat16*)y, n, d, h, w, c);
  return check_launch();
}

int hlbg_nn_concat(const void* a, int32_t ca, const void* b, int32_t cb, void* y, int64_t m, void* stream) {
  k_concat<<<blocks(m * (ca + cb)), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)a, ca,
                                                                      (const __nv_bfloat16*)b, cb,
                                                                      (__nv_bfloat16*)y, m);
  return check_launch();
}

int hlbg_nn_split(const void* y, void* da, int32_t ca, void* db, int32_t cb, int64_t m, int32_t accumulate_b,
                  void* stream) {
  k_split<<<blocks(m * (ca + cb)), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)y, (__nv_bfloat16*)da,
                                                                     ca, (__nv_bfloat16*)db, cb, m, accumulate_b);
  return check_launch();
}

int hlbg_nn_add(void* a, const void* b, int64_t n, void* stream) {
  k_add<<<blocks(n), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16*)a, (const __nv_bfloat16*)b, n);
  return check_launch();
}

int hlbg_nn_mse(const float* pred, const float* target, const float* mask, void* dpred, float* loss, int64_t m,
                int32_t c, float inv_count, void* stream) {
  k_mse<<<blocks(m * c), 256, 0, (cudaStream_t)stream>>>(pred, target, mask, (__nv_bfloat16*)dpred, loss, m, c,
                                                         inv_count);
  return check_launch();
}

int hlbg_nn_adam(float* w, void* wb, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                 float eps, int32_t step, void* stream) {
  const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
  k_adam<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16*)wb, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return check_launch();
}

int hlbg_nn_to_bf16(const float* x, void* y, int64_t n, void* stream) {
  k_f32_to_bf16<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(x, (__nv_bfloat16*)y, n);
  return check_launch();
}

}  // extern "C"
