// 3x3x3 convolution of the warm-start surrogate on the fifth-generation tensor
// cores: tcgen05.mma with the accumulators in tensor memory (TMEM), operands staged
// in shared memory by TMA (cp.async.bulk.tensor), completion tracked on mbarriers.
//
// Implicit GEMM.  One CTA computes an output tile of 8 (x) x 16 (y) x BZ (z)
// voxels for all C_out output channels: BZ MMAs of M = 128 rows (one z-plane each,
// N = C_out, a multiple of 16 up to 256), each with its FP32 accumulator in its
// own TMEM columns.  The reduction runs over C_in in slices of 16 channels and,
// within a slice, over the 27 taps (K = 16 per MMA):
//  * per slice, one TMA load brings the input tile with its halo -- 10 x 18 x 4
//    voxels, 16 channels, in two planes of 8 channels (16-byte rows), positions
//    outside the volume read as zeros, which is the convolution's zero padding --
//    and every tap's A operand is a shared-memory descriptor into that one tile:
//    the core-matrix layout without swizzle puts the 8 rows of a core matrix (8
//    consecutive x) in 128 contiguous bytes and steps 160 bytes (one halo row of 10
//    voxels) from one y to the next, so a tap is only a different start address;
//  * per three taps (one x-row of the stencil; nine -- a z-plane of it -- when
//    C_out > 128), a TMA load brings their weights for the slice (3 or 9 x C_out
//    rows of 32 bytes, in the 32-byte swizzle) into a ring of stages: each tap
//    feeds one MMA per z-plane (BZ = 2 z-planes, each accumulator C_out TMEM
//    columns).
// One thread issues the copies (waiting for a buffer to be free), one thread
// issues the MMAs (waiting for it to be full) and returns each buffer with
// tcgen05.commit.  The four warps then read the accumulators from TMEM (warp w
// owns TMEM lanes 32w..32w+31: the rows y = 4w..4w+3 of the tile), add the bias,
// apply the ReLU and store BF16 (and optionally FP32) channels-last.
//
// Every wait is bounded: a wait that gives up sets g_tc_err (read back by
// hlbg_nn_tc_error), the CTA waits (bounded) for the copies it issued, frees its
// TMEM and returns.  Tensor maps cover this GPU's own memory only (no multicast).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <mutex>

#include "../../include/hemelb_gb300_nn.h"

namespace {

constexpr int kM = 128;                      // rows of one MMA: an 8 x 16 plane of voxels
constexpr int kHX = 10, kHY = 18;            // input tile with its halo in x and y
// z-planes per CTA (MMAs per weight stage): BZ; the input tile is BZ + 2 deep
template <int BZ>
struct Tile {
  static constexpr int kHZ = BZ + 2;
  static constexpr int kAPlane = kHX * kHY * kHZ * 16;  // bytes of 8 channels of the tile
  static constexpr int kATile = 2 * kAPlane;            // one 16-channel slice
};
constexpr int kMaxBStages = 16;
constexpr int64_t kWaitLimit = 1ll << 22;    // polls before a wait gives up

__device__ int g_tc_err;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int64_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1,
                                            int c2, int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6, "
      "%7}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand in the core-matrix layout
// without swizzle (core matrix: 8 rows x 16 bytes, contiguous): start address,
// leading-dimension offset = bytes between the two core matrices along K (the two
// 8-channel planes), stride-dimension offset = bytes between consecutive 8-row
// groups, the descriptor version of tcgen05 (1) and layout code 0 (no swizzle).
__device__ __forceinline__ uint64_t desc_noswizzle(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  return d;
}

// The same for a K-major tile of 32-byte rows (16 BF16) in the 32-byte swizzle
// (the layout TMA writes with CU_TENSOR_MAP_SWIZZLE_32B): 8-row groups 256 bytes
// apart, leading offset unused (1 by convention), layout code 6.
__device__ __forceinline__ uint64_t desc_sw32(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)((256u >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)6u << 61;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = n, M = 128.
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct TcParams {
  int Cin, Cout, N, D, H, W, taps, relu;
  int nbx, nby, nbz;
  int b_stages;          // weight stages in the ring (<= kMaxBStages)
  int tps;               // taps per weight stage (3: one x-row of taps; 1 for a 1x1x1 convolution)
  int b_stride;          // bytes of one weight stage (C_out x 32, rounded up to 128)
  uint32_t ncols;        // TMEM columns allocated (a power of two >= 32 and >= 2 C_out)
  const float* bias;     // [C_out] or null
  __nv_bfloat16* out;    // [voxels][C_out]
  float* out_f32;        // [voxels][C_out] or null
};

template <int BZ>
__global__ void __launch_bounds__(128, 1) k_conv3d_tc(const __grid_constant__ CUtensorMap tin,
                                                      const __grid_constant__ CUtensorMap tw, TcParams p) {
  constexpr int kBZ = BZ, kAPlane = Tile<BZ>::kAPlane, kATile = Tile<BZ>::kATile;
  constexpr int kARegion = (2 * kATile + 1023) / 1024 * 1024;  // the weight stages start 1024-aligned
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // [input slice buffer 0 | buffer 1 | weight stages | barriers | TMEM address]
  const uint32_t a_base = smem_u32(base);
  const uint32_t b_base = a_base + kARegion;
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kARegion + p.b_stages * p.b_stride);
  const uint32_t afull0 = smem_u32(bars), aempty0 = afull0 + 16, bfull0 = afull0 + 32,
                 bempty0 = bfull0 + 8 * kMaxBStages, done = bempty0 + 8 * kMaxBStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 4 + 2 * kMaxBStages + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  int bid = blockIdx.x;
  const int bx = bid % p.nbx;
  bid /= p.nbx;
  const int by = bid % p.nby;
  bid /= p.nby;
  const int bz = bid % p.nbz;
  const int n = bid / p.nbz;
  const int x0 = bx * 8, y0 = by * 16, z0 = bz * kBZ;

  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(afull0 + 8 * s, 1);
      mbar_init(aempty0 + 8 * s, 1);
    }
    for (int s = 0; s < p.b_stages; ++s) {
      mbar_init(bfull0 + 8 * s, 1);
      mbar_init(bempty0 + 8 * s, 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(p.ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const int kslices = p.Cin / 16;
  const int SB = p.b_stages;
  const int groups = p.taps / p.tps;  // weight stages per channel slice
  const uint32_t b_bytes = (uint32_t)(p.tps * p.Cout * 32);
  if (warp == 0 && lane == 0) {
    // producer
    int a_issued = 0, b_issued = 0;
    bool ok = true;
    for (int ks = 0; ks < kslices && ok; ++ks) {
      const int a = ks & 1;
      if (!mbar_wait(aempty0 + 8 * a, ((uint32_t)(ks >> 1) & 1u) ^ 1u)) {
        ok = false;
        break;
      }
      const uint32_t sa = a_base + a * kATile;
      mbar_expect_tx(afull0 + 8 * a, (uint32_t)kATile);
      tma_load_5d(sa, &tin, afull0 + 8 * a, ks * 16, x0 - 1, y0 - 1, z0 - 1, n);
      tma_load_5d(sa + kAPlane, &tin, afull0 + 8 * a, ks * 16 + 8, x0 - 1, y0 - 1, z0 - 1, n);
      ++a_issued;
      for (int tg = 0; tg < groups; ++tg) {
        const int i = ks * groups + tg, s = i % SB;
        if (!mbar_wait(bempty0 + 8 * s, ((uint32_t)(i / SB) & 1u) ^ 1u)) {
          ok = false;
          break;
        }
        const uint32_t sb = b_base + s * p.b_stride;
        mbar_expect_tx(bfull0 + 8 * s, b_bytes);
        tma_load_3d(sb, &tw, bfull0 + 8 * s, ks * 16, 0, tg * p.tps);
        ++b_issued;
      }
    }
    if (!ok) {
      atomicExch(&g_tc_err, 1);
      // the copies in flight land before the CTA's shared memory goes away
      for (int j = a_issued > 2 ? a_issued - 2 : 0; j < a_issued; ++j)
        mbar_wait(afull0 + 8 * (j & 1), (uint32_t)(j >> 1) & 1u);
      for (int j = b_issued > SB ? b_issued - SB : 0; j < b_issued; ++j)
        mbar_wait(bfull0 + 8 * (j % SB), (uint32_t)(j / SB) & 1u);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    const uint32_t idesc = idesc_bf16(p.Cout);
    bool ok = true;
    for (int ks = 0; ks < kslices && ok; ++ks) {
      const int a = ks & 1;
      if (!mbar_wait(afull0 + 8 * a, (uint32_t)(ks >> 1) & 1u)) {
        ok = false;
        break;
      }
      const uint32_t sa = a_base + a * kATile;
      for (int tg = 0; tg < groups; ++tg) {
        const int i = ks * groups + tg, s = i % SB;
        if (!mbar_wait(bfull0 + 8 * s, (uint32_t)(i / SB) & 1u)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int j = 0; j < p.tps; ++j) {
          const int t = tg * p.tps + j;
          // the tap's offset in the halo tile (a 1x1x1 convolution uses the centre)
          const int dz = p.taps == 27 ? t / 9 : 1, dy = p.taps == 27 ? (t / 3) % 3 : 1,
                    dx = p.taps == 27 ? t % 3 : 1;
          const uint64_t bdesc = desc_sw32(b_base + s * p.b_stride + (uint32_t)(j * p.Cout * 32));
#pragma unroll
          for (int pz = 0; pz < kBZ; ++pz) {
            const uint32_t start = sa + (uint32_t)((((pz + dz) * kHY + dy) * kHX + dx) * 16);
            umma_bf16(tmem + (uint32_t)(pz * p.Cout), desc_noswizzle(start, (uint32_t)kAPlane, 160u), bdesc,
                      idesc, (ks | t) != 0 ? 1u : 0u);
          }
        }
        umma_commit(bempty0 + 8 * s);
      }
      umma_commit(aempty0 + 8 * a);
    }
    if (!ok) atomicExch(&g_tc_err, 1);
    umma_commit(done);  // arrives once every MMA issued above has completed
  }
  __syncwarp();

  // epilogue: TMEM lane = voxel row of a plane (x = row % 8, y = row / 8), columns
  // [pz C_out, (pz + 1) C_out) = the output channels of z-plane pz
  const bool finished = mbar_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!finished && lane == 0) atomicExch(&g_tc_err, 1);
  const int row = warp * 32 + lane;
  const int x = x0 + (row & 7), y = y0 + (row >> 3);
  for (int pz = 0; pz < kBZ; ++pz) {
    const int z = z0 + pz;
    const bool inside = finished && x < p.W && y < p.H && z < p.D;
    const int64_t vox = (((int64_t)n * p.D + z) * p.H + y) * p.W + x;
    for (int c0 = 0; c0 < p.Cout; c0 += 16) {
      uint32_t r[16];
      __syncwarp();  // tcgen05.ld is warp-collective: every lane, converged
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(pz * p.Cout + c0), r);
      if (!inside) continue;
      float v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        v[j] = __uint_as_float(r[j]) + (p.bias ? __ldg(p.bias + c0 + j) : 0.f);
        if (p.relu) v[j] = fmaxf(v[j], 0.f);
      }
      uint32_t packed[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        packed[j] = *reinterpret_cast<const uint32_t*>(&h);
      }
      uint4* dst = reinterpret_cast<uint4*>(p.out + vox * p.Cout + c0);
      dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
      dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
      if (p.out_f32) {
        float4* df = reinterpret_cast<float4*>(p.out_f32 + vox * p.Cout + c0);
#pragma unroll
        for (int j = 0; j < 4; ++j) df[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.ncols) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  });
  return fn;
}

}  // namespace

extern "C" {

int hlbg_nn_conv3d_tc(const void* in, int32_t cin, const void* w, const float* bias, void* out, float* out_f32,
                      int32_t cout, int32_t n, int32_t d, int32_t h, int32_t wd, int32_t taps, int32_t relu,
                      void* stream) {
  if (!in || !w || !out || cin <= 0 || cin % 16 || cout < 16 || cout > 256 || cout % 16 || n <= 0 || d <= 0 ||
      h <= 0 || wd <= 0 || (taps != 27 && taps != 1))
    return 1;
  // TMA: 16-byte aligned base addresses; the output is stored in 16-byte vectors
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(w) | reinterpret_cast<uintptr_t>(out) |
       reinterpret_cast<uintptr_t>(out_f32)) & 15u)
    return 1;
  auto enc = encode_fn();
  if (!enc) return 3;
  // z-planes per CTA.  Four planes per weight stage (C_out <= 128) measured slower
  // than two on the network's shapes (fewer CTAs per SM), so two throughout.
  const int bz = 2;
  CUtensorMap tin, tw;
  {
    const cuuint64_t dims[5] = {(cuuint64_t)cin, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
    const cuuint64_t strides[4] = {(cuuint64_t)cin * 2, (cuuint64_t)cin * 2 * wd, (cuuint64_t)cin * 2 * wd * h,
                                   (cuuint64_t)cin * 2 * wd * h * d};
    const cuuint32_t box[5] = {8, (cuuint32_t)kHX, (cuuint32_t)kHY, (cuuint32_t)(bz + 2), 1};
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    if (enc(&tin, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(in), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 3;
  }
  {
    const cuuint64_t dims[3] = {(cuuint64_t)cin, (cuuint64_t)cout, (cuuint64_t)taps};
    const cuuint64_t strides[2] = {(cuuint64_t)cin * 2, (cuuint64_t)cin * 2 * cout};
    const cuuint32_t box[3] = {16, (cuuint32_t)cout, (cuuint32_t)(taps == 27 ? (2 * cout > 256 ? 9 : 3) : 1)};
    const cuuint32_t es[3] = {1, 1, 1};
    if (enc(&tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(w), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 3;
  }
  TcParams p{};
  p.Cin = cin;
  p.Cout = cout;
  p.N = n;
  p.D = d;
  p.H = h;
  p.W = wd;
  p.taps = taps;
  p.relu = relu;
  p.nbx = (wd + 7) / 8;
  p.nby = (h + 15) / 16;
  p.nbz = (d + bz - 1) / bz;
  uint32_t cols = 32;
  while (cols < (uint32_t)(bz * cout)) cols *= 2;
  p.ncols = cols;
  // taps per weight stage: one x-row of the stencil (3), or a whole z-plane of it (9)
  // when 2 C_out > 256 TMEM columns leave the SM to one CTA anyway (measured: 9
  // is faster there, 3 where two or more CTAs share an SM)
  p.tps = taps == 27 ? (2 * cout > 256 ? 9 : 3) : 1;
  p.b_stride = (p.tps * cout * 32 + 1023) / 1024 * 1024;  // swizzled TMA destinations: 1024-byte aligned
  p.bias = bias;
  p.out = static_cast<__nv_bfloat16*>(out);
  p.out_f32 = out_f32;
  // CTAs per SM: at most what its 512 TMEM columns hold (an allocation beyond them
  // would wait), at most 4; each gets an equal share of the
  // SM's shared memory, which is also its floor (so no more CTAs fit), and fills
  // it with weight stages
  const int a_tile = Tile<2>::kATile;
  const int fixed = 1024 + (2 * a_tile + 1023) / 1024 * 1024 + (4 + 2 * kMaxBStages + 1) * 8 + 16;
  // fewer CTAs per SM when four weight stages would not fit in an equal share
  int per_sm = std::min(512 / (int)cols, 4), share = 0;
  for (;; --per_sm) {
    share = 233472 / per_sm - 1024;  // per-SM capacity less the per-CTA reserve
    p.b_stages = std::min(kMaxBStages, (std::min(share, 232448) - fixed) / p.b_stride);
    if (p.b_stages >= 4 || per_sm == 1) break;
  }
  if (p.b_stages < 2) return 1;
  const int smem = std::min(share, 232448);
  // the opt-in shared-memory limit is a per-device attribute of the kernel
  static std::atomic<bool> configured[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 3;
  if (!configured[dev].load()) {
    if (cudaFuncSetAttribute(k_conv3d_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448) != cudaSuccess)
      return 3;
    configured[dev].store(true);
  }
  const int64_t grid = (int64_t)n * p.nbz * p.nby * p.nbx;
  if (grid > 0x7fffffff) return 1;
  k_conv3d_tc<2><<<(unsigned)grid, 128, smem, static_cast<cudaStream_t>(stream)>>>(tin, tw, p);
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

int hlbg_nn_tc_error(int32_t reset) {
  int e = 0;
  if (cudaMemcpyFromSymbol(&e, g_tc_err, sizeof(int)) != cudaSuccess) return -1;
  if (reset && e) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_tc_err, &zero, sizeof(int));
  }
  return e;
}

}  // extern "C"
