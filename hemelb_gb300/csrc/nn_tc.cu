// 3x3x3 convolution of the warm-start surrogate on the fifth-generation tensor
// cores: tcgen05.mma with the accumulator in tensor memory (TMEM), operands staged
// in shared memory by TMA (cp.async.bulk.tensor), completion tracked on mbarriers.
//
// Implicit GEMM.  One CTA computes one output brick of 8 (x) x 4 (y) x 4 (z) = 128
// voxels -- the MMA's M = 128 rows -- for all C_out output channels (N = C_out,
// a multiple of 16 up to 256).  The reduction runs over the 27 taps x C_in input
// channels in steps of K = 16: for tap (dz, dy, dx) and channel slice k, a TMA
// load copies the input brick shifted by (dx, dy, dz), channels [16k, 16k + 16),
// as 128 rows of 32 bytes (coordinates outside the volume read zeros: that is the
// convolution's zero padding), and a second TMA load copies the weights of that
// tap and slice, C_out rows of 32 bytes.  Both land in the 32-byte-swizzled K-major
// layout that the MMA's shared-memory descriptors name.  A ring of kStages such
// stages keeps the copies ahead of the MMAs: one thread issues the copies (waiting
// for a stage to be free), one thread issues the MMAs (waiting for a stage to be
// full) and returns each stage with tcgen05.commit.  The four warps then read the
// accumulator from TMEM (warp w owns TMEM lanes 32w..32w+31, i.e. 32 voxels), add
// the bias, apply the ReLU and store BF16 (and optionally FP32) channels-last.
//
// Every wait is bounded: a wait that gives up sets g_tc_err (read back by
// hlbg_nn_tc_error), the CTA waits (bounded) for the copies it issued, frees its
// TMEM and returns.  Tensor maps cover this GPU's own memory only (no multicast).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "../../include/hemelb_gb300_nn.h"

namespace {

constexpr int kM = 128;                   // voxels per CTA: the MMA's M
constexpr int kStages = 4;                // shared-memory ring depth
constexpr int kASlice = kM * 32;          // one A stage: 128 rows x 16 BF16
constexpr int64_t kWaitLimit = 1ll << 22; // polls before a wait gives up

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

// Shared-memory matrix descriptor of a K-major tile of 32-byte rows in the
// 32-byte swizzle: start address, leading-dimension offset (not used by swizzled
// K-major tiles; 1 by convention), stride between 8-row groups (8 x 32 B), the
// descriptor version of tcgen05 (1) and the layout code of the 32-byte swizzle (6).
__device__ __forceinline__ uint64_t sw32_desc(uint32_t saddr) {
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
  uint32_t ncols;        // TMEM columns allocated (a power of two >= 32 and >= Cout)
  int b_stride;          // bytes of one B stage (C_out x 32, rounded up to 1024)
  const float* bias;     // [C_out] or null
  __nv_bfloat16* out;    // [voxels][C_out]
  float* out_f32;        // [voxels][C_out] or null
};

__global__ void __launch_bounds__(128, 1) k_conv3d_tc(const __grid_constant__ CUtensorMap tin,
                                                      const __grid_constant__ CUtensorMap tw, TcParams p) {
  extern __shared__ uint8_t smem_raw[];
  // stages at a 1024-byte boundary (TMA destinations and swizzle atoms)
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int stage_bytes = kASlice + p.b_stride;
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kStages * stage_bytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 1);
  const uint32_t a0 = smem_u32(base), full0 = smem_u32(bars), empty0 = full0 + 8 * kStages,
                 done = full0 + 16 * kStages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  int bid = blockIdx.x;
  const int bx = bid % p.nbx;
  bid /= p.nbx;
  const int by = bid % p.nby;
  bid /= p.nby;
  const int bz = bid % p.nbz;
  const int n = bid / p.nbz;
  const int x0 = bx * 8, y0 = by * 4, z0 = bz * 4;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
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
  const int ksteps = p.taps * kslices;
  const uint32_t tx_bytes = (uint32_t)(kASlice + p.Cout * 32);
  if (warp == 0 && lane == 0) {
    // producer: the copies of k-step i go to stage i % kStages once it is free
    int issued = 0;
    bool ok = true;
    for (int i = 0; i < ksteps; ++i) {
      const int s = i % kStages;
      const uint32_t ph = (uint32_t)(i / kStages) & 1u;
      if (!mbar_wait(empty0 + 8 * s, ph ^ 1u)) {
        ok = false;
        break;
      }
      const int tap = i / kslices, ks = i % kslices;
      int dz = 0, dy = 0, dx = 0;
      if (p.taps == 27) {
        dz = tap / 9 - 1;
        dy = (tap / 3) % 3 - 1;
        dx = tap % 3 - 1;
      }
      const uint32_t sa = a0 + s * stage_bytes;
      mbar_expect_tx(full0 + 8 * s, tx_bytes);
      tma_load_5d(sa, &tin, full0 + 8 * s, ks * 16, x0 + dx, y0 + dy, z0 + dz, n);
      tma_load_3d(sa + kASlice, &tw, full0 + 8 * s, ks * 16, 0, tap);
      ++issued;
    }
    if (!ok) {
      atomicExch(&g_tc_err, 1);
      // the copies in flight land before the CTA's shared memory goes away
      for (int j = issued > kStages ? issued - kStages : 0; j < issued; ++j)
        mbar_wait(full0 + 8 * (j % kStages), (uint32_t)(j / kStages) & 1u);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: k-step i once its stage is full; the commit returns the stage
    const uint32_t idesc = idesc_bf16(p.Cout);
    for (int i = 0; i < ksteps; ++i) {
      const int s = i % kStages;
      const uint32_t ph = (uint32_t)(i / kStages) & 1u;
      if (!mbar_wait(full0 + 8 * s, ph)) {
        atomicExch(&g_tc_err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = a0 + s * stage_bytes;
      umma_bf16(tmem, sw32_desc(sa), sw32_desc(sa + kASlice), idesc, i > 0 ? 1u : 0u);
      umma_commit(empty0 + 8 * s);
    }
    umma_commit(done);  // arrives once every MMA issued above has completed
  }
  __syncwarp();

  // epilogue: TMEM lane = voxel row of the brick, column = output channel
  const bool finished = mbar_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!finished && lane == 0) atomicExch(&g_tc_err, 1);
  const int row = warp * 32 + lane;
  const int x = x0 + (row & 7), y = y0 + ((row >> 3) & 3), z = z0 + (row >> 5);
  const bool inside = finished && x < p.W && y < p.H && z < p.D;
  const int64_t vox = (((int64_t)n * p.D + z) * p.H + y) * p.W + x;
  for (int c0 = 0; c0 < p.Cout; c0 += 16) {
    uint32_t r[16];
    __syncwarp();  // tcgen05.ld is warp-collective: every lane, converged
    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
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
  CUtensorMap tin, tw;
  {
    const cuuint64_t dims[5] = {(cuuint64_t)cin, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
    const cuuint64_t strides[4] = {(cuuint64_t)cin * 2, (cuuint64_t)cin * 2 * wd, (cuuint64_t)cin * 2 * wd * h,
                                   (cuuint64_t)cin * 2 * wd * h * d};
    const cuuint32_t box[5] = {16, 8, 4, 4, 1};
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    if (enc(&tin, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(in), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 3;
  }
  {
    const cuuint64_t dims[3] = {(cuuint64_t)cin, (cuuint64_t)cout, (cuuint64_t)taps};
    const cuuint64_t strides[2] = {(cuuint64_t)cin * 2, (cuuint64_t)cin * 2 * cout};
    const cuuint32_t box[3] = {16, (cuuint32_t)cout, 1};
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
  p.nby = (h + 3) / 4;
  p.nbz = (d + 3) / 4;
  uint32_t cols = 32;
  while (cols < (uint32_t)cout) cols *= 2;
  p.ncols = cols;
  p.b_stride = (cout * 32 + 1023) / 1024 * 1024;
  p.bias = bias;
  p.out = static_cast<__nv_bfloat16*>(out);
  p.out_f32 = out_f32;
  // shared memory: the stages, the barriers and the TMEM address, plus alignment
  // slack; at least enough that no more CTAs share an SM than its 512 TMEM
  // columns can hold at once (an allocation beyond them would wait)
  const int stage_bytes = kASlice + p.b_stride;
  int smem = 1024 + kStages * stage_bytes + (2 * kStages + 1) * 8 + 16;
  const int per_sm = 512 / (int)cols;
  const int floor_bytes = 232448 / per_sm - 1024;
  if (smem < floor_bytes && per_sm <= 8) smem = floor_bytes;
  if (smem > 232448) return 1;
  static thread_local int configured = 0;
  if (configured < smem) {
    if (cudaFuncSetAttribute(k_conv3d_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448) != cudaSuccess)
      return 3;
    configured = 232448;
  }
  const int64_t grid = (int64_t)n * p.nbz * p.nby * p.nbx;
  if (grid > 0x7fffffff) return 1;
  k_conv3d_tc<<<(unsigned)grid, 128, smem, static_cast<cudaStream_t>(stream)>>>(tin, tw, p);
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
