// gemm_tc.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05).
//
//   C[M, N] = A[M, K] . B[N, K]^T   (A, B bf16 row-major with K contiguous,
//                                    FP32 accumulation in tensor memory)
//
// One CTA computes a 128 x BN tile with 4 warps:
//   * warp 0 / lane 0 issues TMA loads (cp.async.bulk.tensor, 128-byte
//     swizzle) of 128 x 64 A and BN x 64 B tiles into a 4-stage ring;
//   * warp 1 / lane 0 issues tcgen05.mma (kind::f16, BF16 inputs, FP32
//     accumulator in TMEM), 4 MMAs of K = 16 per 64-wide stage, and frees a
//     stage with tcgen05.commit on its "empty" barrier;
//   * all 4 warps drain the accumulator with tcgen05.ld (warp w owns TMEM
//     lanes 32w..32w+31 = tile rows) and apply the fused epilogue:
//     optional bias, ReLU, multiplication by a 0/1 mask taken from a bf16
//     matrix (> 0), FP32 and/or BF16 output.
// Every mbarrier wait is bounded by a wall-clock limit; on timeout the CTA
// records an error flag, stops issuing work, frees its TMEM and returns.
// Requirements: M % 128 == 0, N % BN == 0, K % 64 == 0, 16-byte aligned rows.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gemm_tc.h"

namespace {

constexpr int BM = 128;
constexpr int BK = 64;  // 64 bf16 = 128 bytes = one swizzle row
constexpr int STAGES = 4;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!mbar_try_wait(bar, parity))
    if (now_ns() - t0 > kWaitNs) return false;
  return true;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor, K-major operand with 128-byte swizzle:
// start address >> 4 in bits 0-13, leading offset (unused for this layout)
// in 16-29, stride between 8-row groups (1024 B) >> 4 in 32-45, descriptor
// version 1 in 46-47, swizzle mode 2 (128 B) in 61-63.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 in bits 17-22,
// M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int BN>
__global__ void __launch_bounds__(128, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
              GemmEpilogue ep, int K, unsigned *err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
  unsigned char *sA = smem;
  unsigned char *sB = smem + STAGES * A_BYTES;
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int nk = K / BK;

  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"((uint32_t)BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1)) {
        abort_flag = 1;
        atomicOr(err, 1u);
        break;
      }
      if (*(volatile int *)&abort_flag) break;
      mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
      tma_load_2d(sA + s * A_BYTES, &ta, kb * BK, m0, &full[s]);
      tma_load_2d(sB + s * B_BYTES, &tb, kb * BK, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_bf16(BM, BN);
    bool ok = true;
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full[s], (kb / STAGES) & 1)) {
        abort_flag = 1;
        atomicOr(err, 2u);
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t a0 = smem_u32(sA + s * A_BYTES), b0 = smem_u32(sB + s * B_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 16; kk++)
        umma_bf16(tmem, sdesc_sw128(a0 + kk * 32), sdesc_sw128(b0 + kk * 32), idesc,
                  (kb > 0 || kk > 0) ? 1u : 0u);
      umma_commit(&empty[s]);
    }
    umma_commit(&done);  // arrives once every MMA issued above has completed
    (void)ok;
  }
  __syncwarp();
  // epilogue: every thread waits for the accumulator
  const bool have = mbar_wait(&done, 0);
  if (!have && lane == 0) atomicOr(err, 4u);
  // block-uniform decision: tcgen05.ld below is warp-collective
  const bool drain = __syncthreads_and(have ? 1 : 0) && !abort_flag;
  tc_fence_after();
  if (drain) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      tmem_ld32(tmem + lane_base + (uint32_t)c0, r);
      const int col0 = n0 + c0;
      float v[32];
#pragma unroll
      for (int j = 0; j < 32; j++) {
        float x = __uint_as_float(r[j]);
        if (ep.bias) x += __ldg(ep.bias + col0 + j);
        if (ep.relu) x = fmaxf(x, 0.0f);
        v[j] = x;
      }
      if (ep.mask) {
        const __nv_bfloat16 *mrow = ep.mask + (size_t)row * ep.ldc + col0;
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = __bfloat162float(mrow[j]) > 0.0f ? v[j] : 0.0f;
      }
      if (ep.out32) {
        float4 *o = reinterpret_cast<float4 *>(ep.out32 + (size_t)row * ep.ldc + col0);
#pragma unroll
        for (int j = 0; j < 8; j++) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      }
      if (ep.out16) {
        uint4 *o = reinterpret_cast<uint4 *>(ep.out16 + (size_t)row * ep.ldc + col0);
#pragma unroll
        for (int j = 0; j < 4; j++) {
          __nv_bfloat162 p0 = __floats2bfloat162_rn(v[8 * j], v[8 * j + 1]);
          __nv_bfloat162 p1 = __floats2bfloat162_rn(v[8 * j + 2], v[8 * j + 3]);
          __nv_bfloat162 p2 = __floats2bfloat162_rn(v[8 * j + 4], v[8 * j + 5]);
          __nv_bfloat162 p3 = __floats2bfloat162_rn(v[8 * j + 6], v[8 * j + 7]);
          uint4 u;
          u.x = *reinterpret_cast<uint32_t *>(&p0);
          u.y = *reinterpret_cast<uint32_t *>(&p1);
          u.z = *reinterpret_cast<uint32_t *>(&p2);
          u.w = *reinterpret_cast<uint32_t *>(&p3);
          o[j] = u;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)BN));
  }
}

using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                              const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                              const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encoder() {
  static EncodeFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  }
  return fn;
}

// 2-D tensor map over a row-major bf16 matrix [rows, cols], box 64 x box_rows
bool make_map(CUtensorMap *m, const void *base, int rows, int cols, int box_rows) {
  EncodeFn enc = encoder();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K,
                   const GemmEpilogue &ep, unsigned *err, cudaStream_t st) {
  CUtensorMap ta, tb;
  if (!make_map(&ta, A, M, K, BM) || !make_map(&tb, B, N, K, BN)) return cudaErrorInvalidValue;
  const size_t smem = STAGES * (BM * BK * 2 + BN * BK * 2) + 1024;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid(N / BN, M / BM);
  k_gemm_tc<BN><<<grid, 128, smem, st>>>(ta, tb, ep, K, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t gemm_bf16_tc(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K,
                         const GemmEpilogue &ep, unsigned *err, cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0 || M % BM || K % BK || N % 64) return cudaErrorInvalidValue;
  if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15)
    return cudaErrorInvalidValue;
  if (N % 128 == 0) return launch<128>(A, B, M, N, K, ep, err, st);
  return launch<64>(A, B, M, N, K, ep, err, st);
}
