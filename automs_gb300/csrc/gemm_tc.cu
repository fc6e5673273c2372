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
#include "tc_ptx.cuh"

namespace {

using namespace tc;

constexpr int BM = 128;
constexpr int BK = 64;  // 64 bf16 = 128 bytes = one swizzle row
constexpr int STAGES = 4;

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
    tmem_alloc(&tmem_slot, (uint32_t)BN);
  }
  fence_before();
  __syncthreads();
  fence_after();
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
      fence_after();
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
  fence_after();
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
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, (uint32_t)BN);
  }
}

template <int BN>
cudaError_t launch(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K,
                   const GemmEpilogue &ep, unsigned *err, cudaStream_t st) {
  CUtensorMap ta, tb;
  if (!make_map_bf16(&ta, A, M, K, BM) || !make_map_bf16(&tb, B, N, K, BN)) return cudaErrorInvalidValue;
  const size_t smem = STAGES * (BM * BK * 2 + BN * BK * 2) + 1024;
  static size_t attr_set[AMS_MAX_DEVICES] = {0};
  cudaError_t e = ams_set_smem_atleast(attr_set, k_gemm_tc<BN>, smem);
  if (e != cudaSuccess) return e;
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
