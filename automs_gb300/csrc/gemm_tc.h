// gemm_tc.h -- tcgen05 BF16 GEMM with a fused epilogue (gemm_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

// Epilogue of C = A . B^T (row-major C with leading dimension ldc):
//   x = acc (+ bias[col]) ; relu ; x *= (mask[row, col] > 0) ; store.
struct GemmEpilogue {
  const float *bias = nullptr;
  bool relu = false;
  const __nv_bfloat16 *mask = nullptr;  // same shape as C
  float *out32 = nullptr;
  __nv_bfloat16 *out16 = nullptr;
  int ldc = 0;
};

// A [M, K], B [N, K] bf16 row-major (K contiguous).  M % 128 == 0,
// N % 64 == 0, K % 64 == 0.  err: device flag word, bits set on a timed-out
// wait inside the kernel.
cudaError_t gemm_bf16_tc(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K,
                         const GemmEpilogue &ep, unsigned *err, cudaStream_t st);
