// mlp.cu -- surrogate MLP: training and inference on the tcgen05 GEMM.
//
// No counterpart in the reference (it searches hyper-configs with NNI's
// annealer, physical_exp_nni_main.py:11-29, running the full tracer +
// optimiser per trial).  The surrogate maps a placement descriptor to a
// coverage-gain map and screens candidates so that the tracer only judges the
// best few.
//
// Network: H_l = relu(H_{l-1} W_l^T + b_l), l < L; Y = H_{L-1} W_L^T + b_L.
// Compute is BF16 on the tensor cores with FP32 accumulation; master
// weights, gradients and Adam moments are FP32.  Each weight is kept in two
// BF16 copies, W [out, in] for the forward pass and W^T [in, out] for the
// input gradient, both K-major as the GEMM wants.
//   forward   H_l  = gemm(H_{l-1}, W_l)            epilogue: bias, relu -> bf16
//   loss      dY   = 2 (Y - T) / (B d_L)          rows >= B are zero
//   backward  dW_l = gemm(dZ_l^T, H_{l-1}^T)       fp32
//             db_l = column sums of dZ_l
//             dZ_{l-1} = gemm(dZ_l, W_l^T) o (H_{l-1} > 0)   epilogue mask -> bf16
//   update    Adam on the FP32 masters, then refresh both BF16 copies.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gemm_tc.h"
#include "mlp.h"

namespace {

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
  return x;
}

// W ~ U(-sqrt(6/fan_in), sqrt(6/fan_in)) (He-uniform), b = 0
__global__ void k_init(float *W, int rows, int cols, int cols_used, uint32_t seed, float bound) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)rows * cols) return;
  int c = (int)(i % cols);
  float u = (hash32((uint32_t)i * 2654435761u ^ seed) >> 8) * (1.0f / 16777216.0f);
  W[i] = c < cols_used ? (2.0f * u - 1.0f) * bound : 0.0f;
}

// fp32 [B, d] -> bf16 [Bp, dp] with zero padding
__global__ void k_pack_input(const float *X, int B, int d, int Bp, int dp, __nv_bfloat16 *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)Bp * dp) return;
  int r = (int)(i / dp), c = (int)(i % dp);
  float v = (r < B && c < d) ? X[(size_t)r * d + c] : 0.0f;
  out[i] = __float2bfloat16_rn(v);
}

// bf16 [R, C] -> [C, R]
__global__ void k_transpose(const __nv_bfloat16 *in, int R, int C, __nv_bfloat16 *out) {
  __shared__ __nv_bfloat16 t[32][33];
  int c = blockIdx.x * 32 + threadIdx.x, r0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    int r = r0 + j;
    if (r < R && c < C) t[j][threadIdx.x] = in[(size_t)r * C + c];
  }
  __syncthreads();
  int r = r0 + threadIdx.x;
  for (int j = threadIdx.y; j < 32; j += 8) {
    int cc = blockIdx.x * 32 + j;
    if (cc < C && r < R) out[(size_t)cc * R + r] = t[threadIdx.x][j];
  }
}

// MSE loss over the first B rows and dY (bf16, zero for padded rows)
__global__ void k_loss(const float *Y, const float *T, int B, int Bp, int d, float scale,
                       __nv_bfloat16 *dY, double *part) {
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)Bp * d;
       i += (long long)gridDim.x * blockDim.x) {
    int r = (int)(i / d);
    float g = 0.0f;
    if (r < B) {
      float e = Y[i] - T[i];
      acc += (double)e * e;
      g = 2.0f * e * scale;
    }
    dY[i] = __float2bfloat16_rn(g);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double s[8];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_loss_final(const double *part, int n, float scale, float *loss) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < n; i++) t += part[i];
    *loss = (float)(t * scale);
  }
}

// db[c] = sum_r dZ[r, c]
__global__ void k_colsum(const __nv_bfloat16 *dZ, int R, int C, float *db) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  float s = 0.0f;
  for (int r = 0; r < R; r++) s += __bfloat162float(dZ[(size_t)r * C + c]);
  db[c] = s;
}

// Adam on fp32 masters; refresh W bf16 [rows, cols] and W^T bf16 [cols, rows]
__global__ void k_adam(float *W, float *m, float *v, const float *g, long long n, float lr,
                       float b1, float b2, float eps, float c1, float c2, int rows, int cols,
                       int cols_used, __nv_bfloat16 *Wb, __nv_bfloat16 *Wt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cols > 0 ? (int)(i % cols) : 0;
  float w = W[i];
  if (c < cols_used) {
    float gi = g[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    W[i] = w;
  }
  if (Wb) {
    int r = (int)(i / cols);
    __nv_bfloat16 h = __float2bfloat16_rn(w);
    Wb[i] = h;
    Wt[(size_t)c * rows + r] = h;
  }
}

__global__ void k_to_bf16_pair(const float *W, long long n, int rows, int cols, __nv_bfloat16 *Wb,
                               __nv_bfloat16 *Wt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int r = (int)(i / cols), c = (int)(i % cols);
  __nv_bfloat16 h = __float2bfloat16_rn(W[i]);
  Wb[i] = h;
  Wt[(size_t)c * rows + r] = h;
}

inline int nb(long long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

cudaError_t mlp_init(MlpDev &m, uint32_t seed, cudaStream_t st) {
  for (int l = 1; l <= m.L; l++) {
    const int rows = m.d[l], cols = m.dp[l - 1], used = m.d[l - 1];
    const float bound = sqrtf(6.0f / (float)used);
    k_init<<<nb((long long)rows * cols, 256), 256, 0, st>>>(m.W[l], rows, cols, used,
                                                             seed * 7919u + (uint32_t)l, bound);
    cudaMemsetAsync(m.b[l], 0, sizeof(float) * rows, st);
    cudaMemsetAsync(m.mW[l], 0, sizeof(float) * (size_t)rows * cols, st);
    cudaMemsetAsync(m.vW[l], 0, sizeof(float) * (size_t)rows * cols, st);
    cudaMemsetAsync(m.mb[l], 0, sizeof(float) * rows, st);
    cudaMemsetAsync(m.vb[l], 0, sizeof(float) * rows, st);
  }
  return mlp_refresh_bf16(m, st);
}

cudaError_t mlp_refresh_bf16(MlpDev &m, cudaStream_t st) {
  for (int l = 1; l <= m.L; l++) {
    const long long n = (long long)m.d[l] * m.dp[l - 1];
    k_to_bf16_pair<<<nb(n, 256), 256, 0, st>>>(m.W[l], n, m.d[l], m.dp[l - 1], m.Wb[l], m.Wt[l]);
  }
  return cudaGetLastError();
}

cudaError_t mlp_forward(MlpDev &m, const float *X, int B, float *Y_out, cudaStream_t st) {
  const int Bp = (B + 127) / 128 * 128;
  k_pack_input<<<nb((long long)Bp * m.dp[0], 256), 256, 0, st>>>(X, B, m.d[0], Bp, m.dp[0], m.H[0]);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (int l = 1; l <= m.L; l++) {
    GemmEpilogue ep;
    ep.bias = m.b[l];
    ep.ldc = m.dp[l];
    if (l < m.L) {
      ep.relu = true;
      ep.out16 = m.H[l];
    } else {
      ep.out32 = m.Y;
    }
    e = gemm_bf16_tc(m.H[l - 1], m.Wb[l], Bp, m.dp[l], m.dp[l - 1], ep, m.err, st);
    if (e != cudaSuccess) return e;
  }
  if (Y_out) {
    e = cudaMemcpy2DAsync(Y_out, sizeof(float) * m.d[m.L], m.Y, sizeof(float) * m.dp[m.L],
                          sizeof(float) * m.d[m.L], B, cudaMemcpyDeviceToDevice, st);
  }
  return e;
}

cudaError_t mlp_backward(MlpDev &m, const float *T, int B, float *loss, cudaStream_t st) {
  const int Bp = (B + 127) / 128 * 128;
  const int L = m.L;
  const int dl = m.d[L];
  // targets arrive as [B, d_L]; the output buffer has the same width
  const int nblk = kMlpLossParts;
  k_loss<<<nblk, 256, 0, st>>>(m.Y, T, B, Bp, dl, 1.0f / ((float)B * dl), m.dZ[L], m.part);
  if (loss) k_loss_final<<<1, 32, 0, st>>>(m.part, nblk, 1.0f / ((double)B * dl), loss);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (int l = L; l >= 1; l--) {
    const int dout = m.dp[l], din = m.dp[l - 1];
    // transposes for the weight gradient
    dim3 tb(32, 8);
    k_transpose<<<dim3(nb(dout, 32), nb(Bp, 32)), tb, 0, st>>>(m.dZ[l], Bp, dout, m.tA);
    k_transpose<<<dim3(nb(din, 32), nb(Bp, 32)), tb, 0, st>>>(m.H[l - 1], Bp, din, m.tB);
    GemmEpilogue g1;
    g1.out32 = m.gW[l];
    g1.ldc = din;
    e = gemm_bf16_tc(m.tA, m.tB, dout, din, Bp, g1, m.err, st);
    if (e != cudaSuccess) return e;
    k_colsum<<<nb(dout, 128), 128, 0, st>>>(m.dZ[l], Bp, dout, m.gb[l]);
    if (l > 1) {
      GemmEpilogue g2;
      g2.mask = m.H[l - 1];
      g2.out16 = m.dZ[l - 1];
      g2.ldc = din;
      e = gemm_bf16_tc(m.dZ[l], m.Wt[l], Bp, din, dout, g2, m.err, st);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaGetLastError();
}

cudaError_t mlp_adam(MlpDev &m, float lr, cudaStream_t st) {
  m.step++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f - powf(b1, (float)m.step), c2 = 1.0f - powf(b2, (float)m.step);
  for (int l = 1; l <= m.L; l++) {
    const long long n = (long long)m.d[l] * m.dp[l - 1];
    k_adam<<<nb(n, 256), 256, 0, st>>>(m.W[l], m.mW[l], m.vW[l], m.gW[l], n, lr, b1, b2, eps, c1,
                                       c2, m.d[l], m.dp[l - 1], m.d[l - 1], m.Wb[l], m.Wt[l]);
    k_adam<<<nb(m.d[l], 256), 256, 0, st>>>(m.b[l], m.mb[l], m.vb[l], m.gb[l], m.d[l], lr, b1, b2,
                                            eps, c1, c2, 1, 1, 1, nullptr, nullptr);
  }
  return cudaGetLastError();
}
