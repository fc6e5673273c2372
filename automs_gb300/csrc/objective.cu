// objective.cu -- phase-map coverage objective and its adjoint on GB300.
//
// Reference: Model.get_channel (go.py:107-157, one metasurface hop) and
// Model.forward with loss mode "capacity" (go.py:159-245), differentiated by
// hand instead of autograd.  Channels in the reference orientation:
// H_d [S,R], H_a [S,M], H_r [M,R], code weights W [C,S], complex64.
//
//   U   = (W H_a) o exp(j (phi mod max_phase))            k_prep
//   Y   = W H_d + U H_r        (one streaming pass)        k_pass1
//   per Rx: |Y|, capacity, dropout, max over codes, mask, and the two
//   gradient parts G1 (max term) and G2 (norm term, before 1/||.||)
//   loss = -w sum max + ||masked||                          k_scalars
//   G_U = (G1 + G2/||.||) [H_r; H_d]^H  (second pass)       k_pass2
//   dphi = -Im(conj(G_U) o U) summed over codes,
//   G_W  = G_Wd + (G_U o exp(-j phi')) H_a^H                k_final
//
// Accumulation is FP32 with FP64 for the loss scalars.  When H_r fits in L2
// the second pass reads it from L2, so one evaluation moves H_r from HBM
// once.  Scratch lives in a per-device buffer kept across calls; calls on
// one device must not overlap.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/ams.h"
#include "objective.h"

namespace {

constexpr float kN0 = 1e-9f;                 // 10^(-90/10) mW, go.py:183-184
constexpr float kEps = 1.1920928955078125e-07f;  // float32 eps, go.py:181
constexpr float kInvLn2 = 1.4426950408889634f;

struct c2 { float x, y; };
__device__ __forceinline__ c2 ld2(const float *p, size_t i) {
  float2 v = __ldg(reinterpret_cast<const float2 *>(p) + i);
  return {v.x, v.y};
}
__device__ __forceinline__ void mac(c2 &acc, c2 a, c2 b) {  // acc += a*b
  acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
  acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
}
__device__ __forceinline__ void macc(c2 &acc, c2 a, c2 b) {  // acc += a*conj(b)
  acc.x = fmaf(a.x, b.x, fmaf(a.y, b.y, acc.x));
  acc.y = fmaf(a.y, b.x, fmaf(-a.x, b.y, acc.y));
}

// Python/torch remainder: result has the sign of the divisor
__device__ __forceinline__ float py_mod(float a, float b) {
  float r = fmodf(a, b);
  if (r != 0.f && ((r < 0.f) != (b < 0.f))) r += b;
  return r;
}

// U[c,m] = sum_s W[c,s] H_a[s,m] * exp(j phi'_m)
__global__ void k_prep(const float *W, const float *Ha, const float *phi, float max_phase, int S,
                       int M, int C, float *U) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  int c = blockIdx.y;
  if (m >= M) return;
  c2 v = {0.f, 0.f};
  for (int s = 0; s < S; s++) mac(v, ld2(W, (size_t)c * S + s), ld2(Ha, (size_t)s * M + m));
  float p = py_mod(phi[m], max_phase);  // go.py:133
  float sn, cs;
  sincosf(p, &sn, &cs);
  c2 e = {cs, sn};
  c2 u = {0.f, 0.f};
  mac(u, v, e);
  reinterpret_cast<float2 *>(U)[(size_t)c * M + m] = make_float2(u.x, u.y);
}

// Y over one r per thread, all codes in registers; then the per-Rx loss
// terms and gradient parts.
template <int CB>
__global__ void __launch_bounds__(128) k_pass1(const float *Hd, const float *W, const float *Hr,
                                               const float *U, int S, int M, int R, int C, float w,
                                               const uint8_t *drop, float *G1, float *G2,
                                               double *partials, float *recv_amp) {
  __shared__ c2 sU[64][CB];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = r < R;
  c2 y[CB];
#pragma unroll
  for (int c = 0; c < CB; c++) y[c] = {0.f, 0.f};
  // W H_d
  for (int k0 = 0; k0 < S; k0 += 64) {
    int kn = min(64, S - k0);
    __syncthreads();
    for (int i = threadIdx.x; i < kn * CB; i += blockDim.x) {
      int k = i / CB, c = i % CB;
      sU[k][c] = c < C ? ld2(W, (size_t)c * S + k0 + k) : c2{0.f, 0.f};
    }
    __syncthreads();
    if (live)
      for (int k = 0; k < kn; k++) {
        c2 h = ld2(Hd, (size_t)(k0 + k) * R + r);
#pragma unroll
        for (int c = 0; c < CB; c++) mac(y[c], sU[k][c], h);
      }
  }
  // U H_r
  if (Hr) {
    for (int k0 = 0; k0 < M; k0 += 64) {
      int kn = min(64, M - k0);
      __syncthreads();
      for (int i = threadIdx.x; i < kn * CB; i += blockDim.x) {
        int k = i / CB, c = i % CB;
        sU[k][c] = c < C ? ld2(U, (size_t)c * M + k0 + k) : c2{0.f, 0.f};
      }
      __syncthreads();
      if (live) {
        int k = 0;
        for (; k + 4 <= kn; k += 4) {
          c2 h0 = ld2(Hr, (size_t)(k0 + k) * R + r), h1 = ld2(Hr, (size_t)(k0 + k + 1) * R + r);
          c2 h2 = ld2(Hr, (size_t)(k0 + k + 2) * R + r), h3 = ld2(Hr, (size_t)(k0 + k + 3) * R + r);
#pragma unroll
          for (int c = 0; c < CB; c++) {
            mac(y[c], sU[k][c], h0);
            mac(y[c], sU[k + 1][c], h1);
            mac(y[c], sU[k + 2][c], h2);
            mac(y[c], sU[k + 3][c], h3);
          }
        }
        for (; k < kn; k++) {
          c2 h = ld2(Hr, (size_t)(k0 + k) * R + r);
#pragma unroll
          for (int c = 0; c < CB; c++) mac(y[c], sU[k][c], h);
        }
      }
    }
  }
  double sum_max = 0.0, sum_sq = 0.0;
  if (live) {
    float cap[CB], amp[CB];
    int arg = 0;
    float mx = -1.f;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      if (c >= C) { cap[c] = 0.f; amp[c] = 0.f; continue; }
      amp[c] = sqrtf(y[c].x * y[c].x + y[c].y * y[c].y);
      float a = amp[c] + kEps;
      float v = log2f(1.0f + a * a / kN0);
      if (drop && drop[c]) v = 0.f;
      cap[c] = v;
      if (v > mx) { mx = v; arg = c; }  // first index of the maximum
      if (recv_amp) recv_amp[(size_t)c * R + r] = amp[c];
    }
    sum_max = mx;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      if (c >= C) continue;
      bool dropped = drop && drop[c];
      float msk = (cap[c] != mx) ? cap[c] : 0.f;  // (cap' * mask)
      sum_sq += (double)msk * msk;
      float a = amp[c] + kEps;
      float dcap = (2.0f * a / kN0) / ((1.0f + a * a / kN0)) * kInvLn2;
      float g1 = (c == arg) ? -w : 0.f;
      float g2 = msk;
      if (dropped) { g1 = 0.f; g2 = 0.f; }
      float sc = amp[c] > 0.f ? dcap / amp[c] : 0.f;
      reinterpret_cast<float2 *>(G1)[(size_t)c * R + r] = make_float2(g1 * sc * y[c].x, g1 * sc * y[c].y);
      if (G2)
        reinterpret_cast<float2 *>(G2)[(size_t)c * R + r] = make_float2(g2 * sc * y[c].x, g2 * sc * y[c].y);
    }
  }
  // block partials (deterministic order: warp shuffles then warps in order)
  for (int o = 16; o > 0; o >>= 1) {
    sum_max += __shfl_xor_sync(0xffffffffu, sum_max, o);
    sum_sq += __shfl_xor_sync(0xffffffffu, sum_sq, o);
  }
  __shared__ double sp[2][4];
  int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { sp[0][wid] = sum_max; sp[1][wid] = sum_sq; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < 4; i++) { a += sp[0][i]; b += sp[1][i]; }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

__global__ void k_scalars(const double *partials, int nblocks, float w, float *loss,
                          float *inv_nrm) {
  __shared__ double s[2][256];
  double a = 0, b = 0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) { a += partials[2 * i]; b += partials[2 * i + 1]; }
  s[0][threadIdx.x] = a;
  s[1][threadIdx.x] = b;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) { s[0][threadIdx.x] += s[0][threadIdx.x + h]; s[1][threadIdx.x] += s[1][threadIdx.x + h]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double nrm = sqrt(s[1][0]);
    if (loss) *loss = (float)(-(double)w * s[0][0] + nrm);
    *inv_nrm = nrm > 0 ? (float)(1.0 / nrm) : 0.f;
  }
}

// G_U[c, row] = sum_r G[c,r] conj(Hrow[row, r]) over rows of [H_r; H_d]:
// a warp owns RPW rows, lanes stride over r, G staged in shared memory.
template <int CB, int RPW>
__global__ void __launch_bounds__(128) k_pass2(const float *Hr, const float *Hd, int M, int S,
                                               int R, int C, const float *G1, const float *G2,
                                               const float *inv_nrm, float *GU) {
  constexpr int TR = CB >= 64 ? 64 : 128;
  __shared__ c2 sG[CB][TR];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rows = M + S;
  const int row0 = (blockIdx.x * 4 + warp) * RPW;
  const float inv = G2 ? *inv_nrm : 0.f;
  c2 acc[RPW][CB];
#pragma unroll
  for (int q = 0; q < RPW; q++)
#pragma unroll
    for (int c = 0; c < CB; c++) acc[q][c] = {0.f, 0.f};
  for (int r0 = 0; r0 < R; r0 += TR) {
    __syncthreads();
    for (int i = threadIdx.x; i < CB * TR; i += blockDim.x) {
      int c = i / TR, rr = i % TR;
      c2 g = {0.f, 0.f};
      if (c < C && r0 + rr < R) {
        g = ld2(G1, (size_t)c * R + r0 + rr);
        if (G2) {
          c2 g2 = ld2(G2, (size_t)c * R + r0 + rr);
          g.x = fmaf(g2.x, inv, g.x);
          g.y = fmaf(g2.y, inv, g.y);
        }
      }
      sG[c][rr] = g;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < RPW; q++) {
      int row = row0 + q;
      if (row >= rows) break;
      const float *base = row < M ? Hr + (size_t)row * R * 2 : Hd + (size_t)(row - M) * R * 2;
#pragma unroll
      for (int j = 0; j < TR / 32; j++) {
        int rr = lane + 32 * j;
        if (r0 + rr >= R) break;
        c2 h = ld2(base, (size_t)(r0 + rr));
#pragma unroll
        for (int c = 0; c < CB; c++) macc(acc[q][c], sG[c][rr], h);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < RPW; q++) {
    int row = row0 + q;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      float x = acc[q][c].x, y = acc[q][c].y;
      for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
      }
      if (lane == 0 && row < rows && c < C)
        reinterpret_cast<float2 *>(GU)[(size_t)c * rows + row] = make_float2(x, y);
    }
  }
}

// grad_Y = G1 + G2 / ||masked||
__global__ void k_grad_y(const float *G1, const float *G2, const float *inv_nrm, long long n,
                         float *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float inv = G2 ? *inv_nrm : 0.f;
  c2 g = ld2(G1, i);
  if (G2) {
    c2 h = ld2(G2, i);
    g.x = fmaf(h.x, inv, g.x);
    g.y = fmaf(h.y, inv, g.y);
  }
  reinterpret_cast<float2 *>(out)[i] = make_float2(g.x, g.y);
}

// dphi[m] = -sum_c Im(conj(G_U[c,m]) U[c,m])
__global__ void k_dphi(const float *GU, const float *U, int M, int S, int C, float *dphi) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  float s = 0.f;
  for (int c = 0; c < C; c++) {
    c2 g = ld2(GU, (size_t)c * (M + S) + m), u = ld2(U, (size_t)c * M + m);
    s += g.x * u.y - g.y * u.x;  // Im(conj(g) u)
  }
  dphi[m] = -s;
}

// G_W[c,s] = G_U[c, M+s] + sum_m G_U[c,m] exp(-j phi'_m) conj(H_a[s,m]); one warp per (c,s)
__global__ void k_gradw(const float *GU, const float *Ha, const float *phi, float max_phase,
                        int S, int M, int C, float *GW) {
  int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (wid >= C * S) return;
  int c = wid / S, s = wid % S;
  c2 acc = {0.f, 0.f};
  if (Ha) {
    for (int m = lane; m < M; m += 32) {
      c2 g = ld2(GU, (size_t)c * (M + S) + m);
      float p = py_mod(phi[m], max_phase);
      float sn, cs;
      sincosf(p, &sn, &cs);
      c2 gv = {g.x * cs + g.y * sn, g.y * cs - g.x * sn};  // g * exp(-j p)
      macc(acc, gv, ld2(Ha, (size_t)s * M + m));
    }
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
  }
  if (lane == 0) {
    c2 d = ld2(GU, (size_t)c * (M + S) + M + s);
    reinterpret_cast<float2 *>(GW)[(size_t)c * S + s] = make_float2(acc.x + d.x, acc.y + d.y);
  }
}

int cbucket(int C) {
  int b = 1;
  while (b < C) b <<= 1;
  return b;
}

template <int CB>
cudaError_t launch_pass1(int blocks, cudaStream_t st, const float *Hd, const float *W,
                         const float *Hr, const float *U, int S, int M, int R, int C, float w,
                         const uint8_t *drop, float *G1, float *G2, double *part, float *amp) {
  k_pass1<CB><<<blocks, 128, 0, st>>>(Hd, W, Hr, U, S, M, R, C, w, drop, G1, G2, part, amp);
  return cudaGetLastError();
}

template <int CB, int RPW>
cudaError_t launch_pass2(cudaStream_t st, const float *Hr, const float *Hd, int M, int S, int R,
                         int C, const float *G1, const float *G2, const float *inv, float *GU) {
  int rows = M + S;
  int blocks = (rows + 4 * RPW - 1) / (4 * RPW);
  k_pass2<CB, RPW><<<blocks, 128, 0, st>>>(Hr, Hd, M, S, R, C, G1, G2, inv, GU);
  return cudaGetLastError();
}

}  // namespace

ObjScratchLayout obj_scratch_layout(int S, int M, int R, int C) {
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  ObjScratchLayout L;
  int nb = (R + 127) / 128;
  size_t o = 0;
  L.U = o; o += al(8 * (size_t)C * std::max(M, 1));
  L.G1 = o; o += al(8 * (size_t)C * R);
  L.G2 = o; o += al(8 * (size_t)C * R);
  L.part = o; o += al(16 * (size_t)nb);
  L.GU = o; o += al(8 * (size_t)C * (std::max(M, 0) + S));
  L.inv = o; o += al(16);
  L.total = o;
  return L;
}

cudaError_t obj_run(const ObjArgs &a, char *scratch, cudaStream_t st) {
  const ObjScratchLayout L = obj_scratch_layout(a.S, a.M, a.R, a.C);
  const bool ms = a.Ha && a.Hr;
  const int M = ms ? a.M : 0;
  float *U = reinterpret_cast<float *>(scratch + L.U);
  float *G1 = reinterpret_cast<float *>(scratch + L.G1);
  float *G2 = a.C > 1 ? reinterpret_cast<float *>(scratch + L.G2) : nullptr;
  double *part = reinterpret_cast<double *>(scratch + L.part);
  float *GU = reinterpret_cast<float *>(scratch + L.GU);
  float *inv = reinterpret_cast<float *>(scratch + L.inv);
  cudaError_t e;
  if (ms) {
    dim3 g((M + 255) / 256, a.C);
    k_prep<<<g, 256, 0, st>>>(a.W, a.Ha, a.phi, a.max_phase, a.S, M, a.C, U);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  const int nb = (a.R + 127) / 128;
  const float *Hr = ms ? a.Hr : nullptr;
  switch (cbucket(a.C)) {
#define P1(CB) case CB: e = launch_pass1<CB>(nb, st, a.Hd, a.W, Hr, U, a.S, M, a.R, a.C, a.w, a.drop, G1, G2, part, a.recv_amp); break;
    P1(1) P1(2) P1(4) P1(8) P1(16) P1(32) P1(64)
#undef P1
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  k_scalars<<<1, 256, 0, st>>>(part, nb, a.w, a.loss, inv);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (a.grad_Y) {
    long long n = (long long)a.C * a.R;
    k_grad_y<<<(int)((n + 255) / 256), 256, 0, st>>>(G1, G2, inv, n, a.grad_Y);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (!a.grad_W && !a.grad_phi) return cudaSuccess;
  switch (cbucket(a.C)) {
    case 1: e = launch_pass2<1, 8>(st, Hr, a.Hd, M, a.S, a.R, a.C, G1, G2, inv, GU); break;
    case 2: e = launch_pass2<2, 4>(st, Hr, a.Hd, M, a.S, a.R, a.C, G1, G2, inv, GU); break;
    case 4: e = launch_pass2<4, 2>(st, Hr, a.Hd, M, a.S, a.R, a.C, G1, G2, inv, GU); break;
    case 8: e = launch_pass2<8, 1>(st, Hr, a.Hd, M, a.S, a.R, a.C, G1, G2, inv, GU); break;
    case 16: e = launch_pass2<16, 1>(st, Hr, a.Hd, M, a.S, a.R, a.C, G1, G2, inv, GU); break;
    case 32: e = launch_pass2<32, 1>(st, Hr, a.Hd, M, a.S, a.R, a.C, G1, G2, inv, GU); break;
    case 64: e = launch_pass2<64, 1>(st, Hr, a.Hd, M, a.S, a.R, a.C, G1, G2, inv, GU); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  if (a.grad_phi && ms) {
    k_dphi<<<(M + 255) / 256, 256, 0, st>>>(GU, U, M, a.S, a.C, a.grad_phi);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (a.grad_W) {
    int warps = a.C * a.S;
    k_gradw<<<(warps * 32 + 255) / 256, 256, 0, st>>>(GU, ms ? a.Ha : nullptr, a.phi, a.max_phase,
                                                      a.S, M, a.C, a.grad_W);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

namespace {
// draw_channel + amp_data_to_image (go.py:849-851, 944-964):
// 20 log10 |sum_s H[s,r]|, NaN -> threshold, + offset, clamp below at threshold
__global__ void k_coverage_db(const float *H, int S, int R, float threshold, float offset,
                              float *out) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  double x = 0, y = 0;
  for (int s = 0; s < S; s++) {
    float2 v = __ldg(reinterpret_cast<const float2 *>(H) + (size_t)s * R + r);
    x += v.x;
    y += v.y;
  }
  float a = (float)sqrt(x * x + y * y);
  float d = 20.0f * log10f(a);
  if (isnan(d)) d = threshold;
  d = d + offset;
  out[r] = fmaxf(d, threshold);
}
}  // namespace

cudaError_t coverage_db_run(const float *H, int S, int R, float threshold, float offset,
                            float *out, cudaStream_t st) {
  k_coverage_db<<<(R + 255) / 256, 256, 0, st>>>(H, S, R, threshold, offset, out);
  return cudaGetLastError();
}
