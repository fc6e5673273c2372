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
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/ams.h"
#include "objective.h"
#include "tc_ptx.cuh"

namespace {

constexpr float kN0 = 1e-9f;                 // 10^(-90/10) mW, go.py:183-184
constexpr float kEps = 1.1920928955078125e-07f;  // float32 eps, go.py:181
constexpr float kInvLn2 = 1.4426950408889634f;
// the value of every output of a call whose bounded wait ran out
__device__ __forceinline__ float obj_nan() { return __int_as_float(0x7fc00000); }
// a bounded wait of this call ran out (err may be NULL: a path without waits)
__device__ __forceinline__ bool obj_failed(const unsigned *err) {
  return err != nullptr && __ldcg(err) != 0u;
}

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

// x = hi + lo with hi = bf16(x), lo = bf16(x - hi); a pair of values goes to
// element `pair` of the bf16x2 views of the hi and lo arrays
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}
__device__ __forceinline__ void put_pair(__nv_bfloat16 *hi, __nv_bfloat16 *lo, size_t pair,
                                         float a, float b) {
  __nv_bfloat16 h0, l0, h1, l1;
  split_bf16(a, h0, l0);
  split_bf16(b, h1, l1);
  reinterpret_cast<__nv_bfloat162 *>(hi)[pair] = __halves2bfloat162(h0, h1);
  reinterpret_cast<__nv_bfloat162 *>(lo)[pair] = __halves2bfloat162(l0, l1);
}

// ------------------------------------------------------------------
// Virtual rows k in [0, K), K = M + S: row k < M is H_r[k, :] with
// coefficient U[c, k]; row k >= M is H_d[k - M, :] with coefficient
// W[c, k - M].  Y[c, r] = sum_k coef[c, k] row_k[r].

__device__ __forceinline__ const float *row_ptr(const float *Hr, const float *Hd, int M, int R,
                                                int k) {
  return k < M ? Hr + (size_t)k * R * 2 : Hd + (size_t)(k - M) * R * 2;
}

constexpr int KCHUNK = 256;

// U[c, m] for the streaming path: 8 lanes per (m, c) split the sum over the
// AP elements; the dependent streaming kernel may start before this one ends
// (programmatic dependent launch) and waits for it only before reading U.
__global__ void __launch_bounds__(256) k_prep_wide(ObjArgs a, int M, float *U, unsigned *err) {
  // let the streaming kernel launch now; it waits for this grid before reading U
  cudaTriggerProgrammaticLaunchCompletion();
  // the call's wait-timeout word starts clear (a streaming kernel can set it
  // only after its grid-dependency wait on this grid)
  if (err && blockIdx.x == 0 && threadIdx.x == 0) *err = 0u;
  const long long e = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int sub = threadIdx.x & 7;
  const bool live = e < (long long)M * a.C;
  const int c = live ? (int)(e / M) : 0, m = live ? (int)(e % M) : 0;
  c2 v = {0.f, 0.f};
  if (live)
    for (int s = sub; s < a.S; s += 8) mac(v, ld2(a.W, (size_t)c * a.S + s), ld2(a.Ha, (size_t)s * M + m));
  for (int o = 1; o < 8; o <<= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  if (live && sub == 0) {
    const float p = py_mod(__ldg(a.phi + m), a.max_phase);
    float sn, cs;
    sincosf(p, &sn, &cs);
    c2 u = {0.f, 0.f};
    mac(u, v, c2{cs, sn});
    reinterpret_cast<float2 *>(U)[(size_t)c * M + m] = make_float2(u.x, u.y);
  }
}

// U[c, m] = (sum_s W[c, s] H_a[s, m]) e^{j phi'_m}: one thread per (m, c),
// loads of H_a coalesced over m, issued 8 at a time
__global__ void __launch_bounds__(128) k_prep(ObjArgs a, int M, float *U, unsigned *err) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  // the call's wait-timeout word starts clear (the GEMMs that can set it
  // run after this kernel)
  if (err && m == 0 && c == 0) *err = 0u;
  if (m >= M) return;
  c2 v = {0.f, 0.f};
  int s = 0;
  for (; s + 8 <= a.S; s += 8) {
    c2 h[8], w[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      h[j] = ld2(a.Ha, (size_t)(s + j) * M + m);
      w[j] = ld2(a.W, (size_t)c * a.S + s + j);
    }
#pragma unroll
    for (int j = 0; j < 8; j++) mac(v, w[j], h[j]);
  }
  for (; s < a.S; s++) mac(v, ld2(a.W, (size_t)c * a.S + s), ld2(a.Ha, (size_t)s * M + m));
  const float p = py_mod(__ldg(a.phi + m), a.max_phase);  // go.py:133
  float sn, cs;
  sincosf(p, &sn, &cs);
  c2 u = {0.f, 0.f};
  mac(u, v, c2{cs, sn});
  reinterpret_cast<float2 *>(U)[(size_t)c * M + m] = make_float2(u.x, u.y);
}

// pass 1: partial Y over a k-range; lanes = 32 columns, warps share the rows
template <int CB>
__global__ void __launch_bounds__(256) k_pass1(ObjArgs a, int M, int K, int kper, const float *U,
                                               float *Ypart) {
  __shared__ c2 sC[KCHUNK][CB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = blockIdx.x * 32 + lane;
  const bool live = r < a.R;
  const int k0 = blockIdx.y * kper, k1 = min(K, k0 + kper);
  c2 y[CB];
#pragma unroll
  for (int c = 0; c < CB; c++) y[c] = {0.f, 0.f};
  for (int kc = k0; kc < k1; kc += KCHUNK) {
    const int kn = min(KCHUNK, k1 - kc);
    __syncthreads();
    for (int i = threadIdx.x; i < kn * CB; i += blockDim.x) {
      const int kk = i / CB, c = i % CB, k = kc + kk;
      c2 v = {0.f, 0.f};
      if (c < a.C) v = k < M ? ld2(U, (size_t)c * M + k) : ld2(a.W, (size_t)c * a.S + (k - M));
      sC[kk][c] = v;
    }
    __syncthreads();
    if (live) {
      int kk = warp;
      for (; kk + 24 < kn; kk += 32) {
        const c2 h0 = ld2(row_ptr(a.Hr, a.Hd, M, a.R, kc + kk), r);
        const c2 h1 = ld2(row_ptr(a.Hr, a.Hd, M, a.R, kc + kk + 8), r);
        const c2 h2 = ld2(row_ptr(a.Hr, a.Hd, M, a.R, kc + kk + 16), r);
        const c2 h3 = ld2(row_ptr(a.Hr, a.Hd, M, a.R, kc + kk + 24), r);
#pragma unroll
        for (int c = 0; c < CB; c++) {
          mac(y[c], sC[kk][c], h0);
          mac(y[c], sC[kk + 8][c], h1);
          mac(y[c], sC[kk + 16][c], h2);
          mac(y[c], sC[kk + 24][c], h3);
        }
      }
      for (; kk < kn; kk += 8) {
        const c2 h = ld2(row_ptr(a.Hr, a.Hd, M, a.R, kc + kk), r);
#pragma unroll
        for (int c = 0; c < CB; c++) mac(y[c], sC[kk][c], h);
      }
    }
  }
  // reduce the 8 warps, 8 codes at a time
  __shared__ c2 red[8][32][8];
  for (int cg = 0; cg < CB; cg += 8) {
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (cg + j < CB) red[warp][lane][j] = y[cg + j < CB ? cg + j : 0];
    __syncthreads();
    if (warp == 0 && live) {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int c = cg + j;
        if (c >= CB || c >= a.C) continue;
        c2 t = red[0][lane][j];
        for (int w2 = 1; w2 < 8; w2++) { t.x += red[w2][lane][j].x; t.y += red[w2][lane][j].y; }
        reinterpret_cast<float2 *>(Ypart)[((size_t)blockIdx.y * a.C + c) * a.R + r] =
            make_float2(t.x, t.y);
      }
    }
  }
}

// Sum of the CTAs' (sum_max, sum_sq) pairs by every thread of the last CTA
// (FP64 adds have a long latency on this part; one thread alone would chain
// thousands of them).  Reads bypass L1: the pairs were written by other CTAs.
// The result is valid in thread 0; all threads of the block must call it.
__device__ __forceinline__ void block_sum_pairs(const double *partials, int nb, double &x,
                                                double &z) {
  __threadfence();
  double px = 0.0, pz = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    px += __ldcg(partials + 2 * b);
    pz += __ldcg(partials + 2 * b + 1);
  }
  for (int o = 16; o > 0; o >>= 1) {
    px += __shfl_xor_sync(0xffffffffu, px, o);
    pz += __shfl_xor_sync(0xffffffffu, pz, o);
  }
  __shared__ double red[2][32];
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][wid] = px; red[1][wid] = pz; }
  __syncthreads();
  x = 0.0;
  z = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) { x += red[0][i]; z += red[1][i]; }
}

// epilogue: Y from the partials, per-Rx capacity / dropout / max / mask and
// the gradient parts; the last CTA reduces the block sums into the loss.
template <int CB>
__global__ void __launch_bounds__(256) k_epilogue(ObjArgs a, int kspl, const float *Ypart,
                                                  float *G1, float *G2, double *partials,
                                                  unsigned *counter, float *scal,
                                                  const unsigned *err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  float sum_max = 0.f, sum_sq = 0.f;  // FP32 within a warp, FP64 across warps
  if (r < a.R) {
    c2 y[CB];
    float cap[CB], amp[CB];
    int arg = 0;
    float mx = -1.f;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      y[c] = {0.f, 0.f};
      if (c >= a.C) { cap[c] = 0.f; amp[c] = 0.f; continue; }
      int sp = 0;
      for (; sp + 4 <= kspl; sp += 4) {
        c2 v[4];
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = ld2(Ypart, ((size_t)(sp + j) * a.C + c) * a.R + r);
#pragma unroll
        for (int j = 0; j < 4; j++) { y[c].x += v[j].x; y[c].y += v[j].y; }
      }
      for (; sp < kspl; sp++) {
        c2 v = ld2(Ypart, ((size_t)sp * a.C + c) * a.R + r);
        y[c].x += v.x;
        y[c].y += v.y;
      }
      amp[c] = sqrtf(y[c].x * y[c].x + y[c].y * y[c].y);
      const float aa = amp[c] + kEps;
      float v = log2f(1.0f + aa * aa / kN0);
      if (a.drop && a.drop[c]) v = 0.f;
      cap[c] = v;
      if (v > mx) { mx = v; arg = c; }  // first index of the maximum
      if (a.recv_amp) a.recv_amp[(size_t)c * a.R + r] = amp[c];
    }
    sum_max = mx;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      if (c >= a.C) continue;
      const bool dropped = a.drop && a.drop[c];
      const float msk = (cap[c] != mx) ? cap[c] : 0.f;  // cap' * mask
      sum_sq += msk * msk;
      const float aa = amp[c] + kEps;
      const float dcap = (2.0f * aa / kN0) / (1.0f + aa * aa / kN0) * kInvLn2;
      float g1 = (c == arg) ? -a.w : 0.f, g2 = msk;
      if (dropped) { g1 = 0.f; g2 = 0.f; }
      const float sc = amp[c] > 0.f ? dcap / amp[c] : 0.f;
      reinterpret_cast<float2 *>(G1)[(size_t)c * a.R + r] =
          make_float2(g1 * sc * y[c].x, g1 * sc * y[c].y);
      if (G2)
        reinterpret_cast<float2 *>(G2)[(size_t)c * a.R + r] =
            make_float2(g2 * sc * y[c].x, g2 * sc * y[c].y);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum_max += __shfl_xor_sync(0xffffffffu, sum_max, o);
    sum_sq += __shfl_xor_sync(0xffffffffu, sum_sq, o);
  }
  __shared__ double sp[2][8];
  __shared__ bool last;
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { sp[0][wid] = sum_max; sp[1][wid] = sum_sq; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0, z = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) { x += sp[0][i]; z += sp[1][i]; }
    partials[2 * blockIdx.x] = x;
    partials[2 * blockIdx.x + 1] = z;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    double x, z;
    block_sum_pairs(partials, (int)gridDim.x, x, z);
    if (threadIdx.x == 0) {
      const double nrm = sqrt(z);
      if (a.loss) *a.loss = obj_failed(err) ? obj_nan() : (float)(-(double)a.w * x + nrm);
      scal[0] = nrm > 0 ? (float)(1.0 / nrm) : 0.f;
      *counter = 0u;  // ready for the next call
    }
  }
}

// epilogue for codebooks (CB >= 8): a CTA takes 32 Rx (one per lane) and
// its 8 warps split the codes (warp w: c = w, w + 8, ...), so a thread keeps
// CB / 8 codes.  The max over codes (first index on ties) is reduced across
// the warps in shared memory; then each thread writes its codes' gradient
// parts.  Loss partials and the last-CTA reduction as in k_epilogue.
template <int CB>
__global__ void __launch_bounds__(256) k_epilogue_wide(ObjArgs a, int kspl, const float *Ypart,
                                                       float *G1, float *G2, double *partials,
                                                       unsigned *counter, float *scal) {
  constexpr int CPT = CB / 8;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r = blockIdx.x * 32 + lane;
  const bool live = r < a.R;
  c2 y[CPT];
  float amp[CPT], cap[CPT];
  float mx = -1.f;
  int arg = 0x7fffffff;
  // all loads first (independent across codes), then the arithmetic
  const int rr = live ? r : 0;
  for (int sp = 0; sp < kspl; sp++) {
    c2 v[CPT];
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      const int c = min(wid + 8 * j, a.C - 1);
      v[j] = ld2(Ypart, ((size_t)sp * a.C + c) * a.R + rr);
    }
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      if (sp == 0) y[j] = v[j];
      else { y[j].x += v[j].x; y[j].y += v[j].y; }
    }
  }
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = wid + 8 * j;
    amp[j] = 0.f;
    cap[j] = 0.f;
    if (!live || c >= a.C) continue;
    amp[j] = sqrtf(y[j].x * y[j].x + y[j].y * y[j].y);
    const float aa = amp[j] + kEps;
    float v = log2f(1.0f + aa * aa / kN0);
    if (a.drop && a.drop[c]) v = 0.f;
    cap[j] = v;
    if (v > mx) { mx = v; arg = c; }  // codes ascend within a thread
    if (a.recv_amp) a.recv_amp[(size_t)c * a.R + r] = amp[j];
  }
  __shared__ float smx[8][32];
  __shared__ int sarg[8][32];
  smx[wid][lane] = mx;
  sarg[wid][lane] = arg;
  __syncthreads();
  float M_ = smx[0][lane];
  int A_ = sarg[0][lane];
#pragma unroll
  for (int w2 = 1; w2 < 8; w2++) {
    const float v = smx[w2][lane];
    const int g = sarg[w2][lane];
    if (v > M_ || (v == M_ && g < A_)) { M_ = v; A_ = g; }
  }
  // FP32 within a warp (FP64 arithmetic is slow here), FP64 across warps
  float sum_max = (live && wid == 0) ? M_ : 0.f, sum_sq = 0.f;
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = wid + 8 * j;
    if (!live || c >= a.C) continue;
    const bool dropped = a.drop && a.drop[c];
    const float msk = (cap[j] != M_) ? cap[j] : 0.f;
    sum_sq += msk * msk;
    const float aa = amp[j] + kEps;
    const float dcap = (2.0f * aa / kN0) / (1.0f + aa * aa / kN0) * kInvLn2;
    float g1 = (c == A_) ? -a.w : 0.f, g2 = msk;
    if (dropped) { g1 = 0.f; g2 = 0.f; }
    const float sc = amp[j] > 0.f ? dcap / amp[j] : 0.f;
    reinterpret_cast<float2 *>(G1)[(size_t)c * a.R + r] =
        make_float2(g1 * sc * y[j].x, g1 * sc * y[j].y);
    if (G2)
      reinterpret_cast<float2 *>(G2)[(size_t)c * a.R + r] =
          make_float2(g2 * sc * y[j].x, g2 * sc * y[j].y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum_max += __shfl_xor_sync(0xffffffffu, sum_max, o);
    sum_sq += __shfl_xor_sync(0xffffffffu, sum_sq, o);
  }
  __shared__ double spart[2][8];
  __shared__ bool last;
  if (lane == 0) { spart[0][wid] = sum_max; spart[1][wid] = sum_sq; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0, z = 0;
    for (int i = 0; i < 8; i++) { x += spart[0][i]; z += spart[1][i]; }
    partials[2 * blockIdx.x] = x;
    partials[2 * blockIdx.x + 1] = z;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    double x, z;
    block_sum_pairs(partials, (int)gridDim.x, x, z);
    if (threadIdx.x == 0) {
      const double nrm = sqrt(z);
      if (a.loss) *a.loss = (float)(-(double)a.w * x + nrm);
      scal[0] = nrm > 0 ? (float)(1.0 / nrm) : 0.f;
      *counter = 0u;  // ready for the next call
    }
  }
}

// Two-phase epilogue of the tensor-core path (CB >= 8), same thread layout
// as k_epilogue_wide.  Phase A: loss partials, and per Rx the max over codes
// and its first index.  Phase B: re-reads Y, forms G = G1 + G2 / ||masked||
// and writes it straight into the A operand of the adjoint GEMM (and
// grad_Y), so G1 / G2 are never stored.  Both phases evaluate the capacity
// with the same inline code, so they see bit-identical values.
template <int CPT>
__device__ __forceinline__ void epi_load_y(const ObjArgs &a, int kspl, const float *Ypart, int wid,
                                           int rr, c2 (&y)[CPT]) {
  for (int sp = 0; sp < kspl; sp++) {
    c2 v[CPT];
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      const int c = min(wid + 8 * j, a.C - 1);
      v[j] = ld2(Ypart, ((size_t)sp * a.C + c) * a.R + rr);
    }
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      if (sp == 0) y[j] = v[j];
      else { y[j].x += v[j].x; y[j].y += v[j].y; }
    }
  }
}
__device__ __forceinline__ void epi_cap(const ObjArgs &a, int c, c2 y, float &amp, float &cap) {
  amp = sqrtf(y.x * y.x + y.y * y.y);
  const float aa = amp + kEps;
  float v = log2f(1.0f + aa * aa / kN0);
  if (a.drop && a.drop[c]) v = 0.f;
  cap = v;
}

template <int CB>
__global__ void __launch_bounds__(256) k_tc_epi_a(ObjArgs a, int kspl, const float *Ypart,
                                                  float *maxr, int *argr, double *partials,
                                                  unsigned *counter, float *scal,
                                                  const unsigned *err) {
  constexpr int CPT = CB / 8;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r = blockIdx.x * 32 + lane;
  const bool live = r < a.R;
  c2 y[CPT];
  float cap[CPT];
  epi_load_y<CPT>(a, kspl, Ypart, wid, live ? r : 0, y);
  float mx = -1.f;
  int arg = 0x7fffffff;
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = wid + 8 * j;
    cap[j] = 0.f;
    if (!live || c >= a.C) continue;
    float amp;
    epi_cap(a, c, y[j], amp, cap[j]);
    if (cap[j] > mx) { mx = cap[j]; arg = c; }
    if (a.recv_amp) a.recv_amp[(size_t)c * a.R + r] = amp;
  }
  __shared__ float smx[8][32];
  __shared__ int sarg[8][32];
  smx[wid][lane] = mx;
  sarg[wid][lane] = arg;
  __syncthreads();
  float M_ = smx[0][lane];
  int A_ = sarg[0][lane];
#pragma unroll
  for (int w2 = 1; w2 < 8; w2++) {
    const float v = smx[w2][lane];
    const int g = sarg[w2][lane];
    if (v > M_ || (v == M_ && g < A_)) { M_ = v; A_ = g; }
  }
  if (wid == 0 && live) { maxr[r] = M_; argr[r] = A_; }
  // FP32 within a warp (FP64 arithmetic is slow here), FP64 across warps
  float sum_max = (live && wid == 0) ? M_ : 0.f, sum_sq = 0.f;
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = wid + 8 * j;
    if (!live || c >= a.C) continue;
    const float msk = (cap[j] != M_) ? cap[j] : 0.f;
    sum_sq += msk * msk;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum_max += __shfl_xor_sync(0xffffffffu, sum_max, o);
    sum_sq += __shfl_xor_sync(0xffffffffu, sum_sq, o);
  }
  __shared__ double spart[2][8];
  __shared__ bool last;
  if (lane == 0) { spart[0][wid] = sum_max; spart[1][wid] = sum_sq; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0, z = 0;
    for (int i = 0; i < 8; i++) { x += spart[0][i]; z += spart[1][i]; }
    partials[2 * blockIdx.x] = x;
    partials[2 * blockIdx.x + 1] = z;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    double x, z;
    block_sum_pairs(partials, (int)gridDim.x, x, z);
    if (threadIdx.x == 0) {
      const double nrm = sqrt(z);
      if (a.loss) *a.loss = obj_failed(err) ? obj_nan() : (float)(-(double)a.w * x + nrm);
      scal[0] = nrm > 0 ? (float)(1.0 / nrm) : 0.f;
      *counter = 0u;  // ready for the next call
    }
  }
}

template <int CB>
__global__ void __launch_bounds__(256) k_tc_epi_b(ObjArgs a, int kspl, const float *Ypart,
                                                  const float *maxr, const int *argr,
                                                  const float *scal, int K2p, __nv_bfloat16 *hi,
                                                  __nv_bfloat16 *lo) {
  constexpr int CPT = CB / 8;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r = blockIdx.x * 32 + lane;
  const bool live = r < a.R;
  c2 y[CPT];
  epi_load_y<CPT>(a, kspl, Ypart, wid, live ? r : 0, y);
  const float M_ = live ? maxr[r] : 0.f;
  const int A_ = live ? argr[r] : 0;
  const float inv = a.C > 1 ? scal[0] : 0.f;
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = wid + 8 * j;
    if (c >= a.C) continue;
    c2 g = {0.f, 0.f};
    if (live) {
      float amp, cap;
      epi_cap(a, c, y[j], amp, cap);
      const bool dropped = a.drop && a.drop[c];
      const float msk = (cap != M_) ? cap : 0.f;
      const float aa = amp + kEps;
      const float dcap = (2.0f * aa / kN0) / (1.0f + aa * aa / kN0) * kInvLn2;
      float g1 = (c == A_) ? -a.w : 0.f, g2 = msk;
      if (dropped) { g1 = 0.f; g2 = 0.f; }
      const float sc = amp > 0.f ? dcap / amp : 0.f;
      // G1 + G2 * inv with the rounding of k_tc_make_ag: fmaf(G2, inv, G1)
      const c2 q1 = {g1 * sc * y[j].x, g1 * sc * y[j].y};
      const c2 q2 = {g2 * sc * y[j].x, g2 * sc * y[j].y};
      g.x = fmaf(q2.x, inv, q1.x);
      g.y = fmaf(q2.y, inv, q1.y);
      if (a.grad_Y) reinterpret_cast<float2 *>(a.grad_Y)[(size_t)c * a.R + r] = make_float2(g.x, g.y);
    }
    if (r < K2p / 2) {
      put_pair(hi, lo, ((size_t)(2 * c) * K2p + 2 * r) / 2, g.x, g.y);
      put_pair(hi, lo, ((size_t)(2 * c + 1) * K2p + 2 * r) / 2, g.y, -g.x);
    }
  }
}

// G_U[c, k] = sum over the splits of the partials, one thread per entry
__global__ void k_gu_reduce(const float *GUp, int splits, long long n, float *GU) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = 0.f, y = 0.f;
  for (int s = 0; s < splits; s++) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(GUp) + (size_t)s * n + i);
    x += v.x;
    y += v.y;
  }
  reinterpret_cast<float2 *>(GU)[i] = make_float2(x, y);
}

// pass 2: partial G_U[c, k] = sum_r G[c, r] conj(row_k[r]) over an r-range;
// one warp per row, lanes stride over columns, G staged in shared memory.
template <int CB>
__global__ void __launch_bounds__(256) k_pass2(ObjArgs a, int M, int K, int rper, const float *G1,
                                               const float *G2, const float *scal, float *GUp) {
  constexpr int TR = CB <= 8 ? 256 : (CB <= 32 ? 64 : 32);
  __shared__ c2 sG[CB][TR];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = blockIdx.x * 8 + warp;
  const int r0 = blockIdx.y * rper, r1 = min(a.R, r0 + rper);
  const float inv = G2 ? scal[0] : 0.f;
  const float *row = k < K ? row_ptr(a.Hr, a.Hd, M, a.R, k) : nullptr;
  c2 acc[CB];
#pragma unroll
  for (int c = 0; c < CB; c++) acc[c] = {0.f, 0.f};
  for (int rc = r0; rc < r1; rc += TR) {
    const int rn = min(TR, r1 - rc);
    __syncthreads();
    for (int i = threadIdx.x; i < CB * TR; i += blockDim.x) {
      const int c = i / TR, rr = i % TR;
      c2 g = {0.f, 0.f};
      if (c < a.C && rr < rn) {
        g = ld2(G1, (size_t)c * a.R + rc + rr);
        if (G2) {
          const c2 h = ld2(G2, (size_t)c * a.R + rc + rr);
          g.x = fmaf(h.x, inv, g.x);
          g.y = fmaf(h.y, inv, g.y);
        }
      }
      sG[c][rr] = g;
    }
    __syncthreads();
    if (row) {
#pragma unroll 8
      for (int rr = lane; rr < rn; rr += 32) {
        const c2 h = ld2(row, (size_t)(rc + rr));
#pragma unroll
        for (int c = 0; c < CB; c++) macc(acc[c], sG[c][rr], h);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < CB; c++) {
    float x = acc[c].x, y = acc[c].y;
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if (lane == 0 && row && c < a.C)
      reinterpret_cast<float2 *>(GUp)[((size_t)blockIdx.y * a.C + c) * K + k] = make_float2(x, y);
  }
}

__device__ __forceinline__ c2 gu_sum(const float *GUp, int rspl, int C, int K, int c, int k) {
  c2 g = {0.f, 0.f};
  int sp = 0;
  for (; sp + 4 <= rspl; sp += 4) {
    c2 v[4];
#pragma unroll
    for (int j = 0; j < 4; j++) v[j] = ld2(GUp, ((size_t)(sp + j) * C + c) * K + k);
#pragma unroll
    for (int j = 0; j < 4; j++) { g.x += v[j].x; g.y += v[j].y; }
  }
  for (; sp < rspl; sp++) {
    const c2 v = ld2(GUp, ((size_t)sp * C + c) * K + k);
    g.x += v.x;
    g.y += v.y;
  }
  return g;
}

// final: each CTA owns 32 metasurface rows.  It reduces their G_U partials,
// writes dphi[m] = -sum_c Im(conj(G_U) U) and the partial sums
// sum_m G_U[c,m] e^{-j phi'_m} conj(H_a[s,m]) of dL/dW; the last CTA adds the
// CTAs' partials and the H_d rows G_U[c, M+s] into grad_W.
template <int CB>
__global__ void __launch_bounds__(256) k_final(ObjArgs a, int M, int K, int rspl, const float *U,
                                               const float *GUp, float *gw_part,
                                               unsigned *counter) {
  __shared__ c2 gu[CB][32];
  __shared__ c2 ph[32];
  __shared__ bool last;
  const int m0 = blockIdx.x * 32;
  const int t = threadIdx.x;
  const int nm = max(0, min(32, M - m0));
  for (int i = t; i < CB * 32; i += blockDim.x) {
    const int c = i / 32, j = i % 32;
    gu[c][j] = (c < a.C && j < nm) ? gu_sum(GUp, rspl, a.C, K, c, m0 + j) : c2{0.f, 0.f};
  }
  if (t < 32) {
    c2 e = {0.f, 0.f};
    if (t < nm) {
      const float p = py_mod(__ldg(a.phi + m0 + t), a.max_phase);
      sincosf(p, &e.y, &e.x);
    }
    ph[t] = e;
  }
  __syncthreads();
  if (a.grad_phi && t < nm) {
    float sacc = 0.f;
    for (int c = 0; c < a.C; c++) {
      const c2 g = gu[c][t], u = ld2(U, (size_t)c * M + m0 + t);
      sacc += g.x * u.y - g.y * u.x;  // Im(conj(g) u)
    }
    a.grad_phi[m0 + t] = -sacc;
  }
  if (!a.grad_W) return;
  for (int i = t; i < a.C * a.S; i += blockDim.x) {
    const int c = i / a.S, s2 = i % a.S;
    c2 acc = {0.f, 0.f};
    for (int j = 0; j < nm; j++) {
      const c2 g = gu[c][j], e = ph[j];
      const c2 gv = {g.x * e.x + g.y * e.y, g.y * e.x - g.x * e.y};  // g e^{-j p}
      macc(acc, gv, ld2(a.Ha, (size_t)s2 * M + m0 + j));
    }
    reinterpret_cast<float2 *>(gw_part)[(size_t)blockIdx.x * a.C * a.S + i] = make_float2(acc.x, acc.y);
  }
  __threadfence();
  __syncthreads();
  if (t == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int i = t; i < a.C * a.S; i += blockDim.x) {
    const int c = i / a.S, s2 = i % a.S;
    c2 acc = gu_sum(GUp, rspl, a.C, K, c, M + s2);
    const volatile float2 *pp = reinterpret_cast<const volatile float2 *>(gw_part);
    for (int b = 0; b < (int)gridDim.x; b++) {
      acc.x += pp[(size_t)b * a.C * a.S + i].x;
      acc.y += pp[(size_t)b * a.C * a.S + i].y;
    }
    reinterpret_cast<float2 *>(a.grad_W)[i] = make_float2(acc.x, acc.y);
  }
  if (t == 0) *counter = 0u;  // ready for the next call
}

// dphi[m] = -sum_c Im(conj(G_U[c, m]) U[c, m]); a CTA takes 32 elements
// (lanes) and its 8 warps split the codes
__global__ void __launch_bounds__(256) k_tc_dphi(const float *GU, const float *U, int C, int M,
                                                 int K, float *dphi, const unsigned *err) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int m = blockIdx.x * 32 + lane;
  float acc = 0.f;
  if (m < M)
    for (int c = wid; c < C; c += 8) {
      const float2 g = __ldg(reinterpret_cast<const float2 *>(GU) + (size_t)c * K + m);
      const float2 u = __ldg(reinterpret_cast<const float2 *>(U) + (size_t)c * M + m);
      acc += g.x * u.y - g.y * u.x;
    }
  __shared__ float red[8][32];
  red[wid][lane] = acc;
  __syncthreads();
  if (wid == 0 && m < M) {
    float t = 0.f;
#pragma unroll
    for (int w2 = 0; w2 < 8; w2++) t += red[w2][lane];
    dphi[m] = obj_failed(err) ? obj_nan() : -t;
  }
}

// grad_W[c, s] = G_U[c, M + s] + sum_m G_U[c, m] e^{-j phi'_m} conj(H_a[s, m]).
// k_tc_dw_part: CTA (c, part) takes a slice of the m range, one element per
// thread, keeps 16 AP elements' sums at a time in registers (H_a loads
// coalesced over m) and writes the CTA's sums to dwp[c][part][s];
// k_tc_dw_sum adds the slices and the H_d term.
constexpr int kDwParts = 8;
__global__ void __launch_bounds__(128) k_tc_dw_part(const float *GU, const float *Ha,
                                                    const float *phi, float max_phase, int S,
                                                    int M, int K, float *dwp) {
  constexpr int SB = 16;
  __shared__ float2 red[4][SB];
  const int c = blockIdx.x, part = blockIdx.y;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int per = (M + kDwParts - 1) / kDwParts;
  const int m_lo = part * per, m_hi = min(M, m_lo + per);
  for (int s0 = 0; s0 < S; s0 += SB) {
    c2 acc[SB];
#pragma unroll
    for (int q = 0; q < SB; q++) acc[q] = {0.f, 0.f};
    for (int m = m_lo + threadIdx.x; m < m_hi; m += blockDim.x) {
      const float2 g = __ldg(reinterpret_cast<const float2 *>(GU) + (size_t)c * K + m);
      float sn, cs;
      sincosf(py_mod(__ldg(phi + m), max_phase), &sn, &cs);
      const c2 ge = {g.x * cs + g.y * sn, g.y * cs - g.x * sn};  // g e^{-j p}
#pragma unroll
      for (int q = 0; q < SB; q++)
        if (s0 + q < S) macc(acc[q], ge, ld2(Ha, (size_t)(s0 + q) * M + m));
    }
#pragma unroll
    for (int q = 0; q < SB; q++) {
      float x = acc[q].x, y = acc[q].y;
      for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
      }
      if (lane == 0) red[wid][q] = make_float2(x, y);
    }
    __syncthreads();
    if (threadIdx.x < SB && s0 + threadIdx.x < S) {
      float2 t = red[0][threadIdx.x];
#pragma unroll
      for (int w2 = 1; w2 < 4; w2++) { t.x += red[w2][threadIdx.x].x; t.y += red[w2][threadIdx.x].y; }
      reinterpret_cast<float2 *>(dwp)[((size_t)c * kDwParts + part) * S + s0 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

// out[c][j] = GU[c][k0 + j], j < n (complex), NaN after a run-out wait
__global__ void k_tc_copy_rows(const float *GU, int K, int k0, int n, int C, float *out,
                               const unsigned *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C * n) return;
  const int c = i / n, j = i % n;
  float2 v = __ldg(reinterpret_cast<const float2 *>(GU) + (size_t)c * K + k0 + j);
  if (obj_failed(err)) v = make_float2(obj_nan(), obj_nan());
  reinterpret_cast<float2 *>(out)[i] = v;
}

__global__ void k_tc_dw_sum(const float *GU, const float *dwp, int C, int S, int M, int K,
                            float *grad_W, const unsigned *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C * S) return;
  const int c = i / S, s2 = i % S;
  float2 t = __ldg(reinterpret_cast<const float2 *>(GU) + (size_t)c * K + M + s2);
  for (int q = 0; q < kDwParts; q++) {
    const float2 v = reinterpret_cast<const float2 *>(dwp)[((size_t)c * kDwParts + q) * S + s2];
    t.x += v.x;
    t.y += v.y;
  }
  if (obj_failed(err)) t = make_float2(obj_nan(), obj_nan());
  reinterpret_cast<float2 *>(grad_W)[i] = t;
}

// Streaming paths, after the streaming kernel: one CTA per 32 rows k of
// [H_r; H_d] (lanes, loads coalesced over k), 32 warps.
//   G_U[c, k] = sum_b P1[b][c][k] + (sum_b P2[b][c][k]) / ||masked||, the
//     warps splitting the CTA partials b; every CTA derives 1/||masked|| from
//     the loss partials (CTA 0 also writes the loss);
//   dphi[k] = -sum_c Im(conj(G_U[c, k]) U[c, k]) for metasurface rows;
//   dwp[blk][c][s] = sum over the CTA's metasurface rows of
//     G_U[c, k] e^{-j phi'_k} conj(H_a[s, k]), warp w taking s = w, w + 32, ...
// The last CTA to finish (arrival counter) forms dL/dW: the H_d rows
// G_U[c, M + s] plus the CTAs' dwp, a warp per entry with lanes over CTAs.
template <int CB>
__global__ void __launch_bounds__(1024) k_stream_tail(ObjArgs a, int M, int nparts,
                                                      const float *Ppart, const double *lpart,
                                                      const float *U, float *GU, float *dwp,
                                                      unsigned *counter, const unsigned *err) {
  constexpr int NW = 32;
  const int K = M + a.S;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  // call inputs (not written by the streaming grid) are fetched before the
  // wait: this warp's first H_a row for the dL/dW part and phi for the phase
  const c2 ha_first = warp < a.S && k < M ? ld2(a.Ha, (size_t)warp * M + k) : c2{0.f, 0.f};
  const float phi_k = warp == 0 && k < M ? __ldg(a.phi + k) : 0.f;
  // launched early (programmatic dependent launch): wait for the streaming
  // grid to complete before reading its partials or its wait-timeout word
  cudaGridDependencySynchronize();
  // a bounded wait of the streaming kernel ran out: its partials are
  // incomplete, so every output of the call is NaN
  const bool bad = obj_failed(err);
  __shared__ float inv_s;
  __shared__ c2 r1[NW][CB][32], r2[NW][CB][32];
  __shared__ c2 gv[CB][32];
  // Every loop below issues a batch of UNR independent loads before adding
  // them (in the same order as one load per iteration would), so a warp pays
  // one memory round trip per batch rather than one per partial.
  constexpr int UNR = 8;
  if (warp == 1) {
    double x = 0.0, z = 0.0;
    for (int b0 = lane; b0 < nparts; b0 += 32 * UNR) {
      double xv[UNR], zv[UNR];
#pragma unroll
      for (int u = 0; u < UNR; u++) {
        const int b = b0 + 32 * u;
        xv[u] = b < nparts ? lpart[2 * b] : 0.0;
        zv[u] = b < nparts ? lpart[2 * b + 1] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < UNR; u++) { x += xv[u]; z += zv[u]; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      z += __shfl_xor_sync(0xffffffffu, z, o);
    }
    if (lane == 0) {
      const double nrm = sqrt(z);
      inv_s = nrm > 0 ? (float)(1.0 / nrm) : 0.f;
      if (blockIdx.x == 0 && a.loss) *a.loss = bad ? obj_nan() : (float)(-(double)a.w * x + nrm);
    }
  }
  const float2 *P = reinterpret_cast<const float2 *>(Ppart);
  const int kk = k < K ? k : K - 1;
  c2 s1[CB], s2[CB];
#pragma unroll
  for (int c = 0; c < CB; c++) { s1[c] = {0.f, 0.f}; s2[c] = {0.f, 0.f}; }
  constexpr int UNP = UNR / CB;  // partial loads per batch (registers)
  for (int b0 = warp; b0 < nparts; b0 += NW * UNP) {
    float2 pu[UNP][CB], pv[UNP][CB];
#pragma unroll
    for (int u = 0; u < UNP; u++) {
      const int b = b0 + NW * u;
#pragma unroll
      for (int c = 0; c < CB; c++) {
        const bool on = b < nparts && c < a.C;
        pu[u][c] = on ? __ldg(P + ((size_t)b * 2 * a.C + c) * K + kk) : make_float2(0.f, 0.f);
        if (CB > 1)
          pv[u][c] = on ? __ldg(P + ((size_t)b * 2 * a.C + a.C + c) * K + kk)
                        : make_float2(0.f, 0.f);
      }
    }
#pragma unroll
    for (int u = 0; u < UNP; u++) {
#pragma unroll
      for (int c = 0; c < CB; c++) {
        if (b0 + NW * u >= nparts || c >= a.C) continue;
        s1[c].x += pu[u][c].x;
        s1[c].y += pu[u][c].y;
        if (CB > 1) {
          s2[c].x += pv[u][c].x;
          s2[c].y += pv[u][c].y;
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < CB; c++) { r1[warp][c][lane] = s1[c]; r2[warp][c][lane] = s2[c]; }
  __syncthreads();
  if (warp == 0) {
    const float inv = inv_s;
    c2 e = {1.f, 0.f};
    const bool ms_row = k < M;
    if (ms_row) {
      const float pp = py_mod(phi_k, a.max_phase);
      sincosf(pp, &e.y, &e.x);
    }
    float dph = 0.f;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      c2 g = {0.f, 0.f};
      if (c < a.C && k < K) {
        c2 t1 = {0.f, 0.f}, t2 = {0.f, 0.f};
#pragma unroll 8
        for (int w = 0; w < NW; w++) {
          t1.x += r1[w][c][lane].x; t1.y += r1[w][c][lane].y;
          t2.x += r2[w][c][lane].x; t2.y += r2[w][c][lane].y;
        }
        g = {fmaf(t2.x, inv, t1.x), fmaf(t2.y, inv, t1.y)};
        reinterpret_cast<float2 *>(GU)[(size_t)c * K + k] = make_float2(g.x, g.y);
        if (ms_row) {
          const c2 u = ld2(U, (size_t)c * M + k);
          dph += g.x * u.y - g.y * u.x;  // Im(conj(g) u)
        }
      }
      // g e^{-j phi'} of metasurface rows (zero elsewhere) for the dW sums
      gv[c][lane] = ms_row && c < a.C ? c2{g.x * e.x + g.y * e.y, g.y * e.x - g.x * e.y}
                                      : c2{0.f, 0.f};
    }
    if (ms_row && a.grad_phi) a.grad_phi[k] = bad ? obj_nan() : -dph;
  }
  if (!a.grad_W) return;
  __syncthreads();
  for (int s2 = warp; s2 < a.S; s2 += NW) {
    const c2 h = s2 == warp ? ha_first : k < M ? ld2(a.Ha, (size_t)s2 * M + k) : c2{0.f, 0.f};
#pragma unroll
    for (int c = 0; c < CB; c++) {
      if (c >= a.C) continue;
      c2 d = {0.f, 0.f};
      macc(d, gv[c][lane], h);
      for (int o = 16; o > 0; o >>= 1) {
        d.x += __shfl_xor_sync(0xffffffffu, d.x, o);
        d.y += __shfl_xor_sync(0xffffffffu, d.y, o);
      }
      if (lane == 0)
        reinterpret_cast<float2 *>(dwp)[((size_t)blockIdx.x * a.C + c) * a.S + s2] =
            make_float2(d.x, d.y);
    }
  }
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int i = warp; i < a.C * a.S; i += NW) {
    const int c = i / a.S, s2 = i % a.S;
    const float2 g = __ldcg(reinterpret_cast<const float2 *>(GU) + (size_t)c * K + M + s2);
    c2 acc = {0.f, 0.f};
    for (int b = lane; b < (int)gridDim.x; b += 32) {
      const float2 v = __ldcg(reinterpret_cast<const float2 *>(dwp) + (size_t)b * a.C * a.S + i);
      acc.x += v.x;
      acc.y += v.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) {
      reinterpret_cast<float2 *>(a.grad_W)[i] =
          bad ? make_float2(obj_nan(), obj_nan()) : make_float2(g.x + acc.x, g.y + acc.y);
    }
  }
  if (threadIdx.x == 0) *counter = 0u;  // ready for the next call
}

// grad_Y = G1 + G2 / ||masked||
__global__ void k_grad_y(const float *G1, const float *G2, const float *scal, long long n,
                         float *out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float inv = G2 ? scal[0] : 0.f;
  c2 g = ld2(G1, i);
  if (G2) {
    const c2 h = ld2(G2, i);
    g.x = fmaf(h.x, inv, g.x);
    g.y = fmaf(h.y, inv, g.y);
  }
  reinterpret_cast<float2 *>(out)[i] = make_float2(g.x, g.y);
}

int cbucket(int C) {
  int b = 1;
  while (b < C) b <<= 1;
  return b;
}

// CTAs the CUDA-core split path aims for: a work split that fills a device
// of this size (8 per SM on a 152-SM GB300) and that fixes the scratch
// layout, so it is a constant rather than a device query
constexpr int kTargetBlocks = 1216;

struct Split {
  int K, kspl, kper, rspl, rper, nb_epi;
};

Split make_split(int S, int M, int R) {
  Split sp;
  sp.K = M + S;
  const int bx = (R + 31) / 32;
  sp.kspl = std::max(1, std::min((kTargetBlocks + bx - 1) / bx, (sp.K + 63) / 64));
  sp.kper = (sp.K + sp.kspl - 1) / sp.kspl;
  sp.kspl = (sp.K + sp.kper - 1) / sp.kper;
  const int by = (sp.K + 7) / 8;
  sp.rspl = std::max(1, std::min((kTargetBlocks + by - 1) / by, (R + 255) / 256));
  sp.rper = (R + sp.rspl - 1) / sp.rspl;
  sp.rspl = (R + sp.rper - 1) / sp.rper;
  sp.nb_epi = (R + 127) / 128;
  return sp;
}

template <int CB>
cudaError_t run_cb(const ObjArgs &a, const Split &sp, int M, float *U, float *Ypart, float *G1,
                   float *G2, double *part, unsigned *counter, float *scal, float *GUp,
                   float *gw_part, cudaStream_t st) {
  if (M > 0) {
    dim3 gp((M + 127) / 128, a.C);
    k_prep<<<gp, 128, 0, st>>>(a, M, U, nullptr);
  }
  dim3 g1((a.R + 31) / 32, sp.kspl);
  k_pass1<CB><<<g1, 256, 0, st>>>(a, M, sp.K, sp.kper, U, Ypart);
  if (CB >= 8)
    k_epilogue_wide<(CB >= 8 ? CB : 8)><<<(a.R + 31) / 32, 256, 0, st>>>(a, sp.kspl, Ypart, G1,
                                                                        G2, part, counter, scal);
  else
    k_epilogue<CB><<<sp.nb_epi, 128, 0, st>>>(a, sp.kspl, Ypart, G1, G2, part, counter, scal,
                                              nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (a.grad_Y) {
    const long long n = (long long)a.C * a.R;
    k_grad_y<<<(int)((n + 255) / 256), 256, 0, st>>>(G1, G2, scal, n, a.grad_Y);
  }
  if (!a.grad_W && !a.grad_phi) return cudaGetLastError();
  dim3 g2((sp.K + 7) / 8, sp.rspl);
  k_pass2<CB><<<g2, 256, 0, st>>>(a, M, sp.K, sp.rper, G1, G2, scal, GUp);
  const int nbf = std::max(1, (M + 31) / 32);
  k_final<CB><<<nbf, 256, 0, st>>>(a, M, sp.K, sp.rspl, U, GUp, gw_part, counter + 1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------
// Single-pass streaming path (one HBM read of H_r and H_d).
//
// A persistent CTA per SM walks column tiles of TR Rx.  For each tile the
// TMA engine copies the (M + S) x TR complex block of [H_r; H_d] into a
// 2-stage shared-memory ring (cp.async.bulk.tensor, mbarrier completion);
// the CTA then (A) forms Y for the TR columns, (B) evaluates the per-Rx
// capacity, max and mask and the two gradient parts, and (C) accumulates
// P1[c,k] += sum_col G1[c,col] conj(H[k,col]) (and P2 for the norm term)
// from the same shared-memory tile.  The per-CTA P1/P2 and loss partials are
// reduced by k_stream_gu; k_tc_dphi and k_tc_dw_part / k_tc_dw_sum then form
// dphi and dL/dW.

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// bounded mbarrier wait of the tcgen05 kernels (tc_ptx.cuh): try_wait with a
// suspend-time hint, so waiting warps sleep instead of taking issue slots
// from the other CTA on the SM; false after 2 s
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  return tc::mbar_wait(bar, parity);
}

// the coefficients of the virtual rows into shared memory, coef[k][c]: U for
// metasurface rows, W for the H_d rows.  Four loads per thread are issued
// before their stores, so the staging costs one memory round trip per four
// rows instead of one per row.
template <int NTH, int CB>
__device__ __forceinline__ void stage_coef(const ObjArgs &a, int M, int K, const float *U,
                                           c2 *coef) {
  const int n = K * CB;
  for (int i0 = threadIdx.x; i0 < n; i0 += 4 * NTH) {
    c2 v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int i = i0 + u * NTH, k = i / CB, c = i % CB;
      v[u] = {0.f, 0.f};
      if (i < n && c < a.C)
        v[u] = k < M ? ld2(U, (size_t)c * M + k) : ld2(a.W, (size_t)c * a.S + (k - M));
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (i0 + u * NTH < n) coef[i0 + u * NTH] = v[u];
  }
}

template <int CB, int TR, int KPT>
__global__ void __launch_bounds__(256, 2)
    k_obj_stream(ObjArgs a, const __grid_constant__ CUtensorMap mapR,
                 const __grid_constant__ CUtensorMap mapD, int M, int Mbox, int Mp, int boxR,
                 int stage_bytes, int ntiles, const float *U, float *Ppart, double *lpart,
                 unsigned *err) {
  constexpr int NTH = 256, NW = NTH / 32;
  const int K = M + a.S;
  // H_r rows [0, Mbox) come from boxes of boxR rows, H_d rows start at Mp
  // (a multiple of 16, so every TMA destination is 128-byte aligned)
  const uint32_t tx_bytes = (uint32_t)(Mbox + a.S) * TR * 8;
  extern __shared__ unsigned char smem_dyn[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
  c2 *coef = reinterpret_cast<c2 *>(base + 2 * (size_t)stage_bytes);   // [K][CB]
  __shared__ c2 red[NW][TR][CB];
  __shared__ c2 g1s[CB][TR], g2s[CB][TR];
  __shared__ __align__(8) uint64_t full[2];
  __shared__ int abort_flag;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

  auto issue = [&](int tile, int stage) {
    float2 *dst = reinterpret_cast<float2 *>(base + (size_t)stage * stage_bytes);
    uint64_t *bar = &full[stage];
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(tx_bytes)
                 : "memory");
    const int x = tile * TR * 2;
    for (int m0 = 0; m0 < Mbox; m0 += boxR)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
          " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst + (size_t)m0 * TR)),
          "l"(reinterpret_cast<uint64_t>(&mapR)), "r"(x), "r"(m0), "r"(smem_addr(bar))
          : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst + (size_t)Mp * TR)),
        "l"(reinterpret_cast<uint64_t>(&mapD)), "r"(x), "r"(0), "r"(smem_addr(bar))
        : "memory");
  };
  const int first = blockIdx.x;
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&full[0])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&full[1])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    if (first < ntiles) issue(first, 0);
    if (first + (int)gridDim.x < ntiles) issue(first + gridDim.x, 1);
  }
  // the first tiles are in flight; wait for the U kernel, then stage the
  // coefficients: U for metasurface rows, W for the H_d rows
  cudaGridDependencySynchronize();
  stage_coef<NTH, CB>(a, M, K, U, coef);
  __syncthreads();

  c2 p1[KPT][CB], p2[KPT][CB];
#pragma unroll
  for (int q = 0; q < KPT; q++)
#pragma unroll
    for (int c = 0; c < CB; c++) { p1[q][c] = {0.f, 0.f}; p2[q][c] = {0.f, 0.f}; }
  float sum_max = 0.f, sum_sq = 0.f;  // FP32 within a warp, FP64 across warps
  const int col = t % TR, j = t / TR;
  constexpr int NJ = NTH / TR;

  int it = 0;
  for (int tile = first; tile < ntiles; tile += gridDim.x, it++) {
    const int stg = it & 1;
    if (!mbar_wait_bounded(&full[stg], (it >> 1) & 1)) {
      if (t == 0) atomicOr(err, 1u);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) {
      // before the CTA exits, let the copies it issued land (bounded again):
      // this tile's and, if it was issued, the next tile's in the other stage
      if (t == 0) {
        mbar_wait_bounded(&full[stg], (it >> 1) & 1);
        if (tile + (int)gridDim.x < ntiles) mbar_wait_bounded(&full[stg ^ 1], ((it + 1) >> 1) & 1);
      }
      break;
    }
    const float2 *T = reinterpret_cast<const float2 *>(base + (size_t)stg * stage_bytes);
    // (A) Y for the tile's columns; lanes with equal col are TR apart
    c2 y[CB];
#pragma unroll
    for (int c = 0; c < CB; c++) y[c] = {0.f, 0.f};
#pragma unroll 4
    for (int k = j; k < K; k += NJ) {
      const int row = k < M ? k : Mp + (k - M);
      const float2 h = T[(size_t)row * TR + col];
#pragma unroll
      for (int c = 0; c < CB; c++) mac(y[c], coef[(size_t)k * CB + c], c2{h.x, h.y});
    }
#pragma unroll
    for (int c = 0; c < CB; c++)
      for (int o = TR; o < 32; o <<= 1) {
        y[c].x += __shfl_xor_sync(0xffffffffu, y[c].x, o);
        y[c].y += __shfl_xor_sync(0xffffffffu, y[c].y, o);
      }
    if (lane < TR)
#pragma unroll
      for (int c = 0; c < CB; c++) red[warp][lane][c] = y[c];
    __syncthreads();
    // (B) per-Rx capacity, max, mask, gradient parts
    if (t < TR) {
      const int r = tile * TR + t;
      c2 yy[CB];
      float cap[CB], amp[CB];
#pragma unroll
      for (int c = 0; c < CB; c++) {
        c2 acc = {0.f, 0.f};
#pragma unroll
        for (int w = 0; w < NW; w++) { acc.x += red[w][t][c].x; acc.y += red[w][t][c].y; }
        yy[c] = acc;
      }
      int arg = 0;
      float mx = -1.f;
#pragma unroll
      for (int c = 0; c < CB; c++) {
        if (c >= a.C) { cap[c] = 0.f; amp[c] = 0.f; continue; }
        amp[c] = sqrtf(yy[c].x * yy[c].x + yy[c].y * yy[c].y);
        const float aa = amp[c] + kEps;
        float v = log2f(1.0f + aa * aa / kN0);
        if (a.drop && a.drop[c]) v = 0.f;
        cap[c] = v;
        if (v > mx) { mx = v; arg = c; }
        if (a.recv_amp && r < a.R) a.recv_amp[(size_t)c * a.R + r] = amp[c];
      }
#pragma unroll
      for (int c = 0; c < CB; c++) {
        c2 ga = {0.f, 0.f}, gb = {0.f, 0.f};
        if (c < a.C && r < a.R) {
          const bool dropped = a.drop && a.drop[c];
          const float msk = (cap[c] != mx) ? cap[c] : 0.f;
          sum_sq += msk * msk;
          const float aa = amp[c] + kEps;
          const float dcap = (2.0f * aa / kN0) / (1.0f + aa * aa / kN0) * kInvLn2;
          float g1 = (c == arg) ? -a.w : 0.f, g2 = msk;
          if (dropped) { g1 = 0.f; g2 = 0.f; }
          const float sc = amp[c] > 0.f ? dcap / amp[c] : 0.f;
          ga = {g1 * sc * yy[c].x, g1 * sc * yy[c].y};
          gb = {g2 * sc * yy[c].x, g2 * sc * yy[c].y};
        }
        g1s[c][t] = ga;
        g2s[c][t] = gb;
      }
      if (r < a.R) sum_max += mx;
    }
    __syncthreads();
    // (C) P += G conj(H) over the tile's columns, rows k = t + NTH q; the
    // column order is rotated by the lane so a warp's reads spread over banks
#pragma unroll
    for (int q = 0; q < KPT; q++) {
      const int k = t + NTH * q;
      if (k < K) {
        const int row = k < M ? k : Mp + (k - M);
        const float2 *hr = T + (size_t)row * TR;
#pragma unroll
        for (int cc0 = 0; cc0 < TR; cc0++) {
          const int cc = (cc0 + lane) & (TR - 1);
          const float2 h = hr[cc];
#pragma unroll
          for (int c = 0; c < CB; c++) {
            macc(p1[q][c], g1s[c][cc], c2{h.x, h.y});
            if (CB > 1) macc(p2[q][c], g2s[c][cc], c2{h.x, h.y});
          }
        }
      }
    }
    __syncthreads();
    // the stage is free: order the generic reads before the async-proxy refill
    if (t == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (tile + 2 * (int)gridDim.x < ntiles) issue(tile + 2 * gridDim.x, stg);
    }
  }
  // the tail kernel may launch now; its grid-dependency wait still waits for
  // this grid to complete, with every write below visible
  cudaTriggerProgrammaticLaunchCompletion();
  // partials of this CTA: P1 at [b][c][k], P2 at [b][C + c][k]
#pragma unroll
  for (int q = 0; q < KPT; q++) {
    const int k = t + NTH * q;
    if (k >= K) continue;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      if (c >= a.C) continue;
      float2 *o = reinterpret_cast<float2 *>(Ppart) + ((size_t)blockIdx.x * 2 * a.C + c) * K + k;
      o[0] = make_float2(p1[q][c].x, p1[q][c].y);
      if (CB > 1) o[(size_t)a.C * K] = make_float2(p2[q][c].x, p2[q][c].y);
    }
  }
  if (t < 32) {
    for (int o = 16; o > 0; o >>= 1) {
      sum_max += __shfl_xor_sync(0xffffffffu, sum_max, o);
      sum_sq += __shfl_xor_sync(0xffffffffu, sum_sq, o);
    }
    if (t == 0) {
      lpart[2 * blockIdx.x] = sum_max;
      lpart[2 * blockIdx.x + 1] = sum_sq;
    }
  }
}


using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                              const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                              const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn tmap_encoder() {
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

// complex [rows, R] as a float [rows, 2R] tensor; box (2 TR floats) x box_rows
bool make_cmap(CUtensorMap *m, const float *base, int rows, int R, int TR, int box_rows) {
  EncodeFn enc = tmap_encoder();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)2 * R, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)R * 8};
  cuuint32_t box[2] = {(cuuint32_t)(2 * TR), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct StreamPlan {
  bool ok = false;
  int TR = 0, KPT = 0, Mbox = 0, Mp = 0, boxR = 0, stage_bytes = 0, ntiles = 0, grid = 0;
  size_t smem = 0;
};

int sm_count() { return ams_device_sms(); }

// the single-pass path needs the whole [H_r; H_d] column tile in shared memory
StreamPlan stream_plan(int S, int M, int R, int C, bool grad_y) {
  StreamPlan p;
  const int CB = cbucket(C);
  if (grad_y || CB > 2 || R % 2 || S > 256 || M < 0) return p;
  const int K = M + S;
  const int kpt = (K + 255) / 256;
  int KPT = kpt <= 4 ? 4 : (kpt <= 8 ? 8 : (kpt <= 16 ? 16 : 0));
  if (!KPT || (CB == 2 && KPT > 8)) return p;
  p.boxR = M <= 256 ? std::max(M, 1) : 256;
  p.Mbox = M <= 0 ? 0 : (M + p.boxR - 1) / p.boxR * p.boxR;
  p.Mp = (p.Mbox + 15) / 16 * 16;
  for (int TR : {8, 4, 2}) {
    const size_t stage = ((size_t)(p.Mp + S) * TR * 8 + 1023) / 1024 * 1024;
    const size_t smem = 1024 + 2 * stage + (size_t)K * CB * 8;
    if (smem <= 110 * 1024) {  // two CTAs per SM
      p.TR = TR;
      p.stage_bytes = (int)stage;
      p.smem = smem;
      break;
    }
  }
  if (!p.TR) return p;
  p.KPT = KPT;
  p.ntiles = (R + p.TR - 1) / p.TR;
  p.grid = std::min(2 * sm_count(), p.ntiles);
  p.ok = true;
  return p;
}

template <int CB, int TR, int KPT>
cudaError_t launch_stream_t(const ObjArgs &a, const StreamPlan &pl, const CUtensorMap &mr,
                            const CUtensorMap &md, int M, const float *U, float *Ppart,
                            double *lpart, unsigned *err, cudaStream_t st) {
  auto kfn = k_obj_stream<CB, TR, KPT>;
  static size_t set_bytes[AMS_MAX_DEVICES] = {0};
  {
    cudaError_t e = ams_set_smem_atleast(set_bytes, kfn, pl.smem);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(pl.grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = pl.smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kfn, a, mr, md, M, pl.Mbox, pl.Mp, pl.boxR, pl.stage_bytes,
                            pl.ntiles, U, Ppart, lpart, err);
}

template <int CB, int TR>
cudaError_t launch_stream_k(const ObjArgs &a, const StreamPlan &pl, const CUtensorMap &mr,
                            const CUtensorMap &md, int M, const float *U, float *Ppart,
                            double *lpart, unsigned *err, cudaStream_t st) {
  switch (pl.KPT) {
    case 4: return launch_stream_t<CB, TR, 4>(a, pl, mr, md, M, U, Ppart, lpart, err, st);
    case 8: return launch_stream_t<CB, TR, 8>(a, pl, mr, md, M, U, Ppart, lpart, err, st);
    case 16:
      if (CB == 1) return launch_stream_t<1, TR, 16>(a, pl, mr, md, M, U, Ppart, lpart, err, st);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

template <int CB>
cudaError_t stream_tail(const ObjArgs &a, int M, int nparts, const float *U, const float *Pp,
                        const double *lp, float *GU, float *dwp, unsigned *counter,
                        const unsigned *err, cudaStream_t st);

template <int CB>
cudaError_t run_stream(const ObjArgs &a, const StreamPlan &pl, int M, float *U, float *Ppart,
                       double *lpart, float *GU, float *dwp, unsigned *err, unsigned *counter,
                       cudaStream_t st) {
  CUtensorMap mr, md;
  const float *Hr = M > 0 ? a.Hr : a.Hd;  // no metasurface: mapR is unused (Mbox = 0)
  if (!make_cmap(&mr, Hr, std::max(M, 1), a.R, pl.TR, pl.boxR) ||
      !make_cmap(&md, a.Hd, a.S, a.R, pl.TR, a.S))
    return cudaErrorInvalidValue;
  if (M > 0) {
    const long long n = (long long)M * a.C * 8;
    k_prep_wide<<<(int)((n + 255) / 256), 256, 0, st>>>(a, M, U, err);
  }
  cudaError_t e = obj_begin_call(err, M > 0, st);
  if (e != cudaSuccess) return e;
  switch (pl.TR) {
    case 8: e = launch_stream_k<CB, 8>(a, pl, mr, md, M, U, Ppart, lpart, err, st); break;
    case 4: e = launch_stream_k<CB, 4>(a, pl, mr, md, M, U, Ppart, lpart, err, st); break;
    default: e = launch_stream_k<CB, 2>(a, pl, mr, md, M, U, Ppart, lpart, err, st); break;
  }
  if (e != cudaSuccess) return e;
  return stream_tail<CB>(a, M, pl.grid, U, Ppart, lpart, GU, dwp, counter, err, st);
}

// after a streaming kernel: G_U, dphi and the dL/dW parts, then dL/dW
template <int CB>
cudaError_t stream_tail(const ObjArgs &a, int M, int nparts, const float *U, const float *Pp,
                        const double *lp, float *GU, float *dwp, unsigned *counter,
                        const unsigned *err, cudaStream_t st) {
  const int K = M + a.S, nblk = (K + 31) / 32;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblk);
  cfg.blockDim = dim3(1024);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_stream_tail<CB>, a, M, nparts, Pp, lp, U, GU, dwp, counter,
                            err);
}

// ------------------------------------------------------------------
// Streaming path on a plan's transposed copy HT [Rp][Kp] of [H_r; H_d]
// (row r = column r over all k): a tile of TR Rx is one contiguous block of
// TR * Kp * 8 bytes, fetched by a single cp.async.bulk instead of one 32-byte
// piece per row.  Phases as in k_obj_stream; in (A) warp w takes column
// w % TR and every (NW / TR)-th run of 32 k, lanes over k.

__global__ void __launch_bounds__(256) k_make_ht(const float *Hr, const float *Hd, int M, int S,
                                                 int R, int Rp, int Kp, float *HT) {
  __shared__ float2 tl[32][33];
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32, K = M + S;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int k = k0 + i, r = r0 + threadIdx.x;
    float2 v = make_float2(0.f, 0.f);
    if (k < K && r < R)
      v = __ldg(reinterpret_cast<const float2 *>(k < M ? Hr + (size_t)k * R * 2
                                                        : Hd + (size_t)(k - M) * R * 2) + r);
    tl[i][threadIdx.x] = v;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, k = k0 + threadIdx.x;
    if (r < Rp && k < Kp) reinterpret_cast<float2 *>(HT)[(size_t)r * Kp + k] = tl[threadIdx.x][i];
  }
}

template <int CB, int TR, int KPT>
__global__ void __launch_bounds__(256)
    k_obj_stream_t(ObjArgs a, const float *HT, int M, int Kp, int stage_bytes, int ntiles,
                   const float *U, float *Ppart, double *lpart, unsigned *err) {
  constexpr int NTH = 256, NW = NTH / 32, NPART = NW / TR;
  const int K = M + a.S;
  const uint32_t tile_bytes = (uint32_t)TR * Kp * 8;
  extern __shared__ unsigned char smem_dyn[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
  c2 *coef = reinterpret_cast<c2 *>(base + 2 * (size_t)stage_bytes);  // [K][CB]
  __shared__ c2 red[NW][CB];
  __shared__ c2 g1s[CB][TR], g2s[CB][TR];
  __shared__ __align__(8) uint64_t full[2];
  __shared__ int abort_flag;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

  auto issue = [&](int tile, int stage) {
    uint64_t *bar = &full[stage];
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(tile_bytes)
                 : "memory");
    const float *src = HT + (size_t)tile * TR * Kp * 2;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(base + (size_t)stage * stage_bytes)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(tile_bytes), "r"(smem_addr(bar))
        : "memory");
  };
  const int first = blockIdx.x;
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&full[0])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&full[1])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    if (first < ntiles) issue(first, 0);
    if (first + (int)gridDim.x < ntiles) issue(first + gridDim.x, 1);
  }
  cudaGridDependencySynchronize();
  stage_coef<NTH, CB>(a, M, K, U, coef);
  __syncthreads();

  c2 p1[KPT][CB], p2[KPT][CB];
#pragma unroll
  for (int q = 0; q < KPT; q++)
#pragma unroll
    for (int c = 0; c < CB; c++) { p1[q][c] = {0.f, 0.f}; p2[q][c] = {0.f, 0.f}; }
  float sum_max = 0.f, sum_sq = 0.f;  // FP32 within a warp, FP64 across warps
  const int acol = warp % TR, apart = warp / TR;

  int it = 0;
  for (int tile = first; tile < ntiles; tile += gridDim.x, it++) {
    const int stg = it & 1;
    if (!mbar_wait_bounded(&full[stg], (it >> 1) & 1)) {
      if (t == 0) atomicOr(err, 1u);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) {
      // before the CTA exits, let the copies it issued land (bounded again):
      // this tile's and, if it was issued, the next tile's in the other stage
      if (t == 0) {
        mbar_wait_bounded(&full[stg], (it >> 1) & 1);
        if (tile + (int)gridDim.x < ntiles) mbar_wait_bounded(&full[stg ^ 1], ((it + 1) >> 1) & 1);
      }
      break;
    }
    const float2 *T = reinterpret_cast<const float2 *>(base + (size_t)stg * stage_bytes);
    // (A) Y of column acol over this warp's runs of k
    {
      c2 y[CB];
#pragma unroll
      for (int c = 0; c < CB; c++) y[c] = {0.f, 0.f};
      const float2 *row = T + (size_t)acol * Kp;
#pragma unroll 4
      for (int k = apart * 32 + lane; k < K; k += NPART * 32) {
        const float2 h = row[k];
#pragma unroll
        for (int c = 0; c < CB; c++) mac(y[c], coef[(size_t)k * CB + c], c2{h.x, h.y});
      }
#pragma unroll
      for (int c = 0; c < CB; c++)
        for (int o = 16; o > 0; o >>= 1) {
          y[c].x += __shfl_xor_sync(0xffffffffu, y[c].x, o);
          y[c].y += __shfl_xor_sync(0xffffffffu, y[c].y, o);
        }
      if (lane == 0)
#pragma unroll
        for (int c = 0; c < CB; c++) red[warp][c] = y[c];
    }
    __syncthreads();
    // (B) per-Rx capacity, max, mask, gradient parts
    if (t < TR) {
      const int r = tile * TR + t;
      c2 yy[CB];
      float cap[CB], amp[CB];
#pragma unroll
      for (int c = 0; c < CB; c++) {
        c2 acc = {0.f, 0.f};
#pragma unroll
        for (int pp = 0; pp < NPART; pp++) {
          acc.x += red[pp * TR + t][c].x;
          acc.y += red[pp * TR + t][c].y;
        }
        yy[c] = acc;
      }
      int arg = 0;
      float mx = -1.f;
#pragma unroll
      for (int c = 0; c < CB; c++) {
        if (c >= a.C) { cap[c] = 0.f; amp[c] = 0.f; continue; }
        amp[c] = sqrtf(yy[c].x * yy[c].x + yy[c].y * yy[c].y);
        const float aa = amp[c] + kEps;
        float v = log2f(1.0f + aa * aa / kN0);
        if (a.drop && a.drop[c]) v = 0.f;
        cap[c] = v;
        if (v > mx) { mx = v; arg = c; }
        if (a.recv_amp && r < a.R) a.recv_amp[(size_t)c * a.R + r] = amp[c];
      }
#pragma unroll
      for (int c = 0; c < CB; c++) {
        c2 ga = {0.f, 0.f}, gb = {0.f, 0.f};
        if (c < a.C && r < a.R) {
          const bool dropped = a.drop && a.drop[c];
          const float msk = (cap[c] != mx) ? cap[c] : 0.f;
          sum_sq += msk * msk;
          const float aa = amp[c] + kEps;
          const float dcap = (2.0f * aa / kN0) / (1.0f + aa * aa / kN0) * kInvLn2;
          float g1 = (c == arg) ? -a.w : 0.f, g2 = msk;
          if (dropped) { g1 = 0.f; g2 = 0.f; }
          const float sc = amp[c] > 0.f ? dcap / amp[c] : 0.f;
          ga = {g1 * sc * yy[c].x, g1 * sc * yy[c].y};
          gb = {g2 * sc * yy[c].x, g2 * sc * yy[c].y};
        }
        g1s[c][t] = ga;
        g2s[c][t] = gb;
      }
      if (r < a.R) sum_max += mx;
    }
    __syncthreads();
    // (C) P += G conj(H) over the tile's columns, rows k = t + NTH q
#pragma unroll
    for (int q = 0; q < KPT; q++) {
      const int k = t + NTH * q;
      if (k < K) {
#pragma unroll
        for (int cc = 0; cc < TR; cc++) {
          const float2 h = T[(size_t)cc * Kp + k];
#pragma unroll
          for (int c = 0; c < CB; c++) {
            macc(p1[q][c], g1s[c][cc], c2{h.x, h.y});
            if (CB > 1) macc(p2[q][c], g2s[c][cc], c2{h.x, h.y});
          }
        }
      }
    }
    __syncthreads();
    if (t == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (tile + 2 * (int)gridDim.x < ntiles) issue(tile + 2 * gridDim.x, stg);
    }
  }
  // the tail kernel may launch now; its grid-dependency wait still waits for
  // this grid to complete, with every write below visible
  cudaTriggerProgrammaticLaunchCompletion();
#pragma unroll
  for (int q = 0; q < KPT; q++) {
    const int k = t + NTH * q;
    if (k >= K) continue;
#pragma unroll
    for (int c = 0; c < CB; c++) {
      if (c >= a.C) continue;
      float2 *o = reinterpret_cast<float2 *>(Ppart) + ((size_t)blockIdx.x * 2 * a.C + c) * K + k;
      o[0] = make_float2(p1[q][c].x, p1[q][c].y);
      if (CB > 1) o[(size_t)a.C * K] = make_float2(p2[q][c].x, p2[q][c].y);
    }
  }
  if (t < 32) {
    for (int o = 16; o > 0; o >>= 1) {
      sum_max += __shfl_xor_sync(0xffffffffu, sum_max, o);
      sum_sq += __shfl_xor_sync(0xffffffffu, sum_sq, o);
    }
    if (t == 0) {
      lpart[2 * blockIdx.x] = sum_max;
      lpart[2 * blockIdx.x + 1] = sum_sq;
    }
  }
}

// ------------------------------------------------------------------
// Tensor-core path (tcgen05, 3xBF16 split precision, FP32 accumulation).
//
// A complex product over k becomes one real GEMM on interleaved real views;
// output c occupies the accumulator rows 2c (real part) and 2c+1 (imaginary
// part), which adjacent lanes of one warp read back.
//   forward  Y[c, r] = sum_k coef[c, k] [H_r; H_d][k, r]       (pass 1)
//     A_y row 2c = (Re coef, -Im coef) per k, row 2c+1 = (Im coef, Re coef)
//     B_y = [H_r; H_d]^T as a real [R, 2K] matrix (row r: Re, Im of each k)
//   adjoint  G_U[c, k] = sum_r G[c, r] conj([H_r; H_d][k, r])  (pass 2)
//     A_g row 2c = (Re G, Im G) per r, row 2c+1 = (Im G, -Re G)
//     B_g = [H_r; H_d] as a real [K, 2R] matrix (its native layout)
// Each operand x is held as x_hi = bf16(x) and x_lo = bf16(x - x_hi); the
// product is A_hi B_hi + A_hi B_lo + A_lo B_hi (the dropped A_lo B_lo term is
// below 2^-16 of it).  B_y and B_g are built once per channel set (a plan);
// an evaluation rebuilds only the small A operands.

namespace tcg {
constexpr int BM = 128, BN = 128, BK = 64, STAGES = 3;
constexpr uint32_t A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr size_t SMEM = STAGES * STAGE_BYTES + 1024;
}  // namespace tcg


// B_y [Rp, Kp] from [H_r; H_d] [K, R] complex: 32 x 32 complex tiles turned
// through shared memory (reads coalesced over r, writes over k); entries
// beyond R or K are zero.  Block (32, 8), grid (Rp / 32, Kp / 64).
__global__ void __launch_bounds__(256) k_tc_make_by(const float *Hr, const float *Hd, int M,
                                                    int S, int R, int Rp, int Kp,
                                                    __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  __shared__ float2 t[32][33];
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32, K = M + S;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int k = k0 + i, r = r0 + threadIdx.x;
    float2 v = make_float2(0.f, 0.f);
    if (k < K && r < R)
      v = __ldg(reinterpret_cast<const float2 *>(k < M ? Hr + (size_t)k * R * 2
                                                        : Hd + (size_t)(k - M) * R * 2) + r);
    t[i][threadIdx.x] = v;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, k = k0 + threadIdx.x;
    if (r >= Rp || 2 * k >= Kp) continue;
    const float2 v = t[threadIdx.x][i];
    put_pair(hi, lo, ((size_t)r * Kp + 2 * k) / 2, v.x, v.y);
  }
}

// B_g [Np, K2p] = [H_r; H_d] real view, zero padded; one thread per complex
__global__ void k_tc_make_bg(const float *Hr, const float *Hd, int M, int S, int R, int Np,
                             int K2p, __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ncol = K2p / 2;
  if (i >= (long long)Np * ncol) return;
  const int k = (int)(i / ncol), r = (int)(i % ncol);
  float2 v = make_float2(0.f, 0.f);
  if (k < M + S && r < R)
    v = __ldg(reinterpret_cast<const float2 *>(k < M ? Hr + (size_t)k * R * 2
                                                      : Hd + (size_t)(k - M) * R * 2) + r);
  put_pair(hi, lo, (size_t)i, v.x, v.y);
}

// A_y rows 2c, 2c+1 [., Kp] from coef[c, k] = U[c, k] (k < M), W[c, k - M]
// (M <= k < M + S), zero beyond; one thread per (c, k), c < C
__global__ void k_tc_make_ay(const float *U, const float *W, int C, int M, int S, int Kp,
                             __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int kc = Kp / 2;
  if (i >= (long long)C * kc) return;
  const int c = (int)(i / kc), k = (int)(i % kc);
  float2 v = make_float2(0.f, 0.f);
  if (k < M) v = reinterpret_cast<const float2 *>(U)[(size_t)c * M + k];
  else if (k < M + S) v = __ldg(reinterpret_cast<const float2 *>(W) + (size_t)c * S + (k - M));
  put_pair(hi, lo, ((size_t)(2 * c) * Kp + 2 * k) / 2, v.x, -v.y);
  put_pair(hi, lo, ((size_t)(2 * c + 1) * Kp + 2 * k) / 2, v.y, v.x);
}

// A_g rows 2c, 2c+1 [., K2p] from G = G1 + G2 / ||masked||; one thread per
// (c, r), c < C
__global__ void k_tc_make_ag(const float *G1, const float *G2, const float *scal, int C, int R,
                             int K2p, __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int rc = K2p / 2;
  if (i >= (long long)C * rc) return;
  const int c = (int)(i / rc), r = (int)(i % rc);
  float2 g = make_float2(0.f, 0.f);
  if (r < R) {
    g = reinterpret_cast<const float2 *>(G1)[(size_t)c * R + r];
    if (G2) {
      const float inv = scal[0];
      const float2 h = reinterpret_cast<const float2 *>(G2)[(size_t)c * R + r];
      g.x = fmaf(h.x, inv, g.x);
      g.y = fmaf(h.y, inv, g.y);
    }
  }
  put_pair(hi, lo, ((size_t)(2 * c) * K2p + 2 * r) / 2, g.x, g.y);
  put_pair(hi, lo, ((size_t)(2 * c + 1) * K2p + 2 * r) / 2, g.y, -g.x);
}

// D = sum over this CTA's k-blocks of A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T
// for a 128 x 128 tile, A [Mp, Kd] and B [Np, Kd] bf16 with K contiguous.
// Warp 0 / lane 0 feeds a 3-stage TMA ring (four 16 KB tiles per stage),
// warp 1 / lane 0 issues 12 tcgen05.mma per stage, all 4 warps drain TMEM.
// Rows 2c / 2c+1 of D are stored as out[(z * C + c) * ldo + n] (complex) for
// c < C and n < n_valid, z = blockIdx.z (the split of the k range).
__global__ void __launch_bounds__(128, 1)
    k_cgemm3(const __grid_constant__ CUtensorMap tah, const __grid_constant__ CUtensorMap tal,
             const __grid_constant__ CUtensorMap tbh, const __grid_constant__ CUtensorMap tbl,
             int kb_per, int nkb, int C, int n_valid, long long ldo, float *out, unsigned *err) {
  using namespace tcg;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag, n_issued, n_used;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * BM;
  const int kb0 = blockIdx.z * kb_per;
  const int nk = min(kb_per, nkb - kb0);  // >= 1: the host sizes the grid so
  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) { tc::mbar_init(&full[s], 1); tc::mbar_init(&empty[s], 1); }
    tc::mbar_init(&done, 1);
    abort_flag = 0;
    n_issued = 0;
    n_used = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, (uint32_t)BN);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0 && lane == 0) {
    int kb = 0;
    for (; kb < nk; kb++) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !tc::mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1)) {
        abort_flag = 1;
        atomicOr(err, 1u);
        break;
      }
      if (*(volatile int *)&abort_flag) break;
      unsigned char *sp = smem + s * STAGE_BYTES;
      const int x = (kb0 + kb) * BK;
      tc::mbar_expect_tx(&full[s], STAGE_BYTES);
      tc::tma_load_2d(sp, &tah, x, m0, &full[s]);
      tc::tma_load_2d(sp + A_BYTES, &tal, x, m0, &full[s]);
      tc::tma_load_2d(sp + 2 * A_BYTES, &tbh, x, n0, &full[s]);
      tc::tma_load_2d(sp + 2 * A_BYTES + B_BYTES, &tbl, x, n0, &full[s]);
    }
    n_issued = kb;
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = tc::idesc_bf16(BM, BN);
    int kb = 0;
    for (; kb < nk; kb++) {
      const int s = kb % STAGES;
      if (!tc::mbar_wait(&full[s], (kb / STAGES) & 1)) {
        abort_flag = 1;
        atomicOr(err, 2u);
        break;
      }
      tc::fence_after();
      const uint32_t ah = tc::smem_u32(smem + s * STAGE_BYTES), al = ah + A_BYTES;
      const uint32_t bh = ah + 2 * A_BYTES, bl = bh + B_BYTES;
#pragma unroll
      for (int kk = 0; kk < BK / 16; kk++) {
        const uint32_t o = kk * 32;  // 16 bf16 = 32 bytes along K
        tc::umma_bf16(tmem, tc::sdesc_sw128(ah + o), tc::sdesc_sw128(bh + o), idesc,
                      (kb > 0 || kk > 0) ? 1u : 0u);
        tc::umma_bf16(tmem, tc::sdesc_sw128(ah + o), tc::sdesc_sw128(bl + o), idesc, 1u);
        tc::umma_bf16(tmem, tc::sdesc_sw128(al + o), tc::sdesc_sw128(bh + o), idesc, 1u);
      }
      tc::umma_commit(&empty[s]);
    }
    n_used = kb;
    tc::umma_commit(&done);
  }
  __syncwarp();
  const bool have = tc::mbar_wait(&done, 0);
  if (!have && lane == 0) atomicOr(err, 4u);
  // block-uniform: tcgen05.ld and the shuffles below are warp-collective
  const bool drain = __syncthreads_and(have ? 1 : 0) && !abort_flag;
  // after an abort, the tiles issued but never consumed land before the CTA
  // exits (each stage holds at most one of them; bounded waits again)
  if (abort_flag && tid == 0)
    for (int kb = n_used; kb < n_issued; kb++) tc::mbar_wait(&full[kb % STAGES], (kb / STAGES) & 1);
  tc::fence_after();
  if (drain) {
    const int row = warp * 32 + lane;
    const int c = (m0 + row) >> 1;
    const bool odd = (lane & 1) != 0;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    float2 *o2 = reinterpret_cast<float2 *>(out) + ((size_t)blockIdx.z * C + c) * (size_t)ldo;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      tc::tmem_ld32(tmem + lane_base + (uint32_t)c0, r);
      // the even lane of a pair writes columns 0-15 of the chunk, the odd 16-31
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const float a0 = __uint_as_float(r[j]), a1 = __uint_as_float(r[16 + j]);
        const float b0 = __shfl_xor_sync(0xffffffffu, a0, 1);
        const float b1 = __shfl_xor_sync(0xffffffffu, a1, 1);
        const int n = n0 + c0 + (odd ? 16 : 0) + j;
        if (c < C && n < n_valid)
          o2[n] = odd ? make_float2(b1, a1) : make_float2(a0, b0);
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, (uint32_t)BN);
  }
}

int round_up(long long v, int m) { return (int)((v + m - 1) / m * m); }

// split of a k range of nkb blocks so that the CTAs fill about one wave
void pick_split(int ntiles, int nkb, int sms, int &ks, int &kper) {
  // one CTA fits an SM (shared memory), so keep tiles x splits within a wave
  int want = std::max(1, sms / ntiles);
  want = std::min(want, nkb);
  kper = (nkb + want - 1) / want;
  ks = (nkb + kper - 1) / kper;
}

}  // namespace

namespace {
std::atomic<int> g_inject_timeouts{0};
}  // namespace

// Start of a call on a path with bounded waits, after its first kernel: the
// wait-timeout word is cleared (by that kernel when `cleared`, else here), so
// the word reports this call only.  An injected timeout (test hook of the
// error path) then sets it, as a wait that ran out would.
cudaError_t obj_begin_call(unsigned *err, bool cleared, cudaStream_t st) {
  cudaError_t e = cleared ? cudaSuccess : cudaMemsetAsync(err, 0, 4, st);
  if (e != cudaSuccess) return e;
  int n = g_inject_timeouts.load();
  while (n > 0 && !g_inject_timeouts.compare_exchange_weak(n, n - 1)) {
  }
  if (n > 0) e = cudaMemsetAsync(err, 1, 1, st);
  return e;
}

void obj_inject_timeouts(int calls) { g_inject_timeouts.store(calls > 0 ? calls : 0); }

ObjScratchLayout obj_scratch_layout(int S, int M, int R, int C) {
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const Split sp = make_split(S, M, R);
  ObjScratchLayout L;
  size_t o = 0;
  L.inv = o; o += 256;                                    // control block (see header)
  L.Um = o; o += al(8 * (size_t)C * std::max(M, 1));      // U = (W H_a) e^{j phi'}
  L.gw = o;  // dL/dW partials (k_final CTAs, or the streaming tail CTAs)
  o += al(8 * (size_t)std::max((M + 31) / 32, (M + S + 31) / 32) * C * S);
  L.U = o; o += al(8 * (size_t)sp.kspl * C * R);          // Y partials
  L.G1 = o; o += al(8 * (size_t)C * R);
  L.G2 = o; o += al(8 * (size_t)C * R);
  L.part = o; o += al(16 * (size_t)std::max(sp.nb_epi, (R + 31) / 32));  // either epilogue
  L.GU = o; o += al(8 * (size_t)sp.rspl * C * sp.K);      // G_U partials
  const int nsm = 512;                                    // CTA partials of the streaming path
  L.Pp = o; o += al(8 * (size_t)nsm * 2 * C * sp.K);
  L.lp = o; o += al(16 * (size_t)nsm);
  L.GUs = o; o += al(8 * (size_t)C * sp.K);
  L.total = o;
  return L;
}

cudaError_t obj_run(const ObjArgs &a0, char *scratch, cudaStream_t st) {
  ObjArgs a = a0;
  const bool ms = a.Ha && a.Hr;
  const int M = ms ? a.M : 0;
  if (!ms) { a.Ha = nullptr; a.Hr = nullptr; a.grad_phi = nullptr; }
  const ObjScratchLayout L = obj_scratch_layout(a.S, M, a.R, a.C);
  const Split sp = make_split(a.S, M, a.R);
  float *Ypart = reinterpret_cast<float *>(scratch + L.U);
  float *G1 = reinterpret_cast<float *>(scratch + L.G1);
  float *G2 = a.C > 1 ? reinterpret_cast<float *>(scratch + L.G2) : nullptr;
  double *part = reinterpret_cast<double *>(scratch + L.part);
  float *GUp = reinterpret_cast<float *>(scratch + L.GU);
  float *scal = reinterpret_cast<float *>(scratch + L.inv);
  unsigned *counter = reinterpret_cast<unsigned *>(scratch + L.inv + 32);
  float *Um = reinterpret_cast<float *>(scratch + L.Um);
  float *gw = reinterpret_cast<float *>(scratch + L.gw);
  const StreamPlan pl = stream_plan(a.S, M, a.R, a.C, a.grad_Y != nullptr);
  if (pl.ok && pl.grid <= 512 &&
      !((reinterpret_cast<uintptr_t>(a.Hd) | reinterpret_cast<uintptr_t>(ms ? a.Hr : a.Hd)) & 15)) {
    float *Pp = reinterpret_cast<float *>(scratch + L.Pp);
    double *lp = reinterpret_cast<double *>(scratch + L.lp);
    unsigned *err = reinterpret_cast<unsigned *>(scratch + L.inv + 48);
    float *GUs = reinterpret_cast<float *>(scratch + L.GUs);
    if (cbucket(a.C) == 1) return run_stream<1>(a, pl, M, Um, Pp, lp, GUs, gw, err, counter + 2, st);
    return run_stream<2>(a, pl, M, Um, Pp, lp, GUs, gw, err, counter + 2, st);
  }
  switch (cbucket(a.C)) {
#define CASE(CB) case CB: return run_cb<CB>(a, sp, M, Um, Ypart, G1, G2, part, counter, scal, GUp, gw, st);
    CASE(1) CASE(2) CASE(4) CASE(8) CASE(16) CASE(32) CASE(64)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

// ------------------------------------------------------------------ plans
struct ObjTcPlan {
  const float *Hd, *Ha, *Hr;
  // stream mode (C_max <= 2): transposed FP32 copy and the streaming kernels
  bool stream = false;
  float *HT = nullptr;
  int tKp = 0, tTR = 0, tKPT = 0, tStage = 0, tTiles = 0, tGrid = 0;
  size_t tSmem = 0, oPp = 0, oLp = 0, oGwS = 0;
  int S, M, R, Cmax, K, Kp, Rp, Np, K2p, Mp;
  int ksy, kpy, ksg, kpg;
  __nv_bfloat16 *by_hi, *by_lo, *bg_hi, *bg_lo, *ay_hi, *ay_lo, *ag_hi, *ag_lo;
  CUtensorMap m_byh, m_byl, m_bgh, m_bgl, m_ayh, m_ayl, m_agh, m_agl;
  char *mem;      // one allocation: operands then scratch
  size_t bytes;
  size_t oCtl, oU, oY, oG1, oG2, oPart, oGU, oGUs, oDw;  // byte offsets in mem
};

namespace {
// Stream mode: HT [Rp][Kp] holds [H_r; H_d] transposed (FP32 complex, rows
// padded to an even length so a tile is a whole number of 16-byte units).
cudaError_t plan_stream_create(ObjTcPlan *p, cudaStream_t st, ObjTcPlan **out) {
  const int K = p->K, CB = cbucket(p->Cmax), S = p->S, M = p->M, R = p->R;
  const int kpt = (K + 255) / 256;
  p->tKPT = kpt <= 4 ? 4 : (kpt <= 8 ? 8 : (kpt <= 16 ? 16 : 0));
  if (!p->tKPT || (CB == 2 && p->tKPT > 8)) { delete p; return cudaErrorInvalidValue; }
  p->tKp = (K + 1) / 2 * 2;
  int per_sm = 2;
  for (int TR : {8, 4, 2}) {
    const size_t stage = ((size_t)TR * p->tKp * 8 + 1023) / 1024 * 1024;
    const size_t smem = 1024 + 2 * stage + (size_t)K * CB * 8;
    if (smem <= 110 * 1024) { p->tTR = TR; p->tStage = (int)stage; p->tSmem = smem; break; }
  }
  if (!p->tTR) {  // long columns: two-Rx tiles, one CTA per SM
    const size_t stage = ((size_t)2 * p->tKp * 8 + 1023) / 1024 * 1024;
    const size_t smem = 1024 + 2 * stage + (size_t)K * CB * 8;
    if (smem > 220 * 1024) { delete p; return cudaErrorInvalidValue; }
    p->tTR = 2; p->tStage = (int)stage; p->tSmem = smem;
    per_sm = 1;
  }
  const int Rp = (R + p->tTR - 1) / p->tTR * p->tTR;
  p->tTiles = Rp / p->tTR;
  p->tGrid = std::min(per_sm * sm_count(), p->tTiles);
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  size_t o = 0;
  const size_t oht = o; o += al(8 * (size_t)Rp * p->tKp);
  p->oCtl = o; o += kObjControlBytes;
  p->oU = o; o += al(8 * (size_t)p->Cmax * M);
  p->oPp = o; o += al(8 * (size_t)p->tGrid * 2 * p->Cmax * K);
  p->oLp = o; o += al(16 * (size_t)p->tGrid);
  p->oGwS = o; o += al(8 * (size_t)p->Cmax * K);           // G_U
  p->oDw = o; o += al(8 * (size_t)((K + 31) / 32) * p->Cmax * S);  // dL/dW per tail CTA
  p->bytes = o;
  cudaError_t e = cudaMalloc(&p->mem, o);
  if (e != cudaSuccess) { delete p; return e; }
  p->HT = reinterpret_cast<float *>(p->mem + oht);
  p->stream = true;
  e = cudaMemsetAsync(p->mem + p->oCtl, 0, kObjControlBytes, st);
  if (e == cudaSuccess) {
    dim3 g((Rp + 31) / 32, (p->tKp + 31) / 32), b(32, 8);
    k_make_ht<<<g, b, 0, st>>>(p->Hr, p->Hd, M, S, R, Rp, p->tKp, p->HT);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) { cudaFree(p->mem); delete p; return e; }
  *out = p;
  return cudaSuccess;
}

template <int CB, int TR, int KPT>
cudaError_t launch_stream_ht(ObjTcPlan *p, const ObjArgs &a, const float *U, float *Pp,
                             double *lp, unsigned *err, cudaStream_t st) {
  auto kfn = k_obj_stream_t<CB, TR, KPT>;
  static size_t set_bytes[AMS_MAX_DEVICES] = {0};
  {
    cudaError_t e = ams_set_smem_atleast(set_bytes, kfn, p->tSmem);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p->tGrid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = p->tSmem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kfn, a, (const float *)p->HT, p->M, p->tKp, p->tStage,
                            p->tTiles, U, Pp, lp, err);
}

template <int CB, int TR>
cudaError_t launch_stream_ht_k(ObjTcPlan *p, const ObjArgs &a, const float *U, float *Pp,
                               double *lp, unsigned *err, cudaStream_t st) {
  switch (p->tKPT) {
    case 4: return launch_stream_ht<CB, TR, 4>(p, a, U, Pp, lp, err, st);
    case 8: return launch_stream_ht<CB, TR, 8>(p, a, U, Pp, lp, err, st);
    case 16:
      if (CB == 1) return launch_stream_ht<1, TR, 16>(p, a, U, Pp, lp, err, st);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

template <int CB>
cudaError_t run_plan_stream(ObjTcPlan *p, const ObjArgs &a, cudaStream_t st) {
  const int M = p->M;
  float *U = reinterpret_cast<float *>(p->mem + p->oU);
  float *Pp = reinterpret_cast<float *>(p->mem + p->oPp);
  double *lp = reinterpret_cast<double *>(p->mem + p->oLp);
  float *gw = reinterpret_cast<float *>(p->mem + p->oGwS);
  char *ctl = p->mem + p->oCtl;
  unsigned *counter = reinterpret_cast<unsigned *>(ctl + 40);
  unsigned *err = reinterpret_cast<unsigned *>(ctl + 48);
  const long long n = (long long)M * a.C * 8;
  k_prep_wide<<<(int)((n + 255) / 256), 256, 0, st>>>(a, M, U, err);
  cudaError_t e = obj_begin_call(err, true, st);
  if (e != cudaSuccess) return e;
  switch (p->tTR) {
    case 8: e = launch_stream_ht_k<CB, 8>(p, a, U, Pp, lp, err, st); break;
    case 4: e = launch_stream_ht_k<CB, 4>(p, a, U, Pp, lp, err, st); break;
    default: e = launch_stream_ht_k<CB, 2>(p, a, U, Pp, lp, err, st); break;
  }
  if (e != cudaSuccess) return e;
  return stream_tail<CB>(a, M, p->tGrid, U, Pp, lp, gw, reinterpret_cast<float *>(p->mem + p->oDw),
                         counter, err, st);
}
}  // namespace

cudaError_t obj_tc_plan_create(const float *Hd, const float *Ha, const float *Hr, int S, int M,
                               int R, int Cmax, cudaStream_t st, ObjTcPlan **out,
                               bool force_tc) {
  *out = nullptr;
  if (S <= 0 || M <= 0 || R <= 0 || Cmax <= 0 || Cmax > 64) return cudaErrorInvalidValue;
  ObjTcPlan *p = new ObjTcPlan();
  p->Hd = Hd; p->Ha = Ha; p->Hr = Hr;
  p->S = S; p->M = M; p->R = R; p->Cmax = Cmax;
  p->K = M + S;
  p->Kp = round_up(2LL * p->K, 64);
  p->Rp = round_up(R, tcg::BN);
  p->Np = round_up(p->K, tcg::BN);
  p->K2p = round_up(2LL * R, 64);
  p->Mp = round_up(2LL * Cmax, tcg::BM);
  const int sms = sm_count();
  // stream mode when the streaming kernel's per-thread rows cover K (16 rows
  // a thread for one code, 8 for two); otherwise the tensor-core mode
  const int kpt = (p->K + 255) / 256;
  if (!force_tc && Cmax <= 2 && kpt <= (Cmax == 1 ? 16 : 8)) return plan_stream_create(p, st, out);
  pick_split((p->Rp / tcg::BN) * (p->Mp / tcg::BM), p->Kp / tcg::BK, sms, p->ksy, p->kpy);
  pick_split((p->Np / tcg::BN) * (p->Mp / tcg::BM), p->K2p / tcg::BK, sms, p->ksg, p->kpg);
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  size_t o = 0;
  const size_t nby = (size_t)p->Rp * p->Kp, nbg = (size_t)p->Np * p->K2p;
  const size_t nay = (size_t)p->Mp * p->Kp, nag = (size_t)p->Mp * p->K2p;
  size_t oby = o; o += al(2 * nby) * 2;
  size_t obg = o; o += al(2 * nbg) * 2;
  size_t oay = o; o += al(2 * nay) * 2;
  size_t oag = o; o += al(2 * nag) * 2;
  p->oCtl = o;
  o += kObjControlBytes;
  p->oU = o; o += al(8 * (size_t)Cmax * M);
  p->oY = o; o += al(8 * (size_t)p->ksy * Cmax * R);
  p->oG1 = o; o += al(8 * (size_t)Cmax * R);
  p->oG2 = o; o += al(8 * (size_t)Cmax * R);
  p->oPart = o; o += al(16 * (size_t)((R + 31) / 32));
  p->oGU = o; o += al(8 * (size_t)p->ksg * Cmax * p->K);
  p->oGUs = o; o += al(8 * (size_t)Cmax * p->K);
  p->oDw = o; o += al(8 * (size_t)Cmax * kDwParts * S);
  p->bytes = o;
  cudaError_t e = cudaMalloc(&p->mem, o);
  if (e != cudaSuccess) { delete p; return e; }
  p->by_hi = reinterpret_cast<__nv_bfloat16 *>(p->mem + oby);
  p->by_lo = reinterpret_cast<__nv_bfloat16 *>(p->mem + oby + al(2 * nby));
  p->bg_hi = reinterpret_cast<__nv_bfloat16 *>(p->mem + obg);
  p->bg_lo = reinterpret_cast<__nv_bfloat16 *>(p->mem + obg + al(2 * nbg));
  p->ay_hi = reinterpret_cast<__nv_bfloat16 *>(p->mem + oay);
  p->ay_lo = reinterpret_cast<__nv_bfloat16 *>(p->mem + oay + al(2 * nay));
  p->ag_hi = reinterpret_cast<__nv_bfloat16 *>(p->mem + oag);
  p->ag_lo = reinterpret_cast<__nv_bfloat16 *>(p->mem + oag + al(2 * nag));
  const bool ok =
      tc::make_map_bf16(&p->m_byh, p->by_hi, p->Rp, p->Kp, tcg::BN) &&
      tc::make_map_bf16(&p->m_byl, p->by_lo, p->Rp, p->Kp, tcg::BN) &&
      tc::make_map_bf16(&p->m_bgh, p->bg_hi, p->Np, p->K2p, tcg::BN) &&
      tc::make_map_bf16(&p->m_bgl, p->bg_lo, p->Np, p->K2p, tcg::BN) &&
      tc::make_map_bf16(&p->m_ayh, p->ay_hi, p->Mp, p->Kp, tcg::BM) &&
      tc::make_map_bf16(&p->m_ayl, p->ay_lo, p->Mp, p->Kp, tcg::BM) &&
      tc::make_map_bf16(&p->m_agh, p->ag_hi, p->Mp, p->K2p, tcg::BM) &&
      tc::make_map_bf16(&p->m_agl, p->ag_lo, p->Mp, p->K2p, tcg::BM);
  if (!ok) { cudaFree(p->mem); delete p; return cudaErrorInvalidValue; }
  static size_t attr[AMS_MAX_DEVICES] = {0};
  e = ams_set_smem_atleast(attr, k_cgemm3, tcg::SMEM);
  if (e != cudaSuccess) { cudaFree(p->mem); delete p; return e; }
  // the A operands (rows beyond 2 C stay zero) and the control block
  e = cudaMemsetAsync(p->mem + oay, 0, o - oay, st);
  if (e == cudaSuccess) {
    dim3 gb(p->Rp / 32, p->Kp / 64), bb(32, 8);
    k_tc_make_by<<<gb, bb, 0, st>>>(Hr, Hd, M, S, R, p->Rp, p->Kp, p->by_hi, p->by_lo);
    const long long ng = (long long)p->Np * (p->K2p / 2);
    k_tc_make_bg<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(Hr, Hd, M, S, R, p->Np, p->K2p,
                                                               p->bg_hi, p->bg_lo);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) { cudaFree(p->mem); delete p; return e; }
  *out = p;
  return cudaSuccess;
}

const unsigned *obj_tc_plan_status_word(const ObjTcPlan *p) {
  return p ? reinterpret_cast<const unsigned *>(p->mem + p->oCtl + 48) : nullptr;
}

size_t obj_tc_plan_bytes(const ObjTcPlan *p) { return p ? p->bytes : 0; }
bool obj_tc_plan_streams(const ObjTcPlan *p) { return p && p->stream; }

void obj_tc_plan_destroy(ObjTcPlan *p) {
  if (!p) return;
  cudaFree(p->mem);
  delete p;
}

namespace {
template <int CB>
cudaError_t run_tc(ObjTcPlan *p, const ObjArgs &a, char *ctl, cudaStream_t st) {
  const int M = p->M, R = p->R, C = a.C;
  const bool given = a.U_in != nullptr;
  const float *U = given ? a.U_in : reinterpret_cast<float *>(p->mem + p->oU);
  float *Ypart = reinterpret_cast<float *>(p->mem + p->oY);
  float *G1 = reinterpret_cast<float *>(p->mem + p->oG1);
  float *G2 = C > 1 ? reinterpret_cast<float *>(p->mem + p->oG2) : nullptr;
  double *part = reinterpret_cast<double *>(p->mem + p->oPart);
  float *GUp = reinterpret_cast<float *>(p->mem + p->oGU);
  float *scal = reinterpret_cast<float *>(ctl);
  unsigned *counter = reinterpret_cast<unsigned *>(ctl + 32);
  unsigned *err = reinterpret_cast<unsigned *>(ctl + 48);
  if (!given)
    k_prep<<<dim3((M + 127) / 128, C), 128, 0, st>>>(a, M, reinterpret_cast<float *>(p->mem + p->oU), err);
  {
    cudaError_t e0 = obj_begin_call(err, !given, st);
    if (e0 != cudaSuccess) return e0;
  }
  const long long nay = (long long)C * (p->Kp / 2);
  k_tc_make_ay<<<(unsigned)((nay + 255) / 256), 256, 0, st>>>(U, a.W, C, M, p->S, p->Kp,
                                                              p->ay_hi, p->ay_lo);
  dim3 gy(p->Rp / tcg::BN, p->Mp / tcg::BM, p->ksy);
  k_cgemm3<<<gy, 128, tcg::SMEM, st>>>(p->m_ayh, p->m_ayl, p->m_byh, p->m_byl, p->kpy,
                                        p->Kp / tcg::BK, C, R, R, Ypart, err);
  const bool need_g = a.grad_W || a.grad_phi || a.grad_U;
  if (CB >= 8) {
    constexpr int CW = CB >= 8 ? CB : 8;
    float *maxr = G1;  // G1 / G2 are not needed on this branch: per-Rx max and argmax
    int *argr = reinterpret_cast<int *>(G2 ? G2 : G1 + R);
    const int nb = (R + 31) / 32;
    k_tc_epi_a<CW><<<nb, 256, 0, st>>>(a, p->ksy, Ypart, maxr, argr, part, counter, scal, err);
    if (need_g || a.grad_Y) {
      // with no gradient wanted the A operand is still written (harmless)
      const int nbb = std::max(nb, (p->K2p / 2 + 31) / 32);
      k_tc_epi_b<CW><<<nbb, 256, 0, st>>>(a, p->ksy, Ypart, maxr, argr, scal, p->K2p, p->ag_hi,
                                          p->ag_lo);
    }
  } else {
    k_epilogue<CB><<<(R + 127) / 128, 128, 0, st>>>(a, p->ksy, Ypart, G1, G2, part, counter,
                                                    scal, err);
    if (a.grad_Y) {
      const long long n = (long long)C * R;
      k_grad_y<<<(int)((n + 255) / 256), 256, 0, st>>>(G1, G2, scal, n, a.grad_Y);
    }
    if (need_g) {
      const long long nag = (long long)C * (p->K2p / 2);
      k_tc_make_ag<<<(unsigned)((nag + 255) / 256), 256, 0, st>>>(G1, G2, scal, C, R, p->K2p,
                                                                  p->ag_hi, p->ag_lo);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (!need_g) return cudaGetLastError();
  dim3 gg(p->Np / tcg::BN, p->Mp / tcg::BM, p->ksg);
  k_cgemm3<<<gg, 128, tcg::SMEM, st>>>(p->m_agh, p->m_agl, p->m_bgh, p->m_bgl, p->kpg,
                                        p->K2p / tcg::BK, C, p->K, p->K, GUp, err);
  float *GU = reinterpret_cast<float *>(p->mem + p->oGUs);
  const long long ngu = (long long)C * p->K;
  k_gu_reduce<<<(unsigned)((ngu + 255) / 256), 256, 0, st>>>(GUp, p->ksg, ngu, GU);
  if (given) {
    // dL/dU is G_U's metasurface rows, dL/dW its H_d rows (poisoned like
    // the other outputs when a wait ran out)
    if (a.grad_U)
      k_tc_copy_rows<<<(C * M + 255) / 256, 256, 0, st>>>(GU, p->K, 0, M, C, a.grad_U, err);
    if (a.grad_W)
      k_tc_copy_rows<<<(C * p->S + 255) / 256, 256, 0, st>>>(GU, p->K, M, p->S, C, a.grad_W, err);
    return cudaGetLastError();
  }
  if (a.grad_phi) k_tc_dphi<<<(M + 31) / 32, 256, 0, st>>>(GU, U, C, M, p->K, a.grad_phi, err);
  if (a.grad_W) {
    float *dwp = reinterpret_cast<float *>(p->mem + p->oDw);
    k_tc_dw_part<<<dim3(C, kDwParts), 128, 0, st>>>(GU, p->Ha, a.phi, a.max_phase, p->S, M,
                                                    p->K, dwp);
    k_tc_dw_sum<<<(C * p->S + 127) / 128, 128, 0, st>>>(GU, dwp, C, p->S, M, p->K, a.grad_W,
                                                        err);
  }
  return cudaGetLastError();
}
}  // namespace

cudaError_t obj_tc_run(ObjTcPlan *p, const ObjArgs &a0, cudaStream_t st) {
  if (!p || a0.C <= 0 || a0.C > p->Cmax) return cudaErrorInvalidValue;
  ObjArgs a = a0;
  a.Hd = p->Hd; a.Ha = p->Ha; a.Hr = p->Hr;
  a.S = p->S; a.M = p->M; a.R = p->R;
  // a coefficient-given call needs the tensor-core mode; a call that forms
  // U from W, H_a and phi needs H_a
  if (a.U_in ? p->stream : (p->Ha == nullptr)) return cudaErrorInvalidValue;
  if (p->stream) {
    if (a.grad_Y) return cudaErrorInvalidValue;  // not produced by the streaming kernels
    return cbucket(a.C) == 1 ? run_plan_stream<1>(p, a, st) : run_plan_stream<2>(p, a, st);
  }
  char *ctl = p->mem + p->oCtl;
  switch (cbucket(a.C)) {
#define CASE(CB) case CB: return run_tc<CB>(p, a, ctl, st);
    CASE(1) CASE(2) CASE(4) CASE(8) CASE(16) CASE(32) CASE(64)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
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

namespace {
// complex GEMM, 16 x 16 output tiles through shared memory, FP32
__device__ __forceinline__ float2 cg_ld(const float2 *X, int ld, int op, int r, int c) {
  // element (r, c) of op(X): 0 X, 1 X^T, 2 X^H, 3 conj(X)
  if (op == 0) return X[(size_t)r * ld + c];
  if (op == 3) {
    const float2 v = X[(size_t)r * ld + c];
    return make_float2(v.x, -v.y);
  }
  const float2 v = X[(size_t)c * ld + r];
  return op == 1 ? v : make_float2(v.x, -v.y);
}
__global__ void __launch_bounds__(256) k_cgemm_small(int m, int n, int k, const float2 *A, int lda,
                                                     int opA, const float2 *B, int ldb, int opB,
                                                     float2 *C, int ldc, int accumulate) {
  __shared__ float2 As[16][17], Bs[16][17];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * 16 + ty, col = blockIdx.x * 16 + tx;
  float2 acc = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < k; k0 += 16) {
    As[ty][tx] = (row < m && k0 + tx < k) ? cg_ld(A, lda, opA, row, k0 + tx) : make_float2(0.f, 0.f);
    Bs[ty][tx] = (k0 + ty < k && col < n) ? cg_ld(B, ldb, opB, k0 + ty, col) : make_float2(0.f, 0.f);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const float2 a = As[ty][q], b = Bs[q][tx];
      acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
      acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
    }
    __syncthreads();
  }
  if (row < m && col < n) {
    float2 *o = C + (size_t)row * ldc + col;
    if (accumulate) { acc.x += o->x; acc.y += o->y; }
    *o = acc;
  }
}
}  // namespace

cudaError_t cgemm_run(int m, int n, int k, const float *A, int lda, int opA, const float *B,
                      int ldb, int opB, float *C, int ldc, bool accumulate, cudaStream_t st) {
  if (m <= 0 || n <= 0 || k <= 0 || opA < 0 || opA > 3 || opB < 0 || opB > 3)
    return cudaErrorInvalidValue;
  dim3 grid((n + 15) / 16, (m + 15) / 16), block(16, 16);
  if (grid.y > 65535u) return cudaErrorInvalidValue;
  k_cgemm_small<<<grid, block, 0, st>>>(m, n, k, reinterpret_cast<const float2 *>(A), lda, opA,
                                        reinterpret_cast<const float2 *>(B), ldb, opB,
                                        reinterpret_cast<float2 *>(C), ldc, accumulate ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t coverage_db_run(const float *H, int S, int R, float threshold, float offset,
                            float *out, cudaStream_t st) {
  k_coverage_db<<<(R + 255) / 256, 256, 0, st>>>(H, S, R, threshold, offset, out);
  return cudaGetLastError();
}

// ------------------------------------------------------------------
// Fixed scratch for callers that cannot allocate device memory.  The array
// is part of the module image: every device that loads the library holds
// AMS_OBJECTIVE_NOALLOC_MAX_SCRATCH bytes of it until the process exits.
// Host code must not use the symbol itself as a device address; the address
// is looked up per device with cudaGetSymbolAddress.
static __device__ __align__(256) char g_noalloc_scratch[AMS_OBJECTIVE_NOALLOC_MAX_SCRATCH];

cudaError_t obj_noalloc_scratch(char **out) {
  static std::mutex mu;
  static std::vector<char *> per_device;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)per_device.size() <= dev) per_device.resize(dev + 1, nullptr);
  if (!per_device[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // with `dev` current
    if (e != cudaSuccess) return e;
    per_device[dev] = static_cast<char *>(p);
  }
  *out = per_device[dev];
  return cudaSuccess;
}
