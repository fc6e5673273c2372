// mlp.h -- device state and launchers of the surrogate MLP (mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

constexpr int kMlpMaxLayers = 8;
// CTAs of the loss kernel, each writing one FP64 partial sum (a fixed work
// split, so the loss is summed in the same order on every device)
constexpr int kMlpLossParts = 608;

struct MlpDev {
  int L = 0;                       // weight layers
  int d[kMlpMaxLayers + 1] = {};   // logical widths d[0..L]
  int dp[kMlpMaxLayers + 1] = {};  // stored widths (d[0] padded to 64)
  int max_bp = 0;                  // batch capacity (multiple of 128)
  int step = 0;                    // Adam step count
  float *W[kMlpMaxLayers + 1] = {}, *b[kMlpMaxLayers + 1] = {};
  float *mW[kMlpMaxLayers + 1] = {}, *vW[kMlpMaxLayers + 1] = {};
  float *mb[kMlpMaxLayers + 1] = {}, *vb[kMlpMaxLayers + 1] = {};
  float *gW[kMlpMaxLayers + 1] = {}, *gb[kMlpMaxLayers + 1] = {};
  __nv_bfloat16 *Wb[kMlpMaxLayers + 1] = {}, *Wt[kMlpMaxLayers + 1] = {};
  __nv_bfloat16 *H[kMlpMaxLayers + 1] = {};   // H[0] packed input, H[l] activations
  __nv_bfloat16 *dZ[kMlpMaxLayers + 1] = {};  // gradients of the pre-activations
  __nv_bfloat16 *tA = nullptr, *tB = nullptr;  // transposes for the weight gradients
  float *Y = nullptr;
  double *part = nullptr;
  unsigned *err = nullptr;
};

cudaError_t mlp_init(MlpDev &m, uint32_t seed, cudaStream_t st);
cudaError_t mlp_refresh_bf16(MlpDev &m, cudaStream_t st);
// X [B, d0] fp32; Y_out [B, dL] fp32 (may be NULL: the output stays in m.Y)
cudaError_t mlp_forward(MlpDev &m, const float *X, int B, float *Y_out, cudaStream_t st);
// after mlp_forward on the same batch: gradients into gW/gb, loss (device) if given
cudaError_t mlp_backward(MlpDev &m, const float *T, int B, float *loss, cudaStream_t st);
cudaError_t mlp_adam(MlpDev &m, float lr, cudaStream_t st);
