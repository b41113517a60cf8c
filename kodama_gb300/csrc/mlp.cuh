// The learned relabelling proposal: a 3-layer perceptron (8 -> 64 -> 64 -> 1)
// that scores each landmark whose current label differs from its CV
// prediction, trained on snapshots of plain runs.  BF16 weights and
// activations, FP32 accumulation.  Used by the evolution kernel (evolve.cu)
// to pick which candidates a proposal relabels; every proposal is still
// accepted or rejected by the exact cross-validated accuracy.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kgb {

constexpr int kMlpIn = 8;
constexpr int kMlpHidden = 64;
// parameter vector: W1 (in x hidden, row-major), b1, W2 (hidden x hidden), b2, w3 (hidden), b3
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpIn * kMlpHidden;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpHidden;
constexpr int kMlpParams = kMlpB3 + 1;
constexpr int kMlpGradBlock = 32;  // rows per gradient block (static shared memory)

__device__ __forceinline__ float bf16_round(float v) {
  // round to the nearest bfloat16 (ties to even), kept in a float
  const unsigned u = __float_as_uint(v);
  if ((u & 0x7f800000u) == 0x7f800000u) return v;  // inf / nan unchanged
  const unsigned r = u + 0x7fffu + ((u >> 16) & 1u);
  return __uint_as_float(r & 0xffff0000u);
}

// Logit of one row; p are parameters already rounded to bfloat16 (biases in
// float).  Activations are rounded to bfloat16 between layers.
__device__ __forceinline__ float mlp_logit(const float* __restrict__ p, const float* x_in) {
  float x[kMlpIn];
#pragma unroll
  for (int i = 0; i < kMlpIn; ++i) x[i] = bf16_round(x_in[i]);
  float h1[kMlpHidden];
#pragma unroll 8
  for (int j = 0; j < kMlpHidden; ++j) {
    float a = p[kMlpB1 + j];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) a = fmaf(x[i], p[kMlpW1 + i * kMlpHidden + j], a);
    h1[j] = bf16_round(fmaxf(a, 0.0f));
  }
  float z = p[kMlpB3];
  for (int j = 0; j < kMlpHidden; ++j) {
    float a = p[kMlpB2 + j];
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) a = fmaf(h1[i], p[kMlpW2 + i * kMlpHidden + j], a);
    z = fmaf(bf16_round(fmaxf(a, 0.0f)), p[kMlpW3 + j], z);
  }
  return z;
}

// Rounds a float parameter vector to bfloat16 weights (biases stay float).
int mlp_round_params(const float* master, float* rounded, cudaStream_t st);

// Mean binary cross-entropy gradient of a batch of n rows (rows idx[0..n)
// of feat / target) at `rounded` parameters: grad (kMlpParams floats) and
// the mean loss.  Deterministic: per-block partial sums reduced in order.
// partial holds ceil(n / kMlpGradBlock) x (kMlpParams + 1) floats.
int mlp_gradient(const float* rounded, const float* feat, const uint8_t* target, const int* idx, int n,
                 float* partial, float* grad, float* loss, cudaStream_t st);

// One Adam step on the master parameters (t = step number from 1).
int mlp_adam(float* master, float* m, float* v, const float* grad, float lr, int t, cudaStream_t st);

// Logits of n rows.
int mlp_predict(const float* rounded, const float* feat, int n, float* out, cudaStream_t st);

}  // namespace kgb
