// Training and batch inference of the learned relabelling proposal (mlp.cuh).
//
// Forward: BF16 inputs, weights and activations with FP32 accumulation, the
// arithmetic of the warp-tile tensor-pipe path mlp_logit_warp() (inference)
// up to the order of the float sums.  Backward: FP32 gradients of the mean binary
// cross-entropy, one row per thread for the activations, then one thread per
// parameter summing the block's rows in order; blocks write partial sums that
// a second kernel adds in block order, so training is deterministic.
#include "launch_count.cuh"
#include "mlp.cuh"

#include <math.h>

namespace kgb {

namespace {

constexpr int kB = kMlpGradBlock;
constexpr int kH = kMlpHidden;

__global__ void round_kernel(const float* master, float* rounded) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kMlpParams; e += gridDim.x * blockDim.x) {
    const bool weight = (e >= kMlpW1 && e < kMlpB1) || (e >= kMlpW2 && e < kMlpB2) || (e >= kMlpW3 && e < kMlpB3);
    rounded[e] = weight ? bf16_round(master[e]) : master[e];
  }
}

__global__ void __launch_bounds__(kB) grad_kernel(const float* __restrict__ p, const float* __restrict__ feat,
                                                  const uint8_t* __restrict__ target, const int* __restrict__ idx,
                                                  int n, float* __restrict__ partial) {
  __shared__ float xs[kB][kMlpIn];
  __shared__ float h1s[kB][kH + 1];
  __shared__ float h2s[kB][kH + 1];
  __shared__ float d1s[kB][kH + 1];
  __shared__ float d2s[kB][kH + 1];
  __shared__ float dzs[kB];
  __shared__ float ls[kB];
  const int t = threadIdx.x;
  const int row = blockIdx.x * kB + t;
  if (row < n) {
    const int src = idx[row];
    float x[kMlpIn];
    for (int i = 0; i < kMlpIn; ++i) x[i] = xs[t][i] = bf16_round(feat[static_cast<size_t>(src) * kMlpIn + i]);
    for (int j = 0; j < kH; ++j) {
      float a = p[kMlpB1 + j];
      for (int i = 0; i < kMlpIn; ++i) a = fmaf(x[i], p[kMlpW1 + i * kH + j], a);
      h1s[t][j] = bf16_round(fmaxf(a, 0.0f));
    }
    float z = p[kMlpB3];
    for (int j = 0; j < kH; ++j) {
      float a = p[kMlpB2 + j];
      for (int i = 0; i < kH; ++i) a = fmaf(h1s[t][i], p[kMlpW2 + i * kH + j], a);
      const float h = bf16_round(fmaxf(a, 0.0f));
      h2s[t][j] = h;
      z = fmaf(h, p[kMlpW3 + j], z);
    }
    const float y = target[src] ? 1.0f : 0.0f;
    const float pr = 1.0f / (1.0f + expf(-z));
    const float dz = pr - y;
    dzs[t] = dz;
    ls[t] = fmaxf(z, 0.0f) - z * y + log1pf(expf(-fabsf(z)));
    for (int j = 0; j < kH; ++j) d2s[t][j] = h2s[t][j] > 0.0f ? dz * p[kMlpW3 + j] : 0.0f;
    for (int i = 0; i < kH; ++i) {
      float a = 0.0f;
      if (h1s[t][i] > 0.0f)
        for (int j = 0; j < kH; ++j) a = fmaf(p[kMlpW2 + i * kH + j], d2s[t][j], a);
      d1s[t][i] = a;
    }
  } else {
    for (int i = 0; i < kMlpIn; ++i) xs[t][i] = 0.0f;
    for (int j = 0; j < kH; ++j) h1s[t][j] = h2s[t][j] = d1s[t][j] = d2s[t][j] = 0.0f;
    dzs[t] = 0.0f;
    ls[t] = 0.0f;
  }
  __syncthreads();
  const int rows = min(kB, n - static_cast<int>(blockIdx.x) * kB);
  float* out = partial + static_cast<size_t>(blockIdx.x) * (kMlpParams + 1);
  for (int e = t; e <= kMlpParams; e += kB) {
    float acc = 0.0f;
    if (e == kMlpParams) {
      for (int r = 0; r < rows; ++r) acc += ls[r];
    } else if (e < kMlpB1) {
      const int i = e / kH, j = e % kH;
      for (int r = 0; r < rows; ++r) acc = fmaf(xs[r][i], d1s[r][j], acc);
    } else if (e < kMlpW2) {
      const int j = e - kMlpB1;
      for (int r = 0; r < rows; ++r) acc += d1s[r][j];
    } else if (e < kMlpB2) {
      const int i = (e - kMlpW2) / kH, j = (e - kMlpW2) % kH;
      for (int r = 0; r < rows; ++r) acc = fmaf(h1s[r][i], d2s[r][j], acc);
    } else if (e < kMlpW3) {
      const int j = e - kMlpB2;
      for (int r = 0; r < rows; ++r) acc += d2s[r][j];
    } else if (e < kMlpB3) {
      const int j = e - kMlpW3;
      for (int r = 0; r < rows; ++r) acc = fmaf(dzs[r], h2s[r][j], acc);
    } else {
      for (int r = 0; r < rows; ++r) acc += dzs[r];
    }
    out[e] = acc;
  }
}

__global__ void reduce_kernel(const float* partial, int blocks, int n, float* grad, float* loss) {
  const float inv = 1.0f / static_cast<float>(n > 0 ? n : 1);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e <= kMlpParams; e += gridDim.x * blockDim.x) {
    float acc = 0.0f;
    for (int b = 0; b < blocks; ++b) acc += partial[static_cast<size_t>(b) * (kMlpParams + 1) + e];
    if (e == kMlpParams) *loss = acc * inv;
    else grad[e] = acc * inv;
  }
}

__global__ void adam_kernel(float* master, float* m, float* v, const float* grad, float lr, float c1, float c2) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kMlpParams; e += gridDim.x * blockDim.x) {
    const float g = grad[e];
    m[e] = 0.9f * m[e] + 0.1f * g;
    v[e] = 0.999f * v[e] + 0.001f * g * g;
    master[e] -= lr * (m[e] / c1) / (sqrtf(v[e] / c2) + 1e-8f);
  }
}

__global__ void pack_kernel(const float* __restrict__ p, uint32_t* __restrict__ frag) {
  for (int e = threadIdx.x; e < kMlpFragWords; e += blockDim.x) {
    uint32_t v = 0u;
    if (e < kMlpFragW2) {
      // layer 1 B fragment: n-tile nt, lane (g, tig): W1[2 tig][8 nt + g], W1[2 tig + 1][8 nt + g]
      const int nt = e / 32, lane = e % 32, g = lane >> 2, tig = lane & 3;
      v = bf16_pack(p[kMlpW1 + (2 * tig) * kH + 8 * nt + g], p[kMlpW1 + (2 * tig + 1) * kH + 8 * nt + g]);
    } else if (e < kMlpFragB1) {
      // layer 2 B fragments: (k-slice s, n-tile j), lane, word w = rows 16 s + 8 w + 2 tig (+1)
      const int q = e - kMlpFragW2, w = q & 1, lane = (q >> 1) & 31, sj = q >> 6;
      const int s = sj / 8, j = sj % 8, g = lane >> 2, tig = lane & 3;
      const int k = 16 * s + 8 * w + 2 * tig, col = 8 * j + g;
      v = bf16_pack(p[kMlpW2 + k * kH + col], p[kMlpW2 + (k + 1) * kH + col]);
    } else if (e < kMlpFragB2) {
      v = __float_as_uint(p[kMlpB1 + e - kMlpFragB1]);
    } else if (e < kMlpFragW3) {
      v = __float_as_uint(p[kMlpB2 + e - kMlpFragB2]);
    } else if (e < kMlpFragB3) {
      v = __float_as_uint(bf16_round(p[kMlpW3 + e - kMlpFragW3]));
    } else if (e == kMlpFragB3) {
      v = __float_as_uint(p[kMlpB3]);
    }
    frag[e] = v;
  }
}

// one warp per 32 rows
__global__ void predict_kernel(const uint32_t* __restrict__ frag, const float* __restrict__ feat, int n,
                               float* out) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int base = (blockIdx.x * blockDim.x + threadIdx.x) >> 5 << 5; base < n; base += warps * 32) {
    const int r = base + lane;
    uint32_t fw[4] = {0u, 0u, 0u, 0u};
    if (r < n) {
      float x[kMlpIn];
      for (int i = 0; i < kMlpIn; ++i) x[i] = feat[static_cast<size_t>(r) * kMlpIn + i];
      mlp_pack_row(x, fw);
    }
    const float z = mlp_logit_warp(frag, fw, min(32, n - base));
    if (r < n) out[r] = z;
  }
}

}  // namespace

int mlp_round_params(const float* master, float* rounded, cudaStream_t st) {
  round_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(master, rounded);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int mlp_gradient(const float* rounded, const float* feat, const uint8_t* target, const int* idx, int n,
                 float* partial, float* grad, float* loss, cudaStream_t st) {
  const int blocks = (n + kB - 1) / kB;
  grad_kernel<<<blocks, kB, 0, st>>>(rounded, feat, target, idx, n, partial);
  count_launch();
  reduce_kernel<<<(kMlpParams + 256) / 256, 256, 0, st>>>(partial, blocks, n, grad, loss);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int mlp_adam(float* master, float* m, float* v, const float* grad, float lr, int t, cudaStream_t st) {
  const float c1 = 1.0f - powf(0.9f, static_cast<float>(t)), c2 = 1.0f - powf(0.999f, static_cast<float>(t));
  adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(master, m, v, grad, lr, c1, c2);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int mlp_pack_params(const float* rounded, uint32_t* frag, cudaStream_t st) {
  pack_kernel<<<1, 512, 0, st>>>(rounded, frag);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int mlp_predict(const uint32_t* frag, const float* feat, int n, float* out, cudaStream_t st) {
  const int blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  predict_kernel<<<blocks, 256, 0, st>>>(frag, feat, n, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
