// Exact k-nearest-neighbour graph (self excluded).
//
// Canonical distance: squared Euclidean distance accumulated in float32 over
// coordinates 0..d-1, each term (a-b)*(b-a) as a separately rounded product,
// no fused multiply-add; neighbours ranked by (distance, index); the reported
// distance is sqrtf(d2) (native_knn.cpp:1157-1160 output convention).  This is
// the deterministic stand-in for the reference's approximate HNSW graph
// (native_knn.cpp:125, kodama_matrix.cpp:218-292).
//
// brute-force path: queries are split over CTAs (one query per thread, the
// query held in registers), candidates streamed through shared memory in
// tiles and split over `segments` CTAs along grid.y; each thread keeps a
// sorted top-K list; segment lists are merged by a second kernel.
#include "knn.cuh"
#include "launch_count.cuh"

#include <cuda_runtime.h>
#include <math.h>

namespace kgb {

namespace {

constexpr int kQ = 64;      // queries per CTA
constexpr int kTile = 64;   // candidates per shared-memory tile

// Canonical squared distance of the query (registers) to 4 candidates in
// shared memory (rows padded to dp floats) at once: 4 independent serial
// chains, each in coordinate order without contraction.
template <int NB>
__device__ __forceinline__ void sqdist4(const float (&qv)[16 * NB], const float* cv, int dp, int d,
                                        float (&acc)[4]) {
#pragma unroll
  for (int u = 0; u < 4; ++u) acc[u] = 0.0f;
#pragma unroll
  for (int g = 0; g < 4 * NB; ++g) {
    if (4 * g < d) {
      float4 c4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) c4[u] = *reinterpret_cast<const float4*>(cv + u * dp + 4 * g);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (4 * g + e < d) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const float cvv = e == 0 ? c4[u].x : e == 1 ? c4[u].y : e == 2 ? c4[u].z : c4[u].w;
            const float diff = __fsub_rn(qv[4 * g + e], cvv);
            acc[u] = __fadd_rn(acc[u], __fmul_rn(diff, diff));
          }
        }
      }
    }
  }
}

template <int NB>
__global__ void __launch_bounds__(kQ) knn_segment_kernel(const float* __restrict__ x, int n, int d, int K,
                                                         int seg_len, float* __restrict__ pd, int* __restrict__ pi) {
  extern __shared__ float tile[];
  const int dp = (d + 3) & ~3;
  const int q = blockIdx.x * kQ + threadIdx.x;
  const int seg = blockIdx.y;
  const int c0 = seg * seg_len, c1 = min(n, c0 + seg_len);
  float qv[16 * NB];
  const bool active = q < n;
#pragma unroll
  for (int j = 0; j < 16 * NB; ++j) qv[j] = (active && j < d) ? x[static_cast<size_t>(q) * d + j] : 0.0f;
  float* bd = pd + (static_cast<size_t>(seg) * n + (active ? q : 0)) * K;
  int* bi = pi + (static_cast<size_t>(seg) * n + (active ? q : 0)) * K;
  int cnt = 0;
  float worst = INFINITY;
  for (int t0 = c0; t0 < c1; t0 += kTile) {
    const int tn = min(kTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < kTile * dp; e += kQ) {
      const int c = e / dp, j = e % dp;
      tile[e] = (c < tn && j < d) ? x[static_cast<size_t>(t0 + c) * d + j] : 0.0f;
    }
    __syncthreads();
    if (!active) continue;
    for (int c = 0; c < tn; c += 4) {
      float acc[4];
      sqdist4<NB>(qv, tile + c * dp, dp, d, acc);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = t0 + c + u;
        if (c + u >= tn || j == q) continue;
        const float a = acc[u];
        if (cnt < K || a < worst) {
          // insert after every entry with distance <= a (candidates arrive in
          // increasing index order, so this keeps the index tie-break)
          int pos = cnt < K ? cnt : K - 1;
          while (pos > 0 && bd[pos - 1] > a) {
            bd[pos] = bd[pos - 1];
            bi[pos] = bi[pos - 1];
            --pos;
          }
          bd[pos] = a;
          bi[pos] = j;
          if (cnt < K) ++cnt;
          worst = cnt < K ? INFINITY : bd[K - 1];
        }
      }
    }
  }
  if (!active) return;
  for (int e = cnt; e < K; ++e) {
    bd[e] = INFINITY;
    bi[e] = 0x7fffffff;
  }
}

// Generic d: the query row read from global memory.
__global__ void __launch_bounds__(kQ) knn_segment_generic_kernel(const float* __restrict__ x, int n, int d, int K,
                                                                 int seg_len, float* __restrict__ pd,
                                                                 int* __restrict__ pi) {
  extern __shared__ float tile[];
  const int q = blockIdx.x * kQ + threadIdx.x;
  const int seg = blockIdx.y;
  const int c0 = seg * seg_len, c1 = min(n, c0 + seg_len);
  const bool active = q < n;
  float* bd = pd + (static_cast<size_t>(seg) * n + (active ? q : 0)) * K;
  int* bi = pi + (static_cast<size_t>(seg) * n + (active ? q : 0)) * K;
  int cnt = 0;
  float worst = INFINITY;
  for (int t0 = c0; t0 < c1; t0 += kTile) {
    const int tn = min(kTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < tn * d; e += kQ) tile[e] = x[static_cast<size_t>(t0) * d + e];
    __syncthreads();
    if (!active) continue;
    const float* xq = x + static_cast<size_t>(q) * d;
    for (int c = 0; c < tn; ++c) {
      const int j = t0 + c;
      if (j == q) continue;
      const float* cv = tile + c * d;
      float a = 0.0f;
      for (int k = 0; k < d; ++k) {
        const float diff = __fsub_rn(xq[k], cv[k]);
        a = __fadd_rn(a, __fmul_rn(diff, diff));
      }
      if (cnt < K || a < worst) {
        int pos = cnt < K ? cnt : K - 1;
        while (pos > 0 && bd[pos - 1] > a) {
          bd[pos] = bd[pos - 1];
          bi[pos] = bi[pos - 1];
          --pos;
        }
        bd[pos] = a;
        bi[pos] = j;
        if (cnt < K) ++cnt;
        worst = cnt < K ? INFINITY : bd[K - 1];
      }
    }
  }
  if (!active) return;
  for (int e = cnt; e < K; ++e) {
    bd[e] = INFINITY;
    bi[e] = 0x7fffffff;
  }
}

__global__ void knn_merge_kernel(int n, int K, int segs, const float* __restrict__ pd, const int* __restrict__ pi,
                                 int* __restrict__ idx, float* __restrict__ dist) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int head[kMaxSegments];
  for (int s = 0; s < segs; ++s) head[s] = 0;
  for (int o = 0; o < K; ++o) {
    int bs = -1;
    float bdv = INFINITY;
    int biv = 0x7fffffff;
    for (int s = 0; s < segs; ++s) {
      if (head[s] >= K) continue;
      const size_t off = (static_cast<size_t>(s) * n + q) * K + head[s];
      const float dv = pd[off];
      const int iv = pi[off];
      if (iv == 0x7fffffff) continue;
      if (bs < 0 || dv < bdv || (dv == bdv && iv < biv)) {
        bs = s;
        bdv = dv;
        biv = iv;
      }
    }
    const size_t out = static_cast<size_t>(q) * K + o;
    if (bs < 0) {
      idx[out] = -1;
      dist[out] = INFINITY;
      continue;
    }
    ++head[bs];
    idx[out] = biv;
    dist[out] = __fsqrt_rn(bdv);
  }
}

}  // namespace

size_t knn_bruteforce_scratch(int n, int K, int segments) {
  return static_cast<size_t>(segments) * n * K * (sizeof(float) + sizeof(int));
}

int knn_bruteforce(const float* x, int n, int d, int K, int segments, void* scratch, int* idx, float* dist,
                   cudaStream_t st) {
  if (segments < 1) segments = 1;
  if (segments > kMaxSegments) segments = kMaxSegments;
  float* pd = static_cast<float*>(scratch);
  int* pi = reinterpret_cast<int*>(pd + static_cast<size_t>(segments) * n * K);
  const int seg_len = (n + segments - 1) / segments;
  const dim3 grid((n + kQ - 1) / kQ, segments);
  const size_t smem = sizeof(float) * kTile * ((d + 3) & ~3);
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(knn_segment_generic_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
  }
  if (d <= 16) knn_segment_kernel<1><<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, pd, pi);
  else if (d <= 32) knn_segment_kernel<2><<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, pd, pi);
  else if (d <= 64) knn_segment_kernel<4><<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, pd, pi);
  else knn_segment_generic_kernel<<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, pd, pi);
  knn_merge_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, K, segments, pd, pi, idx, dist);
  count_launch(2);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
