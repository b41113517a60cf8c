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
//
// The same kernels serve the fold-wise cross-validation searches of KNNCV and
// CoreKNN (knncv.cpp:245-308, core.cpp:695-782): candidates restricted to the
// rows of other folds, the inner-product distance (minus the float chain of
// the a * b products) for the cosine and inner-product metrics, and the raw
// internal distance reported (score = -distance, native_knn.cpp:1153).
#include "ext80.h"
#include "knn.cuh"
#include "launch_count.cuh"

#include <cuda_runtime.h>
#include <math.h>

namespace kgb {

namespace {

constexpr int kQ = 64;      // queries per CTA
constexpr int kTile = 64;   // candidates per shared-memory tile

// Canonical distance of the query (registers) to 4 candidates in shared
// memory (rows padded to dp floats) at once: 4 independent serial chains,
// each in coordinate order without contraction.  IP: the chain of products,
// negated by the caller.
template <int NB, bool IP>
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
            if (IP) {
              acc[u] = __fadd_rn(acc[u], __fmul_rn(qv[4 * g + e], cvv));
            } else {
              const float diff = __fsub_rn(qv[4 * g + e], cvv);
              acc[u] = __fadd_rn(acc[u], __fmul_rn(diff, diff));
            }
          }
        }
      }
    }
  }
}

// Inserts candidate j at distance a into the sorted list (bd, bi) of cnt <= K
// entries, after every entry with distance <= a (candidates arrive in
// increasing index order, so this keeps the index tie-break).
__device__ __forceinline__ void topk_insert(float* bd, int* bi, int K, int& cnt, float& worst, float a, int j) {
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

// FOLD: candidates are the rows whose fold differs from the query's (which
// excludes the query itself); otherwise every row but the query.
// Query slot qi is row qrows[qi] for qi < *nq (a row list, e.g. the rows a
// faster search could not certify), or row qi when qrows is null.
__device__ __forceinline__ int query_row(const int* qrows, const int* nq, int n, int qi) {
  if (qrows == nullptr) return qi < n ? qi : -1;
  return qi < *nq ? qrows[qi] : -1;
}

template <int NB, bool IP, bool FOLD>
__global__ void __launch_bounds__(kQ) knn_segment_kernel(const float* __restrict__ x, int n, int d, int K,
                                                         int seg_len, const int* __restrict__ folds,
                                                         const int* __restrict__ qrows, const int* __restrict__ nq,
                                                         float* __restrict__ pd, int* __restrict__ pi) {
  extern __shared__ float tile[];
  __shared__ int tfold[kTile];
  if (qrows != nullptr && static_cast<int>(blockIdx.x) * kQ >= *nq) return;
  const int dp = (d + 3) & ~3;
  const int qi = blockIdx.x * kQ + threadIdx.x;
  const int q = query_row(qrows, nq, n, qi);
  const int seg = blockIdx.y;
  const int c0 = seg * seg_len, c1 = min(n, c0 + seg_len);
  float qv[16 * NB];
  const bool active = q >= 0;
#pragma unroll
  for (int j = 0; j < 16 * NB; ++j) qv[j] = (active && j < d) ? x[static_cast<size_t>(q) * d + j] : 0.0f;
  const int fq = (FOLD && active) ? folds[q] : -1;
  float* bd = pd + (static_cast<size_t>(seg) * n + (active ? qi : 0)) * K;
  int* bi = pi + (static_cast<size_t>(seg) * n + (active ? qi : 0)) * K;
  int cnt = 0;
  float worst = INFINITY;
  for (int t0 = c0; t0 < c1; t0 += kTile) {
    const int tn = min(kTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < kTile * dp; e += kQ) {
      const int c = e / dp, j = e % dp;
      tile[e] = (c < tn && j < d) ? x[static_cast<size_t>(t0 + c) * d + j] : 0.0f;
    }
    if (FOLD)
      for (int c = threadIdx.x; c < kTile; c += kQ) tfold[c] = c < tn ? folds[t0 + c] : -1;
    __syncthreads();
    if (!active) continue;
    for (int c = 0; c < tn; c += 4) {
      float acc[4];
      sqdist4<NB, IP>(qv, tile + c * dp, dp, d, acc);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = t0 + c + u;
        if (c + u >= tn) continue;
        if (FOLD ? tfold[c + u] == fq : j == q) continue;
        topk_insert(bd, bi, K, cnt, worst, IP ? -acc[u] : acc[u], j);
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
template <bool IP, bool FOLD>
__global__ void __launch_bounds__(kQ) knn_segment_generic_kernel(const float* __restrict__ x, int n, int d, int K,
                                                                 int seg_len, const int* __restrict__ folds,
                                                                 const int* __restrict__ qrows,
                                                                 const int* __restrict__ nq,
                                                                 float* __restrict__ pd, int* __restrict__ pi) {
  extern __shared__ float tile[];
  __shared__ int tfold[kTile];
  if (qrows != nullptr && static_cast<int>(blockIdx.x) * kQ >= *nq) return;
  const int qi = blockIdx.x * kQ + threadIdx.x;
  const int q = query_row(qrows, nq, n, qi);
  const int seg = blockIdx.y;
  const int c0 = seg * seg_len, c1 = min(n, c0 + seg_len);
  const bool active = q >= 0;
  const int fq = (FOLD && active) ? folds[q] : -1;
  float* bd = pd + (static_cast<size_t>(seg) * n + (active ? qi : 0)) * K;
  int* bi = pi + (static_cast<size_t>(seg) * n + (active ? qi : 0)) * K;
  int cnt = 0;
  float worst = INFINITY;
  for (int t0 = c0; t0 < c1; t0 += kTile) {
    const int tn = min(kTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < tn * d; e += kQ) tile[e] = x[static_cast<size_t>(t0) * d + e];
    if (FOLD)
      for (int c = threadIdx.x; c < kTile; c += kQ) tfold[c] = c < tn ? folds[t0 + c] : -1;
    __syncthreads();
    if (!active) continue;
    const float* xq = x + static_cast<size_t>(q) * d;
    for (int c = 0; c < tn; ++c) {
      const int j = t0 + c;
      if (FOLD ? tfold[c] == fq : j == q) continue;
      const float* cv = tile + c * d;
      float a = 0.0f;
      if (IP) {
        for (int k = 0; k < d; ++k) a = __fadd_rn(a, __fmul_rn(xq[k], cv[k]));
        a = -a;
      } else {
        for (int k = 0; k < d; ++k) {
          const float diff = __fsub_rn(xq[k], cv[k]);
          a = __fadd_rn(a, __fmul_rn(diff, diff));
        }
      }
      topk_insert(bd, bi, K, cnt, worst, a, j);
    }
  }
  if (!active) return;
  for (int e = cnt; e < K; ++e) {
    bd[e] = INFINITY;
    bi[e] = 0x7fffffff;
  }
}

// Reported distance of an internal one (native_knn_output_distance,
// native_knn.cpp:1157-1164): sqrt for Euclidean, max(0, 1 + v) for cosine,
// 1 + v for inner product; kOutRaw keeps the internal value.
enum OutMode { kOutSqrt = 0, kOutRaw = 1, kOutCosine = 2, kOutInner = 3 };

__device__ __forceinline__ float output_distance(float v, int mode) {
  if (mode == kOutSqrt) return __fsqrt_rn(v);
  if (mode == kOutRaw) return v;
  const float o = __fadd_rn(1.0f, v);
  return mode == kOutCosine ? ((0.0f < o) ? o : 0.0f) : o;
}

__global__ void knn_merge_kernel(int n, int K, int segs, const float* __restrict__ pd, const int* __restrict__ pi,
                                 const int* __restrict__ qrows, const int* __restrict__ nq, int mode,
                                 int* __restrict__ idx, float* __restrict__ dist) {
  const int qi = blockIdx.x * blockDim.x + threadIdx.x;
  const int qrow = query_row(qrows, nq, n, qi);
  if (qrow < 0) return;
  int head[kMaxSegments];
  for (int s = 0; s < segs; ++s) head[s] = 0;
  for (int o = 0; o < K; ++o) {
    int bs = -1;
    float bdv = INFINITY;
    int biv = 0x7fffffff;
    for (int s = 0; s < segs; ++s) {
      if (head[s] >= K) continue;
      const size_t off = (static_cast<size_t>(s) * n + qi) * K + head[s];
      const float dv = pd[off];
      const int iv = pi[off];
      if (iv == 0x7fffffff) continue;
      if (bs < 0 || dv < bdv || (dv == bdv && iv < biv)) {
        bs = s;
        bdv = dv;
        biv = iv;
      }
    }
    const size_t out = static_cast<size_t>(qrow) * K + o;
    if (bs < 0) {
      idx[out] = -1;
      dist[out] = INFINITY;
      continue;
    }
    ++head[bs];
    idx[out] = biv;
    dist[out] = output_distance(bdv, mode);
  }
}

// Cosine search matrix (make_search_matrix): every row multiplied in double
// by 1 / sqrt(sum of squares) when that norm is finite and positive, then
// rounded to float.  mode 0: the squares summed sequentially in double
// (knncv.cpp:85-108); mode 1: summed in x86 80-bit extended precision and
// rounded to double (core.cpp:182-188, ext80.h); mode 2: the extended sum of
// mode 1, the row then scaled in float (normalize_rows_for_cosine,
// kodama_matrix.cpp:155-167).  One thread per row, the coordinates in order.
__global__ void normalize_rows_kernel(const float* __restrict__ x, int n, int d, int mode, float* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float* row = x + static_cast<size_t>(r) * d;
  double ss;
  if (mode == 0) {
    ss = 0.0;
    for (int j = 0; j < d; ++j) ss = __dadd_rn(ss, __dmul_rn(static_cast<double>(row[j]), static_cast<double>(row[j])));
  } else {
    Ext80 acc{0, 0};
    bool finite = true;
    for (int j = 0; j < d; ++j) {
      finite = finite && isfinite(row[j]);
      acc = ext80_add(acc, ext80_float_square(row[j]));
    }
    ss = finite ? ext80_to_double(acc) : INFINITY;
  }
  const double nrm = __dsqrt_rn(ss);
  if (mode == 2) {
    // normalize_rows_for_cosine: the row multiplied in float by the float
    // rounding of 1 / norm; rows with a zero or non-finite norm unchanged
    const bool ok = nrm > 0.0 && isfinite(nrm);
    const float fs = ok ? __double2float_rn(__ddiv_rn(1.0, nrm)) : 1.0f;
    for (int j = 0; j < d; ++j) out[static_cast<size_t>(r) * d + j] = ok ? __fmul_rn(row[j], fs) : row[j];
    return;
  }
  const double scale = (nrm > 0.0 && isfinite(nrm)) ? __ddiv_rn(1.0, nrm) : 1.0;
  for (int j = 0; j < d; ++j)
    out[static_cast<size_t>(r) * d + j] = __double2float_rn(__dmul_rn(static_cast<double>(row[j]), scale));
}

// majority_vote (knncv.cpp:111-131) of each row over its K neighbours (idx -1
// = none): per label the count and the double sum of the scores
// (score = -distance) in neighbour order; the largest count, then the larger
// sum, then the smaller label.  Labels are visited at their first occurrence
// and summed from there, so every sum runs in neighbour order.
__global__ void knn_vote_kernel(const int* __restrict__ idx, const float* __restrict__ dist, int n, int K,
                                const int* __restrict__ labels, int* __restrict__ pred) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int* ri = idx + static_cast<size_t>(r) * K;
  const float* rd = dist + static_cast<size_t>(r) * K;
  int bl = 0, bc = 0;
  double bs = 0.0;
  for (int j = 0; j < K; ++j) {
    if (ri[j] < 0) continue;
    const int l = labels[ri[j]];
    bool first = true;
    for (int i = 0; i < j && first; ++i) first = !(ri[i] >= 0 && labels[ri[i]] == l);
    if (!first) continue;
    int c = 0;
    double sum = 0.0;
    for (int i = j; i < K; ++i) {
      if (ri[i] < 0 || labels[ri[i]] != l) continue;
      ++c;
      sum = __dadd_rn(sum, static_cast<double>(-rd[i]));
    }
    if (bc == 0 || c > bc || (c == bc && sum > bs) || (c == bc && sum == bs && l < bl)) {
      bl = l;
      bc = c;
      bs = sum;
    }
  }
  pred[r] = bl;
}

// Evolution vote tables from the fold-wise neighbours: the first w of each
// row as 16-bit row ids (0xFFFF = none) and scores -distance.
__global__ void knn_fold_tables_kernel(const int* __restrict__ idx, const float* __restrict__ dist, int n, int K,
                                       int w, uint16_t* __restrict__ nb, float* __restrict__ sc) {
  const size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<size_t>(n) * w) return;
  const size_t r = e / w;
  const int j = static_cast<int>(e % w);
  const int id = idx[r * K + j];
  nb[e] = id >= 0 ? static_cast<uint16_t>(id) : static_cast<uint16_t>(0xFFFFu);
  sc[e] = id >= 0 ? -dist[r * K + j] : -INFINITY;
}

template <bool IP, bool FOLD>
int launch_segments(const float* x, int n, int d, int K, int segments, const int* folds, const int* qrows,
                    const int* nq, float* pd, int* pi, cudaStream_t st) {
  const int seg_len = (n + segments - 1) / segments;
  const dim3 grid((n + kQ - 1) / kQ, segments);
  const size_t smem = sizeof(float) * kTile * ((d + 3) & ~3);
  if (d <= 16) {
    knn_segment_kernel<1, IP, FOLD><<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, folds, qrows, nq, pd, pi);
  } else if (d <= 32) {
    knn_segment_kernel<2, IP, FOLD><<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, folds, qrows, nq, pd, pi);
  } else if (d <= 64) {
    knn_segment_kernel<4, IP, FOLD><<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, folds, qrows, nq, pd, pi);
  } else {
    if (smem > 48 * 1024) {
      const cudaError_t e = cudaFuncSetAttribute(knn_segment_generic_kernel<IP, FOLD>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
      if (e != cudaSuccess) return static_cast<int>(e);
    }
    knn_segment_generic_kernel<IP, FOLD><<<grid, kQ, smem, st>>>(x, n, d, K, seg_len, folds, qrows, nq, pd, pi);
  }
  count_launch();
  return static_cast<int>(cudaGetLastError());
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
  const int e = launch_segments<false, false>(x, n, d, K, segments, nullptr, nullptr, nullptr, pd, pi, st);
  if (e != 0) return e;
  knn_merge_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, K, segments, pd, pi, nullptr, nullptr, kOutSqrt, idx, dist);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int knn_bruteforce_rows(const float* x, int n, int d, int K, int segments, const int* rows, const int* nrows,
                        void* scratch, int* idx, float* dist, cudaStream_t st) {
  if (segments < 1) segments = 1;
  if (segments > kMaxSegments) segments = kMaxSegments;
  float* pd = static_cast<float*>(scratch);
  int* pi = reinterpret_cast<int*>(pd + static_cast<size_t>(segments) * n * K);
  const int e = launch_segments<false, false>(x, n, d, K, segments, nullptr, rows, nrows, pd, pi, st);
  if (e != 0) return e;
  knn_merge_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, K, segments, pd, pi, rows, nrows, kOutSqrt, idx, dist);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int knn_fold_search(const float* x, int n, int d, int K, bool inner, const int* folds, int segments, void* scratch,
                    int* idx, float* dist, cudaStream_t st) {
  if (segments < 1) segments = 1;
  if (segments > kMaxSegments) segments = kMaxSegments;
  float* pd = static_cast<float*>(scratch);
  int* pi = reinterpret_cast<int*>(pd + static_cast<size_t>(segments) * n * K);
  const int e = inner ? launch_segments<true, true>(x, n, d, K, segments, folds, nullptr, nullptr, pd, pi, st)
                      : launch_segments<false, true>(x, n, d, K, segments, folds, nullptr, nullptr, pd, pi, st);
  if (e != 0) return e;
  knn_merge_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, K, segments, pd, pi, nullptr, nullptr, kOutRaw, idx, dist);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int knn_bruteforce_inner(const float* x, int n, int d, int K, int metric, int segments, void* scratch, int* idx,
                         float* dist, cudaStream_t st) {
  if (segments < 1) segments = 1;
  if (segments > kMaxSegments) segments = kMaxSegments;
  float* pd = static_cast<float*>(scratch);
  int* pi = reinterpret_cast<int*>(pd + static_cast<size_t>(segments) * n * K);
  const int e = launch_segments<true, false>(x, n, d, K, segments, nullptr, nullptr, nullptr, pd, pi, st);
  if (e != 0) return e;
  knn_merge_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, K, segments, pd, pi, nullptr, nullptr,
                                                   metric == 0 ? kOutCosine : kOutInner, idx, dist);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int normalize_rows(const float* x, int n, int d, int mode, float* out, cudaStream_t st) {
  normalize_rows_kernel<<<(n + 127) / 128, 128, 0, st>>>(x, n, d, mode, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int knn_vote(const int* idx, const float* dist, int n, int K, const int* labels, int* pred, cudaStream_t st) {
  knn_vote_kernel<<<(n + 127) / 128, 128, 0, st>>>(idx, dist, n, K, labels, pred);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int knn_fold_tables(const int* idx, const float* dist, int n, int K, int w, uint16_t* nb, float* sc,
                    cudaStream_t st) {
  const size_t total = static_cast<size_t>(n) * w;
  knn_fold_tables_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(idx, dist, n, K, w, nb, sc);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
