// Graph-side kernels of the KODAMA.matrix path.
//
//   graph_minmax / normalize_external: the caller graph as
//     normalize_external_graph (kodama_matrix.cpp:1292-1330) leaves it:
//     one-based detection, invalid / self / non-finite entries dropped,
//     survivors compacted to the left, distances clamped at 0, width K.
//   normalize_indices: normalize_graph_indices (core.cpp:586-622): positions
//     kept, invalid ids -> -1, non-finite or negative distances -> +inf.
//   build_vote_tables: per problem and landmark row, the first k' valid,
//     non-self, out-of-fold neighbours among landmark rows with score -(d*d)
//     (Euclidean metric) or 1 - d (cosine, inner product; core.cpp:672-677):
//     subset_graph_to_rows (kodama_matrix.cpp:1332-1365) followed by
//     precompute_knn_cv_graph (core.cpp:624-692).
//   project_labels: non-landmark label = majority over the first knn.k
//     landmark neighbours of its graph row, ties to the smaller label, none ->
//     label of the first landmark (kodama_matrix.cpp:3221-3261, :169).
//   dissimilarity: co-label proximity (kodama_matrix.cpp:2685-2776):
//     d' = (1 + d) / (same/valid)^2 or +inf, row stably sorted by (d', id).
#include "graph_ops.cuh"
#include "launch_count.cuh"

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace kgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__global__ void minmax_kernel(const int* __restrict__ idx, size_t total, int* mm) {
  int lo = 0x7fffffff, hi = (-0x7fffffff - 1);
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int v = idx[i];
    if (v < 0) continue;
    lo = min(lo, v);
    hi = max(hi, v);
  }
  lo = __reduce_min_sync(kFull, lo);
  hi = __reduce_max_sync(kFull, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&mm[0], lo);
    atomicMax(&mm[1], hi);
  }
}

__device__ __forceinline__ bool one_based_of(int base, const int* mm, int samples) {
  return base == 1 || (base < 0 && mm[0] >= 1 && mm[1] <= samples);
}

__global__ void normalize_external_kernel(const int* __restrict__ in_idx, const float* __restrict__ in_dist,
                                          int n, int gk, int K, int base, const int* mm,
                                          int* __restrict__ out_idx, float* __restrict__ out_dist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool ob = one_based_of(base, mm, n);
  int col = 0;
  for (int j = 0; j < gk && col < K; ++j) {
    const size_t src = static_cast<size_t>(i) * gk + j;
    int id = in_idx[src];
    if (ob && id > 0) --id;
    if (id < 0 || id >= n || id == i) continue;
    const float d = in_dist[src];
    if (!isfinite(d)) continue;
    out_idx[static_cast<size_t>(i) * K + col] = id;
    out_dist[static_cast<size_t>(i) * K + col] = (0.0f < d) ? d : 0.0f;  // std::max(0.0f, d)
    ++col;
  }
  for (; col < K; ++col) {
    out_idx[static_cast<size_t>(i) * K + col] = -1;
    out_dist[static_cast<size_t>(i) * K + col] = INFINITY;
  }
}

__global__ void normalize_indices_kernel(const int* __restrict__ in_idx, const float* __restrict__ in_dist,
                                         size_t total, int samples, int base, const int* mm,
                                         int* __restrict__ out_idx, float* __restrict__ out_dist) {
  const bool ob = one_based_of(base, mm, samples);
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    int id = in_idx[i];
    if (ob && id > 0) --id;
    if (id < 0 || id >= samples) {
      out_idx[i] = -1;
      out_dist[i] = INFINITY;
      continue;
    }
    out_idx[i] = id;
    const float d = in_dist[i];
    out_dist[i] = (isfinite(d) && d >= 0.0f) ? d : INFINITY;
  }
}

__global__ void scatter_g2l_kernel(const int* __restrict__ land, int problems, int L, int n, int* __restrict__ g2l) {
  const size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<size_t>(problems) * L) return;
  const int p = static_cast<int>(t / L), i = static_cast<int>(t % L);
  g2l[static_cast<size_t>(p) * n + land[t]] = i;
}

// One thread per (problem, row).
__global__ void vote_table_kernel(VoteTableArgs a) {
  const size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<size_t>(a.problems) * a.L) return;
  const int p = static_cast<int>(t / a.L), i = static_cast<int>(t % a.L);
  const int grow = a.land ? a.land[t] : i;
  const int* g2l = a.g2l ? a.g2l + static_cast<size_t>(p) * a.n : nullptr;
  const uint8_t* fo = a.folds + static_cast<size_t>(p) * a.L;
  const int myfold = fo[i];
  uint16_t* nb = a.nb + t * a.w;
  float* sc = a.sc + t * a.w;
  int col = 0;
  // eight neighbours at a time: their ids and distances, then their local
  // ids, then their folds are each loaded together, so a chunk waits on three
  // rounds of loads instead of three per neighbour
  constexpr int kChunk = 8;
  for (int j0 = 0; j0 < a.K && col < a.w; j0 += kChunk) {
    int gnb[kChunk], loc[kChunk], lf[kChunk];
    float dist[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int j = j0 + u;
      const size_t src = static_cast<size_t>(grow) * a.K + j;
      gnb[u] = j < a.K ? a.gidx[src] : -1;
      dist[u] = j < a.K ? a.gdist[src] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < kChunk; ++u)
      loc[u] = (gnb[u] >= 0 && gnb[u] < a.n) ? (g2l ? g2l[gnb[u]] : gnb[u]) : -1;
#pragma unroll
    for (int u = 0; u < kChunk; ++u) lf[u] = loc[u] >= 0 ? fo[loc[u]] : -1;
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      if (col >= a.w) break;
      if (loc[u] < 0 || loc[u] == i) continue;
      if (lf[u] == myfold) continue;
      if (!isfinite(dist[u])) continue;
      const float dc = (0.0f < dist[u]) ? dist[u] : 0.0f;
      nb[col] = static_cast<uint16_t>(loc[u]);
      sc[col] = a.score_one_minus ? __fsub_rn(1.0f, dc) : -__fmul_rn(dc, dc);
      ++col;
    }
  }
  for (; col < a.w; ++col) {
    nb[col] = 0xFFFFu;
    sc[col] = -INFINITY;
  }
}

// One thread per (problem, global row).
__global__ void project_kernel(ProjectArgs a) {
  const size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<size_t>(a.problems) * a.n) return;
  const int p = static_cast<int>(t / a.n), r = static_cast<int>(t % a.n);
  const int* g2l = a.g2l + static_cast<size_t>(p) * a.n;
  const uint16_t* best = a.clbest + static_cast<size_t>(p) * a.L;
  const int* c2l = a.code2label + static_cast<size_t>(p) * a.C0max;
  const int loc = g2l[r];
  int code;
  if (loc >= 0) {
    code = best[loc];
  } else {
    int votes[kMaxProjectK];
    int nv = 0;
    // eight neighbours at a time, each level of dependent loads issued together
    constexpr int kChunk = 8;
    for (int j0 = 0; j0 < a.K && nv < a.pk; j0 += kChunk) {
      int g[kChunk], l[kChunk], b[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u) g[u] = j0 + u < a.K ? a.gidx[static_cast<size_t>(r) * a.K + j0 + u] : -1;
#pragma unroll
      for (int u = 0; u < kChunk; ++u) l[u] = (g[u] >= 0 && g[u] < a.n) ? g2l[g[u]] : -1;
#pragma unroll
      for (int u = 0; u < kChunk; ++u) b[u] = l[u] >= 0 ? best[l[u]] : 0;
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
        if (nv < a.pk && l[u] >= 0) votes[nv++] = b[u];
    }
    if (nv == 0) {
      code = best[0];
    } else {
      int bl = 0x7fffffff, bc = 0;
      for (int q = 0; q < nv; ++q) {
        const int v = votes[q];
        int c = 0;
        for (int u = 0; u < nv; ++u) c += votes[u] == v;
        if (c > bc || (c == bc && v < bl)) {
          bl = v;
          bc = c;
        }
      }
      code = bl;
    }
  }
  a.res[t] = c2l[code];
}

// Reverse adjacency of each problem's vote table: rev_idx[rev_off[v] ..
// rev_off[v+1]) lists the rows r whose table contains v.  One CTA per problem.
__global__ void reverse_table_kernel(ReverseArgs a) {
  extern __shared__ int deg[];
  __shared__ int wsum[32];
  const int p = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = (blockDim.x + 31) / 32;
  const uint16_t* nb = a.nb + static_cast<size_t>(p) * a.L * a.w;
  int* off = a.rev_off + static_cast<size_t>(p) * (a.L + 1);
  uint16_t* idx = a.rev_idx + static_cast<size_t>(p) * a.L * a.w;
  for (int v = tid; v <= a.L; v += blockDim.x) deg[v] = 0;
  __syncthreads();
  const int total = a.L * a.w;  // < 2^22: L < 2^16, w <= 32
  for (int e = tid; e < total; e += blockDim.x) {
    const uint16_t v = nb[e];
    if (v != 0xFFFFu) atomicAdd(&deg[v], 1);
  }
  __syncthreads();
  // exclusive scan of the in-degrees: each thread a contiguous chunk, then
  // the warps' and the block's prefixes
  const int chunk = (a.L + blockDim.x - 1) / blockDim.x;
  const int b = min(a.L, tid * chunk), e = min(a.L, b + chunk);
  int local = 0;
  for (int v = b; v < e; ++v) local += deg[v];
  int incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < nwarps ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nwarps) wsum[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  int run = (warp > 0 ? wsum[warp - 1] : 0) + incl - local;
  for (int v = b; v < e; ++v) {
    const int c = deg[v];
    deg[v] = run;
    off[v] = run;
    run += c;
  }
  if (tid == blockDim.x - 1) off[a.L] = wsum[nwarps - 1];
  __syncthreads();
  for (int e2 = tid; e2 < total; e2 += blockDim.x) {
    const uint16_t v = nb[e2];
    if (v == 0xFFFFu) continue;
    const int slot = atomicAdd(&deg[v], 1);
    idx[slot] = static_cast<uint16_t>(static_cast<unsigned>(e2) / static_cast<unsigned>(a.w));
  }
}

// Label coding of k-means labels 1..k (one CTA per problem): codes are the
// ranks of the labels present, code2label the labels in ascending order.
__global__ void code_labels_kernel(CodingArgs a) {
  extern __shared__ int cmap[];  // k+1 entries
  const int p = blockIdx.x;
  const int* lab = a.labels + static_cast<size_t>(p) * a.n;
  for (int v = threadIdx.x; v <= a.k; v += blockDim.x) cmap[v] = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < a.n; r += blockDim.x) cmap[lab[r]] = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    int* c2l = a.code2label + static_cast<size_t>(p) * a.C0max;
    for (int v = 0; v <= a.k; ++v) {
      if (cmap[v]) {
        c2l[run] = v;
        cmap[v] = run++;
      }
    }
    a.ncodes[p] = run;
  }
  __syncthreads();
  uint16_t* codes = a.codes + static_cast<size_t>(p) * a.n;
  for (int r = threadIdx.x; r < a.n; r += blockDim.x) codes[r] = static_cast<uint16_t>(cmap[lab[r]]);
}

// FNV-1a over the little-endian bytes of each row of a rows x n int matrix
// (hash_integer_vector, kodama_matrix.cpp:1689-1699); one thread per row.
__global__ void fnv_rows_kernel(const int* __restrict__ data, int rows, int n, uint64_t* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const int* v = data + static_cast<size_t>(r) * n;
  uint64_t h = 1469598103934665603ull;
  for (int i = 0; i < n; ++i) {
    const uint32_t b = static_cast<uint32_t>(v[i]);
#pragma unroll
    for (int s = 0; s < 32; s += 8) {
      h ^= static_cast<uint8_t>((b >> s) & 0xffu);
      h *= 1099511628211ull;
    }
  }
  out[r] = h;
}

// 32 x 32 tiles; a CTA walks the run tiles blockIdx.y, blockIdx.y + gridDim.y,
// ... so any number of runs fits the grid's y limit.
__global__ void transpose_kernel(const int* __restrict__ res, int runs, int n, int* __restrict__ out) {
  __shared__ int tile[32][33];
  const int s0 = blockIdx.x * 32;
  const int run_tiles = (runs + 31) / 32;
  for (int rt = blockIdx.y; rt < run_tiles; rt += gridDim.y) {
    const int r0 = rt * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
      const int r = r0 + k, s = s0 + threadIdx.x;
      if (r < runs && s < n) tile[k][threadIdx.x] = res[static_cast<size_t>(r) * n + s];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
      const int s = s0 + k, r = r0 + threadIdx.x;
      if (r < runs && s < n) out[static_cast<size_t>(s) * runs + r] = tile[threadIdx.x][k];
    }
    __syncthreads();
  }
}

// One warp per row; lanes cooperate over runs for each neighbour, then a
// rank sort of the row in shared memory.
__global__ void dissimilarity_kernel(DissimArgs a) {
  extern __shared__ unsigned char dsm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float* kd = reinterpret_cast<float*>(dsm) + static_cast<size_t>(warp) * a.K;
  int* ki = reinterpret_cast<int*>(reinterpret_cast<float*>(dsm) + static_cast<size_t>(wpb) * a.K) +
            static_cast<size_t>(warp) * a.K;
  const int i = blockIdx.x * wpb + warp;
  if (i >= a.n) return;
  const int* li = a.lbs + static_cast<size_t>(i) * a.runs;
  for (int j = 0; j < a.K; ++j) {
    const size_t off = static_cast<size_t>(i) * a.K + j;
    const int stored = a.idx[off];
    const int nb = (stored >= 0 && a.in_one_based) ? stored - 1 : stored;
    float d = a.dist[off];
    if (nb < 0 || nb >= a.n || !isfinite(d)) {
      if (lane == 0) {
        kd[j] = INFINITY;
        ki[j] = stored;
      }
      continue;
    }
    const int* lj = a.lbs + static_cast<size_t>(nb) * a.runs;
    int same = 0, valid = 0;
    for (int r = lane; r < a.runs; r += 32) {
      const int x = li[r], y = lj[r];
      const int pv = (x != 0) & (y != 0);
      valid += pv;
      same += pv & (x == y);
    }
    same = __reduce_add_sync(kFull, same);
    valid = __reduce_add_sync(kFull, valid);
    if (lane == 0) {
      if (same == 0 || valid == 0) {
        d = INFINITY;
      } else {
        const double agr = __ddiv_rn(static_cast<double>(same), static_cast<double>(valid));
        d = static_cast<float>(__ddiv_rn(__dadd_rn(1.0, static_cast<double>(d)), __dmul_rn(agr, agr)));
      }
      kd[j] = d;
      ki[j] = a.out_one_based ? nb + 1 : nb;
    }
  }
  __syncwarp();
  // stable rank sort by (distance, id)
  for (int j = lane; j < a.K; j += 32) {
    const float dj = kd[j];
    const int ij = ki[j];
    int rank = 0;
    for (int q = 0; q < a.K; ++q) {
      const float dq = kd[q];
      const int iq = ki[q];
      const bool less = dq < dj || (!(dj < dq) && iq < ij);
      const bool equal_before = !(dq < dj) && !(dj < dq) && iq == ij && q < j;
      rank += less || equal_before;
    }
    a.out_idx[static_cast<size_t>(i) * a.K + rank] = ij;
    a.out_dist[static_cast<size_t>(i) * a.K + rank] = dj;
  }
}

}  // namespace

int graph_minmax(const int* idx, size_t total, int* mm, cudaStream_t st) {
  const int init[2] = {0x7fffffff, (-0x7fffffff - 1)};
  cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, st);
  const int blocks = static_cast<int>((total + 255) / 256 < 2048 ? (total + 255) / 256 : 2048);
  minmax_kernel<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(idx, total, mm);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int normalize_external(const int* in_idx, const float* in_dist, int n, int gk, int K, int base, const int* mm,
                       int* out_idx, float* out_dist, cudaStream_t st) {
  normalize_external_kernel<<<(n + 255) / 256, 256, 0, st>>>(in_idx, in_dist, n, gk, K, base, mm, out_idx, out_dist);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int normalize_indices(const int* in_idx, const float* in_dist, size_t total, int samples, int base, const int* mm,
                      int* out_idx, float* out_dist, cudaStream_t st) {
  const int blocks = static_cast<int>((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  normalize_indices_kernel<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(in_idx, in_dist, total, samples, base, mm,
                                                                  out_idx, out_dist);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int build_g2l(const int* land, int problems, int L, int n, int* g2l, cudaStream_t st) {
  cudaMemsetAsync(g2l, 0xff, sizeof(int) * static_cast<size_t>(problems) * n, st);
  const size_t total = static_cast<size_t>(problems) * L;
  scatter_g2l_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(land, problems, L, n, g2l);
  return static_cast<int>(cudaGetLastError());
}

int build_vote_tables(const VoteTableArgs& a, cudaStream_t st) {
  const size_t total = static_cast<size_t>(a.problems) * a.L;
  vote_table_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int build_reverse_tables(const ReverseArgs& a, cudaStream_t st) {
  const size_t smem = sizeof(int) * (static_cast<size_t>(a.L) + 1);
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(reverse_table_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  }
  reverse_table_kernel<<<a.problems, 1024, smem, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int project_labels(const ProjectArgs& a, cudaStream_t st) {
  const size_t total = static_cast<size_t>(a.problems) * a.n;
  project_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int code_labels(const CodingArgs& a, cudaStream_t st) {
  const size_t smem = sizeof(int) * (static_cast<size_t>(a.k) + 1);
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(code_labels_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  }
  code_labels_kernel<<<a.problems, 1024, smem, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int fnv_rows(const int* data, int rows, int n, uint64_t* out, cudaStream_t st) {
  fnv_rows_kernel<<<(rows + 63) / 64, 64, 0, st>>>(data, rows, n, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int transpose_runs(const int* res, int runs, int n, int* out, cudaStream_t st) {
  const int run_tiles = (runs + 31) / 32;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((n + 31) / 32, run_tiles < 65535 ? run_tiles : 65535);
  cfg.blockDim = dim3(32, 8);
  cfg.stream = st;
  // the launch's own status (not an error left over from earlier work)
  const cudaError_t e = cudaLaunchKernelEx(&cfg, transpose_kernel, res, runs, n, out);
  count_launch();
  return static_cast<int>(e);
}

int dissimilarity(const DissimArgs& a, cudaStream_t st) {
  const int wpb = 8;
  const size_t smem = static_cast<size_t>(wpb) * a.K * (sizeof(float) + sizeof(int));
  if (smem > 48 * 1024) cudaFuncSetAttribute(dissimilarity_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            static_cast<int>(smem));
  dissimilarity_kernel<<<(a.n + wpb - 1) / wpb, wpb * 32, smem, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
