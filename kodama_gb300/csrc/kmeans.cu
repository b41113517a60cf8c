// Batched k-means that reproduces the reference's CPU k-means bit for bit
// (kodama_matrix.cpp:664-799 kmeans_labels, CPU branch): a batch is P
// independent problems of n rows each (rows picked from one device matrix),
// k clusters, at most max_iter Lloyd iterations with early exit, then a final
// assignment.
//
// Float order contract (the reference is built for x86-64 without FMA):
//   dot(a,b): 16 partial sums p[l] over i = l mod 16 on the leading multiple of
//     16, lanes ((p[l]+p[l+4]) + (p[l+8]+p[l+12])), then ((l0+l1)+l2)+l3, then
//     the tail added one product at a time (dot_float32 :91-122, SSE branch);
//   distance = (|x|^2 + |c|^2) - 2*dot, ties to the lower cluster;
//   centroid sums in ascending row order (:778-791), scaled by 1/size;
//   empty clusters split from a donor picked by a float Fenwick tree over
//   max(0, size-1) with mt19937(1234) uniforms (:566-662).
// Every product and sum uses explicit round-to-nearest intrinsics.
#include "kmeans.cuh"
#include "launch_count.cuh"

#include <cuda_runtime.h>
#include <math.h>

namespace kgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
// std::max(0.0f, v)
__device__ __forceinline__ float pos_part(float v) { return (0.0f < v) ? v : 0.0f; }

// dot in the x86 SSE order; a from registers/global, b from shared/global.
template <class A, class B>
__device__ __forceinline__ float dot_x86(A a, B b, int d) {
  float p[16];
#pragma unroll
  for (int l = 0; l < 16; ++l) p[l] = 0.0f;
  int i = 0;
  for (; i + 15 < d; i += 16) {
#pragma unroll
    for (int l = 0; l < 16; ++l) p[l] = fadd(p[l], fmul(a(i + l), b(i + l)));
  }
  float lane[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) lane[l] = fadd(fadd(p[l], p[4 + l]), fadd(p[8 + l], p[12 + l]));
  float sum = fadd(fadd(fadd(lane[0], lane[1]), lane[2]), lane[3]);
  for (; i < d; ++i) sum = fadd(sum, fmul(a(i), b(i)));
  return sum;
}

__global__ void row_norms_kernel(const float* __restrict__ x, int n, int d, float* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float* xr = x + static_cast<size_t>(r) * d;
  out[r] = dot_x86([&](int j) { return xr[j]; }, [&](int j) { return xr[j]; }, d);
}

__global__ void init_centroids_kernel(KMeansBatch B) {
  const int p = blockIdx.y;
  const int c = blockIdx.x;
  const int orow = B.init_rows[static_cast<size_t>(p) * B.k + c];
  const int grow = B.rows ? B.rows[static_cast<size_t>(p) * B.n + orow] : orow;
  float* cent = B.cent + (static_cast<size_t>(p) * B.k + c) * B.d;
  for (int j = threadIdx.x; j < B.d; j += blockDim.x) cent[j] = B.x[static_cast<size_t>(grow) * B.d + j];
  if (threadIdx.x == 0 && c == 0) {
    B.active[p] = 1;
    B.changed[p] = 0;
  }
}

__global__ void centroid_norms_kernel(KMeansBatch B, int final_pass) {
  const int p = blockIdx.y;
  if (!final_pass && !B.active[p]) return;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.k) return;
  const float* cent = B.cent + (static_cast<size_t>(p) * B.k + c) * B.d;
  B.cnorm[static_cast<size_t>(p) * B.k + c] =
      dot_x86([&](int j) { return cent[j]; }, [&](int j) { return cent[j]; }, B.d);
}

// dot_x86 with the point in registers (NB*16 >= d); every register index is
// a compile-time constant, predicated on d.
template <int NB>
__device__ __forceinline__ float dot_x86_reg(const float (&a)[16 * NB], const float* b, int d) {
  float p[16];
#pragma unroll
  for (int l = 0; l < 16; ++l) p[l] = 0.0f;
  const int nfull = d >> 4;
#pragma unroll
  for (int blk = 0; blk < NB; ++blk) {
    if (blk < nfull) {
#pragma unroll
      for (int l = 0; l < 16; ++l) p[l] = fadd(p[l], fmul(a[16 * blk + l], b[16 * blk + l]));
    }
  }
  float lane[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) lane[l] = fadd(fadd(p[l], p[4 + l]), fadd(p[8 + l], p[12 + l]));
  float sum = fadd(fadd(fadd(lane[0], lane[1]), lane[2]), lane[3]);
#pragma unroll
  for (int i = 0; i < 16 * NB; ++i) {
    if (i >= 16 * nfull && i < d) sum = fadd(sum, fmul(a[i], b[i]));
  }
  return sum;
}

// Two rows per thread; centroids of the problem staged in shared memory with
// rows padded to a multiple of 4 floats so they are read with 128-bit loads.
constexpr int kAssignRows = 2;

template <int NB>
__device__ __forceinline__ void dot2_x86(const float (&a)[kAssignRows][16 * NB], const float (&at)[kAssignRows][16],
                                         const float* b, int d, int nfull, float (&out)[kAssignRows]) {
  float p[kAssignRows][16];
#pragma unroll
  for (int q = 0; q < kAssignRows; ++q)
#pragma unroll
    for (int l = 0; l < 16; ++l) p[q][l] = 0.0f;
#pragma unroll
  for (int blk = 0; blk < NB; ++blk) {
    if (blk < nfull) {
#pragma unroll
      for (int l4 = 0; l4 < 4; ++l4) {
        const float4 c = *reinterpret_cast<const float4*>(b + 16 * blk + 4 * l4);
        const float cv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
#pragma unroll
          for (int q = 0; q < kAssignRows; ++q)
            p[q][4 * l4 + e] = fadd(p[q][4 * l4 + e], fmul(a[q][16 * blk + 4 * l4 + e], cv[e]));
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kAssignRows; ++q) {
    float lane[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) lane[l] = fadd(fadd(p[q][l], p[q][4 + l]), fadd(p[q][8 + l], p[q][12 + l]));
    out[q] = fadd(fadd(fadd(lane[0], lane[1]), lane[2]), lane[3]);
  }
  // tail d - 16*nfull < 16 elements, held separately so indices stay static
  const int tn = d - 16 * nfull;
  const float* bt = b + 16 * nfull;
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    if (t < tn) {
      const float bv = bt[t];
#pragma unroll
      for (int q = 0; q < kAssignRows; ++q) out[q] = fadd(out[q], fmul(at[q][t], bv));
    }
  }
}

template <int NB>
__global__ void assign_kernel(KMeansBatch B, int final_pass) {
  extern __shared__ float cs[];
  const int p = blockIdx.y;
  if (!final_pass && !B.active[p]) return;
  const int k = B.k, d = B.d;
  const int dp = (d + 3) & ~3;
  const float* cent = B.cent + static_cast<size_t>(p) * k * d;
  float* cn = cs + static_cast<size_t>(k) * dp;  // centroid norms, staged after the centroids
  for (int i = threadIdx.x; i < k * dp; i += blockDim.x) {
    const int c = i / dp, j = i % dp;
    cs[i] = j < d ? cent[static_cast<size_t>(c) * d + j] : 0.0f;
  }
  for (int c = threadIdx.x; c < k; c += blockDim.x) cn[c] = B.cnorm[static_cast<size_t>(p) * k + c];
  __syncthreads();
  const int r0 = (blockIdx.x * blockDim.x + threadIdx.x) * kAssignRows;
  if (r0 >= B.n) return;
  int grow[kAssignRows];
  bool live[kAssignRows];
#pragma unroll
  for (int q = 0; q < kAssignRows; ++q) {
    live[q] = r0 + q < B.n;
    const int r = live[q] ? r0 + q : r0;
    grow[q] = B.rows ? B.rows[static_cast<size_t>(p) * B.n + r] : r;
  }
  int best[kAssignRows];
  float bestd[kAssignRows];
  float pn[kAssignRows];
#pragma unroll
  for (int q = 0; q < kAssignRows; ++q) {
    best[q] = 0;
    bestd[q] = INFINITY;
    pn[q] = B.pnorm[grow[q]];
  }
  if constexpr (NB > 0) {
    const int nfull = d >> 4;
    float pt[kAssignRows][16 * NB];
    float ptail[kAssignRows][16];
#pragma unroll
    for (int q = 0; q < kAssignRows; ++q) {
#pragma unroll
      for (int j = 0; j < 16 * NB; ++j) pt[q][j] = j < 16 * nfull ? B.x[static_cast<size_t>(grow[q]) * d + j] : 0.0f;
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const int j = 16 * nfull + t;
        ptail[q][t] = j < d ? B.x[static_cast<size_t>(grow[q]) * d + j] : 0.0f;
      }
    }
    for (int c = 0; c < k; ++c) {
      float dt[kAssignRows];
      dot2_x86<NB>(pt, ptail, cs + static_cast<size_t>(c) * dp, d, nfull, dt);
#pragma unroll
      for (int q = 0; q < kAssignRows; ++q) {
        const float dist = __fsub_rn(fadd(pn[q], cn[c]), fmul(2.0f, dt[q]));
        if (dist < bestd[q] || (dist == bestd[q] && c < best[q])) {
          bestd[q] = dist;
          best[q] = c;
        }
      }
    }
  } else {
    for (int c = 0; c < k; ++c) {
      const float* cc = cs + static_cast<size_t>(c) * dp;
#pragma unroll
      for (int q = 0; q < kAssignRows; ++q) {
        const float* xr = B.x + static_cast<size_t>(grow[q]) * d;
        const float dt = dot_x86([&](int j) { return xr[j]; }, [&](int j) { return cc[j]; }, d);
        const float dist = __fsub_rn(fadd(pn[q], cn[c]), fmul(2.0f, dt));
        if (dist < bestd[q] || (dist == bestd[q] && c < best[q])) {
          bestd[q] = dist;
          best[q] = c;
        }
      }
    }
  }
  int* as = B.assign + static_cast<size_t>(p) * B.n;
#pragma unroll
  for (int q = 0; q < kAssignRows; ++q) {
    if (!live[q]) continue;
    const int r = r0 + q;
    if (final_pass) {
      B.labels[static_cast<size_t>(p) * B.n + r] = best[q] + 1;
    } else if (as[r] != best[q]) {
      as[r] = best[q];
      atomicAdd(&B.changed[p], 1);
    }
  }
}

// Float Fenwick tree over donor weights (kodama_matrix.cpp:566-603).
struct Fenwick {
  float* tree;  // k+1
  float* vals;  // k
  int k;
  __device__ void set(int i, float v) {
    const float delta = __fsub_rn(v, vals[i]);
    vals[i] = v;
    for (unsigned j = static_cast<unsigned>(i) + 1u; j < static_cast<unsigned>(k) + 1u; j += j & (~j + 1u))
      tree[j] = fadd(tree[j], delta);
  }
  __device__ float total() const {
    float s = 0.0f;
    for (unsigned j = static_cast<unsigned>(k); j > 0; j -= j & (~j + 1u)) s = fadd(s, tree[j]);
    return s;
  }
  __device__ int select(float target) const {
    unsigned pos = 0, step = 1;
    const unsigned size = static_cast<unsigned>(k) + 1u;
    while ((step << 1) < size) step <<= 1;
    float prefix = 0.0f;
    for (; step > 0; step >>= 1) {
      const unsigned nxt = pos + step;
      if (nxt < size && fadd(prefix, tree[nxt]) <= target) {
        pos = nxt;
        prefix = fadd(prefix, tree[nxt]);
      }
    }
    return pos < static_cast<unsigned>(k) ? static_cast<int>(pos) : -1;
  }
};

// Update step, part 1 (one CTA of 1024 threads per problem): stable grouping
// of the rows by cluster.  Each warp takes a contiguous range of rows, counts
// its clusters, then places its rows in order at per-(warp, cluster) offsets;
// members[] holds global row ids grouped by cluster in ascending row order.
__global__ void __launch_bounds__(1024) sort_kernel(KMeansBatch B) {
  extern __shared__ int sm[];
  const int p = blockIdx.x;
  if (!B.active[p]) return;
  const int k = B.k, n = B.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* whist = sm;             // 32 x k
  int* cbase = whist + 32 * k; // k+1
  const int* as = B.assign + static_cast<size_t>(p) * n;
  int* mem = B.members + static_cast<size_t>(p) * n;
  int* off = B.offsets + static_cast<size_t>(p) * (k + 1);
  for (int i = threadIdx.x; i < 32 * k; i += blockDim.x) whist[i] = 0;
  __syncthreads();
  const int per = (n + 31) / 32;
  const int beg = warp * per, end = min(n, beg + per);
  for (int base = beg; base < end; base += 32) {
    const int r = base + lane;
    const int c = r < end ? as[r] : -1;
    const unsigned m = __match_any_sync(kFull, c);
    if (c >= 0 && (__ffs(m) - 1) == lane) whist[warp * k + c] += __popc(m);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    int run = 0;
    for (int w = 0; w < 32; ++w) {
      const int v = whist[w * k + c];
      whist[w * k + c] = run;
      run += v;
    }
    cbase[c] = run;  // size for now
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int c = 0; c < k; ++c) {
      const int sz = cbase[c];
      cbase[c] = run;
      off[c] = run;
      run += sz;
    }
    cbase[k] = run;
    off[k] = run;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 32 * k; i += blockDim.x) whist[i] += cbase[i % k];
  __syncthreads();
  const int* rows = B.rows ? B.rows + static_cast<size_t>(p) * n : nullptr;
  for (int base = beg; base < end; base += 32) {
    const int r = base + lane;
    const int c = r < end ? as[r] : -1;
    const unsigned m = __match_any_sync(kFull, c);
    if (c >= 0) {
      const int rank = __popc(m & ((1u << lane) - 1u));
      mem[whist[warp * k + c] + rank] = rows ? rows[r] : r;
    }
    __syncwarp();
    if (c >= 0 && (__ffs(m) - 1) == lane) whist[warp * k + c] += __popc(m);
    __syncwarp();
  }
}

// Update step, part 2 (one warp per problem and cluster, lanes over
// features): centroid sums in ascending row order, scaled by 1/size.
__global__ void sums_kernel(KMeansBatch B) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int p = gw / B.k, c = gw % B.k;
  if (p >= B.problems || !B.active[p]) return;
  const int d = B.d;
  const int* mem = B.members + static_cast<size_t>(p) * B.n;
  const int* off = B.offsets + static_cast<size_t>(p) * (B.k + 1);
  const int b0 = off[c], b1 = off[c + 1];
  float* cent = B.cent + (static_cast<size_t>(p) * B.k + c) * d;
  constexpr int kPref = 8;
  for (int j0 = 0; j0 < d; j0 += 32) {
    const int j = j0 + lane;
    float s = 0.0f;
    for (int q = b0; q < b1; q += kPref) {
      float v[kPref];
#pragma unroll
      for (int t = 0; t < kPref; ++t) {
        const int qq = q + t;
        v[t] = (qq < b1 && j < d) ? B.x[static_cast<size_t>(mem[qq]) * d + j] : 0.0f;
      }
#pragma unroll
      for (int t = 0; t < kPref; ++t) {
        if (q + t < b1) s = fadd(s, v[t]);
      }
    }
    const int cnt = b1 - b0;
    if (cnt != 0) s = fmul(s, __fdiv_rn(1.0f, static_cast<float>(cnt)));
    if (j < d) cent[j] = s;
  }
}

// Update step, part 3 (one thread per problem): empty-cluster splitting and
// the early-exit flag.
__global__ void finalize_kernel(KMeansBatch B) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= B.problems || !B.active[p]) return;
  const int k = B.k, d = B.d, n = B.n;
  const int* off = B.offsets + static_cast<size_t>(p) * (k + 1);
  float* cent = B.cent + static_cast<size_t>(p) * k * d;
  float* fsize = B.fscratch + static_cast<size_t>(p) * (3 * k + 1);
  float* ftree = fsize + k;
  float* fvals = ftree + k + 1;
  bool any_empty = false;
  for (int c = 0; c < k; ++c) {
    fsize[c] = static_cast<float>(off[c + 1] - off[c]);
    any_empty |= off[c + 1] == off[c];
  }
  if (any_empty && n > k) {
    const float eps = 1.0f / 1024.0f;
    Fenwick fw{ftree, fvals, k};
    for (int i = 0; i <= k; ++i) ftree[i] = 0.0f;
    for (int i = 0; i < k; ++i) fvals[i] = 0.0f;
    for (int c = 0; c < k; ++c) fw.set(c, pos_part(__fsub_rn(fsize[c], 1.0f)));
    int u = 0;
    for (int e = 0; e < k; ++e) {
      if (fsize[e] != 0.0f) continue;
      const float total = fw.total();
      int donor = -1;
      if (total > 0.0f) donor = fw.select(fmul(B.split_uniform[u++], total));
      if (donor < 0) {
        donor = 0;
        for (int c = 1; c < k; ++c) if (fsize[c] > fsize[donor]) donor = c;
      }
      float* ec = cent + static_cast<size_t>(e) * d;
      float* dc = cent + static_cast<size_t>(donor) * d;
      for (int j = 0; j < d; ++j) ec[j] = dc[j];
      for (int j = 0; j < d; ++j) {
        if ((j & 1) == 0) {
          ec[j] = fmul(ec[j], fadd(1.0f, eps));
          dc[j] = fmul(dc[j], __fsub_rn(1.0f, eps));
        } else {
          ec[j] = fmul(ec[j], __fsub_rn(1.0f, eps));
          dc[j] = fmul(dc[j], fadd(1.0f, eps));
        }
      }
      fsize[e] = __fdiv_rn(fsize[donor], 2.0f);
      fsize[donor] = __fsub_rn(fsize[donor], fsize[e]);
      fw.set(e, pos_part(__fsub_rn(fsize[e], 1.0f)));
      fw.set(donor, pos_part(__fsub_rn(fsize[donor], 1.0f)));
    }
  }
  if (B.changed[p] == 0) B.active[p] = 0;
  B.changed[p] = 0;
}

}  // namespace

size_t kmeans_sort_smem(int k) { return sizeof(int) * (33 * static_cast<size_t>(k) + 1); }

int kmeans_row_norms(const float* x, int n, int d, float* out, cudaStream_t st) {
  row_norms_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, n, d, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int kmeans_run(const KMeansBatch& B, cudaStream_t st) {
  if (B.problems <= 0) return 0;
  init_centroids_kernel<<<dim3(B.k, B.problems), 64, 0, st>>>(B);
  const size_t cs_bytes = sizeof(float) * (static_cast<size_t>(B.k) * ((B.d + 3) & ~3) + B.k);
  const size_t sort_bytes = kmeans_sort_smem(B.k);
  const dim3 agrid((B.n + 128 * kAssignRows - 1) / (128 * kAssignRows), B.problems);
  const dim3 ngrid((B.k + 127) / 128, B.problems);
  const int sum_warps = B.problems * B.k;
  const int sum_blocks = (sum_warps + 7) / 8;
  auto launch_assign = [&](int final_pass) {
    if (B.d <= 16) assign_kernel<1><<<agrid, 128, cs_bytes, st>>>(B, final_pass);
    else if (B.d <= 32) assign_kernel<2><<<agrid, 128, cs_bytes, st>>>(B, final_pass);
    else if (B.d <= 64) assign_kernel<4><<<agrid, 128, cs_bytes, st>>>(B, final_pass);
    else assign_kernel<0><<<agrid, 128, cs_bytes, st>>>(B, final_pass);
  };
  cudaFuncSetAttribute(assign_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(cs_bytes));
  cudaFuncSetAttribute(assign_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(cs_bytes));
  cudaFuncSetAttribute(assign_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(cs_bytes));
  cudaFuncSetAttribute(assign_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(cs_bytes));
  cudaFuncSetAttribute(sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sort_bytes));
  const int iters = B.max_iter > 1 ? B.max_iter : 1;
  for (int it = 0; it < iters; ++it) {
    centroid_norms_kernel<<<ngrid, 128, 0, st>>>(B, 0);
    launch_assign(0);
    sort_kernel<<<B.problems, 1024, sort_bytes, st>>>(B);
    sums_kernel<<<sum_blocks, 256, 0, st>>>(B);
    finalize_kernel<<<(B.problems + 63) / 64, 64, 0, st>>>(B);
  }
  centroid_norms_kernel<<<ngrid, 128, 0, st>>>(B, 1);
  launch_assign(1);
  count_launch(1 + 5 * iters + 2);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
