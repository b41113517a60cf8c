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

// One thread per row; centroids of the problem staged in shared memory.
template <int NB>
__global__ void assign_kernel(KMeansBatch B, int final_pass) {
  extern __shared__ float cs[];
  const int p = blockIdx.y;
  if (!final_pass && !B.active[p]) return;
  const int k = B.k, d = B.d;
  const float* cent = B.cent + static_cast<size_t>(p) * k * d;
  for (int i = threadIdx.x; i < k * d; i += blockDim.x) cs[i] = cent[i];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B.n) return;
  const int grow = B.rows ? B.rows[static_cast<size_t>(p) * B.n + r] : r;
  const float* xr = B.x + static_cast<size_t>(grow) * d;
  float pt[NB > 0 ? 16 * NB : 1];
  if constexpr (NB > 0) {
#pragma unroll
    for (int j = 0; j < 16 * NB; ++j) pt[j] = j < d ? xr[j] : 0.0f;
  }
  const float pn = B.pnorm[grow];
  const float* cn = B.cnorm + static_cast<size_t>(p) * k;
  int best = 0;
  float bestd = INFINITY;
  for (int c = 0; c < k; ++c) {
    const float* cc = cs + static_cast<size_t>(c) * d;
    float dt;
    if constexpr (NB > 0) {
      dt = dot_x86_reg<NB>(pt, cc, d);
    } else {
      dt = dot_x86([&](int j) { return xr[j]; }, [&](int j) { return cc[j]; }, d);
    }
    const float dist = __fsub_rn(fadd(pn, cn[c]), fmul(2.0f, dt));
    if (dist < bestd || (dist == bestd && c < best)) {
      bestd = dist;
      best = c;
    }
  }
  int* as = B.assign + static_cast<size_t>(p) * B.n;
  if (final_pass) {
    B.labels[static_cast<size_t>(p) * B.n + r] = best + 1;
    return;
  }
  if (as[r] != best) {
    as[r] = best;
    atomicAdd(&B.changed[p], 1);
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

// Update step of one problem per CTA (1024 threads): stable grouping of rows
// by cluster, row-ordered centroid sums, scaling, empty-cluster splitting.
__global__ void __launch_bounds__(1024) update_kernel(KMeansBatch B) {
  extern __shared__ int sm[];
  const int p = blockIdx.x;
  if (!B.active[p]) return;
  const int k = B.k, d = B.d, n = B.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* whist = sm;              // 32 x k
  int* csize = sm + 32 * k;     // k
  int* cbase = csize + k;       // k+1
  float* ftree = reinterpret_cast<float*>(cbase + k + 1);  // k+1
  float* fvals = ftree + k + 1;                           // k
  float* fsize = fvals + k;                               // k
  const int* as = B.assign + static_cast<size_t>(p) * n;
  int* mem = B.members + static_cast<size_t>(p) * n;
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
    csize[c] = run;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int c = 0; c < k; ++c) {
      cbase[c] = run;
      run += csize[c];
    }
    cbase[k] = run;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 32 * k; i += blockDim.x) whist[i] += cbase[i % k];
  __syncthreads();
  for (int base = beg; base < end; base += 32) {
    const int r = base + lane;
    const int c = r < end ? as[r] : -1;
    const unsigned m = __match_any_sync(kFull, c);
    if (c >= 0) {
      const int rank = __popc(m & ((1u << lane) - 1u));
      mem[whist[warp * k + c] + rank] = B.rows ? B.rows[static_cast<size_t>(p) * n + r] : r;
    }
    __syncwarp();
    if (c >= 0 && (__ffs(m) - 1) == lane) whist[warp * k + c] += __popc(m);
    __syncwarp();
  }
  __syncthreads();
  float* cent = B.cent + static_cast<size_t>(p) * k * d;
  // one warp per cluster, lanes over features; members (global rows, in
  // ascending row order) are fetched eight at a time so their loads overlap,
  // and each lane adds its feature in member order
  constexpr int kPref = 8;
  for (int c = warp; c < k; c += 32) {
    const int b0 = cbase[c], b1 = cbase[c + 1];
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
      if (j < d) cent[static_cast<size_t>(c) * d + j] = s;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    bool any_empty = false;
    for (int c = 0; c < k; ++c) {
      fsize[c] = static_cast<float>(csize[c]);
      any_empty |= csize[c] == 0;
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
}

}  // namespace

size_t kmeans_update_smem(int k) { return sizeof(int) * (32 * k + k + k + 1) + sizeof(float) * (k + 1 + k + k); }

int kmeans_row_norms(const float* x, int n, int d, float* out, cudaStream_t st) {
  row_norms_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, n, d, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int kmeans_run(const KMeansBatch& B, cudaStream_t st) {
  if (B.problems <= 0) return 0;
  init_centroids_kernel<<<dim3(B.k, B.problems), 64, 0, st>>>(B);
  const size_t cs_bytes = sizeof(float) * static_cast<size_t>(B.k) * B.d;
  const size_t up_bytes = kmeans_update_smem(B.k);
  const dim3 agrid((B.n + 127) / 128, B.problems);
  const dim3 ngrid((B.k + 127) / 128, B.problems);
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
  cudaFuncSetAttribute(update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(up_bytes));
  const int iters = B.max_iter > 1 ? B.max_iter : 1;
  for (int it = 0; it < iters; ++it) {
    centroid_norms_kernel<<<ngrid, 128, 0, st>>>(B, 0);
    launch_assign(0);
    update_kernel<<<B.problems, 1024, up_bytes, st>>>(B);
  }
  centroid_norms_kernel<<<ngrid, 128, 0, st>>>(B, 1);
  launch_assign(1);
  count_launch(1 + 3 * iters + 2);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
