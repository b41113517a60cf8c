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
#include "bf16_split.cuh"
#include "kmeans.cuh"
#include "knn.cuh"
#include "launch_count.cuh"

#include <cuda_runtime.h>
#include <math.h>

#include <cmath>

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

// The same x86-order dot with the point read from memory (NB*16 >= d).
template <int NB>
__device__ __forceinline__ float dot_x86_mem(const float* a, const float* b, int d) {
  float p[16];
#pragma unroll
  for (int l = 0; l < 16; ++l) p[l] = 0.0f;
  const int nfull = d >> 4;
  for (int blk = 0; blk < nfull; ++blk) {
#pragma unroll
    for (int l = 0; l < 16; ++l) p[l] = fadd(p[l], fmul(a[16 * blk + l], b[16 * blk + l]));
  }
  float lane[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) lane[l] = fadd(fadd(p[l], p[4 + l]), fadd(p[8 + l], p[12 + l]));
  float sum = fadd(fadd(fadd(lane[0], lane[1]), lane[2]), lane[3]);
  for (int i = 16 * nfull; i < d; ++i) sum = fadd(sum, fmul(a[i], b[i]));
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
  bool moved = false;
#pragma unroll
  for (int q = 0; q < kAssignRows; ++q) {
    if (!live[q]) continue;
    const int r = r0 + q;
    if (final_pass) {
      B.labels[static_cast<size_t>(p) * B.n + r] = best[q] + 1;
    } else if (as[r] != best[q]) {
      as[r] = best[q];
      moved = true;
    }
  }
  // the reference only tests whether any assignment changed: one plain store
  // per warp instead of an atomic per row (per-row atomics on one counter
  // serialise in L2)
  const unsigned any = __ballot_sync(__activemask(), moved);
  if (any != 0u && (threadIdx.x & 31) == __ffs(__activemask()) - 1) B.changed[p] = 1;
}

// ---------------------------------------------------------------------------
// Tensor-core assignment.  Approximate distances a_c = (|x|^2 + |c|^2) -
// 2 dot_tc(x, c), where dot_tc is the bf16 hi + lo product (hi.hi + hi.lo +
// lo.hi) accumulated in f32 by mma.sync and the norms are the exact ones of
// the canonical formula; |a_c - dist_c| <= delta = (|x|^2 + max |c|^2) *
// (1e-4 + 2e-6 dp) (the same bound as the kNN candidate search, knn_tc.cu).
// The exact nearest centroid has a_c <= min a + 2 delta, so only those
// centroids get the canonical x86-order distance; the winner among them
// (ties to the lower cluster) is the canonical winner.  Non-finite values
// fail no test and send every centroid to the exact distance.
// ---------------------------------------------------------------------------
constexpr int kTcAssignWarps = 4;

__device__ __forceinline__ void mma_bf16_16816(float* c, const uint32_t* a, uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// cent: the fp32 centroids staged too (else the exact recheck reads them from L2).
size_t assign_tc_smem(int k, int d, int dp, bool cent) {
  const int kpad = (k + 7) / 8 * 8, d4 = (d + 3) & ~3;
  const int half = dp / 2, rw = (half % 16 == 8) ? half : half + 8;
  return sizeof(uint32_t) * 2 * kpad * rw + sizeof(float) * ((cent ? static_cast<size_t>(k) * d4 : 0) + kpad + 1) +
         sizeof(float) * kTcAssignWarps * 16 * (kpad + 1);
}

constexpr size_t kTcSmemLimit = 227 * 1024;

// KS: k-steps of 16 coordinates held in registers (dp <= 16 KS).
template <int KS>
__global__ void __launch_bounds__(32 * kTcAssignWarps) assign_tc_kernel(KMeansBatch B, int final_pass) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int p = blockIdx.y;
  if (!final_pass && !B.active[p]) return;
  const int k = B.k, d = B.d, dp = B.dp, n = B.n;
  const int kpad = (k + 7) / 8 * 8, d4 = (d + 3) & ~3, rw = tc_row_words(dp), ksn = dp >> 4;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
  uint32_t* sch = reinterpret_cast<uint32_t*>(smraw);  // [kpad][rw]
  uint32_t* scl = sch + kpad * rw;
  float* scf = reinterpret_cast<float*>(scl + kpad * rw);  // [k][d4] when staged
  float* scn = scf + (B.tc_cent_smem ? static_cast<size_t>(k) * d4 : 0);  // [kpad] + max
  float* sa = scn + kpad + 1 + warp * 16 * (kpad + 1);     // this warp's [16][kpad + 1]
  const uint16_t* gch = B.ch + static_cast<size_t>(p) * k * dp;
  const uint16_t* gcl = B.cl + static_cast<size_t>(p) * k * dp;
  const float* cent = B.cent + static_cast<size_t>(p) * k * d;
  // centroids staged once per CTA (warps over centroids, lanes over words)
  for (int c = warp; c < kpad; c += kTcAssignWarps) {
    const uint32_t* h32 = reinterpret_cast<const uint32_t*>(gch + static_cast<size_t>(c) * dp);
    const uint32_t* l32 = reinterpret_cast<const uint32_t*>(gcl + static_cast<size_t>(c) * dp);
    for (int w = lane; w < (dp >> 1); w += 32) {
      sch[c * rw + w] = c < k ? h32[w] : 0u;
      scl[c * rw + w] = c < k ? l32[w] : 0u;
    }
    if (c < k && B.tc_cent_smem)
      for (int j = lane; j < d4; j += 32) scf[c * d4 + j] = j < d ? cent[static_cast<size_t>(c) * d + j] : 0.0f;
  }
  for (int c = threadIdx.x; c < kpad; c += blockDim.x)
    scn[c] = c < k ? B.cnorm[static_cast<size_t>(p) * k + c] : 0.0f;
  __syncthreads();
  if (threadIdx.x < 32) {
    float mx = 0.0f;
    for (int c = lane; c < k; c += 32) mx = fmaxf(mx, scn[c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    if (lane == 0) scn[kpad] = mx;
  }
  __syncthreads();
  for (int rb = 0; rb < B.tc_blocks; ++rb) {
    if ((blockIdx.x * B.tc_blocks + rb) * 16 * kTcAssignWarps >= n) break;
    const int r0 = (blockIdx.x * B.tc_blocks + rb) * 16 * kTcAssignWarps + warp * 16;
    auto global_row = [&](int i) {
      const int ii = i < n ? i : n - 1;
      return B.rows ? B.rows[static_cast<size_t>(p) * n + ii] : ii;
    };
    const int ga = global_row(r0 + g), gb = global_row(r0 + g + 8);
    uint32_t ah[KS][4], al[KS][4];
  #pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
      uint2 pa = make_uint2(0u, 0u), pb = pa, qa = pa, qb = pa;
      if (ks < ksn) {
        pa = *reinterpret_cast<const uint2*>(B.xh + static_cast<size_t>(ga) * dp + ks * 16 + 4 * tig);
        pb = *reinterpret_cast<const uint2*>(B.xh + static_cast<size_t>(gb) * dp + ks * 16 + 4 * tig);
        qa = *reinterpret_cast<const uint2*>(B.xl + static_cast<size_t>(ga) * dp + ks * 16 + 4 * tig);
        qb = *reinterpret_cast<const uint2*>(B.xl + static_cast<size_t>(gb) * dp + ks * 16 + 4 * tig);
      }
      ah[ks][0] = pa.x; ah[ks][2] = pa.y; ah[ks][1] = pb.x; ah[ks][3] = pb.y;
      al[ks][0] = qa.x; al[ks][2] = qa.y; al[ks][1] = qb.x; al[ks][3] = qb.y;
    }
    const float pna = B.pnorm[ga], pnb = B.pnorm[gb];
    // approximate distances, eight centroids per n-tile
    for (int nt0 = 0; nt0 < kpad / 8; nt0 += 8) {
      float acc[8][4];
  #pragma unroll
      for (int t = 0; t < 8; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.0f;
  #pragma unroll
      for (int ks = 0; ks < KS; ++ks) {
        if (ks < ksn) {
  #pragma unroll
          for (int t = 0; t < 8; ++t) {
            if (nt0 + t < kpad / 8) {
              const int off = ((nt0 + t) * 8 + g) * rw + ks * 8 + 2 * tig;
              const uint2 bh = *reinterpret_cast<const uint2*>(sch + off);
              const uint2 bl = *reinterpret_cast<const uint2*>(scl + off);
              mma_bf16_16816(acc[t], ah[ks], bh);
              mma_bf16_16816(acc[t], ah[ks], bl);
              mma_bf16_16816(acc[t], al[ks], bh);
            }
          }
        }
      }
  #pragma unroll
      for (int t = 0; t < 8; ++t) {
        if (nt0 + t < kpad / 8) {
          const int c = (nt0 + t) * 8 + 2 * tig;
          sa[g * (kpad + 1) + c] = __fsub_rn(fadd(pna, scn[c]), fmul(2.0f, acc[t][0]));
          sa[g * (kpad + 1) + c + 1] = __fsub_rn(fadd(pna, scn[c + 1]), fmul(2.0f, acc[t][1]));
          sa[(g + 8) * (kpad + 1) + c] = __fsub_rn(fadd(pnb, scn[c]), fmul(2.0f, acc[t][2]));
          sa[(g + 8) * (kpad + 1) + c + 1] = __fsub_rn(fadd(pnb, scn[c + 1]), fmul(2.0f, acc[t][3]));
        }
      }
    }
    __syncwarp();
    // exact distances of the centroids within min a + 2 delta: lanes r and
    // r + 16 take row r, each half of its centroids (by parity)
    {
      const int r = lane & 15, half = lane >> 4;
      const int i = r0 + r;
      const bool valid = i < n;
      const int grow = B.rows ? B.rows[static_cast<size_t>(p) * n + (valid ? i : n - 1)] : (valid ? i : n - 1);
      const float pn = B.pnorm[grow];
      const float* arow = sa + r * (kpad + 1);
      float amin = INFINITY;
      for (int c = half; c < k; c += 2) amin = fminf(amin, arow[c]);
      amin = fminf(amin, __shfl_xor_sync(kFull, amin, 16));
      const float thr = amin + 2.0f * fadd(pn, scn[kpad]) * B.tc_crel;
      // up to 128 coordinates of the row in registers, wider rows read from L1
      constexpr int kRegKS = KS <= 8 ? KS : 1;
      float xv[16 * kRegKS];
      const float* xr = B.x + static_cast<size_t>(grow) * d;
      if constexpr (KS <= 8) {
#pragma unroll
        for (int j = 0; j < 16 * KS; ++j) xv[j] = j < d ? xr[j] : 0.0f;
      }
      int best = k;
      float bestd = INFINITY;
      // each lane walks its own candidates; the lanes compute their dots
      // together (one per lane per round), so the warp never runs a dot for
      // a single lane
      int cpos = half;
      for (;;) {
        while (cpos < k && arow[cpos] > thr) cpos += 2;
        const bool have = cpos < k;
        if (!__any_sync(kFull, have)) break;
        const int c = have ? cpos : 0;
        const float* cc = B.tc_cent_smem ? scf + static_cast<size_t>(c) * d4 : cent + static_cast<size_t>(c) * d;
        float dt;
        if constexpr (KS <= 8) {
          dt = dot_x86_reg<KS>(xv, cc, d);
        } else {
          dt = dot_x86_mem<KS>(xr, cc, d);
        }
        if (have) {
          const float dist = __fsub_rn(fadd(pn, scn[c]), fmul(2.0f, dt));
          if (dist < bestd || (dist == bestd && c < best)) {
            bestd = dist;
            best = c;
          }
          cpos += 2;
        }
      }
      // the pair's winner: smaller distance, then smaller cluster (a NaN
      // distance never wins, as in the full scan; an all-NaN row keeps 0)
      const float od = __shfl_xor_sync(kFull, bestd, 16);
      const int oc = __shfl_xor_sync(kFull, best, 16);
      if (od < bestd || (od == bestd && oc < best)) {
        bestd = od;
        best = oc;
      }
      if (best >= k) best = 0;
      bool moved = false;
      if (valid && half == 0) {
        if (final_pass) {
          B.labels[static_cast<size_t>(p) * n + i] = best + 1;
        } else {
          int* as = B.assign + static_cast<size_t>(p) * n;
          if (as[i] != best) {
            as[i] = best;
            moved = true;
          }
        }
      }
      // only whether any assignment changed matters: one store per warp
      if (__ballot_sync(kFull, moved) != 0u && lane == 0) B.changed[p] = 1;
    }
    __syncwarp();
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

// Update step, part 2 (one CTA per problem and cluster): centroid sums in
// ascending row order, scaled by 1/size.  A cluster can hold thousands of
// rows (in high dimension one centroid often takes most of a mixture
// component), and its features are sequential float chains, so the rows are
// streamed through a ring of kSumStages chunks of kSumChunk rows in shared
// memory with cp.async: every thread copies, the member ids of a chunk are
// read one chunk ahead of its copies, and thread j adds feature j down each
// landed chunk in row order.  Features go in blocks of kSumCols.
constexpr int kSumChunk = 128;
constexpr int kSumStages = 4;
constexpr int kSumCols = 64;
constexpr int kSumThreads = 256;

size_t sums_smem(int d) {
  const int dw = d < kSumCols ? d : kSumCols;
  return sizeof(float) * kSumStages * kSumChunk * dw + sizeof(int) * kSumStages * kSumChunk;
}

__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit_group() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait_groups() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__global__ void __launch_bounds__(kSumThreads) sums_kernel(KMeansBatch B) {
  extern __shared__ float sring[];
  const int p = blockIdx.x / B.k, c = blockIdx.x % B.k;
  if (p >= B.problems || !B.active[p]) return;
  const int d = B.d;
  const int* mem = B.members + static_cast<size_t>(p) * B.n;
  const int* off = B.offsets + static_cast<size_t>(p) * (B.k + 1);
  const int b0 = off[c], b1 = off[c + 1];
  float* cent = B.cent + (static_cast<size_t>(p) * B.k + c) * d;
  const int cnt = b1 - b0;
  const float inv = cnt != 0 ? __fdiv_rn(1.0f, static_cast<float>(cnt)) : 0.0f;
  const int nchunks = (cnt + kSumChunk - 1) / kSumChunk;
  for (int jb = 0; jb < d; jb += kSumCols) {
    const int dw = min(kSumCols, d - jb);
    float* rows_s = sring;                                              // [stage][kSumChunk][dw]
    int* ids_s = reinterpret_cast<int*>(sring + kSumStages * kSumChunk * dw);  // [stage][kSumChunk]
    // stage the ids of the first chunks, then copy chunk i while the ids of
    // chunk i + 1 are read
    auto load_ids = [&](int ch) {
      const int base = b0 + ch * kSumChunk;
      int* ids = ids_s + (ch % kSumStages) * kSumChunk;
      for (int r = threadIdx.x; r < kSumChunk; r += kSumThreads) ids[r] = base + r < b1 ? mem[base + r] : -1;
    };
    auto copy_rows = [&](int ch) {
      const int* ids = ids_s + (ch % kSumStages) * kSumChunk;
      float* dst = rows_s + (ch % kSumStages) * kSumChunk * dw;
      const int m = min(kSumChunk, b1 - (b0 + ch * kSumChunk));
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for (int r = warp; r < m; r += kSumThreads / 32) {
        const float* src = B.x + static_cast<size_t>(ids[r]) * d + jb;
        for (int col = lane; col < dw; col += 32) cp_async4(dst + r * dw + col, src + col);
      }
    };
    float s = 0.0f;
    __syncthreads();
    if (nchunks > 0) load_ids(0);
    __syncthreads();
    // prologue: copies of chunks 0 .. kSumStages-2 in flight
    for (int ch = 0; ch < kSumStages - 1; ++ch) {
      if (ch < nchunks) {
        if (ch + 1 < nchunks) load_ids(ch + 1);
        copy_rows(ch);
      }
      cp_async_commit_group();
      __syncthreads();
    }
    for (int ch = 0; ch < nchunks; ++ch) {
      // keep kSumStages - 1 chunks in flight: issue chunk ch + kSumStages - 1
      const int nx = ch + kSumStages - 1;
      if (nx < nchunks) {
        if (nx + 1 < nchunks) load_ids(nx + 1);
        copy_rows(nx);
      }
      cp_async_commit_group();
      cp_async_wait_groups<kSumStages - 1>();
      __syncthreads();
      if (threadIdx.x < dw) {
        const int m = min(kSumChunk, b1 - (b0 + ch * kSumChunk));
        const float* sc = rows_s + (ch % kSumStages) * kSumChunk * dw + threadIdx.x;
#pragma unroll 8
        for (int r = 0; r < m; ++r) s = fadd(s, sc[r * dw]);
      }
      __syncthreads();
    }
    if (threadIdx.x < dw) cent[jb + threadIdx.x] = cnt != 0 ? fmul(s, inv) : s;
  }
}

// Update step, sort and sums in one (one CTA per cluster and problem, d up
// to 4 x kScanThreads): the CTA scans the problem's assignments in chunks of
// kScanChunk rows -- a ballot per 32 rows, prefix over the warps -- so the
// cluster's members of a chunk land in shared memory in ascending row order;
// thread j then adds columns j, j + 256, ... down them, up to 32 rows' loads
// in flight.  The size goes to offsets[c] (finalize_kernel reads sizes).
// Without the member lists and the one-CTA sort this replaces sort_kernel and
// sums_kernel when each problem's assignments are read by its k CTAs anyway.
constexpr int kScanThreads = 256;
constexpr int kScanChunk = 4 * kScanThreads;
constexpr int kScanCols = 4;  // columns per thread
constexpr int kScanBatch = 16;  // member rows whose loads are issued together

__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(KMeansBatch B) {
  __shared__ int mem[kScanChunk];
  __shared__ int wcount[kScanThreads / 32];
  const int c = blockIdx.x, p = blockIdx.y;
  if (!B.active[p]) return;
  const int n = B.n, d = B.d, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int* as = B.assign + static_cast<size_t>(p) * n;
  const int* rows = B.rows != nullptr ? B.rows + static_cast<size_t>(p) * n : nullptr;
  float s[kScanCols];
#pragma unroll
  for (int q = 0; q < kScanCols; ++q) s[q] = 0.0f;
  int count = 0;
  for (int base = 0; base < n; base += kScanChunk) {
    // warp w scans rows base + 128 w .. + 127, 32 at a time
    unsigned bal[4];
    int cw = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = base + warp * 128 + i * 32 + lane;
      bal[i] = __ballot_sync(kFull, r < n && as[r] == c);
      cw += __popc(bal[i]);
    }
    if (lane == 0) wcount[warp] = cw;
    __syncthreads();
    int off = 0, total = 0;
#pragma unroll
    for (int q = 0; q < kScanThreads / 32; ++q) {
      const int v = wcount[q];
      off += q < warp ? v : 0;
      total += v;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if ((bal[i] >> lane) & 1u) {
        const int r = base + warp * 128 + i * 32 + lane;
        mem[off + __popc(bal[i] & ((1u << lane) - 1u))] = rows != nullptr ? rows[r] : r;
      }
      off += __popc(bal[i]);
    }
    __syncthreads();
    for (int m0 = 0; m0 < total; m0 += kScanBatch) {
      const int mb = min(kScanBatch, total - m0);
#pragma unroll
      for (int q = 0; q < kScanCols; ++q) {
        const int j = tid + q * kScanThreads;
        if (q * kScanThreads < d) {
          float v[kScanBatch];
#pragma unroll
          for (int u = 0; u < kScanBatch; ++u)
            v[u] = (u < mb && j < d) ? B.x[static_cast<size_t>(mem[m0 + u]) * d + j] : 0.0f;
#pragma unroll
          for (int u = 0; u < kScanBatch; ++u)
            if (u < mb) s[q] = fadd(s[q], v[u]);
        }
      }
    }
    count += total;
    __syncthreads();  // mem and wcount are rewritten by the next chunk
  }
  const float inv = count != 0 ? __fdiv_rn(1.0f, static_cast<float>(count)) : 0.0f;
  float* cent = B.cent + (static_cast<size_t>(p) * B.k + c) * d;
#pragma unroll
  for (int q = 0; q < kScanCols; ++q) {
    const int j = tid + q * kScanThreads;
    if (j < d) cent[j] = count != 0 ? fmul(s[q], inv) : s[q];
  }
  if (tid == 0) B.offsets[static_cast<size_t>(p) * (B.k + 1) + c] = count;
}

// Update step, part 3 (one thread per problem): empty-cluster splitting and
// the early-exit flag.  sizes: offsets[c] holds cluster c's size (after
// scan_sums_kernel) rather than its start (after sort_kernel).
__global__ void finalize_kernel(KMeansBatch B, int sizes) {
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
    const int size = sizes ? off[c] : off[c + 1] - off[c];
    fsize[c] = static_cast<float>(size);
    any_empty |= size == 0;
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

// ---------------------------------------------------------------------------
// Persistent batched k-means: one CTA per problem runs every Lloyd iteration
// and the final assignment with block barriers only, so a batch of M
// problems is one launch instead of 5 per iteration.  Same arithmetic as the
// multi-launch path above (tensor-core candidate distances with the exact
// x86-order recheck, centroid sums in ascending row order, the float Fenwick
// split of empty clusters), hence the same labels bit for bit.
//
// Per iteration, in shared memory: the centroids (fp32 and their bf16 hi/lo
// split in the mma B layout), their norms, the problem's assignments,
// per-warp cluster histograms.  The member lists (rows grouped by cluster,
// ascending) go to global memory (L2).
//   assignment: a warp takes 16-row tiles; the mma.sync approximations stay
//     in the accumulator registers, where each quad of lanes finds its two
//     rows' minima, thresholds and candidate masks (shuffles).  A row with
//     finite approximations and a single candidate takes it; the other rows
//     get, for each candidate centroid (ascending), the exact x86-order dot,
//     its 16 partial sums held by 16 lanes (coalesced row loads) and combined
//     by shuffles in the reference's order.  Up to 64 centroids one pass;
//     up to 128 the approximations are computed twice (minima, then masks);
//   grouping: per-warp counts over contiguous row ranges, prefix sums, stable
//     scatter of the row ids into the member lists;
//   sums: a warp per (cluster, 64-column block), taken from a shared queue;
//     lane j keeps the float chains of columns j and j + 32 down the member
//     rows in ascending order, 8 rows' loads in flight;
//   split: one thread, as finalize_kernel.
// ---------------------------------------------------------------------------
constexpr int kPkWarps = 16;
constexpr int kPkThreads = 32 * kPkWarps;

struct PkLayout {
  size_t o_ch, o_cl, o_cf, o_cn, o_as, o_wh, o_off, o_fs, o_misc, total;
};

__host__ __device__ inline size_t pk_align(size_t v) { return (v + 15) & ~static_cast<size_t>(15); }

__host__ __device__ inline PkLayout pk_layout(int n, int k, int d, int dp) {
  const int kpad = (k + 7) / 8 * 8, rw = tc_row_words(dp), d4 = (d + 3) & ~3;
  PkLayout L{};
  size_t o = 0;
  L.o_ch = o; o = pk_align(o + sizeof(uint32_t) * kpad * rw);
  L.o_cl = o; o = pk_align(o + sizeof(uint32_t) * kpad * rw);
  L.o_cf = o; o = pk_align(o + sizeof(float) * static_cast<size_t>(k) * d4);
  L.o_cn = o; o = pk_align(o + sizeof(float) * (kpad + 1));
  L.o_as = o; o = pk_align(o + sizeof(int) * static_cast<size_t>(n));
  L.o_wh = o; o = pk_align(o + sizeof(int) * kPkWarps * k);
  L.o_off = o; o = pk_align(o + sizeof(int) * (k + 1));
  L.o_fs = o; o = pk_align(o + sizeof(float) * (3 * k + 1));
  L.o_misc = o; o = pk_align(o + sizeof(int) * 4);
  L.total = o;
  return L;
}

template <int KS, int NC>
__global__ void __launch_bounds__(kPkThreads, 1) kmeans_persistent_kernel(KMeansBatch B) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int p = blockIdx.x;
  const int k = B.k, d = B.d, dp = B.dp, n = B.n;
  const int kpad = (k + 7) / 8 * 8, rw = tc_row_words(dp), d4 = (d + 3) & ~3, ksn = dp >> 4;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, tig = lane & 3;
  const int half = lane >> 4, hl = lane & 15;
  const PkLayout Ly = pk_layout(n, k, d, dp);
  uint32_t* sch = reinterpret_cast<uint32_t*>(smraw + Ly.o_ch);
  uint32_t* scl = reinterpret_cast<uint32_t*>(smraw + Ly.o_cl);
  float* scf = reinterpret_cast<float*>(smraw + Ly.o_cf);     // [k][d4]
  float* scn = reinterpret_cast<float*>(smraw + Ly.o_cn);     // [kpad] + max
  int* sas = reinterpret_cast<int*>(smraw + Ly.o_as);         // [n] assignments
  int* whist = reinterpret_cast<int*>(smraw + Ly.o_wh);       // [warps][k]
  int* soff = reinterpret_cast<int*>(smraw + Ly.o_off);       // [k + 1]
  float* fsize = reinterpret_cast<float*>(smraw + Ly.o_fs);   // [k], tree [k + 1], vals [k]
  int* misc = reinterpret_cast<int*>(smraw + Ly.o_misc);      // changed, sums queue
  const int* prow = B.rows + static_cast<size_t>(p) * n;
  int* mem = B.members + static_cast<size_t>(p) * n;
  const int nfull = d >> 4, tn = d - 16 * nfull;

  // initial centroids: the problem's rows init_rows[0..k)
  for (int i = tid; i < k * d4; i += kPkThreads) {
    const int c = i / d4, j = i % d4;
    const int grow = prow[B.init_rows[static_cast<size_t>(p) * k + c]];
    scf[i] = j < d ? B.x[static_cast<size_t>(grow) * d + j] : 0.0f;
  }
  for (int i = tid; i < n; i += kPkThreads) sas[i] = -1;
  const int iters = B.max_iter > 1 ? B.max_iter : 1;
  for (int it = 0; it <= iters; ++it) {
    const bool final_pass = it == iters;
    if (tid == 0) misc[0] = 0;
    __syncthreads();
    // centroid norms and the bf16 split of the centroids
    for (int c = tid; c < kpad; c += kPkThreads)
      scn[c] = c < k ? dot_x86([&](int j) { return scf[c * d4 + j]; }, [&](int j) { return scf[c * d4 + j]; }, d)
                     : 0.0f;
    {
      uint16_t* h16 = reinterpret_cast<uint16_t*>(sch);
      uint16_t* l16 = reinterpret_cast<uint16_t*>(scl);
      for (int e = tid; e < kpad * dp; e += kPkThreads) {
        const int c = e / dp, j = e % dp;
        const float v = (c < k && j < d) ? scf[c * d4 + j] : 0.0f;
        const uint32_t hb = bf16_bits(v);
        const uint32_t lb = bf16_bits(__fsub_rn(v, __uint_as_float(hb << 16)));
        h16[c * 2 * rw + perm16(j)] = static_cast<uint16_t>(hb);
        l16[c * 2 * rw + perm16(j)] = static_cast<uint16_t>(lb);
      }
    }
    __syncthreads();
    if (warp == 0) {
      float mx = 0.0f;
      for (int c = lane; c < k; c += 32) mx = fmaxf(mx, scn[c]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
      if (lane == 0) scn[kpad] = mx;
    }
    __syncthreads();

    // ---- assignment ----
    const float crel = B.tc_crel, cmax = scn[kpad];
    const int ntiles = (n + 15) / 16;
    for (int tile = warp; tile < ntiles; tile += kPkWarps) {
      const int r0 = tile * 16;
      const int ga = prow[min(r0 + g, n - 1)], gb = prow[min(r0 + g + 8, n - 1)];
      uint32_t ah[KS][4], al[KS][4];
#pragma unroll
      for (int ks = 0; ks < KS; ++ks) {
        uint2 pa = make_uint2(0u, 0u), pb = pa, qa = pa, qb = pa;
        if (ks < ksn) {
          pa = *reinterpret_cast<const uint2*>(B.xh + static_cast<size_t>(ga) * dp + ks * 16 + 4 * tig);
          pb = *reinterpret_cast<const uint2*>(B.xh + static_cast<size_t>(gb) * dp + ks * 16 + 4 * tig);
          qa = *reinterpret_cast<const uint2*>(B.xl + static_cast<size_t>(ga) * dp + ks * 16 + 4 * tig);
          qb = *reinterpret_cast<const uint2*>(B.xl + static_cast<size_t>(gb) * dp + ks * 16 + 4 * tig);
        }
        ah[ks][0] = pa.x; ah[ks][2] = pa.y; ah[ks][1] = pb.x; ah[ks][3] = pb.y;
        al[ks][0] = qa.x; al[ks][2] = qa.y; al[ks][1] = qb.x; al[ks][3] = qb.y;
      }
      const float pna = B.pnorm[ga], pnb = B.pnorm[gb];
      // approximate distances of rows g (acc[t][0..1]) and g + 8 (acc[t][2..3])
      // to the centroids of n-tile ch * 8 + t, columns 2 tig and 2 tig + 1
      float acc[8][4];
      auto approx = [&](int ch) {
#pragma unroll
        for (int t = 0; t < 8; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.0f;
        // the three products of a k-step go round the 8 n-tiles in turn, so
        // consecutive mma.sync never wait on the same accumulator
#pragma unroll
        for (int ks = 0; ks < KS; ++ks) {
          if (ks < ksn) {
            uint2 bf[8];
#pragma unroll
            for (int t = 0; t < 8; ++t)
              if (ch * 8 + t < kpad / 8)
                bf[t] = *reinterpret_cast<const uint2*>(sch + ((ch * 8 + t) * 8 + g) * rw + ks * 8 + 2 * tig);
#pragma unroll
            for (int t = 0; t < 8; ++t)
              if (ch * 8 + t < kpad / 8) mma_bf16_16816(acc[t], ah[ks], bf[t]);
#pragma unroll
            for (int t = 0; t < 8; ++t)
              if (ch * 8 + t < kpad / 8) mma_bf16_16816(acc[t], al[ks], bf[t]);
#pragma unroll
            for (int t = 0; t < 8; ++t)
              if (ch * 8 + t < kpad / 8)
                bf[t] = *reinterpret_cast<const uint2*>(scl + ((ch * 8 + t) * 8 + g) * rw + ks * 8 + 2 * tig);
#pragma unroll
            for (int t = 0; t < 8; ++t)
              if (ch * 8 + t < kpad / 8) mma_bf16_16816(acc[t], ah[ks], bf[t]);
          }
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int c = (ch * 8 + t) * 8 + 2 * tig;
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int cc = c + (e & 1);
            const float pn = e < 2 ? pna : pnb;
            acc[t][e] = cc < k ? __fsub_rn(fadd(pn, scn[cc]), fmul(2.0f, acc[t][e])) : INFINITY;
          }
        }
      };
      // pass 1: row minima (with the values of a single chunk kept for pass 2)
      float ming = INFINITY, ming8 = INFINITY;
      bool fin_g = true, fin_g8 = true;
#pragma unroll
      for (int ch = 0; ch < NC; ++ch) {
        approx(ch);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int c = (ch * 8 + t) * 8 + 2 * tig;
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            if (c + e < k) {
              ming = fminf(ming, acc[t][e]);
              ming8 = fminf(ming8, acc[t][2 + e]);
              fin_g = fin_g && isfinite(acc[t][e]);
              fin_g8 = fin_g8 && isfinite(acc[t][2 + e]);
            }
          }
        }
      }
#pragma unroll
      for (int o = 1; o <= 2; o <<= 1) {
        ming = fminf(ming, __shfl_xor_sync(kFull, ming, o));
        ming8 = fminf(ming8, __shfl_xor_sync(kFull, ming8, o));
      }
      const float thr_g = ming + 2.0f * fadd(pna, cmax) * crel;
      const float thr_g8 = ming8 + 2.0f * fadd(pnb, cmax) * crel;
      // pass 2: candidate masks (bit c of word c / 32) of both rows
      uint32_t mg[4] = {0u, 0u, 0u, 0u}, mg8[4] = {0u, 0u, 0u, 0u};
#pragma unroll
      for (int ch = 0; ch < NC; ++ch) {
        if (NC > 1) approx(ch);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int c = (ch * 8 + t) * 8 + 2 * tig;
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            if (c + e < k) {
              // column c + e sits in word (ch * 8 + t) / 4 at bit c + e mod 32
              const uint32_t bit = 1u << ((((ch * 8 + t) & 3) << 3) + 2 * tig + e);
              if (!(acc[t][e] > thr_g)) mg[(ch * 8 + t) >> 2] |= bit;
              if (!(acc[t][2 + e] > thr_g8)) mg8[(ch * 8 + t) >> 2] |= bit;
            }
          }
        }
      }
#pragma unroll
      for (int w = 0; w < 4; ++w) {
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
          mg[w] |= __shfl_xor_sync(kFull, mg[w], o);
          mg8[w] |= __shfl_xor_sync(kFull, mg8[w], o);
        }
      }
      {
        // a row whose approximations and norm are all finite and that has a
        // single candidate: that candidate is the exact nearest centroid
        // (the nearest is always a candidate, and an exact tie would make
        // both tied centroids candidates); other rows take the exact recheck
        bool fg = fin_g && isfinite(pna), fg8 = fin_g8 && isfinite(pnb);
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
          fg = __shfl_xor_sync(kFull, static_cast<int>(fg), o) != 0 && fg;
          fg8 = __shfl_xor_sync(kFull, static_cast<int>(fg8), o) != 0 && fg8;
        }
        const int pop_g = __popc(mg[0]) + __popc(mg[1]) + __popc(mg[2]) + __popc(mg[3]);
        const int pop_g8 = __popc(mg8[0]) + __popc(mg8[1]) + __popc(mg8[2]) + __popc(mg8[3]);
        const bool single_g = fg && pop_g == 1, single_g8 = fg8 && pop_g8 == 1;
        auto first_bit = [](const uint32_t (&m)[4]) {
          return m[0] ? __ffs(m[0]) - 1 : m[1] ? 31 + __ffs(m[1]) : m[2] ? 63 + __ffs(m[2]) : 95 + __ffs(m[3]);
        };
        auto put = [&](int i, int best) {
          if (i >= n) return;
          if (final_pass) {
            B.labels[static_cast<size_t>(p) * n + i] = best + 1;
          } else if (sas[i] != best) {
            sas[i] = best;
            misc[0] = 1;
          }
        };
        if (tig == 0) {
          if (single_g) put(r0 + g, first_bit(mg));
          if (single_g8) put(r0 + g + 8, first_bit(mg8));
        }
        // rows left for the exact recheck: bit r of `multi`
        const unsigned bal_g = __ballot_sync(kFull, tig == 0 && !single_g);
        const unsigned bal_g8 = __ballot_sync(kFull, tig == 0 && !single_g8);
        unsigned multi = 0u;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          multi |= ((bal_g >> (4 * q)) & 1u) << q;
          multi |= ((bal_g8 >> (4 * q)) & 1u) << (q + 8);
        }
        while (multi != 0u) {
          const int r = __ffs(multi) - 1;
          multi &= multi - 1u;
          const int i = r0 + r;
          if (i >= n) continue;
          const int src = 4 * (r & 7);
          uint32_t m[4];
#pragma unroll
          for (int w = 0; w < 4; ++w) m[w] = __shfl_sync(kFull, r < 8 ? mg[w] : mg8[w], src);
          const int grow = prow[i];
          const float pn = B.pnorm[grow];
          // the row: lane hl holds coordinates hl + 16 b (b < nfull) and the
          // tail coordinate 16 nfull + hl; both halves compute the same dots
          const float* xr = B.x + static_cast<size_t>(grow) * d;
          float xv[KS];
#pragma unroll
          for (int bb = 0; bb < KS; ++bb) xv[bb] = bb < nfull ? xr[hl + 16 * bb] : 0.0f;
          const float xt = hl < tn ? xr[16 * nfull + hl] : 0.0f;
          int best = k;
          float bestd = INFINITY;
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            uint32_t bits = m[w];
            while (bits != 0u) {
              const int c = 32 * w + __ffs(bits) - 1;
              bits &= bits - 1u;
              const float* cc = scf + c * d4;
              float pp = 0.0f;
#pragma unroll
              for (int bb = 0; bb < KS; ++bb)
                if (bb < nfull) pp = fadd(pp, fmul(xv[bb], cc[hl + 16 * bb]));
              const int hb = half * 16;
              const float q4 = __shfl_sync(kFull, pp, hb + ((hl + 4) & 15));
              const float q8 = __shfl_sync(kFull, pp, hb + ((hl + 8) & 15));
              const float q12 = __shfl_sync(kFull, pp, hb + ((hl + 12) & 15));
              const float lv = fadd(fadd(pp, q4), fadd(q8, q12));
              float sum = fadd(fadd(fadd(__shfl_sync(kFull, lv, hb), __shfl_sync(kFull, lv, hb + 1)),
                                    __shfl_sync(kFull, lv, hb + 2)),
                               __shfl_sync(kFull, lv, hb + 3));
              for (int t = 0; t < tn; ++t)
                sum = fadd(sum, fmul(__shfl_sync(kFull, xt, hb + t), cc[16 * nfull + t]));
              const float dist = __fsub_rn(fadd(pn, scn[c]), fmul(2.0f, sum));
              if (dist < bestd || (dist == bestd && c < best)) {
                bestd = dist;
                best = c;
              }
            }
          }
          if (best >= k) best = 0;
          if (lane == 0) put(i, best);
        }
      }
    }
    __syncthreads();
    if (final_pass) break;

    // ---- grouping: member lists in ascending row order per cluster ----
    for (int i = tid; i < kPkWarps * k; i += kPkThreads) whist[i] = 0;
    __syncthreads();
    const int per = (n + kPkWarps - 1) / kPkWarps;
    const int beg = warp * per, end = min(n, beg + per);
    for (int base = beg; base < end; base += 32) {
      const int r = base + lane;
      const int c = r < end ? sas[r] : -1;
      const unsigned mm = __match_any_sync(kFull, c);
      if (c >= 0 && (__ffs(mm) - 1) == lane) whist[warp * k + c] += __popc(mm);
    }
    __syncthreads();
    for (int c = tid; c < k; c += kPkThreads) {
      int run = 0;
      for (int w = 0; w < kPkWarps; ++w) {
        const int v = whist[w * k + c];
        whist[w * k + c] = run;
        run += v;
      }
      soff[c] = run;  // size for now
    }
    __syncthreads();
    if (tid == 0) {
      int run = 0;
      for (int c = 0; c < k; ++c) {
        const int sz = soff[c];
        soff[c] = run;
        run += sz;
      }
      soff[k] = run;
      misc[1] = 0;
    }
    __syncthreads();
    for (int i = tid; i < kPkWarps * k; i += kPkThreads) whist[i] += soff[i % k];
    __syncthreads();
    for (int base = beg; base < end; base += 32) {
      const int r = base + lane;
      const int c = r < end ? sas[r] : -1;
      const unsigned mm = __match_any_sync(kFull, c);
      if (c >= 0) mem[whist[warp * k + c] + __popc(mm & ((1u << lane) - 1u))] = prow[r];
      __syncwarp();
      if (c >= 0 && (__ffs(mm) - 1) == lane) whist[warp * k + c] += __popc(mm);
      __syncwarp();
    }
    __syncthreads();

    // ---- centroid sums in ascending row order ----
    const int nblk = (d + 63) / 64;
    for (;;) {
      int item = 0;
      if (lane == 0) item = atomicAdd(&misc[1], 1);
      item = __shfl_sync(kFull, item, 0);
      if (item >= k * nblk) break;
      const int c = item / nblk, j0 = (item % nblk) * 64 + lane, j1 = j0 + 32;
      const int b0 = soff[c], b1 = soff[c + 1];
      const int cnt = b1 - b0;
      float s0 = 0.0f, s1 = 0.0f;
      for (int mb = b0; mb < b1; mb += 8) {
        float v0[8], v1[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int id = mb + u < b1 ? mem[mb + u] : -1;
          const float* xr = B.x + static_cast<size_t>(id < 0 ? 0 : id) * d;
          v0[u] = (id >= 0 && j0 < d) ? xr[j0] : 0.0f;
          v1[u] = (id >= 0 && j1 < d) ? xr[j1] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (mb + u < b1) {
            s0 = fadd(s0, v0[u]);
            s1 = fadd(s1, v1[u]);
          }
        }
      }
      const float inv = cnt != 0 ? __fdiv_rn(1.0f, static_cast<float>(cnt)) : 0.0f;
      if (j0 < d) scf[c * d4 + j0] = cnt != 0 ? fmul(s0, inv) : s0;
      if (j1 < d) scf[c * d4 + j1] = cnt != 0 ? fmul(s1, inv) : s1;
    }
    __syncthreads();

    // ---- empty-cluster split (finalize_kernel) ----
    if (tid == 0) {
      float* ftree = fsize + k;
      float* fvals = ftree + k + 1;
      bool any_empty = false;
      for (int c = 0; c < k; ++c) {
        fsize[c] = static_cast<float>(soff[c + 1] - soff[c]);
        any_empty |= soff[c + 1] == soff[c];
      }
      if (any_empty && n > k) {
        const float eps = 1.0f / 1024.0f;
        Fenwick fw{ftree, fvals, k};
        for (int i = 0; i <= k; ++i) ftree[i] = 0.0f;
        for (int i = 0; i < k; ++i) fvals[i] = 0.0f;
        for (int c = 0; c < k; ++c) fw.set(c, pos_part(__fsub_rn(fsize[c], 1.0f)));
        int u = 0;  // the uniforms restart with every split, as in finalize_kernel
        for (int e = 0; e < k; ++e) {
          if (fsize[e] != 0.0f) continue;
          const float total = fw.total();
          int donor = -1;
          if (total > 0.0f) donor = fw.select(fmul(B.split_uniform[u++], total));
          if (donor < 0) {
            donor = 0;
            for (int c = 1; c < k; ++c) if (fsize[c] > fsize[donor]) donor = c;
          }
          float* ec = scf + e * d4;
          float* dc = scf + donor * d4;
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
    }
    __syncthreads();
    // early exit: no assignment changed in this iteration (checked after the
    // update, as the reference does); go to the final assignment
    if (misc[0] == 0) it = iters - 1;
    __syncthreads();
  }
}

}  // namespace

// Above 128 centroids the per-warp distance tiles hold the kernel to one
// 4-warp CTA per SM and the exact assignment is faster.
bool kmeans_tc_supported(int d, int k) {
  if (d < 1 || d > 256 || k < 1 || k > 128) return false;
  return assign_tc_smem(k, d, (d + 15) / 16 * 16, false) <= kTcSmemLimit;
}

size_t kmeans_sort_smem(int k) { return sizeof(int) * (33 * static_cast<size_t>(k) + 1); }

int kmeans_row_norms(const float* x, int n, int d, float* out, cudaStream_t st) {
  row_norms_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, n, d, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

namespace {

// |a - dist| <= (|x|^2 + max |c|^2) * crel: both share RN(|x|^2 + |c|^2);
// 2 |dot_tc - dot_x86| <= 2 (3.1 * 2^-16 [the hi + lo split] +
// 3 dp * 2^-22 [f32 accumulation of 3 dp products, two ulps per add] +
// (d / 16 + 5) 2^-24 [the x86-order dot]) sum|x_i c_i|, with
// sum|x_i c_i| <= 0.51 (|x|^2 + |c|^2); the two final subtractions round
// values of at most 2.03 (|x|^2 + |c|^2) each
float tc_error_factor(int d, int dp) {
  const double tc = 3.1 * std::ldexp(1.0, -16) + 3.0 * dp * std::ldexp(1.0, -22) + (d / 16 + 5) * std::ldexp(1.0, -24);
  return static_cast<float>(1.05 * (1.02 * tc + 4.1 * std::ldexp(1.0, -24)) + 1e-7);
}

// The persistent kernel applies: a batch of several problems given by row
// lists, the tensor-core assignment with d <= 64, and its shared memory fits.
bool persistent_supported(const KMeansBatch& B) {
  if (B.problems < 2 || B.rows == nullptr || B.xh == nullptr || B.members == nullptr) return false;
  if (!kmeans_tc_supported(B.d, B.k) || B.dp > 64 || B.n < 1) return false;
  return pk_layout(B.n, B.k, B.d, B.dp).total <= kTcSmemLimit;
}

}  // namespace

int kmeans_run(const KMeansBatch& B, cudaStream_t st) {
  if (B.problems <= 0) return 0;
  if (persistent_supported(B)) {
    KMeansBatch P = B;
    P.tc_crel = tc_error_factor(B.d, B.dp);
    const size_t bytes = pk_layout(B.n, B.k, B.d, B.dp).total;
    cudaError_t e;
    const int nc = ((B.k + 7) / 8 + 7) / 8;  // 8-n-tile chunks: 1 (k <= 64) or 2 (k <= 128)
    auto go = [&](auto kern) {
      const cudaError_t err =
          cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
      if (err != cudaSuccess) return err;
      kern<<<B.problems, kPkThreads, bytes, st>>>(P);
      return cudaSuccess;
    };
    if (B.dp <= 16) e = nc == 1 ? go(kmeans_persistent_kernel<1, 1>) : go(kmeans_persistent_kernel<1, 2>);
    else if (B.dp <= 32) e = nc == 1 ? go(kmeans_persistent_kernel<2, 1>) : go(kmeans_persistent_kernel<2, 2>);
    else e = nc == 1 ? go(kmeans_persistent_kernel<4, 1>) : go(kmeans_persistent_kernel<4, 2>);
    if (e != cudaSuccess) return static_cast<int>(e);
    count_launch();
    return static_cast<int>(cudaGetLastError());
  }
  init_centroids_kernel<<<dim3(B.k, B.problems), 64, 0, st>>>(B);
  const size_t cs_bytes = sizeof(float) * (static_cast<size_t>(B.k) * ((B.d + 3) & ~3) + B.k);
  const size_t sort_bytes = kmeans_sort_smem(B.k);
  const dim3 agrid((B.n + 128 * kAssignRows - 1) / (128 * kAssignRows), B.problems);
  const dim3 ngrid((B.k + 127) / 128, B.problems);
  const size_t sum_bytes = sums_smem(B.d);
  const bool tc = B.xh != nullptr && kmeans_tc_supported(B.d, B.k);
  const bool cent_smem = tc && assign_tc_smem(B.k, B.d, B.dp, true) <= kTcSmemLimit;
  const size_t tc_bytes = tc ? assign_tc_smem(B.k, B.d, B.dp, cent_smem) : 0;
  const int tc_ks = B.dp <= 64 ? 4 : (B.dp <= 128 ? 8 : 16);
  if (tc) {
    cudaFuncSetAttribute(assign_tc_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tc_bytes));
    cudaFuncSetAttribute(assign_tc_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tc_bytes));
    cudaFuncSetAttribute(assign_tc_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tc_bytes));
  }
  // 64-row blocks per CTA: the centroids are staged once per CTA, but the grid
  // keeps at least two CTAs per SM
  KMeansBatch T = B;
  T.tc_cent_smem = cent_smem ? 1 : 0;
  {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks = static_cast<long long>((B.n + 16 * kTcAssignWarps - 1) / (16 * kTcAssignWarps)) * B.problems;
    long long per = blocks / (2LL * sms);
    T.tc_blocks = static_cast<int>(per < 1 ? 1 : (per > 8 ? 8 : per));
    T.tc_crel = tc_error_factor(B.d, B.dp);
  }
  const int rows_per_cta = 16 * kTcAssignWarps * T.tc_blocks;
  const dim3 tgrid((B.n + rows_per_cta - 1) / rows_per_cta, B.problems);
  auto launch_assign = [&](int final_pass) {
    if (tc) {
      // the centroids' bf16 split (its own launch is counted there)
      bf16_split_rows(B.cent, B.problems * B.k, B.d, B.dp, B.ch, B.cl, st);
      if (tc_ks == 16) assign_tc_kernel<16><<<tgrid, 32 * kTcAssignWarps, tc_bytes, st>>>(T, final_pass);
      else if (tc_ks == 8) assign_tc_kernel<8><<<tgrid, 32 * kTcAssignWarps, tc_bytes, st>>>(T, final_pass);
      else assign_tc_kernel<4><<<tgrid, 32 * kTcAssignWarps, tc_bytes, st>>>(T, final_pass);
      return;
    }
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
  cudaFuncSetAttribute(sums_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sum_bytes));
  const int iters = B.max_iter > 1 ? B.max_iter : 1;
  const bool scan = B.d <= kScanCols * kScanThreads;
  for (int it = 0; it < iters; ++it) {
    centroid_norms_kernel<<<ngrid, 128, 0, st>>>(B, 0);
    launch_assign(0);
    if (scan) {
      scan_sums_kernel<<<dim3(B.k, B.problems), kScanThreads, 0, st>>>(B);
    } else {
      sort_kernel<<<B.problems, 1024, sort_bytes, st>>>(B);
      sums_kernel<<<B.problems * B.k, kSumThreads, sum_bytes, st>>>(B);
    }
    finalize_kernel<<<(B.problems + 63) / 64, 64, 0, st>>>(B, scan ? 1 : 0);
  }
  centroid_norms_kernel<<<ngrid, 128, 0, st>>>(B, 1);
  launch_assign(1);
  count_launch(1 + (scan ? 4 : 5) * iters + 2);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
