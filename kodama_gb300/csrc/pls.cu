// PLS-LDA on the device: the float32 SIMPLS + LDA path of the reference
// (plscv.cpp) restated operation for operation, so that predictions are
// bit-identical to PLSLDACV_CPU / PLSLDAPredict_CPU.
//
//   fold statistics   train_center_scale_float        plscv.cpp:669-698
//   standardisation   subset_scale_float              plscv.cpp:409-424
//   fold Gram         densef_gram                     plscv.cpp:436-447
//   cross-product     centered_label_crossprod_*      plscv.cpp:700-731
//   SIMPLS weights    fit_pls_components_from_crossprod_float  plscv.cpp:816-955
//   LDA               fit_predict_pls_lda_streamed_cpu_float   plscv.cpp:1544-1608
//                     fit_lda_from_score_statistics_float      plscv.cpp:1419-1487
//                     cholesky_solve_float                     plscv.cpp:1379-1412
//
// Every float accumulation of the reference is a sequential chain in a fixed
// order (rows ascending, features ascending, classes ascending); each chain
// here runs in one thread in that order, and the parallelism is across
// chains: slices x features x classes x rows.  Double accumulators of the
// reference (dot_float, mat_vec_float, t_mat_vec_float, power_norm2_float)
// sum exact float products, so each step is one fma(a, b, acc) in double.
// Built with --fmad=false: no other multiply-add is fused.
#include "pls.cuh"
#include "launch_count.cuh"

#include <float.h>
#include <math.h>

namespace kgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEvalThreads = 512;
constexpr int kEvalWarps = kEvalThreads / 32;

// ---------------------------------------------------------------------------
// Preparation (label independent)
// ---------------------------------------------------------------------------

// train_center_scale_float: one thread per (slice, column).
__global__ void stats_kernel(PlsPrepArgs a) {
  const int s = blockIdx.x, r = s / a.F;
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= a.p) return;
  const float* X = a.X + static_cast<size_t>(r) * a.L * a.p;
  const int b = a.train_off[s], e = a.train_off[s + 1], nt = e - b;
  const int* rows = a.train_idx;
  float m = 0.0f;
  if (a.center) {
    for (int t = b; t < e; t += 8) {
      float v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = t + q < e ? X[static_cast<size_t>(rows[t + q]) * a.p + j] : 0.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (t + q < e) m = __fadd_rn(m, v[q]);
    }
    const float inv = nt == 0 ? 0.0f : __fdiv_rn(1.0f, static_cast<float>(nt));
    m = __fmul_rn(m, inv);
  }
  float sd = 1.0f;
  if (a.scale) {
    float acc = 1.0f;  // the reference's scale vector starts at 1
    for (int t = b; t < e; t += 8) {
      float v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = t + q < e ? X[static_cast<size_t>(rows[t + q]) * a.p + j] : 0.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        if (t + q < e) {
          const float d = __fsub_rn(v[q], m);
          acc = __fadd_rn(acc, __fmul_rn(d, d));
        }
      }
    }
    // std::max(1.0f, float(rows.size() - 1)) with size_t arithmetic
    const float den1 = static_cast<float>(static_cast<unsigned long long>(nt) - 1ull);
    const float den = 1.0f < den1 ? den1 : 1.0f;
    const float q = __fsqrt_rn(__fdiv_rn(acc, den));
    sd = (q > 0.0f && isfinite(q)) ? q : 1.0f;
  }
  a.mean[static_cast<size_t>(s) * a.p + j] = m;
  a.sdev[static_cast<size_t>(s) * a.p + j] = sd;
}

// subset_scale_float for every row of every slice (and, in predict mode, for
// the rows to predict).
__global__ void standardize_kernel(PlsPrepArgs a) {
  const size_t per = static_cast<size_t>(a.L) * a.p;
  const size_t total = static_cast<size_t>(a.problems) * a.F * per;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t s = e / per, rem = e - s * per;
    const int j = static_cast<int>(rem % a.p);
    const size_t r = s / a.F;
    const float x = a.X[r * per + rem];
    a.Z[e] = __fdiv_rn(__fsub_rn(x, a.mean[s * a.p + j]), a.sdev[s * a.p + j]);
  }
  if (a.Xv == nullptr) return;
  const size_t pv = static_cast<size_t>(a.NV) * a.p;
  const size_t tv = static_cast<size_t>(a.problems) * pv;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < tv;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t r = e / pv;
    const int j = static_cast<int>((e - r * pv) % a.p);
    const size_t s = r * a.F;
    a.Zv[e] = __fdiv_rn(__fsub_rn(a.Xv[e], a.mean[s * a.p + j]), a.sdev[s * a.p + j]);
  }
}

// Column sums of the standardised training rows in row order (the x_sum of
// the cross-product, label independent).
__global__ void xsum_kernel(PlsPrepArgs a) {
  const int s = blockIdx.x;
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= a.p) return;
  const float* Zs = a.Z + static_cast<size_t>(s) * a.L * a.p;
  const int b = a.train_off[s], e = a.train_off[s + 1];
  float acc = 0.0f;
  for (int t = b; t < e; t += 8) {
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = t + q < e ? Zs[static_cast<size_t>(a.train_idx[t + q]) * a.p + j] : 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (t + q < e) acc = __fadd_rn(acc, v[q]);
  }
  a.xsum[static_cast<size_t>(s) * a.p + j] = acc;
}

// densef_gram: G(j, k) = sum over training rows (ascending) of z_j * z_k, one
// 32 x 32 tile of the lower triangle per CTA (blockIdx.y enumerates tiles),
// written to both triangles.
__global__ void __launch_bounds__(1024) gram_kernel(PlsPrepArgs a, const uint8_t* want) {
  const int s = blockIdx.x;
  if (!want[s]) return;
  // tile index -> (jb, kb), kb <= jb
  int tile = blockIdx.y, jb = 0;
  while (tile > jb) {
    tile -= jb + 1;
    ++jb;
  }
  const int kb = tile;
  __shared__ float zj[32][33];
  __shared__ float zk[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int J = jb * 32 + ty, K = kb * 32 + tx;
  const float* Zs = a.Z + static_cast<size_t>(s) * a.L * a.p;
  const int b = a.train_off[s], e = a.train_off[s + 1];
  float acc = 0.0f;
  for (int t0 = b; t0 < e; t0 += 32) {
    const int t = t0 + ty;
    const int row = t < e ? a.train_idx[t] : -1;
    const int cj = jb * 32 + tx, ck = kb * 32 + tx;
    zj[ty][tx] = (row >= 0 && cj < a.p) ? Zs[static_cast<size_t>(row) * a.p + cj] : 0.0f;
    zk[ty][tx] = (row >= 0 && ck < a.p) ? Zs[static_cast<size_t>(row) * a.p + ck] : 0.0f;
    __syncthreads();
    const int cnt = min(32, e - t0);
    for (int q = 0; q < cnt; ++q) acc = __fadd_rn(acc, __fmul_rn(zj[q][ty], zk[q][tx]));
    __syncthreads();
  }
  if (J < a.p && K < a.p && K <= J) {
    float* G = a.gram + static_cast<size_t>(s) * a.p * a.p;
    G[static_cast<size_t>(J) * a.p + K] = acc;
    G[static_cast<size_t>(K) * a.p + J] = acc;
  }
}

// ---------------------------------------------------------------------------
// Evaluation: one CTA per slice
// ---------------------------------------------------------------------------

struct EvalShared {
  int m, nt, maxr, fitted, nc, stop, best, lab;
  float rn, inv;
};

__device__ __forceinline__ float power_norm2(double sum) {
  if (!isfinite(sum) || sum < 0.0) return INFINITY;
  if (sum <= static_cast<double>(FLT_MAX)) return __fsqrt_rn(__double2float_rn(sum));
  return __double2float_rn(__dsqrt_rn(sum));
}

// Block-wide: out[c] = float(sum_j S[j + c*p] * w[j]) (double chain over j).
__device__ void t_mat_vec(const float* S, int p, int m, const float* w, float* out) {
  for (int c = threadIdx.x; c < m; c += kEvalThreads) {
    const float* col = S + static_cast<size_t>(c) * p;
    double acc = 0.0;
    for (int j = 0; j < p; ++j) acc = fma(static_cast<double>(col[j]), static_cast<double>(w[j]), acc);
    out[c] = __double2float_rn(acc);
  }
}

// Block-wide: out[j] = float(sum_c S[j + c*p] * t[c]) (double chain over c).
__device__ void mat_vec(const float* S, int p, int m, const float* t, float* out) {
  for (int j = threadIdx.x; j < p; j += kEvalThreads) {
    double acc = 0.0;
    for (int c = 0; c < m; ++c)
      acc = fma(static_cast<double>(S[j + static_cast<size_t>(c) * p]), static_cast<double>(t[c]), acc);
    out[j] = __double2float_rn(acc);
  }
}

__device__ void power_refresh(const float* S, int p, int m, float* w, float* tv) {
  for (int it = 0; it < 2; ++it) {
    t_mat_vec(S, p, m, w, tv);
    __syncthreads();
    mat_vec(S, p, m, tv, w);
    __syncthreads();
  }
}

// Serial double sum of squares (dot_float(x, x) and power_norm2_float).
__device__ double sumsq_serial(const float* x, int n) {
  double acc = 0.0;
  for (int i = 0; i < n; ++i) acc = fma(static_cast<double>(x[i]), static_cast<double>(x[i]), acc);
  return acc;
}

// cholesky_solve_float on an n x n matrix A (row-major) for rhs n x m; one thread.
__device__ bool chol_solve(const float* A, int n, const float* rhs, int m, float* Lc, float* sol) {
  for (int row = 0; row < n; ++row) {
    for (int col = 0; col <= row; ++col) {
      float v = A[row * n + col];
      for (int k = 0; k < col; ++k) v = __fsub_rn(v, __fmul_rn(Lc[row * n + k], Lc[col * n + k]));
      if (row == col) {
        if (!isfinite(v) || v <= 0.0f) return false;
        Lc[row * n + col] = __fsqrt_rn(v);
      } else {
        const float d = Lc[col * n + col];
        if (!isfinite(d) || d <= 0.0f) return false;
        Lc[row * n + col] = __fdiv_rn(v, d);
      }
    }
  }
  for (int i = 0; i < n * m; ++i) sol[i] = rhs[i];
  for (int c = 0; c < m; ++c) {
    for (int row = 0; row < n; ++row) {
      float v = sol[row * m + c];
      for (int k = 0; k < row; ++k) v = __fsub_rn(v, __fmul_rn(Lc[row * n + k], sol[k * m + c]));
      sol[row * m + c] = __fdiv_rn(v, Lc[row * n + row]);
    }
    for (int row = n - 1; row >= 0; --row) {
      float v = sol[row * m + c];
      for (int k = row + 1; k < n; ++k) v = __fsub_rn(v, __fmul_rn(Lc[k * n + row], sol[k * m + c]));
      sol[row * m + c] = __fdiv_rn(v, Lc[row * n + row]);
    }
  }
  return true;
}

// Score of one standardised row for component q: sum over features in order.
__device__ __forceinline__ float row_score(const float* z, const float* W, int ldw, int p, int q) {
  float acc = 0.0f;
  for (int j = 0; j < p; ++j) acc = __fadd_rn(acc, __fmul_rn(z[j], W[static_cast<size_t>(j) * ldw + q]));
  return acc;
}

__global__ void __launch_bounds__(kEvalThreads) eval_kernel(PlsEvalArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int s = blockIdx.x, r = s / a.F, f = s % a.F;
  const int p = a.p, L = a.L, C = a.C0max, NCm = a.requested;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  EvalShared& sh = *reinterpret_cast<EvalShared*>(smem);
  size_t off = 64;
  auto carve = [&](size_t bytes) {
    unsigned char* q = smem + off;
    off += (bytes + 15) / 16 * 16;
    return q;
  };
  int* cnt = reinterpret_cast<int*>(carve(sizeof(int) * C));
  int* klist = reinterpret_cast<int*>(carve(sizeof(int) * C));
  float* w = reinterpret_cast<float*>(carve(sizeof(float) * p));
  float* ld = reinterpret_cast<float*>(carve(sizeof(float) * p));
  float* pw = reinterpret_cast<float*>(carve(sizeof(float) * p));
  float* tv = reinterpret_cast<float*>(carve(sizeof(float) * C));
  float* cs = reinterpret_cast<float*>(carve(sizeof(float) * C * NCm));
  float* cp = reinterpret_cast<float*>(carve(sizeof(float) * NCm * NCm));
  float* pooled = reinterpret_cast<float*>(carve(sizeof(float) * NCm * NCm));
  float* cov = reinterpret_cast<float*>(carve(sizeof(float) * NCm * NCm));
  float* Lc = reinterpret_cast<float*>(carve(sizeof(float) * NCm * NCm));
  float* rhs = reinterpret_cast<float*>(carve(sizeof(float) * NCm * C));
  float* sol = reinterpret_cast<float*>(carve(sizeof(float) * NCm * C));
  float* lin = reinterpret_cast<float*>(carve(sizeof(float) * C * NCm));
  float* cst = reinterpret_cast<float*>(carve(sizeof(float) * C));

  const uint16_t* lab = a.labels + static_cast<size_t>(r) * L;
  const int* coff = a.class_off + static_cast<size_t>(r) * (C + 1);
  const uint16_t* crow = a.class_rows + static_cast<size_t>(r) * L;
  const uint8_t* fold = a.predict_mode ? nullptr : a.folds + static_cast<size_t>(r) * L;
  const float* Zs = a.Z + static_cast<size_t>(s) * L * p;
  const int tb = a.train_off[s], te = a.train_off[s + 1];
  const int nv = a.predict_mode ? a.NV : a.val_off[s + 1] - a.val_off[s];
  const int* vidx = a.predict_mode ? nullptr : a.val_idx + a.val_off[s];
  uint16_t* pred = a.pred + static_cast<size_t>(r) * (a.predict_mode ? a.NV : L);
  auto val_row = [&](int v) -> const float* {
    return a.predict_mode ? a.Zv + (static_cast<size_t>(r) * a.NV + v) * p : Zs + static_cast<size_t>(vidx[v]) * p;
  };
  auto val_out = [&](int v) -> int { return a.predict_mode ? v : vidx[v]; };

  // --- fold classes: codes with training rows, ascending -------------------
  for (int c = threadIdx.x; c < C; c += kEvalThreads) cnt[c] = coff[c + 1] - coff[c];
  __syncthreads();
  if (!a.predict_mode)
    for (int v = threadIdx.x; v < nv; v += kEvalThreads) atomicSub(&cnt[lab[vidx[v]]], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = 0;
    for (int c = 0; c < C; ++c)
      if (cnt[c] > 0) klist[m++] = c;
    sh.m = m;
    sh.nt = te - tb;
    a.status[s] = 0;
  }
  __syncthreads();
  const int m = sh.m, nt = sh.nt;
  if (m <= 1) {
    // one training class: it is every prediction (labels.front() without one)
    const int only = m == 1 ? klist[0] : lab[0];
    for (int v = threadIdx.x; v < nv; v += kEvalThreads) pred[val_out(v)] = static_cast<uint16_t>(only);
    if (threadIdx.x == 0) a.eval_comp[s] = 1;
    return;
  }

  // --- label cross-product S (p x m), column k = fold class k -------------
  float* S = a.s_scr + static_cast<size_t>(s) * p * C;
  {
    const int JB = (p + 31) / 32;
    const float inv_n = nt > 0 ? __fdiv_rn(1.0f, static_cast<float>(nt)) : 0.0f;
    for (int it = warp; it < m * JB; it += kEvalWarps) {
      const int k = it / JB, j = (it % JB) * 32 + lane;
      const int code = klist[k];
      const int b = coff[code], e = coff[code + 1];
      float acc = 0.0f;
      for (int base = b; base < e; base += 32) {
        const int row = base + lane < e ? crow[base + lane] : -1;
        const bool ok = row >= 0 && (fold == nullptr || fold[row] != f);
        const unsigned msk = __ballot_sync(kFull, ok);
        float v[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int rq = __shfl_sync(kFull, row, q);
          v[q] = (((msk >> q) & 1u) && j < p) ? Zs[static_cast<size_t>(rq) * p + j] : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 32; ++q)
          if ((msk >> q) & 1u) acc = __fadd_rn(acc, v[q]);
      }
      if (j < p) {
        const float y_mean = __fmul_rn(static_cast<float>(cnt[code]), inv_n);
        S[j + static_cast<size_t>(k) * p] =
            __fsub_rn(acc, __fmul_rn(y_mean, a.xsum[static_cast<size_t>(s) * p + j]));
      }
    }
  }
  __syncthreads();

  // --- SIMPLS weights ------------------------------------------------------
  const int maxr = min(min(a.max_components, p), max(1, nt - 1));
  const int ldw = a.max_components;
  float* Wg = a.W + static_cast<size_t>(s) * p * ldw;
  float* Vg = a.V + static_cast<size_t>(s) * p * ldw;
  const bool gram = a.gram != nullptr && a.use_gram[s];
  const float* G = gram ? a.gram + static_cast<size_t>(s) * p * p : nullptr;
  float* scv = a.sc + static_cast<size_t>(s) * L;
  int fitted = 0;
  for (int comp = 0; comp < maxr; ++comp) {
    for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = comp == 0 ? a.w0[j] : pw[j];
    __syncthreads();
    power_refresh(S, p, m, w, tv);
    if (threadIdx.x == 0) {
      float rn = power_norm2(sumsq_serial(w, p));
      int best = -1;
      if (comp == 0 && !(isfinite(rn) && rn > 1.0e-10f)) {
        // retry on the response column with the largest norm
        double bn = 0.0;
        for (int k = 0; k < m; ++k) {
          const double ns = sumsq_serial(S + static_cast<size_t>(k) * p, p);
          if (isfinite(ns) && ns > bn) {
            bn = ns;
            best = k;
          }
        }
        if (!(best >= 0 && bn > 1.0e-20)) best = -1;
      }
      sh.rn = rn;
      sh.best = best;
    }
    __syncthreads();
    if (sh.best >= 0) {
      const int best = sh.best;
      for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = S[j + static_cast<size_t>(best) * p];
      __syncthreads();
      power_refresh(S, p, m, w, tv);
      if (threadIdx.x == 0) sh.rn = power_norm2(sumsq_serial(w, p));
      __syncthreads();
    }
    const float rn = sh.rn;
    if (!(isfinite(rn) && rn > 1.0e-10f)) break;
    for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = __fdiv_rn(w[j], rn);
    __syncthreads();
    if (gram) {
      for (int i = threadIdx.x; i < p; i += kEvalThreads) {
        double acc = 0.0;
        for (int j = 0; j < p; ++j)
          acc = fma(static_cast<double>(G[static_cast<size_t>(j) * p + i]), static_cast<double>(w[j]), acc);
        ld[i] = __double2float_rn(acc);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double acc = 0.0;
        for (int j = 0; j < p; ++j) acc = fma(static_cast<double>(w[j]), static_cast<double>(ld[j]), acc);
        const float sns = __double2float_rn(acc);
        sh.stop = !(isfinite(sns) && sns > 1.0e-20f);
        sh.inv = sh.stop ? 0.0f : __fdiv_rn(1.0f, __fsqrt_rn(sns));
      }
      __syncthreads();
      if (sh.stop) break;
      const float inv = sh.inv;
      for (int j = threadIdx.x; j < p; j += kEvalThreads) {
        w[j] = __fmul_rn(w[j], inv);
        ld[j] = __fmul_rn(ld[j], inv);
      }
      __syncthreads();
    } else {
      // scores of the training rows, their norm, loading = X^T scores
      for (int t = threadIdx.x; t < nt; t += kEvalThreads) {
        const float* z = Zs + static_cast<size_t>(a.train_idx[tb + t]) * p;
        float acc = 0.0f;
        for (int j = 0; j < p; ++j) acc = __fadd_rn(acc, __fmul_rn(z[j], w[j]));
        scv[t] = acc;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        const float d = __double2float_rn(sumsq_serial(scv, nt));
        const float sn = __fsqrt_rn(0.0f < d ? d : 0.0f);
        sh.stop = !(isfinite(sn) && sn > 1.0e-10f);
        sh.inv = sh.stop ? 0.0f : __fdiv_rn(1.0f, sn);
      }
      __syncthreads();
      if (sh.stop) break;
      const float inv = sh.inv;
      for (int t = threadIdx.x; t < nt; t += kEvalThreads) scv[t] = __fmul_rn(scv[t], inv);
      for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = __fmul_rn(w[j], inv);
      __syncthreads();
      for (int j = threadIdx.x; j < p; j += kEvalThreads) {
        double acc = 0.0;
        for (int t = 0; t < nt; t += 8) {
          float zv[8], sv[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const bool in = t + q < nt;
            zv[q] = in ? Zs[static_cast<size_t>(a.train_idx[tb + t + q]) * p + j] : 0.0f;
            sv[q] = in ? scv[t + q] : 0.0f;
          }
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (t + q < nt) acc = fma(static_cast<double>(zv[q]), static_cast<double>(sv[q]), acc);
        }
        ld[j] = __double2float_rn(acc);
      }
      __syncthreads();
    }
    for (int j = threadIdx.x; j < p; j += kEvalThreads) pw[j] = w[j];
    // Gram-Schmidt against the previous loadings
    for (int q = 0; q < comp; ++q) {
      if (threadIdx.x == 0) {
        float proj = 0.0f;
        for (int j = 0; j < p; ++j) proj = __fadd_rn(proj, __fmul_rn(Vg[static_cast<size_t>(j) * ldw + q], ld[j]));
        sh.inv = proj;
      }
      __syncthreads();
      const float proj = sh.inv;
      for (int j = threadIdx.x; j < p; j += kEvalThreads)
        ld[j] = __fsub_rn(ld[j], __fmul_rn(proj, Vg[static_cast<size_t>(j) * ldw + q]));
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const float d = __double2float_rn(sumsq_serial(ld, p));
      const float ln = __fsqrt_rn(0.0f < d ? d : 0.0f);
      sh.stop = !(isfinite(ln) && ln > 1.0e-10f);
      sh.inv = ln;
    }
    __syncthreads();
    if (sh.stop) break;
    const float ln = sh.inv;
    for (int j = threadIdx.x; j < p; j += kEvalThreads) {
      ld[j] = __fdiv_rn(ld[j], ln);
      Wg[static_cast<size_t>(j) * ldw + comp] = w[j];
      Vg[static_cast<size_t>(j) * ldw + comp] = ld[j];
    }
    __syncthreads();
    // deflate the cross-product
    for (int k = threadIdx.x; k < m; k += kEvalThreads) {
      float acc = 0.0f;
      for (int j = 0; j < p; ++j) acc = __fadd_rn(acc, __fmul_rn(ld[j], S[j + static_cast<size_t>(k) * p]));
      tv[k] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < p * m; e += kEvalThreads) {
      const int j = e % p, k = e / p;
      S[e] = __fsub_rn(S[e], __fmul_rn(ld[j], tv[k]));
    }
    __syncthreads();
    fitted = comp + 1;
  }

  if (fitted < 1) {
    if (a.predict_mode) {
      if (threadIdx.x == 0) a.status[s] = 1;
      return;
    }
    // DegeneratePLSFit: the most frequent training class, smallest on ties
    if (threadIdx.x == 0) {
      int bl = klist[0], bc = -1;
      for (int k = 0; k < m; ++k) {
        if (cnt[klist[k]] > bc) {
          bc = cnt[klist[k]];
          bl = klist[k];
        }
      }
      sh.lab = bl;
      a.eval_comp[s] = 1;
    }
    __syncthreads();
    for (int v = threadIdx.x; v < nv; v += kEvalThreads) pred[val_out(v)] = static_cast<uint16_t>(sh.lab);
    return;
  }

  // --- LDA on the first nc score columns -----------------------------------
  const int nc = a.predict_mode ? fitted : min(a.requested, fitted);
  float* Ts = a.T + static_cast<size_t>(s) * L * NCm;  // by row: Ts[row * nc + q]
  for (int t = threadIdx.x; t < nt; t += kEvalThreads) {
    const int row = a.train_idx[tb + t];
    const float* z = Zs + static_cast<size_t>(row) * p;
    for (int q = 0; q < nc; ++q) Ts[static_cast<size_t>(row) * nc + q] = row_score(z, Wg, ldw, p, q);
  }
  __syncthreads();
  // class sums (rows of each class in order) and score cross-products (all
  // training rows in order): independent chains
  const int ncs = m * nc, ncp = nc * (nc + 1) / 2;
  for (int it = threadIdx.x; it < ncs + ncp; it += kEvalThreads) {
    if (it < ncs) {
      const int k = it / nc, q = it % nc;
      const int code = klist[k];
      float acc = 0.0f;
      for (int i = coff[code]; i < coff[code + 1]; ++i) {
        const int row = crow[i];
        if (fold != nullptr && fold[row] == f) continue;
        acc = __fadd_rn(acc, Ts[static_cast<size_t>(row) * nc + q]);
      }
      cs[k * nc + q] = acc;
    } else {
      int pr = it - ncs, rr = 0;
      while (pr > rr) {
        pr -= rr + 1;
        ++rr;
      }
      const int col = pr;
      float acc = 0.0f;
      for (int t = tb; t < te; t += 8) {
        float x0[8], x1[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int row = t + q < te ? a.train_idx[t + q] : 0;
          x0[q] = Ts[static_cast<size_t>(row) * nc + rr];
          x1[q] = Ts[static_cast<size_t>(row) * nc + col];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (t + q < te) acc = __fadd_rn(acc, __fmul_rn(x0[q], x1[q]));
      }
      cp[rr * nc + col] = acc;
      cp[col * nc + rr] = acc;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < m; ++k) {
      const int c = cnt[klist[k]];
      const float inv = c > 0 ? __fdiv_rn(1.0f, static_cast<float>(c)) : 0.0f;
      for (int q = 0; q < nc; ++q) cs[k * nc + q] = __fmul_rn(cs[k * nc + q], inv);
    }
    const float df = static_cast<float>(max(1, nt - m));
    float trace = 0.0f;
    for (int rr = 0; rr < nc; ++rr) {
      for (int col = 0; col <= rr; ++col) {
        float between = 0.0f;
        for (int k = 0; k < m; ++k)
          between = __fadd_rn(between, __fmul_rn(__fmul_rn(static_cast<float>(cnt[klist[k]]), cs[k * nc + rr]),
                                                 cs[k * nc + col]));
        const float cv = __fdiv_rn(__fsub_rn(cp[rr * nc + col], between), df);
        pooled[rr * nc + col] = cv;
        pooled[col * nc + rr] = cv;
      }
      trace = __fadd_rn(trace, pooled[rr * nc + rr]);
    }
    for (int k = 0; k < m; ++k)
      for (int q = 0; q < nc; ++q) rhs[q * m + k] = cs[k * nc + q];
    const float ridge_scale =
        (isfinite(trace) && trace > 0.0f) ? __fdiv_rn(trace, static_cast<float>(max(1, nc))) : 1.0f;
    const float grid[6] = {1e-8f, 1e-6f, 1e-5f, 1e-4f, 1e-3f, 1e-2f};
    bool ok = false;
    for (int g = 0; g < 6 && !ok; ++g) {
      const float lambda = __fmul_rn(grid[g], ridge_scale);
      for (int i = 0; i < nc * nc; ++i) cov[i] = pooled[i];
      for (int q = 0; q < nc; ++q) cov[q * nc + q] = __fadd_rn(cov[q * nc + q], lambda);
      ok = chol_solve(cov, nc, rhs, m, Lc, sol);
    }
    if (!ok) {
      a.status[s] = 2;
      sh.stop = 1;
    } else {
      const float* lp = a.logprior + a.lp_off[s];
      for (int k = 0; k < m; ++k) {
        float dot_mu = 0.0f;
        for (int q = 0; q < nc; ++q) {
          lin[k * nc + q] = sol[q * m + k];
          dot_mu = __fadd_rn(dot_mu, __fmul_rn(cs[k * nc + q], lin[k * nc + q]));
        }
        cst[k] = __fadd_rn(__fmul_rn(-0.5f, dot_mu), lp[cnt[klist[k]]]);
      }
      sh.stop = 0;
    }
    a.eval_comp[s] = nc;
  }
  __syncthreads();
  if (sh.stop) return;
  for (int v = threadIdx.x; v < nv; v += kEvalThreads) {
    const float* z = val_row(v);
    float sr[16];
    int best = 0;
    float bs = -INFINITY;
    // scores in chunks of 16 components (one chain per component)
    for (int k = 0; k < m; ++k) {
      float sc = cst[k];
      for (int q0 = 0; q0 < nc; q0 += 16) {
        const int cntq = min(16, nc - q0);
        if (k == 0 || nc > 16) {
          for (int q = 0; q < cntq; ++q) sr[q] = row_score(z, Wg, ldw, p, q0 + q);
        }
        for (int q = 0; q < cntq; ++q) sc = __fadd_rn(sc, __fmul_rn(sr[q], lin[k * nc + q0 + q]));
      }
      if (sc > bs) {
        bs = sc;
        best = k;
      }
    }
    pred[val_out(v)] = static_cast<uint16_t>(klist[best]);
  }
}

__global__ void gather_kernel(const float* __restrict__ x, int p, const int* __restrict__ rows, size_t nrows,
                              float* __restrict__ out) {
  const size_t total = nrows * p;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t i = e / p;
    out[e] = x[static_cast<size_t>(rows[i]) * p + (e - i * p)];
  }
}

__global__ void assemble_kernel(int problems, int n, int L, int NV, const int* land, const int* test_rows,
                                const uint16_t* clbest, const uint16_t* proj, const int* c2l, int C0max, int* res) {
  const size_t per = static_cast<size_t>(L) + NV;
  const size_t total = static_cast<size_t>(problems) * per;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t r = e / per, i = e - r * per;
    const int* map = c2l + r * C0max;
    if (i < static_cast<size_t>(L)) {
      res[r * n + land[r * L + i]] = map[clbest[r * L + i]];
    } else {
      const size_t t = i - L;
      res[r * n + test_rows[r * NV + t]] = map[proj[r * NV + t]];
    }
  }
}

}  // namespace

int pls_gather_rows(const float* x, int p, const int* rows, size_t nrows, float* out, cudaStream_t st) {
  gather_kernel<<<4 * 152, 256, 0, st>>>(x, p, rows, nrows, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int pls_assemble_result(int problems, int n, int L, int NV, const int* land, const int* test_rows,
                        const uint16_t* clbest, const uint16_t* proj, const int* code2label, int C0max, int* res,
                        cudaStream_t st) {
  assemble_kernel<<<2 * 152, 256, 0, st>>>(problems, n, L, NV, land, test_rows, clbest, proj, code2label, C0max,
                                           res);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int pls_prepare(const PlsPrepArgs& a, cudaStream_t st) {
  const int S = a.problems * a.F;
  dim3 g1(S, (a.p + 127) / 128);
  stats_kernel<<<g1, 128, 0, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return static_cast<int>(e);
  standardize_kernel<<<4 * 152, 256, 0, st>>>(a);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return static_cast<int>(e);
  xsum_kernel<<<g1, 128, 0, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int pls_build_gram(const PlsPrepArgs& a, const uint8_t* want, cudaStream_t st) {
  const int S = a.problems * a.F;
  const int JB = (a.p + 31) / 32;
  dim3 grid(S, JB * (JB + 1) / 2);
  gram_kernel<<<grid, dim3(32, 32), 0, st>>>(a, want);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

size_t pls_eval_smem(int p, int C0max, int requested) {
  auto al = [](size_t v) { return (v + 15) / 16 * 16; };
  const size_t C = static_cast<size_t>(C0max), N = static_cast<size_t>(requested);
  size_t b = 64;
  b += 2 * al(sizeof(int) * C);
  b += 3 * al(sizeof(float) * p) + al(sizeof(float) * C);
  b += al(sizeof(float) * C * N) + 4 * al(sizeof(float) * N * N) + 2 * al(sizeof(float) * N * C);
  b += al(sizeof(float) * C * N) + al(sizeof(float) * C);
  return b;
}

int pls_evaluate(const PlsEvalArgs& a, cudaStream_t st) {
  const int S = a.problems * a.F;
  const size_t smem = pls_eval_smem(a.p, a.C0max, a.requested);
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
  }
  eval_kernel<<<S, kEvalThreads, smem, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
