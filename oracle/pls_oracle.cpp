// PLS-LDA cross-validation: CPU restatement (the oracle) of the reference's
// float32 SIMPLS + LDA path in plscv.cpp.
//
// TEST INFRASTRUCTURE ONLY.  This file is part of the checker for the CUDA
// path in kodama_gb300/csrc; the product never loads it.
//
// Arithmetic follows the reference operation for operation: float32 values,
// float32 accumulators wherever the reference accumulates in float (in the
// order of its loops), double accumulators where it uses double (dot_float,
// mat_vec_float, t_mat_vec_float, power_norm2_float).  The random start vector
// of SIMPLS and logf() of the LDA priors come from the same libstdc++/libm
// calls as the reference's.  Built with -ffp-contract=off.

#include "pls_oracle.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>
#include <numeric>
#include <random>
#include <stdexcept>

namespace orc {
namespace {

using Vec = std::vector<float>;

// train_center_scale_float (plscv.cpp:669-698): float column sums in row
// order; the squared-deviation sum starts from 1.0f as in the reference.
void center_scale(const float* x, int p, const std::vector<int>& rows, bool center, bool scale, Vec& mean, Vec& sc) {
  mean.assign(static_cast<size_t>(p), 0.0f);
  sc.assign(static_cast<size_t>(p), 1.0f);
  if (center) {
    for (int r : rows)
      for (int j = 0; j < p; ++j) mean[j] += x[static_cast<size_t>(r) * p + j];
    const float inv = rows.empty() ? 0.0f : 1.0f / static_cast<float>(rows.size());
    for (float& v : mean) v *= inv;
  }
  if (scale) {
    for (int r : rows) {
      for (int j = 0; j < p; ++j) {
        const float d = x[static_cast<size_t>(r) * p + j] - mean[j];
        sc[j] += d * d;
      }
    }
    for (int j = 0; j < p; ++j) {
      const float s = std::sqrt(sc[j] / std::max(1.0f, static_cast<float>(rows.size() - 1)));
      sc[j] = s > 0.0f && std::isfinite(s) ? s : 1.0f;
    }
  }
}

// subset_scale_float (plscv.cpp:409-424)
Vec standardize(const float* x, int p, const std::vector<int>& rows, const Vec& mean, const Vec& sc) {
  Vec out(rows.size() * static_cast<size_t>(p));
  for (size_t i = 0; i < rows.size(); ++i)
    for (int j = 0; j < p; ++j)
      out[i * p + j] = (x[static_cast<size_t>(rows[i]) * p + j] - mean[j]) / sc[j];
  return out;
}

// densef_gram (plscv.cpp:436-447): lower triangle, float sums over samples.
Vec gram_of(const Vec& z, int n, int p) {
  // Each entry is its own float chain over the samples in order, as in
  // densef_gram.  The samples are walked in chunks that stay in cache, and
  // within a chunk blocks of 4 x 8 entries advance side by side; an entry's
  // partial sum is carried from chunk to chunk, so its order is unchanged.
  Vec g(static_cast<size_t>(p) * p, 0.0f);
  constexpr int BR = 4, BC = 8, CHUNK = 256;
  for (int s0 = 0; s0 < n; s0 += CHUNK) {
    const int s1 = std::min(n, s0 + CHUNK);
    for (int r0 = 0; r0 < p; r0 += BR) {
      for (int c0 = 0; c0 < r0 + BR && c0 < p; c0 += BC) {
        float acc[BR][BC];
        for (int i = 0; i < BR; ++i)
          for (int j = 0; j < BC; ++j) {
            const int row = std::min(r0 + i, p - 1), col = std::min(c0 + j, p - 1);
            acc[i][j] = g[static_cast<size_t>(row) * p + col];
          }
        if (r0 + BR <= p && c0 + BC <= p) {
          for (int s = s0; s < s1; ++s) {
            const float* zr = z.data() + static_cast<size_t>(s) * p;
            for (int i = 0; i < BR; ++i) {
              const float a = zr[r0 + i];
              for (int j = 0; j < BC; ++j) {
                const float prod = a * zr[c0 + j];
                acc[i][j] = acc[i][j] + prod;
              }
            }
          }
        } else {
          for (int s = s0; s < s1; ++s) {
            const float* zr = z.data() + static_cast<size_t>(s) * p;
            for (int i = 0; i < BR && r0 + i < p; ++i)
              for (int j = 0; j < BC && c0 + j < p; ++j) {
                const float prod = zr[r0 + i] * zr[c0 + j];
                acc[i][j] = acc[i][j] + prod;
              }
          }
        }
        for (int i = 0; i < BR && r0 + i < p; ++i)
          for (int j = 0; j < BC && c0 + j < p; ++j)
            g[static_cast<size_t>(r0 + i) * p + c0 + j] = acc[i][j];
      }
    }
  }
  // mirror the lower triangle (row >= col), as densef_gram stores both halves
  for (int row = 0; row < p; ++row)
    for (int col = 0; col < row; ++col) g[static_cast<size_t>(col) * p + row] = g[static_cast<size_t>(row) * p + col];
  return g;
}

// centered_label_crossprod_colmajor_float (plscv.cpp:700-731): s[j + c*p].
Vec crossprod(const Vec& z, int n, int p, const std::vector<int>& code, int m) {
  Vec s(static_cast<size_t>(p) * m, 0.0f), xs(static_cast<size_t>(p), 0.0f), counts(static_cast<size_t>(m), 0.0f);
  for (int i = 0; i < n; ++i) counts[code[i]] += 1.0f;
  for (int i = 0; i < n; ++i) {
    const int c = code[i];
    for (int j = 0; j < p; ++j) {
      const float v = z[static_cast<size_t>(i) * p + j];
      xs[j] += v;
      s[j + static_cast<size_t>(c) * p] += v;
    }
  }
  const float inv = n > 0 ? 1.0f / static_cast<float>(n) : 0.0f;
  for (int c = 0; c < m; ++c) {
    const float y_mean = counts[c] * inv;
    for (int j = 0; j < p; ++j) s[j + static_cast<size_t>(c) * p] -= y_mean * xs[j];
  }
  return s;
}

// dot_float / norm2_float / power_norm2_float (plscv.cpp:774-794)
float dot_d(const float* a, const float* b, int n) {
  double o = 0.0;
  for (int i = 0; i < n; ++i) o += static_cast<double>(a[i]) * static_cast<double>(b[i]);
  return static_cast<float>(o);
}

float norm2(const Vec& v) {
  return std::sqrt(std::max(0.0f, dot_d(v.data(), v.data(), static_cast<int>(v.size()))));
}

float power_norm2(const Vec& v) {
  double sum = 0.0;
  for (float x : v) sum += static_cast<double>(x) * static_cast<double>(x);
  if (!std::isfinite(sum) || sum < 0.0) return std::numeric_limits<float>::infinity();
  if (sum <= static_cast<double>(std::numeric_limits<float>::max())) return std::sqrt(static_cast<float>(sum));
  return static_cast<float>(std::sqrt(sum));
}

// The randomized start of the first component (plscv.cpp:833-838).
Vec normal_start(int p) {
  std::mt19937 gen(1u);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  Vec w(static_cast<size_t>(p));
  for (float& v : w) v = nd(gen);
  return w;
}

struct Fit {
  int rank = 0;
  Vec w;  // p x rank, weights(j, a) = w[j * rank + a]
};

// fit_pls_components_from_crossprod_float (plscv.cpp:816-955), the parts that
// determine the X weights.  Returns false for DegeneratePLSFit.
bool fit_pls(const Vec& z, int n, int p, Vec s, int m, int max_components, const Vec* gram, Fit& out) {
  const int max_rank = std::min({max_components, p, std::max(1, n - 1)});
  Vec W(static_cast<size_t>(p) * max_rank, 0.0f), V(static_cast<size_t>(p) * max_rank, 0.0f);
  Vec prev;
  int fitted = 0;
  auto tmv = [&](const Vec& w) {
    Vec o(static_cast<size_t>(m));
    for (int c = 0; c < m; ++c) {
      double acc = 0.0;
      for (int j = 0; j < p; ++j) acc += static_cast<double>(s[j + static_cast<size_t>(c) * p]) * static_cast<double>(w[j]);
      o[c] = static_cast<float>(acc);
    }
    return o;
  };
  auto mv = [&](const Vec& r) {
    Vec o(static_cast<size_t>(p));
    for (int j = 0; j < p; ++j) {
      double acc = 0.0;
      for (int c = 0; c < m; ++c) acc += static_cast<double>(s[j + static_cast<size_t>(c) * p]) * static_cast<double>(r[c]);
      o[j] = static_cast<float>(acc);
    }
    return o;
  };
  auto refresh = [&](Vec& w) {
    for (int it = 0; it < 2; ++it) w = mv(tmv(w));
  };
  for (int a = 0; a < max_rank; ++a) {
    Vec w = prev.empty() ? normal_start(p) : prev;
    refresh(w);
    float rn = power_norm2(w);
    if (prev.empty() && (!std::isfinite(rn) || rn <= 1.0e-10f)) {
      int best = -1;
      double bn = 0.0;
      for (int c = 0; c < m; ++c) {
        double ns = 0.0;
        for (int j = 0; j < p; ++j) {
          const double v = static_cast<double>(s[j + static_cast<size_t>(c) * p]);
          ns += v * v;
        }
        if (std::isfinite(ns) && ns > bn) {
          bn = ns;
          best = c;
        }
      }
      if (best >= 0 && bn > 1.0e-20) {
        for (int j = 0; j < p; ++j) w[j] = s[j + static_cast<size_t>(best) * p];
        refresh(w);
        rn = power_norm2(w);
      }
    }
    if (!std::isfinite(rn) || rn <= 1.0e-10f) break;
    for (float& v : w) v /= rn;
    Vec loading(static_cast<size_t>(p));
    if (gram != nullptr) {
      for (int i = 0; i < p; ++i) {
        double acc = 0.0;
        for (int j = 0; j < p; ++j)
          acc += static_cast<double>((*gram)[static_cast<size_t>(i) * p + j]) * static_cast<double>(w[j]);
        loading[i] = static_cast<float>(acc);
      }
      const float sns = dot_d(w.data(), loading.data(), p);
      if (!std::isfinite(sns) || sns <= 1.0e-20f) break;
      const float inv = 1.0f / std::sqrt(sns);
      for (float& v : w) v *= inv;
      for (float& v : loading) v *= inv;
    } else {
      Vec sc(static_cast<size_t>(n));
      for (int i = 0; i < n; ++i) {
        float v = 0.0f;
        for (int j = 0; j < p; ++j) v += z[static_cast<size_t>(i) * p + j] * w[j];
        sc[i] = v;
      }
      const float sn = norm2(sc);
      if (!std::isfinite(sn) || sn <= 1.0e-10f) break;
      const float inv = 1.0f / sn;
      for (float& v : sc) v *= inv;
      for (float& v : w) v *= inv;
      for (int j = 0; j < p; ++j) {
        double acc = 0.0;
        for (int i = 0; i < n; ++i) acc += static_cast<double>(z[static_cast<size_t>(i) * p + j]) * static_cast<double>(sc[i]);
        loading[j] = static_cast<float>(acc);
      }
    }
    prev = w;
    for (int q = 0; q < a; ++q) {
      float proj = 0.0f;
      for (int j = 0; j < p; ++j) proj += V[static_cast<size_t>(j) * max_rank + q] * loading[j];
      for (int j = 0; j < p; ++j) loading[j] -= proj * V[static_cast<size_t>(j) * max_rank + q];
    }
    const float ln = norm2(loading);
    if (!std::isfinite(ln) || ln <= 1.0e-10f) break;
    for (float& v : loading) v /= ln;
    for (int j = 0; j < p; ++j) {
      W[static_cast<size_t>(j) * max_rank + a] = w[j];
      V[static_cast<size_t>(j) * max_rank + a] = loading[j];
    }
    Vec vs(static_cast<size_t>(m));
    for (int c = 0; c < m; ++c) {
      float v = 0.0f;
      for (int j = 0; j < p; ++j) v += loading[j] * s[j + static_cast<size_t>(c) * p];
      vs[c] = v;
    }
    for (int j = 0; j < p; ++j)
      for (int c = 0; c < m; ++c) s[j + static_cast<size_t>(c) * p] -= loading[j] * vs[c];
    fitted = a + 1;
  }
  if (fitted < 1) return false;
  out.rank = fitted;
  out.w.assign(static_cast<size_t>(p) * fitted, 0.0f);
  for (int j = 0; j < p; ++j)
    for (int a = 0; a < fitted; ++a) out.w[static_cast<size_t>(j) * fitted + a] = W[static_cast<size_t>(j) * max_rank + a];
  return true;
}

// cholesky_solve_float (plscv.cpp:1379-1412); rhs / sol are n x m row-major.
bool chol_solve(const Vec& A, int n, const Vec& rhs, int m, Vec& sol) {
  Vec L(static_cast<size_t>(n) * n, 0.0f);
  for (int row = 0; row < n; ++row) {
    for (int col = 0; col <= row; ++col) {
      float v = A[static_cast<size_t>(row) * n + col];
      for (int k = 0; k < col; ++k) v -= L[static_cast<size_t>(row) * n + k] * L[static_cast<size_t>(col) * n + k];
      if (row == col) {
        if (!std::isfinite(v) || v <= 0.0f) return false;
        L[static_cast<size_t>(row) * n + col] = std::sqrt(v);
      } else {
        const float d = L[static_cast<size_t>(col) * n + col];
        if (!std::isfinite(d) || d <= 0.0f) return false;
        L[static_cast<size_t>(row) * n + col] = v / d;
      }
    }
  }
  sol = rhs;
  for (int c = 0; c < m; ++c) {
    for (int row = 0; row < n; ++row) {
      float v = sol[static_cast<size_t>(row) * m + c];
      for (int k = 0; k < row; ++k) v -= L[static_cast<size_t>(row) * n + k] * sol[static_cast<size_t>(k) * m + c];
      sol[static_cast<size_t>(row) * m + c] = v / L[static_cast<size_t>(row) * n + row];
    }
    for (int row = n - 1; row >= 0; --row) {
      float v = sol[static_cast<size_t>(row) * m + c];
      for (int k = row + 1; k < n; ++k) v -= L[static_cast<size_t>(k) * n + row] * sol[static_cast<size_t>(k) * m + c];
      sol[static_cast<size_t>(row) * m + c] = v / L[static_cast<size_t>(row) * n + row];
    }
  }
  return true;
}

// fit_predict_pls_lda_streamed_cpu_float (plscv.cpp:1544-1608) with
// fit_lda_from_score_statistics_float (:1419-1487).  Returns class codes.
std::vector<int> lda_streamed(const Vec& zt, int nt, const std::vector<int>& code, const Vec& zv, int nv, int p,
                              const Fit& fit, int m, int nc) {
  Vec cs(static_cast<size_t>(m) * nc, 0.0f), cp(static_cast<size_t>(nc) * nc, 0.0f), sr(static_cast<size_t>(nc));
  std::vector<int> counts(static_cast<size_t>(m), 0);
  for (int i = 0; i < nt; ++i) counts[code[i]]++;
  // the weights padded to 8 lanes per feature (zeros past nc), so that the
  // nc float chains of a score row run as unconditional vector lanes
  const int nb = (nc + 7) / 8;
  Vec wp(static_cast<size_t>(p) * nb * 8, 0.0f);
  for (int j = 0; j < p; ++j)
    for (int a = 0; a < nc; ++a) wp[(static_cast<size_t>(j) * nb + a / 8) * 8 + a % 8] = fit.w[static_cast<size_t>(j) * fit.rank + a];
  auto score_row = [&](const Vec& z, int i) {
    const float* zr = z.data() + static_cast<size_t>(i) * p;
    for (int b = 0; b < nb; ++b) {
      float acc[8] = {};
      for (int j = 0; j < p; ++j) {
        const float v = zr[j];
        const float* wr = wp.data() + (static_cast<size_t>(j) * nb + b) * 8;
        for (int a = 0; a < 8; ++a) {
          const float prod = v * wr[a];
          acc[a] = acc[a] + prod;
        }
      }
      for (int a = 0; a < 8 && b * 8 + a < nc; ++a) sr[b * 8 + a] = acc[a];
    }
  };
  for (int i = 0; i < nt; ++i) {
    score_row(zt, i);
    const int c = code[i];
    for (int a = 0; a < nc; ++a) cs[static_cast<size_t>(c) * nc + a] += sr[a];
    for (int r = 0; r < nc; ++r)
      for (int col = 0; col <= r; ++col) cp[static_cast<size_t>(r) * nc + col] += sr[r] * sr[col];
  }
  for (int r = 0; r < nc; ++r)
    for (int col = 0; col < r; ++col) cp[static_cast<size_t>(col) * nc + r] = cp[static_cast<size_t>(r) * nc + col];
  // LDA from the score statistics
  for (int c = 0; c < m; ++c) {
    const float inv = counts[c] > 0 ? 1.0f / static_cast<float>(counts[c]) : 0.0f;
    for (int a = 0; a < nc; ++a) cs[static_cast<size_t>(c) * nc + a] *= inv;
  }
  Vec pooled(static_cast<size_t>(nc) * nc, 0.0f);
  const float df = static_cast<float>(std::max(1, nt - m));
  float trace = 0.0f;
  for (int r = 0; r < nc; ++r) {
    for (int col = 0; col <= r; ++col) {
      float between = 0.0f;
      for (int c = 0; c < m; ++c)
        between += static_cast<float>(counts[c]) * cs[static_cast<size_t>(c) * nc + r] * cs[static_cast<size_t>(c) * nc + col];
      const float cov = (cp[static_cast<size_t>(r) * nc + col] - between) / df;
      pooled[static_cast<size_t>(r) * nc + col] = cov;
      pooled[static_cast<size_t>(col) * nc + r] = cov;
    }
    trace += pooled[static_cast<size_t>(r) * nc + r];
  }
  Vec rhs(static_cast<size_t>(nc) * m);
  for (int c = 0; c < m; ++c)
    for (int a = 0; a < nc; ++a) rhs[static_cast<size_t>(a) * m + c] = cs[static_cast<size_t>(c) * nc + a];
  const float ridge_scale = std::isfinite(trace) && trace > 0.0f ? trace / static_cast<float>(std::max(1, nc)) : 1.0f;
  const float grid[] = {1e-8f, 1e-6f, 1e-5f, 1e-4f, 1e-3f, 1e-2f};
  Vec sol;
  bool ok = false;
  for (float ridge : grid) {
    Vec cov = pooled;
    const float lambda = ridge * ridge_scale;
    for (int a = 0; a < nc; ++a) cov[static_cast<size_t>(a) * nc + a] += lambda;
    if (chol_solve(cov, nc, rhs, m, sol)) {
      ok = true;
      break;
    }
  }
  if (!ok) throw std::runtime_error("Float32 PLS-LDA Cholesky factorization failed.");
  Vec lin(static_cast<size_t>(m) * nc), cst(static_cast<size_t>(m));
  for (int c = 0; c < m; ++c) {
    float dot_mu = 0.0f;
    for (int a = 0; a < nc; ++a) {
      lin[static_cast<size_t>(c) * nc + a] = sol[static_cast<size_t>(a) * m + c];
      dot_mu += cs[static_cast<size_t>(c) * nc + a] * lin[static_cast<size_t>(c) * nc + a];
    }
    const float prior = std::max(static_cast<float>(counts[c]) / static_cast<float>(std::max(1, nt)),
                                 std::numeric_limits<float>::min());
    cst[c] = -0.5f * dot_mu + std::log(prior);
  }
  std::vector<int> pred(static_cast<size_t>(nv), 0);
  for (int i = 0; i < nv; ++i) {
    score_row(zv, i);
    int best = 0;
    float bs = -std::numeric_limits<float>::infinity();
    for (int c = 0; c < m; ++c) {
      float sc = cst[c];
      for (int a = 0; a < nc; ++a) sc += sr[a] * lin[static_cast<size_t>(c) * nc + a];
      if (sc > bs) {
        bs = sc;
        best = c;
      }
    }
    pred[i] = best;
  }
  return pred;
}

std::vector<int> sorted_unique(std::vector<int> v) {
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
  return v;
}

std::vector<int> encode(const std::vector<int>& y, const std::vector<int>& classes) {
  std::vector<int> code(y.size());
  for (size_t i = 0; i < y.size(); ++i)
    code[i] = static_cast<int>(std::lower_bound(classes.begin(), classes.end(), y[i]) - classes.begin());
  return code;
}

}  // namespace

// solve_linear_float (plscv.cpp:1346-1377): Gauss-Jordan with partial
// pivoting on a + 1e-9 I (row-major n x n), right-hand sides b (n x m).
Vec solve_linear(Vec a, int n, Vec b, int m) {
  for (int i = 0; i < n; ++i) a[static_cast<size_t>(i) * n + i] += 1.0e-9f;
  for (int col = 0; col < n; ++col) {
    int pivot = col;
    float best = std::abs(a[static_cast<size_t>(col) * n + col]);
    for (int r = col + 1; r < n; ++r) {
      const float val = std::abs(a[static_cast<size_t>(r) * n + col]);
      if (val > best) {
        best = val;
        pivot = r;
      }
    }
    if (best < 1.0e-12f) continue;
    if (pivot != col) {
      for (int j = 0; j < n; ++j) std::swap(a[static_cast<size_t>(col) * n + j], a[static_cast<size_t>(pivot) * n + j]);
      for (int j = 0; j < m; ++j) std::swap(b[static_cast<size_t>(col) * m + j], b[static_cast<size_t>(pivot) * m + j]);
    }
    const float div = a[static_cast<size_t>(col) * n + col];
    for (int j = col; j < n; ++j) a[static_cast<size_t>(col) * n + j] /= div;
    for (int j = 0; j < m; ++j) b[static_cast<size_t>(col) * m + j] /= div;
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const float f = a[static_cast<size_t>(r) * n + col];
      if (f == 0.0f) continue;
      for (int j = col; j < n; ++j) a[static_cast<size_t>(r) * n + j] -= f * a[static_cast<size_t>(col) * n + j];
      for (int j = 0; j < m; ++j) b[static_cast<size_t>(r) * m + j] -= f * b[static_cast<size_t>(col) * m + j];
    }
  }
  return b;
}

// The PLS-DA branch of run_plscv_host (plscv.cpp:2428-2443): scores of the
// training and validation rows (transform_pls_scores_float :995), class means
// (label_means_float :1210), one-hot regression coefficients
// (regression_coefficients_centered_one_hot_float :1222-1265) and the
// prediction argmax (predict_pls_da_labels_float :1267-1292).
std::vector<int> da_predict(const Vec& zt, int nt, const std::vector<int>& code, const Vec& zv, int nv, int p,
                            const Fit& fit, int m, int nc) {
  auto scores = [&](const Vec& z, int rows) {
    Vec t(static_cast<size_t>(rows) * nc, 0.0f);
    for (int i = 0; i < rows; ++i) {
      float* out = t.data() + static_cast<size_t>(i) * nc;
      for (int j = 0; j < p; ++j) {
        const float v = z[static_cast<size_t>(i) * p + j];
        const float* wr = fit.w.data() + static_cast<size_t>(j) * fit.rank;
        for (int a = 0; a < nc; ++a) out[a] += v * wr[a];
      }
    }
    return t;
  };
  const Vec tt = scores(zt, nt), tv = scores(zv, nv);
  std::vector<float> ymean(static_cast<size_t>(m), 0.0f);
  for (int i = 0; i < nt; ++i) ymean[code[i]] += 1.0f;
  const float inv_n = nt > 0 ? 1.0f / static_cast<float>(nt) : 0.0f;
  for (float& v : ymean) v *= inv_n;
  Vec lhs(static_cast<size_t>(nc) * nc), rhs(static_cast<size_t>(nc) * m, 0.0f);
  std::vector<double> ssum(static_cast<size_t>(nc), 0.0), lacc(static_cast<size_t>(nc) * nc, 0.0);
  for (int r = 0; r < nt; ++r) {
    const int c = code[r];
    const float* tr = tt.data() + static_cast<size_t>(r) * nc;
    for (int a = 0; a < nc; ++a) {
      const double value = tr[a];
      rhs[static_cast<size_t>(a) * m + c] += static_cast<float>(value);
      ssum[a] += value;
      for (int b = a; b < nc; ++b) lacc[static_cast<size_t>(a) * nc + b] += value * static_cast<double>(tr[b]);
    }
  }
  for (int a = 0; a < nc; ++a)
    for (int b = a; b < nc; ++b) {
      const float v = static_cast<float>(lacc[static_cast<size_t>(a) * nc + b]);
      lhs[static_cast<size_t>(a) * nc + b] = v;
      lhs[static_cast<size_t>(b) * nc + a] = v;
    }
  for (int a = 0; a < nc; ++a)
    for (int c = 0; c < m; ++c)
      rhs[static_cast<size_t>(a) * m + c] -= static_cast<float>(ssum[a] * static_cast<double>(ymean[c]));
  const Vec coef = solve_linear(lhs, nc, rhs, m);
  std::vector<int> pred(static_cast<size_t>(nv), 0);
  for (int i = 0; i < nv; ++i) {
    int best = 0;
    float bs = -std::numeric_limits<float>::infinity();
    for (int c = 0; c < m; ++c) {
      float sc = ymean[c];
      for (int a = 0; a < nc; ++a) sc += tv[static_cast<size_t>(i) * nc + a] * coef[static_cast<size_t>(a) * m + c];
      if (sc > bs) {
        bs = sc;
        best = c;
      }
    }
    pred[i] = best;
  }
  return pred;
}

// get_pls_fold_x_cache_float (plscv.cpp:593-667) and the uncached branch of
// run_plscv_host (:2371-2381) compute the same per-fold data.
PLSFoldCache pls_fold_cache(const float* x, int n, int p, const std::vector<int>& folds, const PLSOpts& o) {
  PLSFoldCache cache;
  cache.folds = folds;
  cache.fold_ids = sorted_unique(folds);
  for (int f : cache.fold_ids) {
    PLSFoldData d;
    for (int i = 0; i < n; ++i) (folds[i] == f ? d.validation : d.train).push_back(i);
    center_scale(x, p, d.train, o.center, o.scale, d.mean, d.scale);
    d.x_train = standardize(x, p, d.train, d.mean, d.scale);
    d.x_val = standardize(x, p, d.validation, d.mean, d.scale);
    cache.data.push_back(std::move(d));
  }
  return cache;
}

// The Gram is only built for folds with at least as many training rows as
// columns (plscv.cpp:611-613).
void pls_build_grams(PLSFoldCache& cache, int p) {
  for (PLSFoldData& d : cache.data) {
    const int nt = static_cast<int>(d.train.size());
    if (p <= nt) d.gram = gram_of(d.x_train, nt, p);
  }
  cache.gram_built = true;
}

PLSCVOut plsldacv_on_cache(const PLSFoldCache& cache, int n, int p, const std::vector<int>& labels,
                           const PLSOpts& o, bool use_gram) {
  PLSCVOut out;
  out.folds = cache.folds;
  out.predicted.assign(static_cast<size_t>(n), labels.empty() ? 0 : labels.front());
  out.accuracy_by_components.assign(static_cast<size_t>(o.max_components), 0.0);
  const int requested = o.fixed_components > 0 ? o.fixed_components : o.max_components;
  int evaluated = requested;
  for (const PLSFoldData& d : cache.data) {
    const int nt = static_cast<int>(d.train.size());
    std::vector<int> y(d.train.size());
    for (size_t i = 0; i < d.train.size(); ++i) y[i] = labels[d.train[i]];
    const std::vector<int> classes = sorted_unique(y);
    if (classes.size() <= 1) {
      const int lab = classes.empty() ? (labels.empty() ? 0 : labels.front()) : classes.front();
      evaluated = std::min(evaluated, 1);
      for (int r : d.validation) out.predicted[r] = lab;
      continue;
    }
    const int m = static_cast<int>(classes.size());
    const std::vector<int> code = encode(y, classes);
    Fit fit;
    const Vec* g = use_gram && !d.gram.empty() ? &d.gram : nullptr;
    if (!fit_pls(d.x_train, nt, p, crossprod(d.x_train, nt, p, code, m), m, o.max_components, g, fit)) {
      // DegeneratePLSFit: the most frequent training label (smallest on ties)
      std::map<int, int> counts;
      for (int l : y) ++counts[l];
      int lab = classes.front(), best = -1;
      for (const auto& kv : counts) {
        if (kv.second > best) {
          lab = kv.first;
          best = kv.second;
        }
      }
      evaluated = std::min(evaluated, 1);
      for (int r : d.validation) out.predicted[r] = lab;
      continue;
    }
    const int a = std::min(requested, fit.rank);
    evaluated = std::min(evaluated, a);
    const std::vector<int> pc =
        o.da ? da_predict(d.x_train, nt, code, d.x_val, static_cast<int>(d.validation.size()), p, fit, m, a)
             : lda_streamed(d.x_train, nt, code, d.x_val, static_cast<int>(d.validation.size()), p, fit, m, a);
    for (size_t i = 0; i < d.validation.size(); ++i) out.predicted[d.validation[i]] = classes[pc[i]];
  }
  const int best = std::min(evaluated, o.max_components);
  size_t ok = 0;
  for (int i = 0; i < n; ++i) ok += labels[i] == out.predicted[i];
  out.accuracy_by_components[static_cast<size_t>(best - 1)] = static_cast<double>(ok) / static_cast<double>(n);
  out.selected_components = best;
  return out;
}

PLSCVOut plsldacv(const float* x, int n, int p, const std::vector<int>& labels, const std::vector<int>& constrain,
                  const PLSOpts& o) {
  if (o.max_components < 1) throw std::invalid_argument("PLSOptions::max_components must be positive.");
  if (o.fixed_components < 0) throw std::invalid_argument("PLSOptions::fixed_components must be non-negative.");
  if (o.fixed_components > o.max_components)
    throw std::invalid_argument("PLSOptions::fixed_components cannot exceed max_components.");
  const std::vector<int> folds = make_folds(labels, constrain, o.folds, o.stratified, o.cv_seed);
  const PLSFoldCache cache = pls_fold_cache(x, n, p, folds, o);
  return plsldacv_on_cache(cache, n, p, labels, o, false);
}

std::vector<int> plslda_predict(const float* train, int n, int p, const std::vector<int>& labels, const float* test,
                                int nt, const PLSOpts& o) {
  if (n == 0 || nt == 0 || p == 0) return {};
  const std::vector<int> classes = sorted_unique(labels);
  if (classes.empty()) return {};
  if (classes.size() == 1) return std::vector<int>(static_cast<size_t>(nt), classes.front());
  std::vector<int> rows(static_cast<size_t>(n)), trows(static_cast<size_t>(nt));
  std::iota(rows.begin(), rows.end(), 0);
  std::iota(trows.begin(), trows.end(), 0);
  Vec mean, sc;
  center_scale(train, p, rows, o.center, o.scale, mean, sc);
  const Vec zt = standardize(train, p, rows, mean, sc);
  const Vec zq = standardize(test, p, trows, mean, sc);
  const int requested = o.fixed_components > 0 ? o.fixed_components : o.max_components;
  const int ncomp = std::max(1, std::min({requested, p, std::max(1, n - 1)}));
  const int m = static_cast<int>(classes.size());
  const std::vector<int> code = encode(labels, classes);
  Fit fit;
  if (!fit_pls(zt, n, p, crossprod(zt, n, p, code, m), m, ncomp, nullptr, fit))
    throw std::runtime_error("CPU float32 SIMPLS found no supervised latent direction.");
  const std::vector<int> pc = lda_streamed(zt, n, code, zq, nt, p, fit, m, fit.rank);
  std::vector<int> out(static_cast<size_t>(nt));
  for (int i = 0; i < nt; ++i) out[i] = classes[pc[i]];
  return out;
}

}  // namespace orc
