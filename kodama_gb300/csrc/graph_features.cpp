// Graph-only KODAMA.matrix: Laplacian features of a caller graph (host).
//
// KODAMAMatrixFromGraph (kodama_matrix.cpp:4640-4657, and its CUDA variant
// :4740-4760, which computes the same features on the host) turns a
// neighbour graph without data into feature columns and then runs the
// graph-input path on them.  The features are
// graph_laplacian_operator_features (kodama_matrix.cpp:1575-1603):
//   * the graph normalised as normalize_external_graph (:1292-1330);
//   * self-tuning Gaussian weights exp(-d^2 / (s_i s_j)) with s_i the median
//     of row i's distances (graph_local_scales, :1367-1399), symmetrised by
//     the larger weight, normalised by sqrt(deg_i deg_j)
//     (make_sparse_graph_operator, :1401-1482);
//   * columns drawn from std::normal_distribution<float> on
//     std::mt19937_64(seed), centred and Gram-Schmidt orthonormalised in
//     double (:1501-1548), then max(8, steps) rounds of operator application
//     (:1550-1573) and orthonormalisation, then per-column standardisation
//     (:1484-1499).
// The steps, their order and the containers whose iteration order fixes a
// floating-point sum (the per-row std::unordered_map of edge weights) are
// kept as the reference has them, so the features are the same floats on a
// host with the same C library.
#include "graph_features.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <random>
#include <stdexcept>
#include <unordered_map>
#include <utility>

namespace kgb {
namespace {

struct Graph {
  int K = 0;
  std::vector<int> idx;
  std::vector<float> dist;
};

Graph normalize_graph(const int* idx, const float* dist, int n, int gk, int index_base) {
  if (n < 2) throw std::invalid_argument("NeighborGraph samples must be at least 2.");
  if (gk <= 0) throw std::invalid_argument("NeighborGraph.neighbors must be positive.");
  int min_index = std::numeric_limits<int>::max(), max_index = std::numeric_limits<int>::min();
  const size_t total = static_cast<size_t>(n) * gk;
  for (size_t e = 0; e < total; ++e) {
    if (idx[e] < 0) continue;
    min_index = std::min(min_index, idx[e]);
    max_index = std::max(max_index, idx[e]);
  }
  const bool one_based = index_base == 1 || (index_base < 0 && min_index >= 1 && max_index <= n);
  Graph g;
  g.K = gk;
  g.idx.assign(total, -1);
  g.dist.assign(total, std::numeric_limits<float>::infinity());
  for (int i = 0; i < n; ++i) {
    int col = 0;
    for (int j = 0; j < gk && col < gk; ++j) {
      const size_t src = static_cast<size_t>(i) * gk + j;
      int id = idx[src];
      if (one_based && id > 0) --id;
      if (id < 0 || id >= n || id == i) continue;
      const float d = dist[src];
      if (!std::isfinite(d)) continue;
      g.idx[static_cast<size_t>(i) * gk + col] = id;
      g.dist[static_cast<size_t>(i) * gk + col] = std::max(0.0f, d);
      ++col;
    }
  }
  return g;
}

std::vector<float> local_scales(const Graph& g, int n) {
  std::vector<float> scales(static_cast<size_t>(n), 1.0f);
  std::vector<float> row;
  row.reserve(static_cast<size_t>(g.K));
  for (int i = 0; i < n; ++i) {
    row.clear();
    for (int j = 0; j < g.K; ++j) {
      const size_t e = static_cast<size_t>(i) * g.K + j;
      if (g.idx[e] < 0 || !std::isfinite(g.dist[e])) continue;
      row.push_back(std::max(0.0f, g.dist[e]));
    }
    if (row.empty()) continue;
    const size_t mid = row.size() / 2;
    std::nth_element(row.begin(), row.begin() + static_cast<std::ptrdiff_t>(mid), row.end());
    float s = row[mid];
    if (s <= 1.0e-6f) {
      double mean = 0.0;
      for (float d : row) mean += static_cast<double>(d);
      s = static_cast<float>(mean / static_cast<double>(row.size()));
    }
    scales[static_cast<size_t>(i)] = std::max(s, 1.0e-6f);
  }
  return scales;
}

struct Operator {
  std::vector<int> indptr, indices;
  std::vector<float> weights;
};

Operator make_operator(const Graph& g, int n) {
  const std::vector<float> scales = local_scales(g, n);
  std::vector<std::unordered_map<int, float>> rows(static_cast<size_t>(n));
  for (auto& r : rows) r.reserve(static_cast<size_t>(std::max(1, g.K)));
  auto weight = [&](int i, int j, float d) {
    d = std::max(0.0f, d);
    const double denom = std::max(1.0e-12, static_cast<double>(scales[i]) * static_cast<double>(scales[j]));
    return static_cast<float>(std::exp(-(static_cast<double>(d) * static_cast<double>(d)) / denom));
  };
  auto add = [&](int from, int to, float w) {
    if (from < 0 || from >= n || to < 0 || to >= n || from == to || !std::isfinite(w) || w <= 0.0f) return;
    auto& r = rows[static_cast<size_t>(from)];
    auto it = r.find(to);
    if (it == r.end()) r.emplace(to, w);
    else it->second = std::max(it->second, w);
  };
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < g.K; ++j) {
      const size_t e = static_cast<size_t>(i) * g.K + j;
      const int nb = g.idx[e];
      if (nb < 0 || nb >= n) continue;
      const float d = g.dist[e];
      if (!std::isfinite(d)) continue;
      const float w = weight(i, nb, d);
      add(i, nb, w);
      add(nb, i, w);
    }
  }
  std::vector<double> degree(static_cast<size_t>(n), 0.0);
  for (int i = 0; i < n; ++i)
    for (const auto& kv : rows[static_cast<size_t>(i)]) degree[static_cast<size_t>(i)] += static_cast<double>(kv.second);
  Operator op;
  op.indptr.assign(static_cast<size_t>(n) + 1, 0);
  size_t nnz = 0;
  for (int i = 0; i < n; ++i) {
    op.indptr[static_cast<size_t>(i)] = static_cast<int>(nnz);
    nnz += rows[static_cast<size_t>(i)].size();
  }
  op.indptr[static_cast<size_t>(n)] = static_cast<int>(nnz);
  op.indices.reserve(nnz);
  op.weights.reserve(nnz);
  for (int i = 0; i < n; ++i) {
    std::vector<std::pair<int, float>> ordered(rows[static_cast<size_t>(i)].begin(), rows[static_cast<size_t>(i)].end());
    std::sort(ordered.begin(), ordered.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    const double row_degree = std::max(degree[static_cast<size_t>(i)], 1.0e-12);
    for (const auto& kv : ordered) {
      const double denom = std::sqrt(row_degree * std::max(degree[static_cast<size_t>(kv.first)], 1.0e-12));
      op.indices.push_back(kv.first);
      op.weights.push_back(static_cast<float>(static_cast<double>(kv.second) / denom));
    }
  }
  return op;
}

void apply(const Operator& op, int n, const std::vector<float>& cur, std::vector<float>& next, int p) {
  std::fill(next.begin(), next.end(), 0.0f);
  for (int i = 0; i < n; ++i) {
    const size_t rb = static_cast<size_t>(i) * p;
    for (int e = op.indptr[static_cast<size_t>(i)]; e < op.indptr[static_cast<size_t>(i) + 1]; ++e) {
      const size_t nb = static_cast<size_t>(op.indices[static_cast<size_t>(e)]) * p;
      const float w = op.weights[static_cast<size_t>(e)];
      for (int c = 0; c < p; ++c) next[rb + c] += w * cur[nb + c];
    }
  }
}

void center_columns(std::vector<float>& x, int n, int p) {
  for (int c = 0; c < p; ++c) {
    double mean = 0.0;
    for (int i = 0; i < n; ++i) mean += static_cast<double>(x[static_cast<size_t>(i) * p + c]);
    mean /= static_cast<double>(std::max(1, n));
    for (int i = 0; i < n; ++i)
      x[static_cast<size_t>(i) * p + c] = static_cast<float>(static_cast<double>(x[static_cast<size_t>(i) * p + c]) - mean);
  }
}

void orthonormalize(std::vector<float>& x, int n, int p) {
  center_columns(x, n, p);
  for (int c = 0; c < p; ++c) {
    for (int prev = 0; prev < c; ++prev) {
      double dot = 0.0;
      for (int i = 0; i < n; ++i)
        dot += static_cast<double>(x[static_cast<size_t>(i) * p + c]) * static_cast<double>(x[static_cast<size_t>(i) * p + prev]);
      for (int i = 0; i < n; ++i)
        x[static_cast<size_t>(i) * p + c] = static_cast<float>(static_cast<double>(x[static_cast<size_t>(i) * p + c]) -
                                                               dot * static_cast<double>(x[static_cast<size_t>(i) * p + prev]));
    }
    double norm2 = 0.0;
    for (int i = 0; i < n; ++i) {
      const double v = static_cast<double>(x[static_cast<size_t>(i) * p + c]);
      norm2 += v * v;
    }
    if (norm2 <= 1.0e-20) {
      for (int i = 0; i < n; ++i) x[static_cast<size_t>(i) * p + c] = 0.0f;
      if (n > 0) x[static_cast<size_t>(c % n) * p + c] = 1.0f;
      center_columns(x, n, p);
      norm2 = 0.0;
      for (int i = 0; i < n; ++i) {
        const double v = static_cast<double>(x[static_cast<size_t>(i) * p + c]);
        norm2 += v * v;
      }
    }
    const float inv = static_cast<float>(1.0 / std::sqrt(std::max(norm2, 1.0e-20)));
    for (int i = 0; i < n; ++i) x[static_cast<size_t>(i) * p + c] *= inv;
  }
}

void standardize_columns(std::vector<float>& x, int n, int p) {
  for (int c = 0; c < p; ++c) {
    double mean = 0.0;
    for (int i = 0; i < n; ++i) mean += static_cast<double>(x[static_cast<size_t>(i) * p + c]);
    mean /= static_cast<double>(std::max(1, n));
    double ss = 0.0;
    for (int i = 0; i < n; ++i) {
      float& v = x[static_cast<size_t>(i) * p + c];
      v = static_cast<float>(static_cast<double>(v) - mean);
      ss += static_cast<double>(v) * static_cast<double>(v);
    }
    const double scale = ss > 0.0 ? std::sqrt(ss / static_cast<double>(std::max(1, n - 1))) : 1.0;
    const float inv = static_cast<float>(1.0 / std::max(scale, 1.0e-6));
    for (int i = 0; i < n; ++i) x[static_cast<size_t>(i) * p + c] *= inv;
  }
}

}  // namespace

std::vector<float> graph_laplacian_features(const int* idx, const float* dist, int n, int gk, int index_base,
                                            int components, int steps, uint64_t seed) {
  const Graph g = normalize_graph(idx, dist, n, gk, index_base);
  const Operator op = make_operator(g, n);
  const int p = std::max(1, std::min(components, n));
  const int iterations = std::max(8, steps);
  std::vector<float> cur(static_cast<size_t>(n) * p, 0.0f), next(cur.size(), 0.0f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> normal(0.0f, 1.0f);
  for (float& v : cur) v = normal(rng);
  orthonormalize(cur, n, p);
  for (int it = 0; it < iterations; ++it) {
    apply(op, n, cur, next, p);
    orthonormalize(next, n, p);
    cur.swap(next);
  }
  standardize_columns(cur, n, p);
  return cur;
}

}  // namespace kgb
