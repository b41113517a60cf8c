// Laplacian features of a neighbour graph (graph_features.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace kgb {

// n x min(components, n) float features (row-major) of the graph idx/dist
// (n x gk; index_base 0, 1 or -1 = detect), graph_laplacian_operator_features
// (kodama_matrix.cpp:1575-1603) with max(8, steps) iterations.
std::vector<float> graph_laplacian_features(const int* idx, const float* dist, int n, int gk, int index_base,
                                            int components, int steps, uint64_t seed);

}  // namespace kgb
