// Test driver of the compiled drop-in boundary (tests/test_boundary_cxx.py):
// the reference's C++ core, linked with kodama_gb300/cxx/kodama_cuda_backend.cpp
// and libkodama_gb300.so, called through its public dispatching functions.
//
// Every Backend::CUDA call must reach the GB300 library: on a host without a
// GPU each one ends in the library's own error ("no CUDA device"), never in
// the reference's CPU-build stub ("requires a CUDA build").  The CPU backend
// of the same binary still runs the reference's own code.  One line per call:
// "<entry point>\t<ok | exception message>".

#include "kodama/kodama.hpp"
#include "kodama_matrix_cuda.hpp"

#include <cstdio>
#include <functional>
#include <random>
#include <string>
#include <vector>

namespace {

void report(const char* name, const std::function<void()>& f) {
  try {
    f();
    std::printf("%s\tok\n", name);
  } catch (const std::exception& e) {
    std::string m = e.what();
    for (char& c : m)
      if (c == '\n' || c == '\t') c = ' ';
    std::printf("%s\t%s\n", name, m.c_str());
  }
}

}  // namespace

int main() {
  using namespace kodama;
  const int n = 300, d = 6;
  std::mt19937 rng(7);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  std::vector<float> x(static_cast<size_t>(n) * d);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) x[static_cast<size_t>(i) * d + j] = nd(rng) + static_cast<float>(3 * (i % 3));
  const MatrixView view(x.data(), n, d);
  std::vector<int> labels(n);
  for (int i = 0; i < n; ++i) labels[i] = 1 + i % 3;

  KODAMAMatrixOptions mo;
  mo.runs = 2;
  mo.cycles = 3;
  mo.graph_neighbors = 10;
  mo.compute_visual_init = false;
  mo.knn.k = 5;

  // the CPU backend: the reference's own code in the same binary
  report("KODAMAMatrix[CPU]", [&] { (void)KODAMAMatrix(view, {}, {}, {}, mo); });

  KODAMAMatrixOptions cu = mo;
  cu.backend = Backend::CUDA;
  report("KODAMAMatrix_CUDA", [&] { (void)KODAMAMatrix(view, {}, {}, {}, cu); });

  KODAMAGraphOptions go;
  go.neighbors = 10;
  go.backend = Backend::CUDA;
  report("KODAMAGraph_CUDA", [&] { (void)KODAMAGraph(view, go); });

  // a host graph handed to the CUDA backend: the reference orchestrates the
  // runs and calls CoreKNNGraph_CUDA for each run's evolution
  KODAMAGraphOptions gcpu = go;
  gcpu.backend = Backend::CPU;
  gcpu.materialize_graph = true;
  KODAMAGraphResult graph = KODAMAGraph(view, gcpu);
  report("KODAMAMatrix(graph)->CoreKNNGraph_CUDA", [&] { (void)KODAMAMatrix(view, graph, {}, {}, {}, cu); });
  report("KODAMAMatrixFromGraphData_CUDA", [&] { (void)KODAMAMatrixFromGraphData(view, graph.knn, {}, {}, {}, cu); });
  report("KODAMAMatrixFromGraph_CUDA", [&] { (void)KODAMAMatrixFromGraph(graph.knn, n, {}, {}, {}, cu); });

  KNNOptions ko;
  ko.backend = Backend::CUDA;
  report("KNNCV_CUDA", [&] { (void)KNNCV(view, labels, {}, ko); });

  CoreOptions co;
  co.cycles = 3;
  co.knn.backend = Backend::CUDA;
  co.pls.backend = Backend::CUDA;
  report("CoreKNN_CUDA", [&] { (void)CoreKNN(view, labels, {}, {}, co); });
  report("CorePLSLDA_CUDA", [&] { (void)CorePLSLDA(view, labels, {}, {}, co); });

  PLSOptions po;
  po.backend = Backend::CUDA;
  po.max_components = 2;
  report("PLSLDACV_CUDA", [&] { (void)PLSLDACV(view, labels, {}, po); });
  report("PLSDACV_CUDA", [&] { (void)PLSDACV(view, labels, {}, po); });
  report("PLSLDAPredict_CUDA", [&] { (void)PLSLDAPredict(view, labels, view, po); });

  NeighborGraph one = graph.knn;
  if (one.index_base != GraphIndexBase::One)
    for (int& v : one.indices) v += v >= 0 ? 1 : 0;
  one.index_base = GraphIndexBase::One;
  std::vector<int> res(static_cast<size_t>(2) * n, 1);
  report("apply_kodama_dissimilarity_cuda",
         [&] { detail::apply_kodama_dissimilarity_cuda(one, res, 2, n, 0, true, true); });
  return 0;
}
