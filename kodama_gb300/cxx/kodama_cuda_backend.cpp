// Strong definitions of the reference's *_CUDA entry points
// (inst/include/kodama/kodama.hpp:871-1249) on top of the C ABI of
// libkodama_gb300 (include/kodama_gb300.h).
//
// A build of the reference's C++ core that links this translation unit and
// libkodama_gb300.so answers `backend = "cuda"` with the GB300 library: these
// definitions take the place of the CPU build's throwing stubs (core.cpp,
// knncv.cpp, plscv.cpp, kodama_matrix.cpp), and
// detail::apply_kodama_dissimilarity_cuda is the CUDA branch of
// KODAMADissimilarityInPlace (kodama_matrix.cpp:4412-4423).  Compile with the
// reference's include directories (inst/include and src, for the option and
// result types and the host helpers of common.hpp) and this repository's
// include directory.
//
// Marshalling: MatrixView rows become a row-major float buffer
// (value_float); std::vector inputs are passed as pointers (empty = NULL);
// every result field the reference's CUDA variants fill is filled here, the
// summary fields (per-fold accuracy, global accuracy, confusion) by the
// reference's own host helpers.  Status codes become exceptions:
// KGB_EINVAL -> std::invalid_argument, others -> std::runtime_error, with the
// library's message.

#include "kodama/kodama.hpp"
#include "common.hpp"
#include "kodama_matrix_cuda.hpp"

#include "kodama_gb300.h"

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

using namespace kodama;

void check(int rc) {
  if (rc == KGB_OK) return;
  char msg[2048];
  kgb_last_error(msg, sizeof msg);
  if (rc == KGB_EINVAL) throw std::invalid_argument(msg);
  throw std::runtime_error(std::string("kodama_gb300: ") + msg);
}

class Timer {
 public:
  double seconds() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }

 private:
  std::chrono::steady_clock::time_point t0_ = std::chrono::steady_clock::now();
};

std::vector<float> as_float(MatrixView x) {
  std::vector<float> f(x.rows * x.cols);
  for (std::size_t i = 0; i < x.rows; ++i)
    for (std::size_t j = 0; j < x.cols; ++j) f[i * x.cols + j] = x.value_float(i, j);
  return f;
}

const int32_t* opt_ptr(const std::vector<int>& v) { return v.empty() ? nullptr : v.data(); }

void check_rows(const std::vector<int>& v, std::size_t n, const char* what) {
  if (!v.empty() && v.size() != n)
    throw std::invalid_argument(std::string(what) + " size must be zero or match number of rows.");
}

int metric_of(DistanceMetric m) {
  return m == DistanceMetric::Cosine ? KGB_METRIC_COSINE
       : m == DistanceMetric::InnerProduct ? KGB_METRIC_INNER_PRODUCT : KGB_METRIC_EUCLIDEAN;
}

int base_of(GraphIndexBase b) { return b == GraphIndexBase::One ? 1 : (b == GraphIndexBase::Zero ? 0 : -1); }

kgb_policy policy_of(const EvolutionPolicy& p) {
  kgb_policy k{};
  k.prediction_guidance = p.prediction_guidance;
  k.adaptive_proposal_size = p.adaptive_proposal_size;
  k.transition_proposal = p.transition_proposal;
  k.stochastic_acceptance = p.stochastic_acceptance;
  k.diversity_multiplier = p.diversity_multiplier;
  k.pls_transition_coarsening = p.pls_transition_coarsening;
  k.pls_fragmentation_penalty = p.pls_fragmentation_penalty;
  k.reject_single_class = p.reject_single_class;
  return k;
}

kgb_matrix_options matrix_options_of(const KODAMAMatrixOptions& o) {
  if (o.spatial_cols > 0 || !o.spatial.empty())
    throw std::invalid_argument("kodama_gb300: spatial KODAMA.matrix options are not supported by the CUDA backend");
  kgb_matrix_options k{};
  k.runs = o.runs;
  k.cycles = o.cycles;
  k.landmarks = o.landmarks;
  k.splitting = o.splitting;
  k.graph_neighbors = o.graph_neighbors;
  k.folds = o.folds;
  k.knn_k = o.knn.k;
  k.classifier = o.classifier == CoreClassifier::KNN ? 0 : 1;
  k.components = o.components;
  k.materialize_graph = o.materialize_graph ? 1 : 0;
  k.apply_dissimilarity = o.apply_kodama_dissimilarity ? 1 : 0;
  k.metric = metric_of(o.metric);
  k.device = o.knn.gpu_device;
  k.host_threads = o.n_threads;
  k.first_run = 1;
  k.seed = o.seed;
  k.policy = policy_of(o.evolution);
  return k;
}

kgb_core_options core_options_of(const CoreOptions& o) {
  kgb_core_options k{};
  k.cycles = o.cycles;
  k.k = o.knn.k;
  k.folds = o.knn.cv.folds;
  k.stratified = o.knn.cv.stratified ? 1 : 0;
  k.evolutionary_search = o.evolutionary_search ? 1 : 0;
  k.guarded_diversity = o.guarded_diversity ? 1 : 0;
  k.many_to_one_absorption = o.many_to_one_absorption ? 1 : 0;
  k.adaptive_proposal_size = o.adaptive_proposal_size ? 1 : 0;
  k.device = o.knn.gpu_device;
  k.auto_class_coarsening = o.auto_class_coarsening ? 1 : 0;
  k.metric = metric_of(o.knn.metric);
  k.seed = o.seed;
  k.cv_seed = o.knn.cv.seed;
  k.policy = policy_of(o.evolution);
  return k;
}

kgb_pls_options pls_options_of(const PLSOptions& o) {
  kgb_pls_options p{};
  p.folds = o.cv.folds;
  p.stratified = o.cv.stratified ? 1 : 0;
  p.max_components = o.max_components;
  p.fixed_components = o.fixed_components;
  p.center = o.center ? 1 : 0;
  p.scale = o.scale ? 1 : 0;
  p.device = o.gpu_device;
  p.cv_seed = o.cv.seed;
  return p;
}

// ---------------------------------------------------------------------------
// KODAMA.matrix: the C call with every output buffer, then the result struct.
// ---------------------------------------------------------------------------
struct MatrixCall {
  const float* x = nullptr;
  int n = 0, d = 0;
  const NeighborGraph* graph = nullptr;  // caller graph (graph-input path)
};

KODAMAMatrixResult run_matrix(const MatrixCall& c, const std::vector<int>& starting, const std::vector<int>& con,
                              const std::vector<int>& fixed, const KODAMAMatrixOptions& o) {
  Timer timer;
  const int n = c.n;
  check_rows(starting, static_cast<std::size_t>(n), "starting_labels");
  check_rows(con, static_cast<std::size_t>(n), "constrain");
  check_rows(fixed, static_cast<std::size_t>(n), "fixed");
  kgb_matrix_options ko = matrix_options_of(o);
  ko.starting_labels = opt_ptr(starting);
  ko.constrain = opt_ptr(con);
  ko.fixed = opt_ptr(fixed);
  const int runs = o.runs, cycles = std::max(0, o.cycles);
  KODAMAMatrixResult r;
  r.res.assign(static_cast<std::size_t>(runs) * n, 0);
  r.acc.assign(static_cast<std::size_t>(runs), 0.0);
  r.v.assign(static_cast<std::size_t>(runs) * cycles, 0.0);
  std::vector<uint64_t> hashes(static_cast<std::size_t>(runs) * 3);
  std::vector<int32_t> counters(static_cast<std::size_t>(runs) * 8);
  std::vector<int32_t> diag(static_cast<std::size_t>(runs) * cycles * 5);
  std::vector<int32_t> pls(static_cast<std::size_t>(runs) * 2);
  const int cap = std::max(1, c.graph != nullptr ? c.graph->neighbors : o.graph_neighbors);
  std::vector<int32_t> kidx(o.materialize_graph ? static_cast<std::size_t>(n) * cap : 0);
  std::vector<float> kdist(kidx.size());
  kgb_matrix_result out{};
  out.res = r.res.data();
  out.acc = r.acc.data();
  out.v = r.v.data();
  out.run_hashes = hashes.data();
  out.run_counters = counters.data();
  out.cycle_diag = diag.data();
  out.knn_idx = kidx.empty() ? nullptr : kidx.data();
  out.knn_dist = kdist.empty() ? nullptr : kdist.data();
  out.knn_cap = cap;
  out.pls_counters = pls.data();
  if (c.graph != nullptr) {
    check(kgb_kodama_matrix_from_graph_data(c.x, n, c.d, c.graph->indices.data(), c.graph->distances.data(),
                                            c.graph->neighbors, base_of(c.graph->index_base), &ko, &out));
  } else {
    check(kgb_kodama_matrix(c.x, n, c.d, &ko, &out));
  }
  r.runs = runs;
  r.samples = n;
  r.cycles = cycles;
  r.effective_landmarks = out.effective_landmarks;
  r.n_threads = o.n_threads;
  r.backend = Backend::CUDA;
  r.graph_backend = Backend::CUDA;
  r.optimization_backend = Backend::CUDA;
  r.dissimilarity_backend = Backend::CUDA;
  r.graph_index_type = KNNIndexType::CudaExact;
  r.graph_builds = c.graph == nullptr ? 1 : 0;
  r.run_diagnostics.resize(static_cast<std::size_t>(runs));
  for (int i = 0; i < runs; ++i) {
    CoreRunDiagnostic& rd = r.run_diagnostics[static_cast<std::size_t>(i)];
    const int32_t* ct = counters.data() + 8 * static_cast<std::size_t>(i);
    rd.run = ct[0];
    rd.cycles_completed = ct[1];
    rd.transition_attempted = ct[2];
    rd.transition_accepted = ct[3];
    rd.many_to_one_attempted = ct[4];
    rd.many_to_one_accepted = ct[5];
    rd.cv_evaluations = ct[6];
    rd.pls_coarsening_attempted = pls[2 * static_cast<std::size_t>(i)];
    rd.pls_coarsening_accepted = pls[2 * static_cast<std::size_t>(i) + 1];
    rd.landmark_rows_hash = hashes[3 * static_cast<std::size_t>(i)];
    rd.initial_labels_hash = hashes[3 * static_cast<std::size_t>(i) + 1];
    rd.fold_assignments_hash = hashes[3 * static_cast<std::size_t>(i) + 2];
  }
  r.cycle_diagnostics.resize(static_cast<std::size_t>(runs) * cycles);
  for (int i = 0; i < runs; ++i) {
    for (int cy = 0; cy < cycles; ++cy) {
      const std::size_t at = static_cast<std::size_t>(i) * cycles + cy;
      const int32_t* dg = diag.data() + 5 * at;
      CoreCycleDiagnostic& cd = r.cycle_diagnostics[at];
      cd.run = r.run_diagnostics[static_cast<std::size_t>(i)].run;
      cd.cycle = cy + 1;
      cd.proposal_size = dg[0];
      cd.active_classes = dg[1];
      cd.accepted = static_cast<unsigned char>(dg[2]);
      cd.improving_acceptance = static_cast<unsigned char>(dg[3]);
      cd.temperature_acceptance = static_cast<unsigned char>(dg[4]);
    }
  }
  if (o.materialize_graph && out.knn_k > 0) {
    // one-based, as make_graph_indices_one_based leaves the reference's knn
    const int k = out.knn_k;
    r.knn.neighbors = k;
    r.knn.index_base = GraphIndexBase::One;
    r.knn.indices.resize(static_cast<std::size_t>(n) * k);
    r.knn.distances.resize(static_cast<std::size_t>(n) * k);
    for (int i = 0; i < n; ++i) {
      std::copy_n(kidx.data() + static_cast<std::size_t>(i) * cap, k,
                  r.knn.indices.data() + static_cast<std::size_t>(i) * k);
      std::copy_n(kdist.data() + static_cast<std::size_t>(i) * cap, k,
                  r.knn.distances.data() + static_cast<std::size_t>(i) * k);
    }
    r.knn_is_kodama_corrected = o.apply_kodama_dissimilarity;
  }
  // stage timings of the device call (host seconds), as the reference lists its steps
  static const char* const kSteps[] = {"total", "knn_graph", "shared_landmark_partition", "landmark_initialization",
                                       "core_evolution", "landmark_sampling", "kodama_dissimilarity", "label_coding"};
  double acc_s = 0.0;
  for (int s = 0; s < 8; ++s) {
    acc_s += s > 0 ? out.timings[s] : 0.0;
    r.timings.push_back(KODAMAStageTiming{kSteps[s], out.timings[s], s > 0 ? acc_s : out.timings[0]});
  }
  r.graph_seconds = out.timings[1];
  r.shared_landmark_partition_seconds = out.timings[2];
  r.optimization_wall_seconds = out.timings[4];
  r.dissimilarity_seconds = out.timings[6];
  r.runtime_seconds = timer.seconds();
  return r;
}

// ---------------------------------------------------------------------------
// Core*: a CoreResult with its output buffers.
// ---------------------------------------------------------------------------
struct CoreCall {
  CoreResult r;
  std::vector<uint8_t> flags;
  kgb_core_result out{};
  CoreCall(int samples, int cycles) : flags(3 * static_cast<std::size_t>(std::max(cycles, 0))) {
    r.clbest.resize(static_cast<std::size_t>(samples));
    r.cvpredbest.resize(static_cast<std::size_t>(samples));
    r.fold_assignments.resize(static_cast<std::size_t>(samples));
    const std::size_t c = static_cast<std::size_t>(std::max(cycles, 0));
    r.vect_acc.resize(c);
    r.vect_score.resize(c);
    r.proposal_size.resize(c);
    r.active_classes.resize(c);
    out.clbest = r.clbest.data();
    out.cvpredbest = r.cvpredbest.data();
    out.fold_assignments = r.fold_assignments.data();
    out.vect_acc = r.vect_acc.data();
    out.vect_score = r.vect_score.data();
    out.proposal_size = r.proposal_size.data();
    out.active_classes = r.active_classes.data();
    out.flags = flags.data();
  }
  CoreResult finish(double seconds) {
    r.accbest = out.accbest;
    r.scorebest = out.scorebest;
    const std::size_t c = r.vect_acc.size();
    r.accepted.resize(c);
    r.improving_acceptance.resize(c);
    r.temperature_acceptance.resize(c);
    for (std::size_t i = 0; i < c; ++i) {
      r.accepted[i] = flags[3 * i];
      r.improving_acceptance[i] = flags[3 * i + 1];
      r.temperature_acceptance[i] = flags[3 * i + 2];
    }
    const int32_t* k = out.counters;
    r.cycles_completed = k[0];
    r.proposals_evaluated = k[1];
    r.best_state_updates = k[2];
    r.current_state_accepts = k[3];
    r.stochastic_state_attempts = k[4];
    r.stochastic_state_accepts = k[5];
    r.current_state_rejections = k[6];
    r.coarsening_moves = k[7];
    r.absorption_moves = k[8];
    r.transition_attempted = k[9];
    r.transition_accepted = k[10];
    r.many_to_one_attempted = k[11];
    r.many_to_one_accepted = k[12];
    r.cv_evaluations = k[13];
    r.success = k[14] != 0;
    r.pls_coarsening_attempted = k[16];
    r.pls_coarsening_accepted = k[17];
    r.runtime_seconds = seconds;
    return r;
  }
};

// Per-fold accuracy, global accuracy and confusion of a cross-validation, by
// the reference's host helpers (knncv.cpp:462-480, common.cpp).
template <class Result>
void summarise(Result& r, const std::vector<int>& labels) {
  for (int fold : detail::sorted_unique_folds(r.fold_assignments)) {
    const std::vector<int> validation = detail::indices_where_fold(r.fold_assignments, fold, true);
    const std::vector<int> train = detail::indices_where_fold(r.fold_assignments, fold, false);
    r.folds.push_back(FoldResult{fold, static_cast<int>(train.size()), static_cast<int>(validation.size()),
                                 detail::accuracy_on_indices(labels, r.predicted_labels, validation)});
  }
  r.global_accuracy = detail::accuracy(labels, r.predicted_labels);
  r.confusion = detail::make_confusion(labels, r.predicted_labels);
}

PLSCVResult run_plscv(MatrixView x, const std::vector<int>& labels, const std::vector<int>& con,
                      const PLSOptions& o, bool da) {
  Timer timer;
  check_rows(labels, x.rows, "labels");
  check_rows(con, x.rows, "constrain");
  const std::vector<float> f = as_float(x);
  const kgb_pls_options po = pls_options_of(o);
  PLSCVResult r;
  r.true_labels = labels;
  r.predicted_labels.resize(x.rows);
  r.fold_assignments.resize(x.rows);
  r.accuracy_by_components.resize(static_cast<std::size_t>(std::max(1, o.max_components)));
  int32_t selected = 0;
  check((da ? kgb_plsdacv : kgb_plsldacv)(f.data(), static_cast<int32_t>(x.rows), static_cast<int32_t>(x.cols),
                                          labels.data(), opt_ptr(con), &po, r.predicted_labels.data(),
                                          r.fold_assignments.data(), &selected, r.accuracy_by_components.data()));
  r.selected_components = selected;
  summarise(r, labels);
  r.parameters.backend = Backend::CUDA;
  r.parameters.mode = da ? PLSMode::PLS_DA : PLSMode::PLS_LDA;
  r.parameters.max_components = o.max_components;
  r.parameters.selected_components = selected;
  r.parameters.fixed_components = o.fixed_components;
  r.parameters.center = o.center;
  r.parameters.scale = o.scale;
  r.parameters.gpu_device = o.gpu_device;
  r.parameters.n_threads = o.n_threads;
  r.runtime_seconds = timer.seconds();
  return r;
}

}  // namespace

namespace kodama {

KODAMAMatrixResult KODAMAMatrix_CUDA(MatrixView x, const std::vector<int>& starting_labels,
                                     const std::vector<int>& constrain, const std::vector<int>& fixed,
                                     const KODAMAMatrixOptions& options) {
  const std::vector<float> f = as_float(x);
  MatrixCall c;
  c.x = f.data();
  c.n = static_cast<int>(x.rows);
  c.d = static_cast<int>(x.cols);
  return run_matrix(c, starting_labels, constrain, fixed, options);
}

KODAMAMatrixResult KODAMAMatrixFromGraphData_CUDA(MatrixView x, const NeighborGraph& graph,
                                                  const std::vector<int>& starting_labels,
                                                  const std::vector<int>& constrain, const std::vector<int>& fixed,
                                                  const KODAMAMatrixOptions& options) {
  const std::vector<float> f = as_float(x);
  MatrixCall c;
  c.x = f.data();
  c.n = static_cast<int>(x.rows);
  c.d = static_cast<int>(x.cols);
  c.graph = &graph;
  return run_matrix(c, starting_labels, constrain, fixed, options);
}

// As the reference's CUDA variant does (kodama_matrix.cpp:4743-4762): the
// graph's Laplacian features by the reference's own host code
// (KODAMAGraphFeatures_CPU), then the graph-input path on the device with the
// features as the data.
KODAMAMatrixResult KODAMAMatrixFromGraph_CUDA(const NeighborGraph& graph, int samples,
                                              const std::vector<int>& starting_labels,
                                              const std::vector<int>& constrain, const std::vector<int>& fixed,
                                              const KODAMAMatrixOptions& options) {
  Timer feature_timer;
  std::vector<float> features = KODAMAGraphFeatures_CPU(graph, samples, options);
  const double feature_seconds = feature_timer.seconds();
  MatrixCall c;
  c.x = features.data();
  c.n = samples;
  c.d = static_cast<int>(features.size() / static_cast<std::size_t>(samples));
  c.graph = &graph;
  KODAMAMatrixResult r = run_matrix(c, starting_labels, constrain, fixed, options);
  r.graph_feature_seconds = feature_seconds;
  return r;
}

// The exact graph, materialised on the host (knn, zero-based as
// self_knn_graph leaves it).  The reference's resident handle type has its
// implementation in kodama_matrix.cpp, so the result carries no handle:
// KODAMAMatrix(x, graph) then takes the graph-input path with graph.knn.
KODAMAGraphResult KODAMAGraph_CUDA(MatrixView x, const KODAMAGraphOptions& options) {
  Timer timer;
  if (!options.samples.empty())
    throw std::invalid_argument("kodama_gb300: KODAMAGraphOptions::samples is not supported by the CUDA backend");
  const int n = static_cast<int>(x.rows), d = static_cast<int>(x.cols);
  if (n < 2 || d < 1) throw std::invalid_argument("KODAMAGraph requires at least two rows and one column.");
  const int K = std::max(1, std::min(options.neighbors, n - 1));
  const std::vector<float> f = as_float(x);
  KODAMAGraphResult g;
  g.samples = n;
  g.dimensions = d;
  g.neighbors = K;
  g.backend = Backend::CUDA;
  g.index_type = KNNIndexType::CudaExact;
  g.knn.neighbors = K;
  g.knn.index_base = GraphIndexBase::Zero;
  g.knn.indices.resize(static_cast<std::size_t>(n) * K);
  g.knn.distances.resize(static_cast<std::size_t>(n) * K);
  Timer gt;
  check(kgb_knn_graph_metric(f.data(), n, d, K, metric_of(options.metric), options.gpu_device,
                             g.knn.indices.data(), g.knn.distances.data()));
  g.graph_seconds = gt.seconds();
  g.graph_builds = 1;
  g.runtime_seconds = timer.seconds();
  return g;
}

KODAMAGraphResult KODAMAGraph_CUDA(MatrixView, MatrixView, const KODAMAGraphOptions&) {
  throw std::invalid_argument("kodama_gb300: spatial KODAMAGraph is not supported by the CUDA backend");
}

CoreResult CoreKNNGraph_CUDA(const NeighborGraph& graph, int samples, const std::vector<int>& initial_clbest,
                             const std::vector<int>& constrain, const std::vector<int>& fixed,
                             const CoreOptions& options) {
  Timer timer;
  if (initial_clbest.size() != static_cast<std::size_t>(samples))
    throw std::invalid_argument("labels size must match NeighborGraph samples.");
  check_rows(constrain, static_cast<std::size_t>(samples), "constrain");
  check_rows(fixed, static_cast<std::size_t>(samples), "fixed");
  const kgb_core_options ko = core_options_of(options);
  CoreCall c(samples, options.cycles);
  check(kgb_core_knn_graph(graph.indices.data(), graph.distances.data(), samples, graph.neighbors,
                           base_of(graph.index_base), initial_clbest.data(), opt_ptr(constrain), opt_ptr(fixed), &ko,
                           &c.out));
  return c.finish(timer.seconds());
}

CoreResult CoreKNN_CUDA(MatrixView x, const std::vector<int>& clbest, const std::vector<int>& constrain,
                        const std::vector<int>& fixed, const CoreOptions& options) {
  Timer timer;
  check_rows(clbest, x.rows, "labels");
  check_rows(constrain, x.rows, "constrain");
  check_rows(fixed, x.rows, "fixed");
  const std::vector<float> f = as_float(x);
  const kgb_core_options ko = core_options_of(options);
  CoreCall c(static_cast<int>(x.rows), options.cycles);
  check(kgb_core_knn(f.data(), static_cast<int32_t>(x.rows), static_cast<int32_t>(x.cols),
                     metric_of(options.knn.metric), clbest.data(), opt_ptr(constrain), opt_ptr(fixed), &ko, &c.out));
  return c.finish(timer.seconds());
}

CoreResult CorePLSLDA_CUDA(MatrixView x, const std::vector<int>& clbest, const std::vector<int>& constrain,
                           const std::vector<int>& fixed, const CoreOptions& options) {
  Timer timer;
  check_rows(clbest, x.rows, "labels");
  check_rows(constrain, x.rows, "constrain");
  check_rows(fixed, x.rows, "fixed");
  const std::vector<float> f = as_float(x);
  const kgb_core_options ko = core_options_of(options);
  const kgb_pls_options po = pls_options_of(static_cast<PLSOptions>(options.pls));
  CoreCall c(static_cast<int>(x.rows), options.cycles);
  check(kgb_core_plslda(f.data(), static_cast<int32_t>(x.rows), static_cast<int32_t>(x.cols), clbest.data(),
                        opt_ptr(constrain), opt_ptr(fixed), &ko, &po, &c.out));
  return c.finish(timer.seconds());
}

KNNCVResult KNNCV_CUDA(MatrixView x, const std::vector<int>& labels, const std::vector<int>& constrain,
                       const KNNOptions& options) {
  Timer timer;
  check_rows(labels, x.rows, "labels");
  check_rows(constrain, x.rows, "constrain");
  const std::vector<float> f = as_float(x);
  kgb_knn_options ko{};
  ko.folds = options.cv.folds;
  ko.stratified = options.cv.stratified ? 1 : 0;
  ko.k = options.k;
  ko.metric = metric_of(options.metric);
  ko.device = options.gpu_device;
  ko.cv_seed = options.cv.seed;
  KNNCVResult r;
  r.true_labels = labels;
  r.predicted_labels.resize(x.rows);
  r.fold_assignments.resize(x.rows);
  check(kgb_knncv(f.data(), static_cast<int32_t>(x.rows), static_cast<int32_t>(x.cols), labels.data(),
                  opt_ptr(constrain), &ko, r.predicted_labels.data(), r.fold_assignments.data()));
  summarise(r, labels);
  r.parameters.backend = Backend::CUDA;
  r.parameters.index_type = KNNIndexType::CudaExact;
  r.parameters.metric = options.metric;
  r.parameters.k = options.k;
  r.parameters.gpu_device = options.gpu_device;
  r.parameters.n_threads = options.n_threads;
  r.runtime_seconds = timer.seconds();
  return r;
}

PLSCVResult PLSLDACV_CUDA(MatrixView x, const std::vector<int>& labels, const std::vector<int>& constrain,
                          const PLSOptions& options) {
  return run_plscv(x, labels, constrain, options, false);
}

PLSCVResult PLSDACV_CUDA(MatrixView x, const std::vector<int>& labels, const std::vector<int>& constrain,
                         const PLSOptions& options) {
  return run_plscv(x, labels, constrain, options, true);
}

std::vector<int> PLSLDAPredict_CUDA(MatrixView train, const std::vector<int>& labels, MatrixView test,
                                    const PLSOptions& options) {
  check_rows(labels, train.rows, "labels");
  if (train.cols != test.cols) throw std::invalid_argument("train and test must have the same columns.");
  const std::vector<float> tr = as_float(train), te = as_float(test);
  const kgb_pls_options po = pls_options_of(options);
  std::vector<int> pred(test.rows);
  check(kgb_plslda_predict(tr.data(), static_cast<int32_t>(train.rows), static_cast<int32_t>(train.cols),
                           labels.data(), te.data(), static_cast<int32_t>(test.rows), &po, pred.data()));
  return pred;
}

namespace detail {

// The CUDA branch of KODAMADissimilarityInPlace (kodama_matrix.cpp:4412-4423):
// co-label proximity of a one-based graph, rewritten in place.
void apply_kodama_dissimilarity_cuda(NeighborGraph& graph, const std::vector<int>& res, int runs, int samples,
                                     int gpu_device, bool input_one_based_indices, bool output_one_based_indices) {
  if (!input_one_based_indices || !output_one_based_indices)
    throw std::invalid_argument("kodama_gb300: the CUDA proximity takes and returns one-based graph indices");
  check(kgb_dissimilarity_inplace(graph.indices.data(), graph.distances.data(), samples, graph.neighbors, res.data(),
                                  runs, gpu_device));
}

}  // namespace detail

}  // namespace kodama
