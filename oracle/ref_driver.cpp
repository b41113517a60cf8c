// Reference-side driver: a thin extern "C" shim over the reference's own
// public C++ API (inst/include/kodama/kodama.hpp), compiled together with the
// reference CPU sources by oracle/build_ref.sh into oracle/_ref/libkodama_ref.so.
//
// TEST INFRASTRUCTURE ONLY.  Used to pin the CPU restatement in
// oracle/kodama_oracle.cpp and to generate tests/golden fixtures.  Nothing in
// the product (kodama_gb300/) links or loads it.
//
// Every function returns 0 on success and 1 on a C++ exception, whose message
// is kept for ref_last_error().

#include "kodama/kodama.hpp"

#include <chrono>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

namespace {

thread_local std::string g_error;

// Option block layout shared with oracle/oracle.py (int32 slots).
enum Opt {
  O_RUNS = 0, O_CYCLES, O_LANDMARKS, O_SPLITTING, O_GRAPH_NEIGHBORS, O_FOLDS,
  O_KNN_K, O_THREADS, O_MATERIALIZE, O_CLASSIFIER, O_COMPONENTS, O_APPLY_DISSIM,
  O_FIRST_RUN, O_METRIC,
  O_COUNT
};

kodama::DistanceMetric metric_of(int m) {
  return m == 0 ? kodama::DistanceMetric::Cosine :
    (m == 1 ? kodama::DistanceMetric::InnerProduct : kodama::DistanceMetric::Euclidean);
}

kodama::KODAMAMatrixOptions matrix_options(const int* o, unsigned long long seed) {
  kodama::KODAMAMatrixOptions opt;
  opt.runs = o[O_RUNS];
  opt.cycles = o[O_CYCLES];
  opt.landmarks = o[O_LANDMARKS];
  opt.splitting = o[O_SPLITTING];
  opt.graph_neighbors = o[O_GRAPH_NEIGHBORS];
  opt.folds = o[O_FOLDS];
  opt.knn.k = o[O_KNN_K];
  opt.n_threads = o[O_THREADS];
  opt.materialize_graph = o[O_MATERIALIZE] != 0;
  opt.classifier = o[O_CLASSIFIER] == 1 ? kodama::CoreClassifier::PLS_LDA : kodama::CoreClassifier::KNN;
  opt.components = o[O_COMPONENTS];
  opt.apply_kodama_dissimilarity = o[O_APPLY_DISSIM] != 0;
  opt.seed = seed;
  opt.metric = metric_of(o[O_METRIC]);
  opt.backend = kodama::Backend::CPU;
  opt.compute_visual_init = false;
  opt.progress = false;
  return opt;
}

void export_matrix_result(
  const kodama::KODAMAMatrixResult& r, int n, int runs, int cycles,
  int* res, double* acc, double* v, unsigned long long* hashes, int* run_counters,
  int* cycle_diag, int* out_idx, float* out_dist, int* out_k, double* timings, int* pls_counters
) {
  std::memcpy(res, r.res.data(), sizeof(int) * static_cast<size_t>(runs) * n);
  std::memcpy(acc, r.acc.data(), sizeof(double) * runs);
  std::memcpy(v, r.v.data(), sizeof(double) * static_cast<size_t>(runs) * cycles);
  for (int i = 0; i < runs; ++i) {
    const auto& d = r.run_diagnostics[i];
    hashes[3 * i + 0] = d.landmark_rows_hash;
    hashes[3 * i + 1] = d.initial_labels_hash;
    hashes[3 * i + 2] = d.fold_assignments_hash;
    int* c = run_counters + 8 * i;
    c[0] = d.run; c[1] = d.cycles_completed; c[2] = d.transition_attempted;
    c[3] = d.transition_accepted; c[4] = d.many_to_one_attempted;
    c[5] = d.many_to_one_accepted; c[6] = d.cv_evaluations;
    c[7] = r.effective_landmarks;
    if (pls_counters) {
      pls_counters[2 * i] = d.pls_coarsening_attempted;
      pls_counters[2 * i + 1] = d.pls_coarsening_accepted;
    }
  }
  for (size_t i = 0; i < r.cycle_diagnostics.size(); ++i) {
    const auto& d = r.cycle_diagnostics[i];
    int* c = cycle_diag + 5 * i;
    c[0] = d.proposal_size; c[1] = d.active_classes; c[2] = d.accepted;
    c[3] = d.improving_acceptance; c[4] = d.temperature_acceptance;
  }
  *out_k = r.knn.neighbors;
  if (out_idx && !r.knn.indices.empty()) {
    std::memcpy(out_idx, r.knn.indices.data(), sizeof(int) * r.knn.indices.size());
    std::memcpy(out_dist, r.knn.distances.data(), sizeof(float) * r.knn.distances.size());
  }
  if (timings) {
    timings[0] = r.runtime_seconds;
    timings[1] = r.graph_seconds;
    timings[2] = r.optimization_wall_seconds;
    timings[3] = r.dissimilarity_seconds;
    timings[4] = r.shared_landmark_partition_seconds;
  }
}

}  // namespace

extern "C" {

int ref_last_error(char* buf, int len) {
  if (len <= 0) return 0;
  std::strncpy(buf, g_error.c_str(), static_cast<size_t>(len - 1));
  buf[len - 1] = '\0';
  return static_cast<int>(g_error.size());
}

// KODAMAMatrixFromGraphData_CPU (kodama.hpp:1206): data + caller graph.
int ref_kodama_matrix_graph_data_ex(
  const float* x, int n, int d, const int* gidx, const float* gdist, int gk, int index_base,
  const int* o, unsigned long long seed,
  int* res, double* acc, double* v, unsigned long long* hashes, int* run_counters,
  int* cycle_diag, int* out_idx, float* out_dist, int* out_k, double* timings, int* pls_counters,
  const int* starting, const int* constrain, const int* fixed
) {
  try {
    const std::vector<int> st = starting ? std::vector<int>(starting, starting + n) : std::vector<int>();
    const std::vector<int> co = constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    const std::vector<int> fx = fixed ? std::vector<int>(fixed, fixed + n) : std::vector<int>();
    kodama::MatrixView view(x, static_cast<size_t>(n), static_cast<size_t>(d));
    kodama::NeighborGraph g;
    g.neighbors = gk;
    g.indices.assign(gidx, gidx + static_cast<size_t>(n) * gk);
    g.distances.assign(gdist, gdist + static_cast<size_t>(n) * gk);
    g.index_base = index_base == 1 ? kodama::GraphIndexBase::One :
      (index_base == 0 ? kodama::GraphIndexBase::Zero : kodama::GraphIndexBase::Auto);
    const auto opt = matrix_options(o, seed);
    const auto t0 = std::chrono::steady_clock::now();
    const auto r = kodama::KODAMAMatrixFromGraphData_CPU(view, g, st, co, fx, opt);
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    export_matrix_result(r, n, opt.runs, opt.cycles, res, acc, v, hashes, run_counters,
                         cycle_diag, out_idx, out_dist, out_k, timings, pls_counters);
    if (timings) timings[5] = wall;
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

int ref_kodama_matrix_graph_data(
  const float* x, int n, int d, const int* gidx, const float* gdist, int gk, int index_base,
  const int* o, unsigned long long seed,
  int* res, double* acc, double* v, unsigned long long* hashes, int* run_counters,
  int* cycle_diag, int* out_idx, float* out_dist, int* out_k, double* timings, int* pls_counters
) {
  return ref_kodama_matrix_graph_data_ex(x, n, d, gidx, gdist, gk, index_base, o, seed, res, acc, v, hashes,
                                         run_counters, cycle_diag, out_idx, out_dist, out_k, timings,
                                         pls_counters, nullptr, nullptr, nullptr);
}

kodama::NeighborGraph make_graph(const int* gidx, const float* gdist, int n, int gk, int index_base) {
  kodama::NeighborGraph g;
  g.neighbors = gk;
  g.indices.assign(gidx, gidx + static_cast<size_t>(n) * gk);
  g.distances.assign(gdist, gdist + static_cast<size_t>(n) * gk);
  g.index_base = index_base == 1 ? kodama::GraphIndexBase::One :
    (index_base == 0 ? kodama::GraphIndexBase::Zero : kodama::GraphIndexBase::Auto);
  return g;
}

// KODAMAMatrix_CPU (kodama.hpp:1069): raw data, the reference's own HNSW graph.
int ref_kodama_matrix_raw(
  const float* x, int n, int d, const int* o, unsigned long long seed,
  int* res, double* acc, double* v, unsigned long long* hashes, int* run_counters,
  int* cycle_diag, int* out_idx, float* out_dist, int* out_k, double* timings, int* pls_counters
) {
  try {
    kodama::MatrixView view(x, static_cast<size_t>(n), static_cast<size_t>(d));
    const auto opt = matrix_options(o, seed);
    const auto t0 = std::chrono::steady_clock::now();
    const auto r = kodama::KODAMAMatrix_CPU(view, {}, {}, {}, opt);
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    export_matrix_result(r, n, opt.runs, opt.cycles, res, acc, v, hashes, run_counters,
                         cycle_diag, out_idx, out_dist, out_k, timings, pls_counters);
    if (timings) timings[5] = wall;
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// CoreKNNGraph_CPU (kodama.hpp:1034).
// copts: cycles, k, folds, stratified, evolutionary, guarded, absorption, adaptive
// scal_out: accbest, scorebest; int_out: counters (16).
int ref_core_knn_graph(
  const int* gidx, const float* gdist, int samples, int gk, int index_base,
  const int* labels, const int* constrain, int has_constrain, const int* fixed, int has_fixed,
  const int* copts, unsigned long long seed, unsigned long long cv_seed,
  int* clbest, int* cvpredbest, int* folds, double* vect_acc, double* vect_score,
  int* proposal_size, int* active_classes, unsigned char* flags3, double* scal_out, int* int_out
) {
  try {
    kodama::NeighborGraph g;
    g.neighbors = gk;
    g.indices.assign(gidx, gidx + static_cast<size_t>(samples) * gk);
    g.distances.assign(gdist, gdist + static_cast<size_t>(samples) * gk);
    g.index_base = index_base == 1 ? kodama::GraphIndexBase::One :
      (index_base == 0 ? kodama::GraphIndexBase::Zero : kodama::GraphIndexBase::Auto);
    kodama::CoreOptions opt;
    opt.cycles = copts[0];
    opt.knn.k = copts[1];
    opt.knn.cv.folds = copts[2];
    opt.knn.cv.stratified = copts[3] != 0;
    opt.evolutionary_search = copts[4] != 0;
    opt.guarded_diversity = copts[5] != 0;
    opt.many_to_one_absorption = copts[6] != 0;
    opt.adaptive_proposal_size = copts[7] != 0;
    opt.knn.metric = metric_of(copts[8]);
    opt.seed = seed;
    opt.knn.cv.seed = cv_seed;
    std::vector<int> lab(labels, labels + samples);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + samples) : std::vector<int>();
    std::vector<int> fix = has_fixed ? std::vector<int>(fixed, fixed + samples) : std::vector<int>();
    const auto r = kodama::CoreKNNGraph_CPU(g, samples, lab, con, fix, opt);
    std::memcpy(clbest, r.clbest.data(), sizeof(int) * samples);
    std::memcpy(cvpredbest, r.cvpredbest.data(), sizeof(int) * samples);
    std::memcpy(folds, r.fold_assignments.data(), sizeof(int) * samples);
    for (int c = 0; c < opt.cycles; ++c) {
      vect_acc[c] = r.vect_acc[c];
      vect_score[c] = r.vect_score[c];
      proposal_size[c] = r.proposal_size[c];
      active_classes[c] = r.active_classes[c];
      flags3[3 * c + 0] = r.accepted[c];
      flags3[3 * c + 1] = r.improving_acceptance[c];
      flags3[3 * c + 2] = r.temperature_acceptance[c];
    }
    scal_out[0] = r.accbest;
    scal_out[1] = r.scorebest;
    const int counters[16] = {
      r.cycles_completed, r.proposals_evaluated, r.best_state_updates, r.current_state_accepts,
      r.stochastic_state_attempts, r.stochastic_state_accepts, r.current_state_rejections,
      r.coarsening_moves, r.absorption_moves, r.transition_attempted, r.transition_accepted,
      r.many_to_one_attempted, r.many_to_one_accepted, r.cv_evaluations, r.success ? 1 : 0, 0};
    std::memcpy(int_out, counters, sizeof(counters));
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// KODAMADissimilarityInPlace (kodama.hpp:1181), one-based graph in place.
int ref_dissimilarity(int* gidx, float* gdist, int samples, int gk, const int* res, int runs, int threads) {
  try {
    kodama::NeighborGraph g;
    g.neighbors = gk;
    g.indices.assign(gidx, gidx + static_cast<size_t>(samples) * gk);
    g.distances.assign(gdist, gdist + static_cast<size_t>(samples) * gk);
    g.index_base = kodama::GraphIndexBase::One;
    std::vector<int> labels(res, res + static_cast<size_t>(runs) * samples);
    kodama::KODAMADissimilarityInPlace(g, labels, runs, samples, kodama::Backend::CPU, threads);
    std::memcpy(gidx, g.indices.data(), sizeof(int) * g.indices.size());
    std::memcpy(gdist, g.distances.data(), sizeof(float) * g.distances.size());
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// PLSLDACV_CPU (kodama.hpp:906), or PLSDACV_CPU (:899) with popts[7] != 0.
// popts: folds, stratified, max_components, fixed_components, center, scale,
// threads, da.
int ref_plsldacv(
  const float* x, int n, int d, const int* labels, const int* constrain, int has_constrain,
  const int* popts, unsigned long long cv_seed, int* predicted, int* folds,
  int* selected_components, double* accuracy_by_components, double* seconds
) {
  try {
    kodama::MatrixView view(x, static_cast<size_t>(n), static_cast<size_t>(d));
    kodama::PLSOptions opt;
    opt.cv.folds = popts[0];
    opt.cv.stratified = popts[1] != 0;
    opt.cv.seed = cv_seed;
    opt.max_components = popts[2];
    opt.fixed_components = popts[3];
    opt.center = popts[4] != 0;
    opt.scale = popts[5] != 0;
    opt.n_threads = popts[6];
    std::vector<int> lab(labels, labels + n);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    const auto t0 = std::chrono::steady_clock::now();
    const auto r = popts[7] != 0 ? kodama::PLSDACV_CPU(view, lab, con, opt) : kodama::PLSLDACV_CPU(view, lab, con, opt);
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::memcpy(predicted, r.predicted_labels.data(), sizeof(int) * n);
    std::memcpy(folds, r.fold_assignments.data(), sizeof(int) * n);
    *selected_components = r.selected_components;
    for (size_t i = 0; i < r.accuracy_by_components.size() && i < static_cast<size_t>(opt.max_components); ++i) {
      accuracy_by_components[i] = r.accuracy_by_components[i];
    }
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// PLSLDAPredict_CPU (kodama.hpp:934).
int ref_plsldapredict(
  const float* train, int n, int d, const int* labels, const float* test, int nt,
  const int* popts, int* predicted
) {
  try {
    kodama::MatrixView tv(train, static_cast<size_t>(n), static_cast<size_t>(d));
    kodama::MatrixView qv(test, static_cast<size_t>(nt), static_cast<size_t>(d));
    kodama::PLSOptions opt;
    opt.max_components = popts[2];
    opt.fixed_components = popts[3];
    opt.center = popts[4] != 0;
    opt.scale = popts[5] != 0;
    opt.n_threads = popts[6];
    std::vector<int> lab(labels, labels + n);
    const auto r = kodama::PLSLDAPredict_CPU(tv, lab, qv, opt);
    std::memcpy(predicted, r.data(), sizeof(int) * nt);
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// CorePLSLDA_CPU (kodama.hpp:986).  copts as ref_core_knn_graph plus
// copts[8] = auto_class_coarsening; popts as ref_plsldacv; int_out has 18
// counters (the 16 of ref_core_knn_graph, then pls_coarsening attempted /
// accepted).
int ref_core_plslda(
  const float* x, int samples, int d, const int* labels, const int* constrain, int has_constrain,
  const int* fixed, int has_fixed, const int* copts, const int* popts, unsigned long long seed,
  unsigned long long cv_seed, int* clbest, int* cvpredbest, int* folds, double* vect_acc, double* vect_score,
  int* proposal_size, int* active_classes, unsigned char* flags3, double* scal_out, int* int_out
) {
  try {
    kodama::MatrixView view(x, static_cast<size_t>(samples), static_cast<size_t>(d));
    kodama::CoreOptions opt;
    opt.classifier = kodama::CoreClassifier::PLS_LDA;
    opt.cycles = copts[0];
    opt.evolutionary_search = copts[4] != 0;
    opt.guarded_diversity = copts[5] != 0;
    opt.many_to_one_absorption = copts[6] != 0;
    opt.adaptive_proposal_size = copts[7] != 0;
    opt.auto_class_coarsening = copts[8] != 0;
    opt.seed = seed;
    opt.pls.cv.folds = popts[0];
    opt.pls.cv.stratified = popts[1] != 0;
    opt.pls.cv.seed = cv_seed;
    opt.pls.max_components = popts[2];
    opt.pls.fixed_components = popts[3];
    opt.pls.center = popts[4] != 0;
    opt.pls.scale = popts[5] != 0;
    opt.pls.n_threads = popts[6];
    std::vector<int> lab(labels, labels + samples);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + samples) : std::vector<int>();
    std::vector<int> fix = has_fixed ? std::vector<int>(fixed, fixed + samples) : std::vector<int>();
    const auto r = kodama::CorePLSLDA_CPU(view, lab, con, fix, opt);
    std::memcpy(clbest, r.clbest.data(), sizeof(int) * samples);
    std::memcpy(cvpredbest, r.cvpredbest.data(), sizeof(int) * samples);
    std::memcpy(folds, r.fold_assignments.data(), sizeof(int) * samples);
    for (int c = 0; c < opt.cycles; ++c) {
      vect_acc[c] = r.vect_acc[c];
      vect_score[c] = r.vect_score[c];
      proposal_size[c] = r.proposal_size[c];
      active_classes[c] = r.active_classes[c];
      flags3[3 * c + 0] = r.accepted[c];
      flags3[3 * c + 1] = r.improving_acceptance[c];
      flags3[3 * c + 2] = r.temperature_acceptance[c];
    }
    scal_out[0] = r.accbest;
    scal_out[1] = r.scorebest;
    const int counters[18] = {
      r.cycles_completed, r.proposals_evaluated, r.best_state_updates, r.current_state_accepts,
      r.stochastic_state_attempts, r.stochastic_state_accepts, r.current_state_rejections,
      r.coarsening_moves, r.absorption_moves, r.transition_attempted, r.transition_accepted,
      r.many_to_one_attempted, r.many_to_one_accepted, r.cv_evaluations, r.success ? 1 : 0, 0,
      r.pls_coarsening_attempted, r.pls_coarsening_accepted};
    std::memcpy(int_out, counters, sizeof(counters));
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// KNNCV_CPU (kodama.hpp:864): the reference's HNSW fold-wise kNN.
int ref_knncv(
  const float* x, int n, int d, const int* labels, int k, int folds, int stratified,
  int metric, unsigned long long cv_seed, int threads, int* predicted, int* fold_out, double* seconds
) {
  try {
    kodama::MatrixView view(x, static_cast<size_t>(n), static_cast<size_t>(d));
    kodama::KNNOptions opt;
    opt.k = k;
    opt.cv.folds = folds;
    opt.cv.stratified = stratified != 0;
    opt.cv.seed = cv_seed;
    opt.metric = metric == 2 ? kodama::DistanceMetric::Euclidean :
      (metric == 1 ? kodama::DistanceMetric::InnerProduct : kodama::DistanceMetric::Cosine);
    opt.n_threads = threads;
    std::vector<int> lab(labels, labels + n);
    const auto t0 = std::chrono::steady_clock::now();
    const auto r = kodama::KNNCV_CPU(view, lab, {}, opt);
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::memcpy(predicted, r.predicted_labels.data(), sizeof(int) * n);
    std::memcpy(fold_out, r.fold_assignments.data(), sizeof(int) * n);
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// CoreKNN_CPU (core.cpp:1648-1667): the reference's HNSW fold-wise kNN under
// maximize_core.  Outputs as ref_core_knn_graph.
int ref_core_knn(
  const float* x, int n, int d, int metric,
  const int* labels, const int* constrain, int has_constrain, const int* fixed, int has_fixed,
  const int* copts, unsigned long long seed, unsigned long long cv_seed,
  int* clbest, int* cvpredbest, int* folds, double* vect_acc, double* vect_score,
  int* proposal_size, int* active_classes, unsigned char* flags3, double* scal_out, int* int_out
) {
  try {
    kodama::MatrixView view(x, static_cast<size_t>(n), static_cast<size_t>(d));
    kodama::CoreOptions opt;
    opt.cycles = copts[0];
    opt.knn.k = copts[1];
    opt.knn.cv.folds = copts[2];
    opt.knn.cv.stratified = copts[3] != 0;
    opt.evolutionary_search = copts[4] != 0;
    opt.guarded_diversity = copts[5] != 0;
    opt.many_to_one_absorption = copts[6] != 0;
    opt.adaptive_proposal_size = copts[7] != 0;
    opt.knn.metric = metric == 2 ? kodama::DistanceMetric::Euclidean :
      (metric == 1 ? kodama::DistanceMetric::InnerProduct : kodama::DistanceMetric::Cosine);
    opt.knn.hnsw_tune_k = std::max(50, opt.knn.k);
    opt.seed = seed;
    opt.knn.cv.seed = cv_seed;
    std::vector<int> lab(labels, labels + n);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    std::vector<int> fix = has_fixed ? std::vector<int>(fixed, fixed + n) : std::vector<int>();
    const auto r = kodama::CoreKNN_CPU(view, lab, con, fix, opt);
    std::memcpy(clbest, r.clbest.data(), sizeof(int) * n);
    std::memcpy(cvpredbest, r.cvpredbest.data(), sizeof(int) * n);
    std::memcpy(folds, r.fold_assignments.data(), sizeof(int) * n);
    for (int c = 0; c < opt.cycles; ++c) {
      vect_acc[c] = r.vect_acc[c];
      vect_score[c] = r.vect_score[c];
      proposal_size[c] = r.proposal_size[c];
      active_classes[c] = r.active_classes[c];
      flags3[3 * c + 0] = r.accepted[c];
      flags3[3 * c + 1] = r.improving_acceptance[c];
      flags3[3 * c + 2] = r.temperature_acceptance[c];
    }
    scal_out[0] = r.accbest;
    scal_out[1] = r.scorebest;
    const int counters[16] = {
      r.cycles_completed, r.proposals_evaluated, r.best_state_updates, r.current_state_accepts,
      r.stochastic_state_attempts, r.stochastic_state_accepts, r.current_state_rejections,
      r.coarsening_moves, r.absorption_moves, r.transition_attempted, r.transition_accepted,
      r.many_to_one_attempted, r.many_to_one_accepted, r.cv_evaluations, r.success ? 1 : 0, 0};
    std::memcpy(int_out, counters, sizeof(counters));
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

}  // extern "C"
