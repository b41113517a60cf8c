/*
 * kodama_gb300 — C ABI of the GB300 (sm_103a) implementation of KODAMA.matrix's
 * label-evolution hot path.
 *
 * This is the drop-in boundary behind the reference's `backend = "cuda"` seam.
 * The reference exposes the path as C++ functions in
 * inst/include/kodama/kodama.hpp whose CUDA variants are only declared in the
 * reference tree (the kernels live outside it).  Each entry point below
 * replaces one of those declarations; a C++ `*_CUDA` definition marshals its
 * std::vector arguments into these plain pointers.
 *
 * Conventions
 *   - All pointers are HOST pointers; arrays are row-major, C-contiguous.
 *   - Every function returns KGB_OK (0) or a KGB_E* status; no C++ exception
 *     crosses the boundary.  kgb_last_error() returns the message of the last
 *     failure on the calling thread.
 *   - There is no CPU fallback: without a usable CUDA device every compute
 *     entry point returns KGB_ECUDA.
 *   - Calls may come from several host threads; each call runs on its own
 *     stream of the selected device and synchronises before returning.
 */
#ifndef KODAMA_GB300_H
#define KODAMA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KGB_OK 0
#define KGB_EINVAL 1    /* invalid argument (std::invalid_argument in the reference) */
#define KGB_ENOMEM 2    /* device allocation failed */
#define KGB_ECUDA 3     /* CUDA runtime error or no device */
#define KGB_ETIMEOUT 4  /* a bounded device-side wait gave up */
#define KGB_EINTERNAL 5 /* internal consistency check failed (std::runtime_error) */

/* DistanceMetric (kodama.hpp:27-31). */
#define KGB_METRIC_COSINE 0
#define KGB_METRIC_INNER_PRODUCT 1
#define KGB_METRIC_EUCLIDEAN 2

/* Evolution-policy switches (kodama.hpp:49-61 EvolutionPolicy). 1 = on. */
typedef struct kgb_policy {
  int32_t prediction_guidance;
  int32_t adaptive_proposal_size;
  int32_t transition_proposal;
  int32_t stochastic_acceptance;
  int32_t diversity_multiplier;
  int32_t pls_transition_coarsening;
  int32_t pls_fragmentation_penalty;
  int32_t reject_single_class;
} kgb_policy;

/* KODAMA.matrix options (kodama.hpp KODAMAMatrixOptions, the subset the
 * label-evolution path reads). */
typedef struct kgb_matrix_options {
  int32_t runs;              /* M */
  int32_t cycles;            /* Tcycle */
  int32_t landmarks;         /* default 10000 */
  int32_t splitting;         /* 0 = 100 if n < 40000 else 300 */
  int32_t graph_neighbors;   /* K, default 100 */
  int32_t folds;             /* default 5 */
  int32_t knn_k;             /* default 30 */
  int32_t classifier;        /* 0 = kNN, 1 = PLS-LDA */
  int32_t components;        /* PLS components, default 50 */
  int32_t materialize_graph; /* return the (corrected) graph */
  int32_t apply_dissimilarity;
  int32_t metric;            /* KGB_METRIC_* (KODAMAMatrixOptions::metric, default Euclidean):
                                the exact graph's metric and the vote score rule */
  int32_t device;            /* CUDA device ordinal */
  int32_t host_threads;      /* host worker threads for per-run set-up, 0 = auto */
  int32_t first_run;         /* id of the first run (default 1): runs first_run .. first_run+runs-1
                                use seeds seed+id, so runs can be sharded across devices */
  int32_t reserved;
  uint64_t seed;             /* default 1234 */
  kgb_policy policy;
  /* Learned relabelling proposal (kNN classifier): NULL = the plain proposal
   * of the reference; else the 4801 network parameters of
   * kgb_proposal_train.  No counterpart in the reference. */
  const float* proposal_weights;
  int32_t snapshot_cycle;    /* cycle whose starting state kgb_matrix_result.snapshot_* record */
  int32_t proposal_greedy;   /* 0 = sample the relabelled candidates from the network's softmax
                                (Gumbel top-k, default); 1 = take the top-scored ones */
  /* Semi-supervised inputs of KODAMAMatrix (kodama.hpp:1077-1083), n entries
   * each or NULL: starting_labels replace the k-means start (and switch the
   * evolution to greedy acceptance), constrain groups the samples (every
   * result row takes its group's majority label), fixed (non-zero) rows keep
   * their labels. */
  const int32_t* starting_labels;
  const int32_t* constrain;
  const int32_t* fixed;
} kgb_matrix_options;

/* Caller-allocated outputs of a KODAMA.matrix call. NULL = not wanted
 * (res, acc and v are required). */
typedef struct kgb_matrix_result {
  int32_t* res;              /* runs x n labels (KODAMAMatrixResult::res) */
  double* acc;               /* runs (best CV accuracy per run) */
  double* v;                 /* runs x cycles (accuracy trace) */
  uint64_t* run_hashes;      /* runs x 3: landmark rows, initial labels, folds (FNV-1a) */
  int32_t* run_counters;     /* runs x 8: run, cycles, transition att/acc, m2o att/acc, cv_evals, landmarks */
  int32_t* cycle_diag;       /* runs x cycles x 5: proposal size, active classes, accepted, improving, temperature */
  int32_t* knn_idx;          /* n x knn_cap one-based neighbour ids (materialize_graph) */
  float* knn_dist;           /* n x knn_cap */
  int32_t knn_cap;           /* capacity (columns) of knn_idx/knn_dist */
  int32_t knn_k;             /* out: columns written */
  int32_t effective_landmarks; /* out */
  double timings[8];         /* out: host seconds: total, graph, atlas, landmarks+init, evolution+projection,
                                landmark sampling (part of landmarks+init), dissimilarity+outputs,
                                label coding (part of landmarks+init) */
  double kernel_ms[8];       /* out: CUDA-event milliseconds on the call's stream: graph build, atlas k-means,
                                landmark planning + k-means, vote tables, evolution kernel, projection,
                                dissimilarity, whole device span */
  int32_t res_on_device;     /* in: 1 = `res` is a device pointer (the label matrix stays in HBM) */
  int32_t reserved;
  int32_t* pls_counters;     /* runs x 2: PLS coarsening attempted / accepted (classifier 1), or NULL */
  /* Training data for the learned proposal (kNN classifier), or NULL: the
   * state at the start of cycle opt->snapshot_cycle of every run, per
   * landmark 8 features (runs x L x 8, L = effective_landmarks) and flags
   * (runs x L): bit 0 = candidate (label differs from its CV prediction),
   * bit 1 = the run's final best label equals that prediction. */
  float* snapshot_features;
  uint8_t* snapshot_flags;
} kgb_matrix_result;

/* Replaces KODAMAMatrix_CUDA (kodama.hpp:1077-1083; dispatch
 * kodama_matrix.cpp:4521-4531): raw data in, the exact kNN graph is built on
 * the device (graph-input semantics of kodama_matrix.cpp:3528-3558). */
int kgb_kodama_matrix(const float* x, int32_t n, int32_t d, const kgb_matrix_options* opt,
                      kgb_matrix_result* out);

/* Same as kgb_kodama_matrix with `x` already resident in device memory (a
 * CUDA device pointer on opt->device).  Set out->res_on_device to keep the
 * label matrix in HBM as well.  Used to time the path without host copies. */
int kgb_kodama_matrix_resident(const float* x_device, int32_t n, int32_t d, const kgb_matrix_options* opt,
                               kgb_matrix_result* out);

/* Resident graph: KODAMAGraph_CUDA (kodama.hpp:1112-1115,
 * kodama_matrix.cpp:4057-4216) keeps the data and the exact kNN graph
 * (neighbors columns, at most n - 1) in device memory behind an opaque
 * handle, as KODAMAGraphHandle does (kodama.hpp:481-504); every call on a
 * handle holds its lock.  kgb_graph_materialize copies the graph out
 * (indices one-based, KODAMAGraphMaterialize); kgb_kodama_matrix_graph is
 * KODAMAMatrix(x, KODAMAGraphResult) (kodama.hpp:1156-1163): the
 * graph-input path on the resident data and graph, its first
 * min(neighbors, graph width) columns. */
typedef struct kgb_graph_handle kgb_graph_handle;
/* metric: KODAMAGraphOptions::metric (KGB_METRIC_*; the graph as
 * kgb_knn_graph_metric builds it).  The matrix on a handle scores neighbours
 * by its own kgb_matrix_options::metric and, like the reference's
 * graph-input path, first clamps the graph's distances at zero. */
int kgb_graph_create(const float* x, int32_t n, int32_t d, int32_t neighbors, int32_t metric, int32_t device,
                     kgb_graph_handle** out);
int kgb_graph_info(const kgb_graph_handle* graph, int32_t* n, int32_t* d, int32_t* neighbors);
int kgb_graph_materialize(kgb_graph_handle* graph, int32_t* idx, float* dist);
int kgb_kodama_matrix_graph(kgb_graph_handle* graph, const kgb_matrix_options* opt, kgb_matrix_result* out);
void kgb_graph_destroy(kgb_graph_handle* graph);

/* A batch of independent KODAMA.matrix problems (each as kgb_kodama_matrix
 * with raw data; no semi-supervised inputs, learned proposal or snapshots).
 * Not a reference entry point: the reference runs such a batch as separate
 * KODAMAMatrix calls, and every problem's result here equals that call's.
 * All problems are captured into one CUDA graph of `lanes` independent
 * chains; the schedule is autotuned on the first call for a batch shape
 * (lanes/order 0) and the graph is replayed while the shape stays. */
typedef struct kgb_matrix_problem {
  const float* x;               /* n x d, row-major, host memory */
  int32_t n, d;
  kgb_matrix_options options;   /* options.device is ignored (the batch's device is used) */
  kgb_matrix_result* result;    /* host buffers, as for kgb_kodama_matrix */
} kgb_matrix_problem;

typedef struct kgb_batch_options {
  int32_t device;
  int32_t lanes;                /* concurrent chains, 1..64; 0 = autotuned */
  int32_t order;                /* 1 = longest first to the least loaded lane, 2 = round robin; 0 = autotuned */
  int32_t reserved;
} kgb_batch_options;

typedef struct kgb_batch_report {
  int32_t lanes, order;         /* the schedule used */
  int32_t graph_nodes;          /* nodes of the captured graph */
  int32_t kernel_nodes;         /* kernel launches per replay */
  int32_t rebuilt;              /* 1 = this call captured (and possibly tuned) the graph */
  int32_t reserved;
  double device_ms;             /* CUDA-event time of the graph launch */
  double tune_ms;               /* host wall time spent autotuning in this call */
} kgb_batch_report;

int kgb_kodama_matrix_batch(const kgb_matrix_problem* problems, int32_t count, const kgb_batch_options* options,
                            kgb_batch_report* report);

/* Replaces KODAMAMatrixFromGraphData_CUDA (kodama.hpp:1215-1222,
 * kodama_matrix.cpp:4676-4699): data plus a caller graph (n x gk, indices
 * zero- or one-based: index_base 0, 1, or -1 = auto as GraphIndexBase::Auto). */
int kgb_kodama_matrix_from_graph_data(const float* x, int32_t n, int32_t d, const int32_t* gidx,
                                      const float* gdist, int32_t gk, int32_t index_base,
                                      const kgb_matrix_options* opt, kgb_matrix_result* out);

/* Core options (kodama.hpp:280-314 CoreOptions with its KNNOptions cv block). */
typedef struct kgb_core_options {
  int32_t cycles;
  int32_t k;                 /* knn.k */
  int32_t folds;             /* knn.cv.folds */
  int32_t stratified;        /* knn.cv.stratified */
  int32_t evolutionary_search;
  int32_t guarded_diversity;
  int32_t many_to_one_absorption;
  int32_t adaptive_proposal_size;
  int32_t device;
  int32_t auto_class_coarsening; /* CoreOptions::auto_class_coarsening (PLS-LDA classifier only) */
  int32_t metric;            /* knn.metric, KGB_METRIC_* (0 = cosine, the KNNOptions default):
                                the graph vote scores -(d*d) for Euclidean, 1 - d otherwise
                                (core.cpp:672-677); the raw-data search metric of kgb_core_knn is
                                its own argument */
  uint64_t seed;
  uint64_t cv_seed;
  kgb_policy policy;
} kgb_core_options;

/* CoreResult (kodama.hpp:316-349) for one problem; caller-allocated. */
typedef struct kgb_core_result {
  int32_t* clbest;           /* samples */
  int32_t* cvpredbest;       /* samples */
  int32_t* fold_assignments; /* samples */
  double* vect_acc;          /* cycles */
  double* vect_score;        /* cycles */
  int32_t* proposal_size;    /* cycles */
  int32_t* active_classes;   /* cycles */
  uint8_t* flags;            /* cycles x 3: accepted, improving, temperature */
  double accbest;            /* out */
  double scorebest;          /* out */
  int32_t counters[18];      /* out: cycles_completed, proposals_evaluated, best_state_updates,
                                current_state_accepts, stochastic_attempts, stochastic_accepts,
                                current_state_rejections, coarsening_moves, absorption_moves,
                                transition_attempted, transition_accepted, many_to_one_attempted,
                                many_to_one_accepted, cv_evaluations, success, 0,
                                pls_coarsening_attempted, pls_coarsening_accepted */
} kgb_core_result;

/* Replaces CoreKNNGraph_CUDA (kodama.hpp:1043-1050, core.cpp:1684-1700):
 * label evolution over a precomputed neighbour graph.  constrain / fixed may
 * be NULL (empty vectors in the reference). */
int kgb_core_knn_graph(const int32_t* gidx, const float* gdist, int32_t samples, int32_t gk,
                       int32_t index_base, const int32_t* labels, const int32_t* constrain,
                       const int32_t* fixed, const kgb_core_options* opt, kgb_core_result* out);

/* ---- Raw-data fold-wise kNN (KNNCV, CoreKNN) ------------------------------
 * The exact search of the CUDA backend (KNNIndexType::CudaExact): for each
 * row the k nearest rows of the other folds by the internal distance
 * (squared L2 for KGB_METRIC_EUCLIDEAN; minus the inner product for
 * KGB_METRIC_INNER_PRODUCT and for KGB_METRIC_COSINE on rows scaled to unit
 * norm), float32 chains in coordinate order, ties to the smaller row; vote
 * score = -distance (native_knn.cpp:1153).  At most 65535 rows. */

/* KNNOptions (kodama.hpp:151-166) as KNNCV uses them. */
typedef struct kgb_knn_options {
  int32_t folds;             /* cv.folds (default 10) */
  int32_t stratified;        /* cv.stratified (default 1) */
  int32_t k;                 /* default 10 */
  int32_t metric;            /* KGB_METRIC_* (default cosine) */
  int32_t device;
  int32_t reserved;
  uint64_t cv_seed;          /* cv.seed (default 1) */
} kgb_knn_options;

/* Replaces KNNCV_CUDA (kodama.hpp:871, knncv.cpp:421-488): cross-validated
 * kNN predictions of `labels` from x (n x d); majority vote by count, then
 * score sum, then the smaller label (knncv.cpp:111-131).  constrain may be
 * NULL.  predicted and fold_assignments have n entries. */
int kgb_knncv(const float* x, int32_t n, int32_t d, const int32_t* labels, const int32_t* constrain,
              const kgb_knn_options* opt, int32_t* predicted, int32_t* fold_assignments);

/* Replaces CoreKNN_CUDA (kodama.hpp:1036, core.cpp:1782-1808): label
 * evolution over the fold-wise neighbour tables of x (precompute_knn_cv_cuda,
 * core.cpp:695-782); metric is KGB_METRIC_*.  opt->k <= 32.  constrain /
 * fixed may be NULL. */
int kgb_core_knn(const float* x, int32_t n, int32_t d, int32_t metric, const int32_t* labels,
                 const int32_t* constrain, const int32_t* fixed, const kgb_core_options* opt,
                 kgb_core_result* out);

/* Batched CoreKNNGraph: `problems` independent evolutions over ONE graph
 * (labels is problems x samples; seeds[p] / cv_seeds[p] per problem; out is
 * an array of `problems` results).  All problems run in one persistent launch.
 * No single counterpart in the reference: it is the M-lane scheduler
 * (kodama_matrix.cpp:3823-3850) applied to CoreKNNGraph_CUDA. */
int kgb_core_knn_graph_batch(const int32_t* gidx, const float* gdist, int32_t samples, int32_t gk,
                             int32_t index_base, int32_t problems, const int32_t* labels,
                             const uint64_t* seeds, const uint64_t* cv_seeds,
                             const kgb_core_options* opt, kgb_core_result* out);

/* PLS options (kodama.hpp:177-188 PLSOptions / CorePLSLDAOptions). */
typedef struct kgb_pls_options {
  int32_t folds;             /* cv.folds (default 10) */
  int32_t stratified;        /* cv.stratified (default 1) */
  int32_t max_components;    /* default 10 */
  int32_t fixed_components;  /* default 0 = evaluate max_components */
  int32_t center;            /* default 1 */
  int32_t scale;             /* default 1 */
  int32_t device;
  int32_t reserved;
  uint64_t cv_seed;          /* cv.seed (default 1) */
} kgb_pls_options;

/* Replaces PLSLDACV_CUDA (kodama.hpp:920; CPU semantics of run_plscv_host,
 * plscv.cpp:2293-2507): cross-validated PLS-LDA predictions of `labels` from
 * x (n x p).  constrain may be NULL.  accuracy_by_components has
 * max_components entries (only the selected one is non-zero, as in the
 * reference). */
int kgb_plsldacv(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                 const kgb_pls_options* opt, int32_t* predicted, int32_t* fold_assignments,
                 int32_t* selected_components, double* accuracy_by_components);

/* Replaces PLSDACV_CUDA (kodama.hpp:913; CPU semantics of run_plscv_host in
 * PLSMode::PLS_DA, plscv.cpp:2428-2443): the same folds and SIMPLS fits as
 * kgb_plsldacv, with the class chosen by the one-hot least-squares
 * regression on the scores instead of LDA. */
int kgb_plsdacv(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                const kgb_pls_options* opt, int32_t* predicted, int32_t* fold_assignments,
                int32_t* selected_components, double* accuracy_by_components);

/* Replaces PLSLDAPredict_CUDA (kodama.hpp:941; CPU semantics
 * plscv.cpp:2976-3005): fit PLS-LDA on train (n x p, labels) and predict
 * test (nt x p). */
int kgb_plslda_predict(const float* train, int32_t n, int32_t p, const int32_t* labels, const float* test,
                       int32_t nt, const kgb_pls_options* opt, int32_t* predicted);

/* Replaces CorePLSLDA_CUDA (kodama.hpp:1002; CPU semantics core.cpp:1626-1646):
 * label evolution with PLSLDACV as the predictor.  Non-stratified folds only
 * (the fold cache of plscv.cpp:593-667 applies); constrain / fixed may be NULL. */
int kgb_core_plslda(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                    const int32_t* fixed, const kgb_core_options* opt, const kgb_pls_options* pls,
                    kgb_core_result* out);

/* ---- Learned relabelling proposal (no counterpart in the reference) ------
 * A 3-layer perceptron (8 -> 64 -> 64 -> 1, bfloat16 weights and
 * activations, float accumulation) that ranks the landmarks whose label
 * differs from their CV prediction; kgb_matrix_options.proposal_weights makes
 * a KODAMA.matrix run relabel the best-ranked candidates instead of uniformly
 * drawn ones, every move still accepted or rejected by the exact CV accuracy.
 * Parameters: 4801 floats (W1 8x64, b1 64, W2 64x64, b2 64, w3 64, b3). */
#define KGB_PROPOSAL_PARAMS 4801

/* Trains the network on n rows of features (n x 8) and 0/1 targets with
 * Adam (mean binary cross-entropy), minibatches drawn in a seeded order.
 * weights_init may be NULL (seeded He-uniform start).  loss_per_epoch has
 * `epochs` entries (may be NULL). */
int kgb_proposal_train(const float* features, const uint8_t* targets, int32_t n, int32_t epochs, int32_t batch,
                       float learning_rate, uint64_t seed, const float* weights_init, int32_t device,
                       float* weights_out, float* loss_per_epoch);

/* Gradient of the mean loss over n rows at `weights` (4801 floats) and the loss. */
int kgb_proposal_gradient(const float* weights, const float* features, const uint8_t* targets, int32_t n,
                          int32_t device, float* grad, float* loss);

/* Logits of n rows. */
int kgb_proposal_predict(const float* weights, const float* features, int32_t n, int32_t device, float* logits);

/* Exact kNN graph on the device: for each row its K nearest other rows by
 * squared Euclidean distance (float32, coordinate order, no FMA), ties by
 * index; idx zero-based, dist = sqrtf(d2).  Built by bf16 tensor-core
 * candidate search with an exact re-rank where it applies (KGB_KNN_*).  Replaces
 * native_cuda_exact_knn_search (native_cuda_backend.hpp:165) as used by
 * self_knn_graph (kodama_matrix.cpp:391-533). */
int kgb_knn_graph(const float* x, int32_t n, int32_t d, int32_t K, int32_t device, int32_t* idx,
                  float* dist);

/* Search methods of the exact graph (all give the same result). */
#define KGB_KNN_AUTO 0        /* the tensor-core search where it applies, else the brute force */
#define KGB_KNN_BRUTE_FORCE 1 /* float32 brute force in the canonical order */
#define KGB_KNN_TENSOR 2      /* bf16 hi+lo tensor-core candidates, canonical re-rank, per-row
                                 certificate, brute force for uncertified rows; d <= 256, K <= 96 */

/* kgb_knn_graph with an explicit method; fallback_rows (may be NULL) receives
 * how many rows were computed by the brute force. */
int kgb_knn_graph_ex(const float* x, int32_t n, int32_t d, int32_t K, int32_t device, int32_t method,
                     int32_t* idx, float* dist, int32_t* fallback_rows);

/* The exact graph under a metric (KGB_METRIC_*), as self_knn_graph
 * (kodama_matrix.cpp:391-533) asks native_cuda_exact_knn_search for it: K
 * neighbours, self excluded, ties by index.  Euclidean: kgb_knn_graph.
 * Inner product: internal distance minus the inner product (float32,
 * coordinate order, no FMA), reported 1 + internal; cosine: the same on rows
 * scaled as normalize_rows_for_cosine (kodama_matrix.cpp:155-167), reported
 * max(0, 1 + internal) (native_knn.cpp:1157-1164). */
int kgb_knn_graph_metric(const float* x, int32_t n, int32_t d, int32_t K, int32_t metric, int32_t device,
                         int32_t* idx, float* dist);

/* Replaces the Backend::CUDA branch of KODAMADissimilarityInPlace
 * (kodama.hpp:1181-1189, kodama_matrix.cpp:4383-4463): co-label proximity on a
 * one-based graph, in place.  res is runs x samples. */
int kgb_dissimilarity_inplace(int32_t* gidx, float* gdist, int32_t samples, int32_t gk,
                              const int32_t* res, int32_t runs, int32_t device);

/* The same co-label proximity as kgb_dissimilarity_inplace, on DEVICE
 * pointers (gidx, gdist: samples x gk one-based graph, rewritten in place;
 * res: runs x samples labels) and on the caller's `stream` (a cudaStream_t;
 * NULL = the legacy default stream) of `device`.  Before it returns, the call
 * synchronises that stream to read back its index-check flag, so the
 * results are complete when it returns.  It allocates no device memory: for callers that cannot call
 * cudaMalloc/cudaFree, such as a process whose caching allocator already
 * holds the GPU, or a serving loop where cudaFree would stall the device.
 * Its scratch is a fixed 16 MiB array inside the library, so
 * samples * runs <= 4194240 and gk <= 2048; larger inputs return KGB_EINVAL
 * (use kgb_dissimilarity_inplace).  Every call looks up that array's
 * address on the device; the first call on a device may load the module
 * there, so make it before any stream capture.  Calls that overlap on one
 * device share the scratch and race: serialise them.  No counterpart in the
 * reference. */
int kgb_dissimilarity_inplace_device(int32_t* gidx, float* gdist, int32_t samples, int32_t gk,
                                     const int32_t* res, int32_t runs, int32_t device, void* stream);

/* Number of kernels this library has launched since it was loaded. */
int64_t kgb_launch_count(void);

/* Message of the last failure on this thread; returns its full length. */
int kgb_last_error(char* buf, size_t len);

/* Library version string. */
const char* kgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* KODAMA_GB300_H */
