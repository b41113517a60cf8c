"""kodama_gb300: GB300-native KODAMA.matrix label-evolution hot path.

Python mirror of the reference's C++ entry points for the path
(inst/include/kodama/kodama.hpp): same names, argument meaning and error
behaviour (ValueError where the reference throws std::invalid_argument).
Every call goes through the C ABI (include/kodama_gb300.h) into the CUDA
library; there is no CPU fallback.

    KODAMA_matrix(x, graph=None, ...)   KODAMAMatrix_CUDA / KODAMAMatrixFromGraphData_CUDA
    CoreKNNGraph(graph_idx, graph_dist, labels, ...)   CoreKNNGraph_CUDA
    CoreKNNGraph_batch(...)             M independent CoreKNNGraph problems, one launch
    knn_graph(x, K)                     exact kNN graph (native_cuda_exact_knn_search)
    KODAMADissimilarityInPlace(...)     KODAMADissimilarityInPlace(backend=CUDA)
    PLSLDACV(x, labels, ...)            PLSLDACV_CUDA
    PLSLDAPredict(train, labels, test)  PLSLDAPredict_CUDA
    CorePLSLDA(x, labels, ...)          CorePLSLDA_CUDA
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

__all__ = ["KODAMADissimilarityInPlace_device", "PLSDACV", "KODAMAGraph", "KODAMA_matrix_batch", "train_proposal", "proposal_gradient", "proposal_predict", "KODAMA_matrix", "CoreKNNGraph", "CoreKNNGraph_batch", "knn_graph",
           "KODAMADissimilarityInPlace", "PLSLDACV", "PLSLDAPredict", "CorePLSLDA", "PLSCVResult", "MatrixResult", "CoreResult", "EvolutionPolicy",
           "library_path", "version", "launch_count"]


def library_path() -> str:
    return N.LIB_PATH


def version() -> str:
    return N.load().kgb_version().decode()


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class EvolutionPolicy:
    """EvolutionPolicy (kodama.hpp:49-61); from_name mirrors core.cpp:35-61."""
    prediction_guidance: bool = True
    adaptive_proposal_size: bool = True
    transition_proposal: bool = True
    stochastic_acceptance: bool = True
    diversity_multiplier: bool = True
    pls_transition_coarsening: bool = True
    pls_fragmentation_penalty: bool = True
    reject_single_class: bool = True

    @staticmethod
    def from_name(name: str) -> "EvolutionPolicy":
        p = EvolutionPolicy()
        flag = {"no_prediction_guidance": "prediction_guidance",
                "fixed_proposal_budget": "adaptive_proposal_size",
                "no_transition_proposal": "transition_proposal",
                "greedy_acceptance": "stochastic_acceptance",
                "raw_cv_score": "diversity_multiplier",
                "no_pls_transition_coarsening": "pls_transition_coarsening",
                "no_pls_fragmentation_penalty": "pls_fragmentation_penalty"}
        if name == "full":
            return p
        if name not in flag:
            raise ValueError(
                f"Unknown evolution policy '{name}'. Expected full, no_prediction_guidance, "
                "fixed_proposal_budget, no_transition_proposal, greedy_acceptance, raw_cv_score, "
                "no_pls_transition_coarsening, or no_pls_fragmentation_penalty.")
        setattr(p, flag[name], False)
        return p

    def _c(self) -> N.Policy:
        return N.Policy(*[int(getattr(self, f)) for f, _ in N.Policy._fields_])


@dataclass
class MatrixResult:
    """KODAMAMatrixResult (kodama.hpp:604-682): the fields of the path."""
    res: np.ndarray
    acc: np.ndarray
    v: np.ndarray
    run_hashes: np.ndarray
    run_counters: np.ndarray
    cycle_diag: np.ndarray
    knn_idx: np.ndarray | None
    knn_dist: np.ndarray | None
    effective_landmarks: int
    timings: dict = field(default_factory=dict)
    kernel_ms: dict = field(default_factory=dict)
    pls_counters: np.ndarray | None = None   # (runs, 2): PLS coarsening attempted / accepted
    snapshot_features: np.ndarray | None = None  # (runs, L, 8) learned-proposal training features
    snapshot_flags: np.ndarray | None = None     # (runs, L): bit 0 candidate, bit 1 target


_TIMING_NAMES = ("total", "knn_graph", "shared_landmark_partition", "landmark_initialization",
                 "core_evolution", "landmark_sampling", "kodama_dissimilarity", "label_coding")
_KERNEL_NAMES = ("knn_graph", "atlas_kmeans", "landmark_kmeans", "vote_tables", "evolution",
                 "projection", "dissimilarity", "device_span")


def _matrix_options(runs, cycles, landmarks, splitting, graph_neighbors, folds, knn_k, seed,
                    materialize_graph, apply_dissimilarity, device, host_threads, policy, first_run=1,
                    classifier=0, components=50, metric=2):
    pol = policy if isinstance(policy, EvolutionPolicy) else EvolutionPolicy.from_name(policy or "full")
    return N.MatrixOptions(runs=runs, cycles=cycles, landmarks=landmarks, splitting=splitting,
                           graph_neighbors=graph_neighbors, folds=folds, knn_k=knn_k,
                           classifier=classifier, components=components,
                           materialize_graph=int(materialize_graph),
                           apply_dissimilarity=int(apply_dissimilarity), metric=metric, device=device,
                           host_threads=host_threads, first_run=first_run, reserved=0, seed=seed,
                           policy=pol._c())


class KODAMAGraph:
    """KODAMAGraph with backend="cuda" (kgb_graph_create): the data and its
    exact kNN graph kept resident on the device; ``matrix`` runs
    KODAMA.matrix on them without rebuilding the graph (KODAMAMatrix(x,
    KODAMAGraphResult)).  Use as a context manager or call ``close``."""

    def __init__(self, x, neighbors=100, device=0, metric="euclidean"):
        xa = np.ascontiguousarray(x, dtype=np.float32)
        if xa.ndim != 2:
            raise ValueError("x must be a 2-D matrix")
        self.n, self.d = xa.shape
        self.device = device
        h = ctypes.c_void_p()
        N.check(N.load().kgb_graph_create(_ptr(xa), self.n, self.d, neighbors, _metric(metric), device,
                                          ctypes.byref(h)))
        self._h = h
        k = ctypes.c_int32()
        N.check(N.load().kgb_graph_info(self._h, None, None, ctypes.byref(k)))
        self.neighbors = k.value

    def graph(self):
        """The resident graph: (indices one-based, distances), n x neighbors."""
        idx = np.zeros((self.n, self.neighbors), np.int32)
        dist = np.zeros((self.n, self.neighbors), np.float32)
        N.check(N.load().kgb_graph_materialize(self._h, _ptr(idx), _ptr(dist)))
        return idx, dist

    def matrix(self, **kw) -> "MatrixResult":
        """KODAMA_matrix on the resident data and graph (same keywords as
        KODAMA_matrix, without the data and graph arguments)."""
        if self._h is None:
            raise ValueError("the graph handle is closed")
        return KODAMA_matrix(None, _handle=self, **kw)

    def close(self):
        if self._h is not None:
            N.load().kgb_graph_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def KODAMA_matrix(x, graph=None, *, runs=100, cycles=20, landmarks=10000, splitting=0,
                  graph_neighbors=100, folds=5, knn_k=30, seed=1234, materialize_graph=False,
                  apply_dissimilarity=True, index_base=-1, device=0, host_threads=0,
                  policy="full", res_out=None, first_run=1, classifier="knn",
                  components=50, proposal_weights=None, snapshot_cycle=None,
                  proposal_greedy=False, starting_labels=None, constrain=None,
                  fixed=None, _handle=None, metric="euclidean") -> MatrixResult:
    """KODAMA.matrix on the GPU with the kNN (``classifier="knn"``) or PLS-LDA
    (``classifier="pls"``, ``components`` latent components) classifier.
    ``proposal_weights`` (the 4801 parameters of ``train_proposal``) selects
    the learned relabelling proposal, which samples the relabelled candidates
    from the network's softmax (``proposal_greedy=True``: takes the
    top-scored ones); ``snapshot_cycle`` records its training data
    (``snapshot_features`` / ``snapshot_flags``) at that cycle.

    Semi-supervised inputs (n integers each, KODAMAMatrix's starting_labels /
    constrain / fixed, kodama.hpp:1077-1083): ``starting_labels`` replace the
    k-means start and make the evolution greedy, ``constrain`` groups the
    samples (every result row takes its group's majority label), non-zero
    ``fixed`` rows keep their labels.

    ``graph`` = (indices, distances) of shape (n, K) runs the graph-input path
    (KODAMAMatrixFromGraphData_CUDA); without it the exact kNN graph is built
    on the device (KODAMAMatrix_CUDA with exact-graph semantics).
    ``x`` may also be a CUDA torch tensor (float32, contiguous): the data is
    then read in place from HBM (kgb_kodama_matrix_resident); pass
    ``res_out`` (a CUDA int32 tensor of shape (runs, n)) to keep the label
    matrix on the device too.
    ``metric`` ("euclidean", "cosine", "inner_product") is
    KODAMAMatrixOptions::metric: the metric of the exact graph built from raw
    data and the vote score rule (-(d*d) for Euclidean, 1 - d otherwise).
    Defaults are those of KODAMAMatrixOptions (kodama.hpp:535-570).
    """
    x_dev = None
    if _handle is not None:
        n, d = _handle.n, _handle.d
    elif hasattr(x, "is_cuda") and x.is_cuda:
        if graph is not None:
            raise ValueError("device-resident input is supported for raw data only")
        x_dev = x
        n, d = int(x.shape[0]), int(x.shape[1])
    else:
        x = np.ascontiguousarray(x, dtype=np.float32)
        if x.ndim != 2:
            raise ValueError("x must be a 2-D matrix")
        n, d = x.shape
    cls = {"knn": 0, "pls": 1, "pls-lda": 1, 0: 0, 1: 1}.get(classifier)
    if cls is None:
        raise ValueError("Unsupported KODAMA.matrix classifier.")
    opt = _matrix_options(runs, cycles, landmarks, splitting, graph_neighbors, folds, knn_k, seed,
                          materialize_graph, apply_dissimilarity, device, host_threads, policy, first_run,
                          cls, components, _metric(metric))
    res = np.zeros((runs, n), np.int32)
    acc = np.zeros(runs, np.float64)
    v = np.zeros((runs, max(cycles, 0)), np.float64)
    hashes = np.zeros((runs, 3), np.uint64)
    counters = np.zeros((runs, 8), np.int32)
    cdiag = np.zeros((runs, max(cycles, 0), 5), np.int32)
    plsc = np.zeros((runs, 2), np.int32)
    cap = max(1, graph_neighbors if graph is None else np.asarray(graph[0]).shape[1])
    kidx = np.zeros((n, cap), np.int32) if materialize_graph else None
    kdist = np.zeros((n, cap), np.float32) if materialize_graph else None
    out = N.MatrixResult()
    if res_out is not None:
        if tuple(res_out.shape) != (runs, n) or not res_out.is_cuda:
            raise ValueError("res_out must be a CUDA int32 tensor of shape (runs, n)")
        out.res = ctypes.cast(ctypes.c_void_p(res_out.data_ptr()), ctypes.POINTER(ctypes.c_int32))
        out.res_on_device = 1
    else:
        out.res = res.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    out.acc = acc.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    out.v = v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    out.run_hashes = hashes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    out.run_counters = counters.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    out.cycle_diag = cdiag.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    out.pls_counters = plsc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    wts = None
    if proposal_weights is not None:
        wts = np.ascontiguousarray(proposal_weights, dtype=np.float32)
        if wts.shape != (N.PROPOSAL_PARAMS,):
            raise ValueError(f"proposal_weights must hold {N.PROPOSAL_PARAMS} floats")
        opt.proposal_weights = wts.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        opt.proposal_greedy = 1 if proposal_greedy else 0
    semi = {}
    for name, vec, msg in (
            ("starting_labels", starting_labels, "starting_labels size must match number of rows."),
            ("constrain", constrain, "constrain size must be zero or match number of rows."),
            ("fixed", fixed, "fixed size must be zero or match number of rows.")):
        if vec is None or len(vec) == 0:
            continue
        a = np.ascontiguousarray(vec, dtype=np.int32)
        if a.shape != (n,):
            raise ValueError(msg)
        semi[name] = a
        setattr(opt, name, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    snap_f = snap_g = None
    if snapshot_cycle is not None:
        if not 0 <= snapshot_cycle < cycles:
            raise ValueError("snapshot_cycle must lie in [0, cycles)")
        opt.snapshot_cycle = int(snapshot_cycle)
        snap_f = np.zeros(runs * n * 8, np.float32)  # the landmarks are fewer than n
        snap_g = np.zeros(runs * n, np.uint8)
        out.snapshot_features = snap_f.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        out.snapshot_flags = snap_g.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    if materialize_graph:
        out.knn_idx = kidx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        out.knn_dist = kdist.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    out.knn_cap = cap
    lib = N.load()
    if _handle is not None:
        rc = lib.kgb_kodama_matrix_graph(_handle._h, ctypes.byref(opt), ctypes.byref(out))
    elif x_dev is not None:
        rc = lib.kgb_kodama_matrix_resident(ctypes.c_void_p(x_dev.data_ptr()), n, d, ctypes.byref(opt),
                                            ctypes.byref(out))
    elif graph is None:
        rc = lib.kgb_kodama_matrix(_ptr(x), n, d, ctypes.byref(opt), ctypes.byref(out))
    else:
        gi = np.ascontiguousarray(graph[0], dtype=np.int32)
        gd = np.ascontiguousarray(graph[1], dtype=np.float32)
        if gi.shape != gd.shape or gi.shape[0] != n:
            raise ValueError("NeighborGraph indices/distances size must equal samples * neighbors.")
        rc = lib.kgb_kodama_matrix_from_graph_data(_ptr(x), n, d, _ptr(gi), _ptr(gd), gi.shape[1],
                                                   index_base, ctypes.byref(opt), ctypes.byref(out))
    N.check(rc)
    k = out.knn_k
    return MatrixResult(
        res=res, acc=acc, v=v, run_hashes=hashes, run_counters=counters, cycle_diag=cdiag,
        knn_idx=kidx[:, :k].copy() if (materialize_graph and k) else None,
        knn_dist=kdist[:, :k].copy() if (materialize_graph and k) else None,
        effective_landmarks=out.effective_landmarks,
        timings=dict(zip(_TIMING_NAMES, list(out.timings))),
        kernel_ms=dict(zip(_KERNEL_NAMES, list(out.kernel_ms))), pls_counters=plsc,
        snapshot_features=None if snap_f is None else
        snap_f[: runs * out.effective_landmarks * 8].reshape(runs, out.effective_landmarks, 8),
        snapshot_flags=None if snap_g is None else
        snap_g[: runs * out.effective_landmarks].reshape(runs, out.effective_landmarks))


@dataclass
class BatchReport:
    """Schedule and timing of one kgb_kodama_matrix_batch call."""
    lanes: int
    order: int
    graph_nodes: int
    kernel_nodes: int
    rebuilt: bool
    device_ms: float
    tune_ms: float


def KODAMA_matrix_batch(problems, *, runs=100, cycles=20, landmarks=10000, splitting=0, graph_neighbors=100,
                        folds=5, knn_k=30, seed=1234, components=50, policy="full", device=0, lanes=0,
                        order=0, materialize_graph=False, apply_dissimilarity=True):
    """Independent KODAMA.matrix problems in one captured CUDA graph.

    ``problems``: list of dicts with ``x`` (n x d float32) and optionally
    ``classifier`` ("knn" / "pls") and any per-problem override of the
    keyword options.  Returns (list of MatrixResult, BatchReport); each result
    equals KODAMA_matrix on that problem alone.  ``lanes`` / ``order`` fix the
    schedule (0 = autotuned on the first call for this batch shape)."""
    count = len(problems)
    if count < 1:
        raise ValueError("a batch needs at least one problem")
    base = dict(runs=runs, cycles=cycles, landmarks=landmarks, splitting=splitting,
                graph_neighbors=graph_neighbors, folds=folds, knn_k=knn_k, seed=seed, components=components)
    arr = (N.MatrixProblem * count)()
    keep, outs = [], []
    for i, pr in enumerate(problems):
        x = np.ascontiguousarray(pr["x"], dtype=np.float32)
        if x.ndim != 2:
            raise ValueError("x must be a 2-D matrix")
        n, d = x.shape
        kw = {k: pr.get(k, v) for k, v in base.items()}
        cls = {"knn": 0, "pls": 1, "pls-lda": 1, 0: 0, 1: 1}.get(pr.get("classifier", "knn"))
        if cls is None:
            raise ValueError("Unsupported KODAMA.matrix classifier.")
        opt = _matrix_options(kw["runs"], kw["cycles"], kw["landmarks"], kw["splitting"], kw["graph_neighbors"],
                              kw["folds"], kw["knn_k"], kw["seed"], materialize_graph, apply_dissimilarity,
                              device, 0, policy, 1, cls, kw["components"], _metric(pr.get("metric", "euclidean")))
        M, T = kw["runs"], kw["cycles"]
        b = dict(x=x, res=np.zeros((M, n), np.int32), acc=np.zeros(M, np.float64),
                 v=np.zeros((M, max(T, 0)), np.float64), hashes=np.zeros((M, 3), np.uint64),
                 counters=np.zeros((M, 8), np.int32), cdiag=np.zeros((M, max(T, 0), 5), np.int32),
                 plsc=np.zeros((M, 2), np.int32))
        cap = max(1, min(kw["graph_neighbors"] if kw["graph_neighbors"] > 0 else 100, n))
        if materialize_graph:
            b["kidx"] = np.zeros((n, cap), np.int32)
            b["kdist"] = np.zeros((n, cap), np.float32)
        out = N.MatrixResult()
        out.res = b["res"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        out.acc = b["acc"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        out.v = b["v"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        out.run_hashes = b["hashes"].ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        out.run_counters = b["counters"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        out.cycle_diag = b["cdiag"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        out.pls_counters = b["plsc"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        if materialize_graph:
            out.knn_idx = b["kidx"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            out.knn_dist = b["kdist"].ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        out.knn_cap = cap
        b["out"] = out
        arr[i].x = x.ctypes.data
        arr[i].n = n
        arr[i].d = d
        arr[i].options = opt
        arr[i].result = ctypes.pointer(out)
        keep.append(b)
    bo = N.BatchOptions(device=device, lanes=lanes, order=order, reserved=0)
    rep = N.BatchReport()
    N.check(N.load().kgb_kodama_matrix_batch(arr, count, ctypes.byref(bo), ctypes.byref(rep)))
    for b in keep:
        out = b["out"]
        k = out.knn_k
        outs.append(MatrixResult(
            res=b["res"], acc=b["acc"], v=b["v"], run_hashes=b["hashes"], run_counters=b["counters"],
            cycle_diag=b["cdiag"],
            knn_idx=b["kidx"][:, :k].copy() if (materialize_graph and k) else None,
            knn_dist=b["kdist"][:, :k].copy() if (materialize_graph and k) else None,
            effective_landmarks=out.effective_landmarks,
            timings=dict(zip(_TIMING_NAMES, list(out.timings))),
            kernel_ms=dict(zip(_KERNEL_NAMES, list(out.kernel_ms))), pls_counters=b["plsc"],
            snapshot_features=None, snapshot_flags=None))
    return outs, BatchReport(lanes=rep.lanes, order=rep.order, graph_nodes=rep.graph_nodes,
                             kernel_nodes=rep.kernel_nodes, rebuilt=bool(rep.rebuilt), device_ms=rep.device_ms,
                             tune_ms=rep.tune_ms)


def launch_count() -> int:
    """Kernels launched by the CUDA library since it was loaded."""
    return int(N.load().kgb_launch_count())


@dataclass
class CoreResult:
    """CoreResult (kodama.hpp:316-349)."""
    clbest: np.ndarray
    cvpredbest: np.ndarray
    fold_assignments: np.ndarray
    vect_acc: np.ndarray
    vect_score: np.ndarray
    proposal_size: np.ndarray
    active_classes: np.ndarray
    flags: np.ndarray
    accbest: float
    scorebest: float
    counters: np.ndarray


def _core_options(cycles, k, folds, stratified, evolutionary_search, guarded_diversity,
                  many_to_one_absorption, adaptive_proposal_size, seed, cv_seed, device, policy,
                  metric="cosine"):
    pol = policy if isinstance(policy, EvolutionPolicy) else EvolutionPolicy.from_name(policy or "full")
    return N.CoreOptions(cycles=cycles, k=k, folds=folds, stratified=int(stratified),
                         evolutionary_search=int(evolutionary_search),
                         guarded_diversity=int(guarded_diversity),
                         many_to_one_absorption=int(many_to_one_absorption),
                         adaptive_proposal_size=int(adaptive_proposal_size), device=device,
                         auto_class_coarsening=0, metric=_metric(metric), seed=seed, cv_seed=cv_seed,
                         policy=pol._c())


def _alloc_core(samples, cycles):
    bufs = dict(clbest=np.zeros(samples, np.int32), cvpredbest=np.zeros(samples, np.int32),
                fold_assignments=np.zeros(samples, np.int32),
                vect_acc=np.zeros(max(cycles, 1), np.float64),
                vect_score=np.zeros(max(cycles, 1), np.float64),
                proposal_size=np.zeros(max(cycles, 1), np.int32),
                active_classes=np.zeros(max(cycles, 1), np.int32),
                flags=np.zeros((max(cycles, 1), 3), np.uint8))
    r = N.CoreResult()
    for name, arr in bufs.items():
        ctype = dict(N.CoreResult._fields_)[name]
        setattr(r, name, arr.ctypes.data_as(ctype))
    return r, bufs


def _wrap_core(r, bufs, cycles):
    return CoreResult(
        clbest=bufs["clbest"], cvpredbest=bufs["cvpredbest"], fold_assignments=bufs["fold_assignments"],
        vect_acc=bufs["vect_acc"][:cycles], vect_score=bufs["vect_score"][:cycles],
        proposal_size=bufs["proposal_size"][:cycles], active_classes=bufs["active_classes"][:cycles],
        flags=bufs["flags"][:cycles], accbest=r.accbest, scorebest=r.scorebest,
        counters=np.array(list(r.counters), np.int32))


def CoreKNNGraph_batch(graph_idx, graph_dist, labels, seeds, cv_seeds, *, cycles=100, k=30,
                       folds=10, stratified=True, evolutionary_search=False,
                       guarded_diversity=False, many_to_one_absorption=False,
                       adaptive_proposal_size=True, index_base=-1, device=0,
                       policy="full", metric="cosine") -> list[CoreResult]:
    """`len(seeds)` independent CoreKNNGraph evolutions over one graph in one launch.
    ``metric`` is KNNOptions::metric (default cosine, as in the reference):
    the vote scores -(d*d) for "euclidean", 1 - d otherwise."""
    gi = np.ascontiguousarray(graph_idx, dtype=np.int32)
    gd = np.ascontiguousarray(graph_dist, dtype=np.float32)
    samples, gk = gi.shape
    lab = np.ascontiguousarray(labels, dtype=np.int32).reshape(-1, samples)
    problems = lab.shape[0]
    s = np.ascontiguousarray(seeds, dtype=np.uint64)
    cs = np.ascontiguousarray(cv_seeds, dtype=np.uint64)
    if s.shape[0] != problems or cs.shape[0] != problems:
        raise ValueError("one seed and one cv seed per problem")
    opt = _core_options(cycles, k, folds, stratified, evolutionary_search, guarded_diversity,
                        many_to_one_absorption, adaptive_proposal_size, 0, 0, device, policy, metric)
    arr = (N.CoreResult * problems)()
    keep = []
    for p in range(problems):
        r, bufs = _alloc_core(samples, cycles)
        arr[p] = r
        keep.append(bufs)
    rc = N.load().kgb_core_knn_graph_batch(_ptr(gi), _ptr(gd), samples, gk, index_base, problems,
                                           _ptr(lab), _ptr(s), _ptr(cs), ctypes.byref(opt), arr)
    N.check(rc)
    return [_wrap_core(arr[p], keep[p], cycles) for p in range(problems)]


def CoreKNNGraph(graph_idx, graph_dist, labels, *, constrain=None, fixed=None, cycles=100, k=30,
                 folds=10, stratified=True, evolutionary_search=False, guarded_diversity=False,
                 many_to_one_absorption=False, adaptive_proposal_size=True, seed=1, cv_seed=1,
                 index_base=-1, device=0, policy="full", metric="cosine") -> CoreResult:
    """CoreKNNGraph_CUDA (kodama.hpp:1043): label evolution over a neighbour graph.
    ``metric`` is KNNOptions::metric (default cosine, as in the reference):
    the vote scores -(d*d) for "euclidean", 1 - d otherwise (core.cpp:672-677)."""
    gi = np.ascontiguousarray(graph_idx, dtype=np.int32)
    gd = np.ascontiguousarray(graph_dist, dtype=np.float32)
    samples, gk = gi.shape
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    if lab.shape[0] != samples:
        raise ValueError("initial labels size must match NeighborGraph samples.")
    con = None if constrain is None else np.ascontiguousarray(constrain, dtype=np.int32)
    fix = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.int32)
    opt = _core_options(cycles, k, folds, stratified, evolutionary_search, guarded_diversity,
                        many_to_one_absorption, adaptive_proposal_size, seed, cv_seed, device, policy, metric)
    r, bufs = _alloc_core(samples, cycles)
    rc = N.load().kgb_core_knn_graph(_ptr(gi), _ptr(gd), samples, gk, index_base, _ptr(lab),
                                     _ptr(con), _ptr(fix), ctypes.byref(opt), ctypes.byref(r))
    N.check(rc)
    return _wrap_core(r, bufs, cycles)


@dataclass
class FoldResult:
    """FoldResult (kodama.hpp:222-227)."""
    fold: int
    n_train: int
    n_validation: int
    accuracy: float


@dataclass
class ConfusionMatrix:
    """ConfusionMatrix (kodama.hpp:229-237): counts[truth, predicted] over the
    sorted distinct true labels; predictions outside them are not counted."""
    labels: np.ndarray
    counts: np.ndarray


@dataclass
class KNNCVResult:
    """The KNNCVResult fields of the path (kodama.hpp:256-266)."""
    predicted_labels: np.ndarray
    true_labels: np.ndarray
    fold_assignments: np.ndarray
    folds: list
    global_accuracy: float
    confusion: ConfusionMatrix


def _metric(metric) -> int:
    if isinstance(metric, str):
        if metric not in N.METRICS:
            raise ValueError(f"unknown metric {metric!r}")
        return N.METRICS[metric]
    return int(metric)


def _cv_summary(truth, pred, folds):
    """Fold results, global accuracy and confusion (knncv.cpp:462-485,
    common.cpp:226-255)."""
    out = []
    for f in np.unique(folds):
        val = folds == f
        out.append(FoldResult(int(f), int((~val).sum()), int(val.sum()), float(np.mean(truth[val] == pred[val]))))
    labels = np.unique(truth)
    pos = {int(v): i for i, v in enumerate(labels)}
    counts = np.zeros((len(labels), len(labels)), np.int64)
    for t, p in zip(truth.tolist(), pred.tolist()):
        if p in pos:
            counts[pos[t], pos[p]] += 1
    return out, float(np.mean(truth == pred)), ConfusionMatrix(labels, counts)


def KNNCV(x, labels, *, constrain=None, folds=10, stratified=True, seed=1, k=10, metric="cosine",
          device=0) -> KNNCVResult:
    """KNNCV with backend "cuda" (R/kodama.R:160, knncv.cpp:421-488): fold-wise
    exact kNN votes; ``seed`` is cv.seed."""
    xa = np.ascontiguousarray(x, dtype=np.float32)
    if xa.ndim != 2:
        raise ValueError("x must be a 2-D matrix")
    n, d = xa.shape
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    if lab.shape[0] != n:
        raise ValueError("labels size must match number of rows.")
    con = None if constrain is None else np.ascontiguousarray(constrain, dtype=np.int32)
    if con is not None and con.shape[0] != n:
        raise ValueError("constrain size must be zero or match number of rows.")
    pred = np.zeros(n, np.int32)
    fo = np.zeros(n, np.int32)
    opt = N.KnnOptions(folds=folds, stratified=int(stratified), k=k, metric=_metric(metric), device=device,
                       reserved=0, cv_seed=seed)
    N.check(N.load().kgb_knncv(_ptr(xa), n, d, _ptr(lab), _ptr(con), ctypes.byref(opt), _ptr(pred), _ptr(fo)))
    fr, acc, cm = _cv_summary(lab, pred, fo)
    return KNNCVResult(pred, lab, fo, fr, acc, cm)


def CoreKNN(x, labels, *, constrain=None, fixed=None, cycles=100, folds=10, stratified=True, seed=1, k=30,
            metric="euclidean", evolutionary_search=False, guarded_diversity=False,
            many_to_one_absorption=False, adaptive_proposal_size=True, cv_seed=None, device=0,
            policy="full") -> CoreResult:
    """CoreKNN with backend "cuda" (R/kodama.R:266, core.cpp:1782-1808): label
    evolution over the fold-wise exact kNN tables of x.  ``seed`` seeds both
    the evolution and the folds unless ``cv_seed`` is given (core_impl_cpp,
    kodama_r.cpp:1140-1145)."""
    xa = np.ascontiguousarray(x, dtype=np.float32)
    if xa.ndim != 2:
        raise ValueError("x must be a 2-D matrix")
    n, d = xa.shape
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    if lab.shape[0] != n:
        raise ValueError("labels size must match number of rows.")
    con = None if constrain is None else np.ascontiguousarray(constrain, dtype=np.int32)
    fix = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.int32)
    if con is not None and con.shape[0] != n:
        raise ValueError("constrain size must be zero or match number of rows.")
    if fix is not None and fix.shape[0] != n:
        raise ValueError("fixed size must be zero or match number of rows.")
    opt = _core_options(cycles, k, folds, stratified, evolutionary_search, guarded_diversity,
                        many_to_one_absorption, adaptive_proposal_size, seed,
                        seed if cv_seed is None else cv_seed, device, policy)
    r, bufs = _alloc_core(n, cycles)
    N.check(N.load().kgb_core_knn(_ptr(xa), n, d, _metric(metric), _ptr(lab), _ptr(con), _ptr(fix),
                                  ctypes.byref(opt), ctypes.byref(r)))
    return _wrap_core(r, bufs, cycles)


KNN_METHODS = {"auto": 0, "brute_force": 1, "tensor": 2}


def knn_graph(x, K: int, *, device: int = 0, method: str = "auto", return_fallback: bool = False,
              metric: str = "euclidean"):
    """Exact kNN graph: zero-based (n, K) indices and the reference's reported
    distances (sqrt for "euclidean"; 1 - <x,y> for "inner_product";
    max(0, 1 - cos) for "cosine").  ``method`` ("auto", "brute_force" or
    "tensor", same result) and ``return_fallback`` (rows computed by the
    brute force) apply to the Euclidean search."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    idx = np.zeros((n, K), np.int32)
    dist = np.zeros((n, K), np.float32)
    if _metric(metric) != N.METRICS["euclidean"]:
        N.check(N.load().kgb_knn_graph_metric(_ptr(x), n, d, K, _metric(metric), device, _ptr(idx), _ptr(dist)))
        return (idx, dist, n) if return_fallback else (idx, dist)
    fb = ctypes.c_int32(0)
    N.check(N.load().kgb_knn_graph_ex(_ptr(x), n, d, K, device, KNN_METHODS[method], _ptr(idx), _ptr(dist),
                                      ctypes.byref(fb)))
    return (idx, dist, int(fb.value)) if return_fallback else (idx, dist)


def KODAMADissimilarityInPlace(graph_idx: np.ndarray, graph_dist: np.ndarray, run_labels: np.ndarray,
                               *, device: int = 0) -> None:
    """Co-label proximity correction of a one-based graph, in place."""
    if graph_idx.dtype != np.int32 or graph_dist.dtype != np.float32:
        raise ValueError("graph arrays must be int32 / float32")
    if not (graph_idx.flags.c_contiguous and graph_dist.flags.c_contiguous):
        raise ValueError("graph arrays must be C-contiguous")
    res = np.ascontiguousarray(run_labels, dtype=np.int32)
    samples, gk = graph_idx.shape
    N.check(N.load().kgb_dissimilarity_inplace(_ptr(graph_idx), _ptr(graph_dist), samples, gk, _ptr(res),
                                               res.shape[0], device))


def KODAMADissimilarityInPlace_device(graph_idx, graph_dist, run_labels, *, device: int = 0) -> None:
    """KODAMADissimilarityInPlace on CUDA torch tensors (graph_idx int32 and
    graph_dist float32 of shape (n, K), one-based, rewritten in place;
    run_labels int32 of shape (runs, n)), on torch's current stream, through
    kgb_dissimilarity_inplace_device: no device memory is allocated, at most
    samples * runs = 4,194,240 labels and K = 2048."""
    import torch

    for t, dt in ((graph_idx, torch.int32), (graph_dist, torch.float32), (run_labels, torch.int32)):
        if not (t.is_cuda and t.dtype == dt and t.is_contiguous()):
            raise ValueError("graph_idx / graph_dist / run_labels must be contiguous CUDA int32 / float32 / int32")
    n, k = int(graph_idx.shape[0]), int(graph_idx.shape[1])
    stream = torch.cuda.current_stream(device)
    N.check(N.load().kgb_dissimilarity_inplace_device(
        ctypes.c_void_p(graph_idx.data_ptr()), ctypes.c_void_p(graph_dist.data_ptr()), n, k,
        ctypes.c_void_p(run_labels.data_ptr()), int(run_labels.shape[0]), device,
        ctypes.c_void_p(stream.cuda_stream)))


def _pls_options(folds, stratified, max_components, fixed_components, center, scale, cv_seed, device):
    return N.PlsOptions(folds=folds, stratified=int(stratified), max_components=max_components,
                        fixed_components=fixed_components, center=int(center), scale=int(scale),
                        device=device, reserved=0, cv_seed=cv_seed)


@dataclass
class PLSCVResult:
    """The PLSCVResult fields of the path (kodama.hpp:263-275)."""
    predicted_labels: np.ndarray
    fold_assignments: np.ndarray
    selected_components: int
    accuracy_by_components: np.ndarray
    global_accuracy: float


def PLSLDACV(x, labels, *, constrain=None, folds=10, stratified=True, max_components=10,
             fixed_components=0, center=True, scale=True, cv_seed=1, device=0) -> PLSCVResult:
    """PLSLDACV: cross-validated PLS-LDA predictions (plscv.cpp:2920)."""
    xa = np.ascontiguousarray(x, dtype=np.float32)
    n, p = xa.shape
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    con = None if constrain is None else np.ascontiguousarray(constrain, dtype=np.int32)
    pred = np.zeros(n, np.int32)
    fo = np.zeros(n, np.int32)
    sel = ctypes.c_int32(0)
    abc = np.zeros(max(1, max_components), np.float64)
    opt = _pls_options(folds, stratified, max_components, fixed_components, center, scale, cv_seed, device)
    N.check(N.load().kgb_plsldacv(_ptr(xa), n, p, _ptr(lab), _ptr(con), ctypes.byref(opt), _ptr(pred),
                                  _ptr(fo), ctypes.byref(sel), _ptr(abc)))
    return PLSCVResult(pred, fo, int(sel.value), abc, float(np.mean(pred == lab)))


def PLSDACV(x, labels, *, constrain=None, folds=10, stratified=True, max_components=10,
            fixed_components=0, center=True, scale=True, cv_seed=1, device=0) -> PLSCVResult:
    """PLSDACV: cross-validated PLS-DA predictions (plscv.cpp:2897, PLSMode::PLS_DA)."""
    xa = np.ascontiguousarray(x, dtype=np.float32)
    n, p = xa.shape
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    con = None if constrain is None else np.ascontiguousarray(constrain, dtype=np.int32)
    pred = np.zeros(n, np.int32)
    fo = np.zeros(n, np.int32)
    sel = ctypes.c_int32(0)
    abc = np.zeros(max(1, max_components), np.float64)
    opt = _pls_options(folds, stratified, max_components, fixed_components, center, scale, cv_seed, device)
    N.check(N.load().kgb_plsdacv(_ptr(xa), n, p, _ptr(lab), _ptr(con), ctypes.byref(opt), _ptr(pred),
                                 _ptr(fo), ctypes.byref(sel), _ptr(abc)))
    return PLSCVResult(pred, fo, int(sel.value), abc, float(np.mean(pred == lab)))


def PLSLDAPredict(train, labels, test, *, max_components=10, fixed_components=0, center=True,
                  scale=True, device=0) -> np.ndarray:
    """PLSLDAPredict: fit on (train, labels), predict test (plscv.cpp:3068)."""
    tr = np.ascontiguousarray(train, dtype=np.float32)
    te = np.ascontiguousarray(test, dtype=np.float32)
    n, p = tr.shape
    if te.ndim != 2 or te.shape[1] != p:
        raise ValueError("PLSLDAPredict train/test column mismatch.")
    if len(labels) != n:
        raise ValueError("PLSLDAPredict labels size must match training rows.")
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    out = np.zeros(te.shape[0], np.int32)
    opt = _pls_options(2, False, max_components, fixed_components, center, scale, 1, device)
    N.check(N.load().kgb_plslda_predict(_ptr(tr), n, p, _ptr(lab), _ptr(te), te.shape[0],
                                        ctypes.byref(opt), _ptr(out)))
    return out


def CorePLSLDA(x, labels, *, constrain=None, fixed=None, cycles=100, folds=10, stratified=True,
               max_components=10, fixed_components=0, center=True, scale=True,
               evolutionary_search=False, guarded_diversity=False, many_to_one_absorption=False,
               adaptive_proposal_size=True, auto_class_coarsening=False, seed=1, cv_seed=1,
               device=0, policy="full") -> CoreResult:
    """CorePLSLDA: label evolution with PLSLDACV as the predictor (core.cpp:1626).
    counters has 18 entries: CoreResult's 16, then PLS coarsening attempted / accepted."""
    xa = np.ascontiguousarray(x, dtype=np.float32)
    n, p = xa.shape
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    con = None if constrain is None else np.ascontiguousarray(constrain, dtype=np.int32)
    fix = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.int32)
    opt = _core_options(cycles, 1, folds, stratified, evolutionary_search, guarded_diversity,
                        many_to_one_absorption, adaptive_proposal_size, seed, cv_seed, device, policy)
    opt.auto_class_coarsening = int(auto_class_coarsening)
    popt = _pls_options(folds, stratified, max_components, fixed_components, center, scale, cv_seed, device)
    r, bufs = _alloc_core(n, cycles)
    N.check(N.load().kgb_core_plslda(_ptr(xa), n, p, _ptr(lab), _ptr(con), _ptr(fix), ctypes.byref(opt),
                                     ctypes.byref(popt), ctypes.byref(r)))
    return _wrap_core(r, bufs, cycles)


# ---------------------------------------------------------------------------
# Learned relabelling proposal (no counterpart in the reference)
# ---------------------------------------------------------------------------

def train_proposal(features, targets, *, epochs=20, batch=4096, learning_rate=2e-3, seed=1,
                   weights_init=None, device=0):
    """Trains the proposal network (kgb_proposal_train): returns (weights, loss per epoch)."""
    f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 8)
    t = np.ascontiguousarray(targets, dtype=np.uint8).reshape(-1)
    if len(t) != len(f):
        raise ValueError("one target per feature row")
    w = np.zeros(N.PROPOSAL_PARAMS, np.float32)
    losses = np.zeros(max(epochs, 1), np.float32)
    init = None if weights_init is None else np.ascontiguousarray(weights_init, dtype=np.float32)
    N.check(N.load().kgb_proposal_train(_ptr(f), _ptr(t), len(f), epochs, batch, learning_rate, seed, _ptr(init),
                                        device, _ptr(w), _ptr(losses)))
    return w, losses[:epochs]


def proposal_gradient(weights, features, targets, *, device=0):
    """Mean-loss gradient of the proposal network on the GPU: (grad, loss)."""
    w = np.ascontiguousarray(weights, dtype=np.float32)
    f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 8)
    t = np.ascontiguousarray(targets, dtype=np.uint8).reshape(-1)
    g = np.zeros(N.PROPOSAL_PARAMS, np.float32)
    loss = ctypes.c_float(0.0)
    N.check(N.load().kgb_proposal_gradient(_ptr(w), _ptr(f), _ptr(t), len(f), device, _ptr(g), ctypes.byref(loss)))
    return g, float(loss.value)


def proposal_predict(weights, features, *, device=0):
    """Logits of the proposal network on the GPU."""
    w = np.ascontiguousarray(weights, dtype=np.float32)
    f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 8)
    out = np.zeros(len(f), np.float32)
    N.check(N.load().kgb_proposal_predict(_ptr(w), _ptr(f), len(f), device, _ptr(out)))
    return out
