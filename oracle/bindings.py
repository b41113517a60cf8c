"""ctypes bindings shared by the two CPU checkers (TEST INFRASTRUCTURE ONLY):

* ``oracle.ref``    -> oracle/_ref/libkodama_ref.so, the reference's own CPU core
                       compiled from its sources by oracle/build_ref.sh (only where
                       the reference checkout exists);
* ``oracle.oracle`` -> oracle/_build/liboracle.so, the CPU restatement in
                       oracle/kodama_oracle.cpp (builds anywhere, travels).

Both export the same C functions under the prefixes ``ref_`` and ``orc_``.
"""

from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))

OPT_FIELDS = ("runs", "cycles", "landmarks", "splitting", "graph_neighbors", "folds",
              "knn_k", "threads", "materialize", "classifier", "components", "apply_dissim", "first_run",
              "metric")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C")


class _Lib:
    """Resolves ``name`` to ``<prefix>name`` in a lazily loaded library."""

    def __init__(self, path: str, prefix: str):
        self.path, self.prefix, self._h = path, prefix, None

    def available(self) -> bool:
        return os.path.exists(self.path)

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        if self._h is None:
            if not self.available():
                raise RuntimeError(f"{self.path} is not built")
            self._h = ctypes.CDLL(self.path)
        return getattr(self._h, self.prefix + name)


def _err(L) -> str:
    buf = ctypes.create_string_buffer(4096)
    L.last_error(buf, 4096)
    return buf.value.decode()


@dataclass
class MatrixResult:
    res: np.ndarray          # (runs, n) int32
    acc: np.ndarray          # (runs,) float64
    v: np.ndarray            # (runs, cycles) float64
    hashes: np.ndarray       # (runs, 3) uint64: landmark rows, initial labels, folds
    run_counters: np.ndarray # (runs, 8) int32
    cycle_diag: np.ndarray   # (runs, cycles, 5) int32
    knn_idx: np.ndarray | None
    knn_dist: np.ndarray | None
    timings: np.ndarray      # runtime, graph, optimisation, dissimilarity, atlas, wall
    pls_counters: np.ndarray # (runs, 2) int32: PLS coarsening attempted / accepted


def matrix_options(**kw) -> np.ndarray:
    defaults = dict(runs=100, cycles=20, landmarks=10000, splitting=0, graph_neighbors=100,
                    folds=5, knn_k=30, threads=1, materialize=0, classifier=0, components=50,
                    apply_dissim=1, first_run=1, metric=2)
    defaults.update(kw)
    return np.array([defaults[f] for f in OPT_FIELDS], dtype=np.int32)


def _alloc_matrix(n, opts):
    runs, cycles = int(opts[0]), int(opts[1])
    k_cap = max(1, int(opts[4]))
    return dict(
        res=np.zeros(runs * n, np.int32), acc=np.zeros(runs, np.float64),
        v=np.zeros(runs * cycles, np.float64), hashes=np.zeros(runs * 3, np.uint64),
        run_counters=np.zeros(runs * 8, np.int32), cycle_diag=np.zeros(runs * cycles * 5, np.int32),
        out_idx=np.zeros(n * k_cap, np.int32), out_dist=np.zeros(n * k_cap, np.float32),
        out_k=ctypes.c_int(0), timings=np.zeros(6, np.float64), pls=np.zeros(runs * 2, np.int32))


def _wrap(n, opts, b) -> MatrixResult:
    runs, cycles = int(opts[0]), int(opts[1])
    k = b["out_k"].value
    has_graph = bool(opts[8]) and k > 0
    return MatrixResult(
        res=b["res"].reshape(runs, n), acc=b["acc"], v=b["v"].reshape(runs, cycles),
        hashes=b["hashes"].reshape(runs, 3), run_counters=b["run_counters"].reshape(runs, 8),
        cycle_diag=b["cycle_diag"].reshape(runs, cycles, 5),
        knn_idx=b["out_idx"][: n * k].reshape(n, k).copy() if has_graph else None,
        knn_dist=b["out_dist"][: n * k].reshape(n, k).copy() if has_graph else None,
        timings=b["timings"], pls_counters=b["pls"].reshape(runs, 2))


def _opt_vec(v, n):
    if v is None:
        return None, ctypes.c_void_p(0)
    a = np.ascontiguousarray(v, np.int32)
    if a.shape != (n,):
        raise ValueError("starting / constrain / fixed need one entry per row")
    return a, a.ctypes.data_as(ctypes.c_void_p)


def kodama_matrix_graph_data(L, x: np.ndarray, gidx: np.ndarray, gdist: np.ndarray,
                             index_base: int, seed: int = 1234, starting=None, constrain=None, fixed=None,
                             **kw) -> MatrixResult:
    """KODAMAMatrixFromGraphData_CPU: data plus a caller-supplied graph, with
    optional starting labels, constraint groups and fixed flags."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    gk = gidx.shape[1]
    opts = matrix_options(**kw)
    opts[4] = opts[4] if opts[4] > 0 else 100
    b = _alloc_matrix(n, opts)
    keep = [_opt_vec(v, n) for v in (starting, constrain, fixed)]
    rc = L.kodama_matrix_graph_data_ex(
        x.ctypes.data_as(ctypes.c_void_p), n, d,
        np.ascontiguousarray(gidx, np.int32).ctypes.data_as(ctypes.c_void_p),
        np.ascontiguousarray(gdist, np.float32).ctypes.data_as(ctypes.c_void_p), gk, index_base,
        opts.ctypes.data_as(ctypes.c_void_p), ctypes.c_ulonglong(seed),
        *[b[f].ctypes.data_as(ctypes.c_void_p) for f in
          ("res", "acc", "v", "hashes", "run_counters", "cycle_diag", "out_idx", "out_dist")],
        ctypes.byref(b["out_k"]), b["timings"].ctypes.data_as(ctypes.c_void_p),
        b["pls"].ctypes.data_as(ctypes.c_void_p), *[k[1] for k in keep])
    if rc != 0:
        raise RuntimeError(_err(L))
    return _wrap(n, opts, b)


def kodama_matrix_raw(L, x: np.ndarray, seed: int = 1234, **kw) -> MatrixResult:
    """KODAMAMatrix_CPU: raw data, the reference's own HNSW graph."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    opts = matrix_options(**kw)
    opts[4] = opts[4] if opts[4] > 0 else 100
    b = _alloc_matrix(n, opts)
    rc = L.kodama_matrix_raw(
        x.ctypes.data_as(ctypes.c_void_p), n, d, opts.ctypes.data_as(ctypes.c_void_p),
        ctypes.c_ulonglong(seed),
        *[b[f].ctypes.data_as(ctypes.c_void_p) for f in
          ("res", "acc", "v", "hashes", "run_counters", "cycle_diag", "out_idx", "out_dist")],
        ctypes.byref(b["out_k"]), b["timings"].ctypes.data_as(ctypes.c_void_p),
        b["pls"].ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError(_err(L))
    return _wrap(n, opts, b)


@dataclass
class CoreResult:
    clbest: np.ndarray
    cvpredbest: np.ndarray
    folds: np.ndarray
    vect_acc: np.ndarray
    vect_score: np.ndarray
    proposal_size: np.ndarray
    active_classes: np.ndarray
    flags: np.ndarray        # (cycles, 3): accepted, improving, temperature
    accbest: float
    scorebest: float
    counters: np.ndarray     # 16 ints (18 for core_plslda)


def core_knn_graph(L, gidx, gdist, labels, *, index_base=-1, constrain=None, fixed=None, cycles=20,
                   k=10, folds=10, stratified=True, evolutionary=False, guarded=False,
                   absorption=False, adaptive=True, seed=1, cv_seed=1, metric=2) -> CoreResult:
    """CoreKNNGraph_CPU; metric is KNNOptions::metric (0 cosine, 1 inner
    product, 2 Euclidean): the vote score 1 - d or -(d*d)."""
    samples, gk = gidx.shape
    lab = np.ascontiguousarray(labels, np.int32)
    con = np.ascontiguousarray(constrain if constrain is not None else np.zeros(samples), np.int32)
    fix = np.ascontiguousarray(fixed if fixed is not None else np.zeros(samples), np.int32)
    copts = np.array([cycles, k, folds, int(stratified), int(evolutionary), int(guarded),
                      int(absorption), int(adaptive), metric], np.int32)
    out = dict(clbest=np.zeros(samples, np.int32), cvpredbest=np.zeros(samples, np.int32),
               folds=np.zeros(samples, np.int32), vect_acc=np.zeros(cycles, np.float64),
               vect_score=np.zeros(cycles, np.float64), proposal_size=np.zeros(cycles, np.int32),
               active_classes=np.zeros(cycles, np.int32), flags=np.zeros(cycles * 3, np.uint8),
               scal=np.zeros(2, np.float64), counters=np.zeros(16, np.int32))
    rc = L.core_knn_graph(
        np.ascontiguousarray(gidx, np.int32).ctypes.data_as(ctypes.c_void_p),
        np.ascontiguousarray(gdist, np.float32).ctypes.data_as(ctypes.c_void_p),
        samples, gk, index_base, lab.ctypes.data_as(ctypes.c_void_p),
        con.ctypes.data_as(ctypes.c_void_p), int(constrain is not None),
        fix.ctypes.data_as(ctypes.c_void_p), int(fixed is not None),
        copts.ctypes.data_as(ctypes.c_void_p), ctypes.c_ulonglong(seed), ctypes.c_ulonglong(cv_seed),
        *[out[f].ctypes.data_as(ctypes.c_void_p) for f in
          ("clbest", "cvpredbest", "folds", "vect_acc", "vect_score", "proposal_size",
           "active_classes", "flags", "scal", "counters")])
    if rc != 0:
        raise RuntimeError(_err(L))
    return CoreResult(out["clbest"], out["cvpredbest"], out["folds"], out["vect_acc"],
                      out["vect_score"], out["proposal_size"], out["active_classes"],
                      out["flags"].reshape(cycles, 3), float(out["scal"][0]),
                      float(out["scal"][1]), out["counters"])


def core_plslda(L, x, labels, *, constrain=None, fixed=None, cycles=20, folds=10, stratified=True,
                components=5, fixed_components=None, center=True, scale=True, threads=1,
                evolutionary=False, guarded=False, absorption=False, adaptive=True,
                coarsening=False, seed=1, cv_seed=1) -> CoreResult:
    """CorePLSLDA_CPU; counters has 18 entries (16 of CoreKNNGraph, then PLS
    coarsening attempted / accepted)."""
    x = np.ascontiguousarray(x, np.float32)
    samples, d = x.shape
    lab = np.ascontiguousarray(labels, np.int32)
    con = np.ascontiguousarray(constrain if constrain is not None else np.zeros(samples), np.int32)
    fix = np.ascontiguousarray(fixed if fixed is not None else np.zeros(samples), np.int32)
    fc = components if fixed_components is None else fixed_components
    copts = np.array([cycles, 0, folds, int(stratified), int(evolutionary), int(guarded),
                      int(absorption), int(adaptive), int(coarsening)], np.int32)
    popts = np.array([folds, int(stratified), components, fc, int(center), int(scale), threads], np.int32)
    out = dict(clbest=np.zeros(samples, np.int32), cvpredbest=np.zeros(samples, np.int32),
               folds=np.zeros(samples, np.int32), vect_acc=np.zeros(cycles, np.float64),
               vect_score=np.zeros(cycles, np.float64), proposal_size=np.zeros(cycles, np.int32),
               active_classes=np.zeros(cycles, np.int32), flags=np.zeros(cycles * 3, np.uint8),
               scal=np.zeros(2, np.float64), counters=np.zeros(18, np.int32))
    rc = L.core_plslda(
        x.ctypes.data_as(ctypes.c_void_p), samples, d, lab.ctypes.data_as(ctypes.c_void_p),
        con.ctypes.data_as(ctypes.c_void_p), int(constrain is not None),
        fix.ctypes.data_as(ctypes.c_void_p), int(fixed is not None),
        copts.ctypes.data_as(ctypes.c_void_p), popts.ctypes.data_as(ctypes.c_void_p),
        ctypes.c_ulonglong(seed), ctypes.c_ulonglong(cv_seed),
        *[out[f].ctypes.data_as(ctypes.c_void_p) for f in
          ("clbest", "cvpredbest", "folds", "vect_acc", "vect_score", "proposal_size",
           "active_classes", "flags", "scal", "counters")])
    if rc != 0:
        raise RuntimeError(_err(L))
    return CoreResult(out["clbest"], out["cvpredbest"], out["folds"], out["vect_acc"],
                      out["vect_score"], out["proposal_size"], out["active_classes"],
                      out["flags"].reshape(cycles, 3), float(out["scal"][0]),
                      float(out["scal"][1]), out["counters"])


def dissimilarity(L, gidx1: np.ndarray, gdist: np.ndarray, res: np.ndarray, threads: int = 1):
    """KODAMADissimilarityInPlace on a one-based graph; returns new arrays."""
    idx = np.ascontiguousarray(gidx1, np.int32).copy()
    dist = np.ascontiguousarray(gdist, np.float32).copy()
    samples, gk = idx.shape
    runs = res.shape[0]
    r = np.ascontiguousarray(res, np.int32)
    rc = L.dissimilarity(idx.ctypes.data_as(ctypes.c_void_p), dist.ctypes.data_as(ctypes.c_void_p),
                                 samples, gk, r.ctypes.data_as(ctypes.c_void_p), runs, threads)
    if rc != 0:
        raise RuntimeError(_err(L))
    return idx, dist


def plsldacv(L, x, labels, *, folds=10, stratified=True, max_components=10, fixed_components=0,
             center=True, scale=True, threads=1, cv_seed=1, constrain=None, da=False):
    """PLSLDACV_CPU (PLSDACV_CPU with da=True): returns (predicted, folds,
    selected_components, acc_by_comp, seconds)."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    lab = np.ascontiguousarray(labels, np.int32)
    con = np.ascontiguousarray(constrain if constrain is not None else np.zeros(n), np.int32)
    popts = np.array([folds, int(stratified), max_components, fixed_components, int(center),
                      int(scale), threads, int(da)], np.int32)
    pred = np.zeros(n, np.int32)
    fo = np.zeros(n, np.int32)
    sel = ctypes.c_int(0)
    abc = np.zeros(max(1, max_components), np.float64)
    sec = ctypes.c_double(0)
    rc = L.plsldacv(x.ctypes.data_as(ctypes.c_void_p), n, d, lab.ctypes.data_as(ctypes.c_void_p),
                            con.ctypes.data_as(ctypes.c_void_p), int(constrain is not None),
                            popts.ctypes.data_as(ctypes.c_void_p), ctypes.c_ulonglong(cv_seed),
                            pred.ctypes.data_as(ctypes.c_void_p), fo.ctypes.data_as(ctypes.c_void_p),
                            ctypes.byref(sel), abc.ctypes.data_as(ctypes.c_void_p), ctypes.byref(sec))
    if rc != 0:
        raise RuntimeError(_err(L))
    return pred, fo, sel.value, abc, sec.value


def plsldapredict(L, train, labels, test, *, components=5, center=True, scale=True, threads=1):
    train = np.ascontiguousarray(train, np.float32)
    test = np.ascontiguousarray(test, np.float32)
    n, d = train.shape
    popts = np.array([2, 0, components, components, int(center), int(scale), threads], np.int32)
    pred = np.zeros(test.shape[0], np.int32)
    rc = L.plsldapredict(train.ctypes.data_as(ctypes.c_void_p), n, d,
                                 np.ascontiguousarray(labels, np.int32).ctypes.data_as(ctypes.c_void_p),
                                 test.ctypes.data_as(ctypes.c_void_p), test.shape[0],
                                 popts.ctypes.data_as(ctypes.c_void_p), pred.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError(_err(L))
    return pred


def knncv(L, x, labels, *, constrain=None, k=10, folds=10, stratified=True, metric=0, cv_seed=1, threads=1):
    """KNNCV: predictions and fold assignments (and, from the reference, its
    runtime in seconds; 0.0 from the restatement)."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    pred = np.zeros(n, np.int32)
    fo = np.zeros(n, np.int32)
    con = np.ascontiguousarray(constrain if constrain is not None else np.zeros(n), np.int32)
    lab = np.ascontiguousarray(labels, np.int32)
    sec = ctypes.c_double(0)
    if L.prefix == "orc_":
        rc = L.knncv(x.ctypes.data_as(ctypes.c_void_p), n, d, lab.ctypes.data_as(ctypes.c_void_p),
                     con.ctypes.data_as(ctypes.c_void_p), int(constrain is not None), k, folds,
                     int(stratified), metric, ctypes.c_ulonglong(cv_seed),
                     pred.ctypes.data_as(ctypes.c_void_p), fo.ctypes.data_as(ctypes.c_void_p))
    else:
        if constrain is not None:
            raise ValueError("the reference shim takes no constrain")
        rc = L.knncv(x.ctypes.data_as(ctypes.c_void_p), n, d, lab.ctypes.data_as(ctypes.c_void_p),
                     k, folds, int(stratified), metric, ctypes.c_ulonglong(cv_seed), threads,
                     pred.ctypes.data_as(ctypes.c_void_p), fo.ctypes.data_as(ctypes.c_void_p),
                     ctypes.byref(sec))
    if rc != 0:
        raise RuntimeError(_err(L))
    return pred, fo, sec.value


def core_knn(L, x, labels, *, metric=2, constrain=None, fixed=None, cycles=20, k=30, folds=10,
             stratified=True, evolutionary=False, guarded=False, absorption=False, adaptive=True,
             seed=1, cv_seed=1) -> CoreResult:
    """CoreKNN on raw data (metric 0 cosine, 1 inner product, 2 Euclidean)."""
    x = np.ascontiguousarray(x, np.float32)
    samples, d = x.shape
    lab = np.ascontiguousarray(labels, np.int32)
    con = np.ascontiguousarray(constrain if constrain is not None else np.zeros(samples), np.int32)
    fix = np.ascontiguousarray(fixed if fixed is not None else np.zeros(samples), np.int32)
    copts = np.array([cycles, k, folds, int(stratified), int(evolutionary), int(guarded),
                      int(absorption), int(adaptive), metric], np.int32)
    out = dict(clbest=np.zeros(samples, np.int32), cvpredbest=np.zeros(samples, np.int32),
               folds=np.zeros(samples, np.int32), vect_acc=np.zeros(cycles, np.float64),
               vect_score=np.zeros(cycles, np.float64), proposal_size=np.zeros(cycles, np.int32),
               active_classes=np.zeros(cycles, np.int32), flags=np.zeros(cycles * 3, np.uint8),
               scal=np.zeros(2, np.float64), counters=np.zeros(16, np.int32))
    rc = L.core_knn(
        x.ctypes.data_as(ctypes.c_void_p), samples, d, metric, lab.ctypes.data_as(ctypes.c_void_p),
        con.ctypes.data_as(ctypes.c_void_p), int(constrain is not None),
        fix.ctypes.data_as(ctypes.c_void_p), int(fixed is not None),
        copts.ctypes.data_as(ctypes.c_void_p), ctypes.c_ulonglong(seed), ctypes.c_ulonglong(cv_seed),
        *[out[f].ctypes.data_as(ctypes.c_void_p) for f in
          ("clbest", "cvpredbest", "folds", "vect_acc", "vect_score", "proposal_size",
           "active_classes", "flags", "scal", "counters")])
    if rc != 0:
        raise RuntimeError(_err(L))
    return CoreResult(out["clbest"], out["cvpredbest"], out["folds"], out["vect_acc"],
                      out["vect_score"], out["proposal_size"], out["active_classes"],
                      out["flags"].reshape(cycles, 3), float(out["scal"][0]),
                      float(out["scal"][1]), out["counters"])


def exact_knn(L, x, K, threads=1):
    """Canonical exact kNN: zero-based (n, K) indices and sqrt distances."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    idx = np.zeros((n, K), np.int32)
    dist = np.zeros((n, K), np.float32)
    rc = L.exact_knn(x.ctypes.data_as(ctypes.c_void_p), n, d, K, idx.ctypes.data_as(ctypes.c_void_p),
                     dist.ctypes.data_as(ctypes.c_void_p), threads)
    if rc != 0:
        raise RuntimeError(_err(L))
    return idx, dist


def exact_knn_metric(L, x, K, metric, threads=1):
    """Exact graph under a metric (0 cosine, 1 inner product, 2 Euclidean):
    zero-based indices and the reference's reported distances."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    idx = np.zeros((n, K), np.int32)
    dist = np.zeros((n, K), np.float32)
    rc = L.exact_knn_metric(x.ctypes.data_as(ctypes.c_void_p), n, d, K, int(metric),
                            idx.ctypes.data_as(ctypes.c_void_p), dist.ctypes.data_as(ctypes.c_void_p), threads)
    if rc != 0:
        raise RuntimeError(_err(L))
    return idx, dist


def exact_knn_rows(L, x, K, rows, threads=1):
    """exact_knn for the listed query rows only: (len(rows), K) results."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    rows = np.ascontiguousarray(rows, np.int32)
    idx = np.zeros((len(rows), K), np.int32)
    dist = np.zeros((len(rows), K), np.float32)
    rc = L.exact_knn_rows(x.ctypes.data_as(ctypes.c_void_p), n, d, K, rows.ctypes.data_as(ctypes.c_void_p),
                          len(rows), idx.ctypes.data_as(ctypes.c_void_p), dist.ctypes.data_as(ctypes.c_void_p),
                          threads)
    if rc != 0:
        raise RuntimeError(_err(L))
    return idx, dist


def kmeans(L, x, k, rng_seed, discard=0, max_iter=10):
    x = np.ascontiguousarray(x, np.float32)
    n, p = x.shape
    out = np.zeros(n, np.int32)
    rc = L.kmeans(x.ctypes.data_as(ctypes.c_void_p), n, p, k, ctypes.c_ulonglong(rng_seed), discard,
                  max_iter, out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError(_err(L))
    return out


def dot_x86(L, a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = ctypes.c_float(0)
    L.dot_x86(a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p), len(a), ctypes.byref(out))
    return out.value


def quota_sample(L, offsets, rows, target, seed, discard=0):
    offsets = np.ascontiguousarray(offsets, np.int32)
    rows = np.ascontiguousarray(rows, np.int32)
    out = np.zeros(target, np.int32)
    rc = L.quota_sample(offsets.ctypes.data_as(ctypes.c_void_p), len(offsets) - 1,
                        rows.ctypes.data_as(ctypes.c_void_p), len(rows), target,
                        ctypes.c_ulonglong(seed), discard, out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError(_err(L))
    return out
