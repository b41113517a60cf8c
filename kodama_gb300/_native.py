"""ctypes declarations of the C ABI in include/kodama_gb300.h.

Loads kodama_gb300/_lib/libkodama_gb300.so (built in-tree by
kodama_gb300/build.py).  There is no fallback: if the library is missing or
no CUDA device is usable, every call raises.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libkodama_gb300.so")

PROPOSAL_PARAMS = 4801
KGB_OK, KGB_EINVAL, KGB_ENOMEM, KGB_ECUDA, KGB_ETIMEOUT, KGB_EINTERNAL = range(6)

EXPORTED = (
    "kgb_kodama_matrix",
    "kgb_kodama_matrix_from_graph_data",
    "kgb_kodama_matrix_resident",
    "kgb_kodama_matrix_batch",
    "kgb_graph_create",
    "kgb_graph_info",
    "kgb_graph_materialize",
    "kgb_kodama_matrix_graph",
    "kgb_graph_destroy",
    "kgb_launch_count",
    "kgb_core_knn_graph",
    "kgb_core_knn_graph_batch",
    "kgb_knncv",
    "kgb_knn_graph_ex",
    "kgb_knn_graph_metric",
    "kgb_core_knn",
    "kgb_plsldacv",
    "kgb_plsdacv",
    "kgb_plslda_predict",
    "kgb_core_plslda",
    "kgb_proposal_train",
    "kgb_proposal_gradient",
    "kgb_proposal_predict",
    "kgb_knn_graph",
    "kgb_dissimilarity_inplace",
    "kgb_dissimilarity_inplace_device",
    "kgb_last_error",
    "kgb_version",
)


class Policy(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "prediction_guidance", "adaptive_proposal_size", "transition_proposal",
        "stochastic_acceptance", "diversity_multiplier", "pls_transition_coarsening",
        "pls_fragmentation_penalty", "reject_single_class")]


class MatrixOptions(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "runs", "cycles", "landmarks", "splitting", "graph_neighbors", "folds", "knn_k",
        "classifier", "components", "materialize_graph", "apply_dissimilarity", "metric",
        "device", "host_threads", "first_run", "reserved")] + [
        ("seed", ctypes.c_uint64), ("policy", Policy), ("proposal_weights", ctypes.POINTER(ctypes.c_float)),
        ("snapshot_cycle", ctypes.c_int32), ("proposal_greedy", ctypes.c_int32),
        ("starting_labels", ctypes.POINTER(ctypes.c_int32)), ("constrain", ctypes.POINTER(ctypes.c_int32)),
        ("fixed", ctypes.POINTER(ctypes.c_int32))]


class MatrixResult(ctypes.Structure):
    _fields_ = [
        ("res", ctypes.POINTER(ctypes.c_int32)),
        ("acc", ctypes.POINTER(ctypes.c_double)),
        ("v", ctypes.POINTER(ctypes.c_double)),
        ("run_hashes", ctypes.POINTER(ctypes.c_uint64)),
        ("run_counters", ctypes.POINTER(ctypes.c_int32)),
        ("cycle_diag", ctypes.POINTER(ctypes.c_int32)),
        ("knn_idx", ctypes.POINTER(ctypes.c_int32)),
        ("knn_dist", ctypes.POINTER(ctypes.c_float)),
        ("knn_cap", ctypes.c_int32),
        ("knn_k", ctypes.c_int32),
        ("effective_landmarks", ctypes.c_int32),
        ("timings", ctypes.c_double * 8),
        ("kernel_ms", ctypes.c_double * 8),
        ("res_on_device", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("pls_counters", ctypes.POINTER(ctypes.c_int32)),
        ("snapshot_features", ctypes.POINTER(ctypes.c_float)),
        ("snapshot_flags", ctypes.POINTER(ctypes.c_uint8)),
    ]


class MatrixProblem(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("n", ctypes.c_int32), ("d", ctypes.c_int32),
                ("options", MatrixOptions), ("result", ctypes.POINTER(MatrixResult))]


class BatchOptions(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("device", "lanes", "order", "reserved")]


class BatchReport(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("lanes", "order", "graph_nodes", "kernel_nodes", "rebuilt",
                                              "reserved")] + [("device_ms", ctypes.c_double),
                                                              ("tune_ms", ctypes.c_double)]


class CoreOptions(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "cycles", "k", "folds", "stratified", "evolutionary_search", "guarded_diversity",
        "many_to_one_absorption", "adaptive_proposal_size", "device", "auto_class_coarsening", "metric")] + [
        ("seed", ctypes.c_uint64), ("cv_seed", ctypes.c_uint64), ("policy", Policy)]


class CoreResult(ctypes.Structure):
    _fields_ = [
        ("clbest", ctypes.POINTER(ctypes.c_int32)),
        ("cvpredbest", ctypes.POINTER(ctypes.c_int32)),
        ("fold_assignments", ctypes.POINTER(ctypes.c_int32)),
        ("vect_acc", ctypes.POINTER(ctypes.c_double)),
        ("vect_score", ctypes.POINTER(ctypes.c_double)),
        ("proposal_size", ctypes.POINTER(ctypes.c_int32)),
        ("active_classes", ctypes.POINTER(ctypes.c_int32)),
        ("flags", ctypes.POINTER(ctypes.c_uint8)),
        ("accbest", ctypes.c_double),
        ("scorebest", ctypes.c_double),
        ("counters", ctypes.c_int32 * 18),
    ]


class KnnOptions(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "folds", "stratified", "k", "metric", "device", "reserved")] + [("cv_seed", ctypes.c_uint64)]


METRICS = {"cosine": 0, "inner_product": 1, "euclidean": 2}


class PlsOptions(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "folds", "stratified", "max_components", "fixed_components", "center", "scale", "device",
        "reserved")] + [("cv_seed", ctypes.c_uint64)]


_lib = None


def load():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m kodama_gb300.build` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    i32 = ctypes.c_int32
    lib.kgb_kodama_matrix.argtypes = [P, i32, i32, ctypes.POINTER(MatrixOptions), ctypes.POINTER(MatrixResult)]
    lib.kgb_kodama_matrix_resident.argtypes = [P, i32, i32, ctypes.POINTER(MatrixOptions),
                                               ctypes.POINTER(MatrixResult)]
    lib.kgb_kodama_matrix_batch.argtypes = [ctypes.POINTER(MatrixProblem), i32, ctypes.POINTER(BatchOptions),
                                            ctypes.POINTER(BatchReport)]
    lib.kgb_graph_create.argtypes = [P, i32, i32, i32, i32, i32, ctypes.POINTER(ctypes.c_void_p)]
    lib.kgb_graph_info.argtypes = [P, P, P, P]
    lib.kgb_graph_materialize.argtypes = [P, P, P]
    lib.kgb_kodama_matrix_graph.argtypes = [P, ctypes.POINTER(MatrixOptions), ctypes.POINTER(MatrixResult)]
    lib.kgb_graph_destroy.argtypes = [P]
    lib.kgb_graph_destroy.restype = None
    lib.kgb_launch_count.restype = ctypes.c_int64
    lib.kgb_launch_count.argtypes = []
    lib.kgb_kodama_matrix_from_graph_data.argtypes = [
        P, i32, i32, P, P, i32, i32, ctypes.POINTER(MatrixOptions), ctypes.POINTER(MatrixResult)]
    lib.kgb_core_knn_graph.argtypes = [P, P, i32, i32, i32, P, P, P, ctypes.POINTER(CoreOptions),
                                       ctypes.POINTER(CoreResult)]
    lib.kgb_core_knn_graph_batch.argtypes = [P, P, i32, i32, i32, i32, P, P, P, ctypes.POINTER(CoreOptions),
                                             ctypes.POINTER(CoreResult)]
    lib.kgb_knn_graph.argtypes = [P, i32, i32, i32, i32, P, P]
    lib.kgb_knn_graph_ex.argtypes = [P, i32, i32, i32, i32, i32, P, P, P]
    lib.kgb_knn_graph_metric.argtypes = [P, i32, i32, i32, i32, i32, P, P]
    lib.kgb_knncv.argtypes = [P, i32, i32, P, P, ctypes.POINTER(KnnOptions), P, P]
    lib.kgb_core_knn.argtypes = [P, i32, i32, i32, P, P, P, ctypes.POINTER(CoreOptions), ctypes.POINTER(CoreResult)]
    lib.kgb_dissimilarity_inplace.argtypes = [P, P, i32, i32, P, i32, i32]
    lib.kgb_proposal_train.argtypes = [P, P, i32, i32, i32, ctypes.c_float, ctypes.c_uint64, P, i32, P, P]
    lib.kgb_proposal_gradient.argtypes = [P, P, P, i32, i32, P, P]
    lib.kgb_proposal_predict.argtypes = [P, P, i32, i32, P]
    lib.kgb_plsldacv.argtypes = [P, i32, i32, P, P, ctypes.POINTER(PlsOptions), P, P, P, P]
    lib.kgb_plsdacv.argtypes = [P, i32, i32, P, P, ctypes.POINTER(PlsOptions), P, P, P, P]
    lib.kgb_plslda_predict.argtypes = [P, i32, i32, P, P, i32, ctypes.POINTER(PlsOptions), P]
    lib.kgb_core_plslda.argtypes = [P, i32, i32, P, P, P, ctypes.POINTER(CoreOptions),
                                    ctypes.POINTER(PlsOptions), ctypes.POINTER(CoreResult)]
    lib.kgb_dissimilarity_inplace_device.argtypes = [P, P, i32, i32, P, i32, i32, P]
    lib.kgb_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.kgb_version.restype = ctypes.c_char_p
    for name in EXPORTED:
        if name not in ("kgb_version", "kgb_launch_count", "kgb_graph_destroy"):
            getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


class KodamaError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[kgb status {code}] {message}")
        self.code = code


def check(rc: int) -> None:
    if rc == KGB_OK:
        return
    buf = ctypes.create_string_buffer(4096)
    load().kgb_last_error(buf, 4096)
    msg = buf.value.decode(errors="replace")
    if rc == KGB_EINVAL:
        raise ValueError(msg)
    raise KodamaError(rc, msg)
