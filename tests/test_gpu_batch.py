"""Batched KODAMA.matrix (kgb_kodama_matrix_batch): every problem of a
captured batch gives the result of its own kgb_kodama_matrix call, whatever
the schedule, and a replay of the captured graph gives it again."""

import numpy as np
import pytest

from kodama_gb300 import datasets

pytestmark = pytest.mark.gpu

KW = dict(runs=4, cycles=6, knn_k=10, components=3, graph_neighbors=20, folds=5, seed=21)
FIELDS = ("res", "acc", "v", "run_hashes", "run_counters", "cycle_diag", "pls_counters")


def _problems():
    shapes = [(300, 10, "knn"), (800, 50, "pls"), (1500, 100, "knn"), (2500, 10, "pls"), (650, 100, "pls"),
              (1200, 50, "knn")]
    out = []
    for i, (n, d, cls) in enumerate(shapes):
        x, _ = datasets.gaussian_mixture(n=n, d=d, clusters=3 + i, mean_scale=3.0, seed=100 + i)
        out.append({"x": x, "classifier": cls})
    return out


def _same(a, b):
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


@pytest.fixture(scope="module")
def singles(kg):
    return [kg.KODAMA_matrix(p["x"], classifier=p["classifier"], **KW) for p in _problems()]


@pytest.mark.parametrize("lanes,order", [(1, 2), (3, 1), (8, 2)])
def test_batch_equals_single_calls(kg, singles, lanes, order):
    res, rep = kg.KODAMA_matrix_batch(_problems(), lanes=lanes, order=order, **KW)
    assert rep.lanes == lanes and rep.order == order
    assert rep.kernel_nodes > 0 and rep.device_ms > 0.0
    for r, s in zip(res, singles):
        _same(r, s)


def test_batch_replay_and_autotune(kg, singles):
    probs = _problems()
    res1, rep1 = kg.KODAMA_matrix_batch(probs, **KW)
    assert rep1.rebuilt and rep1.lanes in (4, 8, 16, 32) and rep1.order in (1, 2)
    res2, rep2 = kg.KODAMA_matrix_batch(probs, **KW)
    assert not rep2.rebuilt and (rep2.lanes, rep2.order) == (rep1.lanes, rep1.order)
    for a, b, s in zip(res1, res2, singles):
        _same(a, s)
        _same(b, s)


def test_batch_materialized_graph(kg):
    probs = _problems()[:3]
    res, _ = kg.KODAMA_matrix_batch(probs, lanes=2, order=1, materialize_graph=True, **KW)
    for p, r in zip(probs, res):
        s = kg.KODAMA_matrix(p["x"], classifier=p["classifier"], materialize_graph=True, **KW)
        _same(r, s)
        assert np.array_equal(r.knn_idx, s.knn_idx) and np.array_equal(r.knn_dist, s.knn_dist)


def test_batch_rejects_semi_supervised_inputs(kg):
    import ctypes
    from kodama_gb300 import _native as N
    p = _problems()[0]
    x = np.ascontiguousarray(p["x"], np.float32)
    arr = (N.MatrixProblem * 1)()
    out = N.MatrixResult()
    res = np.zeros((2, x.shape[0]), np.int32)
    acc = np.zeros(2)
    v = np.zeros((2, 3))
    out.res = res.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    out.acc = acc.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    out.v = v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    con = np.arange(x.shape[0], dtype=np.int32)
    opt = N.MatrixOptions(runs=2, cycles=3, folds=5, knn_k=10, graph_neighbors=20)
    opt.constrain = con.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    arr[0].x = x.ctypes.data
    arr[0].n, arr[0].d = x.shape
    arr[0].options = opt
    arr[0].result = ctypes.pointer(out)
    rc = N.load().kgb_kodama_matrix_batch(arr, 1, ctypes.byref(N.BatchOptions(0, 1, 1, 0)), None)
    assert rc == N.KGB_EINVAL
