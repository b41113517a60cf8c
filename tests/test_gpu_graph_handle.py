"""KODAMAGraph on the device (kgb_graph_create / kgb_kodama_matrix_graph):
KODAMA.matrix on a resident graph gives the result of the raw-data call with
the same options, for the full graph width and for a narrower one."""

import numpy as np
import pytest

from kodama_gb300 import datasets

pytestmark = pytest.mark.gpu

FIELDS = ("res", "acc", "v", "run_hashes", "run_counters", "cycle_diag", "pls_counters", "knn_idx", "knn_dist")


def _same(a, b):
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


@pytest.fixture(scope="module")
def data():
    return datasets.gaussian_mixture(n=3000, d=20, clusters=7, mean_scale=3.0, seed=31)[0]


def test_resident_graph_is_the_exact_graph(kg, data):
    with kg.KODAMAGraph(data, neighbors=40) as g:
        idx, dist = g.graph()
    gi, gd = kg.knn_graph(data, 40)
    assert np.array_equal(idx, gi + 1) and np.array_equal(dist, gd)


@pytest.mark.parametrize("kw", [
    dict(graph_neighbors=40),
    dict(graph_neighbors=25),
    dict(graph_neighbors=40, classifier="pls", components=3),
    dict(graph_neighbors=30, knn_k=15, splitting=30),
])
def test_matrix_on_handle_equals_raw_call(kg, data, kw):
    base = dict(runs=4, cycles=8, folds=5, knn_k=10, seed=5, materialize_graph=True)
    base.update(kw)
    with kg.KODAMAGraph(data, neighbors=40) as g:
        r1 = g.matrix(**base)
        r2 = g.matrix(**base)  # the handle is reusable
    s = kg.KODAMA_matrix(data, **base)
    _same(r1, s)
    _same(r2, s)


def test_semi_supervised_on_handle(kg, data):
    rng = np.random.default_rng(2)
    start = rng.integers(1, 6, len(data)).astype(np.int32)
    con = (np.arange(len(data)) // 3).astype(np.int32)
    base = dict(runs=3, cycles=6, folds=5, knn_k=10, seed=9, graph_neighbors=30, starting_labels=start,
                constrain=con)
    with kg.KODAMAGraph(data, neighbors=30) as g:
        r = g.matrix(**base)
    _same(r, kg.KODAMA_matrix(data, **base))


def test_closed_handle_raises(kg, data):
    g = kg.KODAMAGraph(data[:500], neighbors=10)
    g.close()
    with pytest.raises(ValueError):
        g.matrix(runs=2, cycles=2)
