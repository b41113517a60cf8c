"""CPU suite: the CPU restatement against the reference itself (where the
reference core was compiled here) and against committed golden fixtures."""

import numpy as np
import pytest

from kodama_gb300 import datasets
from oracle import ref


needs_ref = pytest.mark.skipif(not ref.available(), reason="reference core not built here")


@needs_ref
def test_matrix_spirals_vs_reference(orc):
    x = datasets.spirals()[0].astype(np.float32)
    gi, gd = orc.exact_knn(x, 50, threads=4)
    kw = dict(runs=6, cycles=15, landmarks=10000, splitting=0, graph_neighbors=50, folds=10, knn_k=10,
              threads=4, materialize=1)
    r = ref.kodama_matrix_graph_data(x, gi + 1, gd, 1, seed=1234, **kw)
    o = orc.kodama_matrix_graph_data(x, gi + 1, gd, 1, seed=1234, **kw)
    for f in ("res", "acc", "v", "hashes", "run_counters", "cycle_diag", "knn_idx", "knn_dist"):
        assert np.array_equal(getattr(r, f), getattr(o, f)), f


@needs_ref
@pytest.mark.parametrize("constrained", [False, True])
@pytest.mark.parametrize("evolutionary", [False, True])
def test_core_knn_graph_vs_reference(orc, constrained, evolutionary):
    x, _ = datasets.gaussian_mixture(n=1500, d=20, seed=4)
    gi, gd = orc.exact_knn(x, 30, threads=8)
    rng = np.random.default_rng(1)
    labels = rng.integers(1, 7, 1500).astype(np.int32)
    con = rng.integers(0, 500, 1500).astype(np.int32) if constrained else None
    fix = (rng.random(1500) < 0.05).astype(np.int32)
    kw = dict(index_base=0, constrain=con, fixed=fix, cycles=15, k=10, folds=5, seed=3, cv_seed=4,
              evolutionary=evolutionary, guarded=evolutionary, absorption=evolutionary,
              stratified=not evolutionary)
    a = ref.core_knn_graph(gi, gd, labels, **kw)
    b = orc.core_knn_graph(gi, gd, labels, **kw)
    for f in ("clbest", "cvpredbest", "folds", "vect_acc", "vect_score", "proposal_size",
              "active_classes", "flags", "counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert a.accbest == b.accbest and a.scorebest == b.scorebest


@needs_ref
def test_dissimilarity_vs_reference(orc):
    rng = np.random.default_rng(2)
    n, K, M = 800, 15, 12
    x, _ = datasets.gaussian_mixture(n=n, d=8, seed=2)
    gi, gd = orc.exact_knn(x, K)
    gi1 = (gi + 1).astype(np.int32)
    gi1[rng.random(gi1.shape) < 0.05] = -1
    res = rng.integers(0, 4, (M, n)).astype(np.int32)
    a = ref.dissimilarity(gi1, gd, res)
    b = orc.dissimilarity(gi1, gd, res)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
