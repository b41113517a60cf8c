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
@pytest.mark.parametrize("metric", [0, 1])
def test_matrix_metric_vs_reference(orc, metric):
    """KODAMA.matrix under the cosine (0) and inner-product (1) metrics on
    the exact graph of that metric: the vote scores 1 - d (core.cpp:672-677)
    and the caller graph's distances (1 - <x,y> can be negative for the
    inner product) clamped at zero (kodama_matrix.cpp:1292-1330)."""
    # overlapping clusters and knn.k = 4: count ties are frequent, and the
    # two score rules order some tied sums differently; scaled by 0.2 the
    # inner-product graph has both negative (clamped) and positive distances
    x, _ = datasets.gaussian_mixture(n=1800, d=12, clusters=6, mean_scale=1.0, seed=8)
    x = (x * 0.2).astype(np.float32)
    gi, gd = orc.exact_knn_metric(x, 30, metric, threads=8)
    if metric == 1:
        assert (gd < 0).any() and (gd > 0).any(), "the inner-product case should exercise clamping"
    kw = dict(runs=5, cycles=12, landmarks=10000, splitting=20, graph_neighbors=30, folds=10, knn_k=4,
              threads=4, materialize=1, metric=metric)
    r = ref.kodama_matrix_graph_data(x, gi, gd, 0, seed=99, **kw)
    o = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=99, **kw)
    for f in ("res", "acc", "v", "hashes", "run_counters", "cycle_diag", "knn_idx", "knn_dist"):
        assert np.array_equal(getattr(r, f), getattr(o, f)), f
    e = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=99, **dict(kw, metric=2))
    assert not (np.array_equal(e.res, o.res) and np.array_equal(e.cycle_diag, o.cycle_diag)), \
        "the score rule should change the evolution"


@needs_ref
def test_core_knn_graph_cosine_vs_reference(orc):
    """CoreKNNGraph with KNNOptions' default cosine metric (score 1 - d)."""
    x, _ = datasets.gaussian_mixture(n=1200, d=16, seed=6)
    gi, gd = orc.exact_knn_metric(x, 25, 0, threads=8)
    labels = np.random.default_rng(3).integers(1, 6, 1200).astype(np.int32)
    kw = dict(index_base=0, cycles=15, k=10, folds=5, seed=3, cv_seed=4, evolutionary=True, guarded=True,
              absorption=True, stratified=False, metric=0)
    a = ref.core_knn_graph(gi, gd, labels, **kw)
    b = orc.core_knn_graph(gi, gd, labels, **kw)
    for f in ("clbest", "cvpredbest", "folds", "vect_acc", "vect_score", "proposal_size",
              "active_classes", "flags", "counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert a.accbest == b.accbest and a.scorebest == b.scorebest


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


def _low_rank_noisy(n, d, seed, flip=0.3):
    x, y = datasets.low_rank(n=n, d=d, seed=seed)
    rng = np.random.default_rng(seed)
    lab = y.copy()
    f = rng.random(n) < flip
    lab[f] = rng.integers(1, 9, int(f.sum()))
    return x, lab.astype(np.int32)


@needs_ref
@pytest.mark.parametrize("n,d,stratified,maxc,fixc", [(300, 20, True, 5, 0), (500, 40, False, 5, 5),
                                                       (200, 300, False, 4, 4), (120, 10, True, 12, 0)])
def test_plsldacv_vs_reference(orc, n, d, stratified, maxc, fixc):
    x, lab = _low_rank_noisy(n, d, seed=n + d)
    kw = dict(folds=10, stratified=stratified, max_components=maxc, fixed_components=fixc, cv_seed=7)
    a = ref.plsldacv(x, lab, **kw)
    b = orc.plsldacv(x, lab, **kw)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2] == b[2] and np.array_equal(a[3], b[3])
    half = n // 2
    pa = ref.plsldapredict(x[:half], lab[:half], x[half:], components=maxc)
    pb = orc.plsldapredict(x[:half], lab[:half], x[half:], components=maxc)
    assert np.array_equal(pa, pb)


@needs_ref
@pytest.mark.parametrize("stratified,coarsening", [(False, True), (True, True), (False, False)])
def test_core_plslda_vs_reference(orc, stratified, coarsening):
    x, _ = datasets.low_rank(n=400, d=30, seed=5)
    labels = np.random.default_rng(6).integers(1, 12, 400).astype(np.int32)
    kw = dict(cycles=15, folds=5, stratified=stratified, components=4, evolutionary=True, guarded=True,
              absorption=True, coarsening=coarsening, seed=11, cv_seed=12,
              constrain=np.arange(1, 401, dtype=np.int32))
    a = ref.core_plslda(x, labels, **kw)
    b = orc.core_plslda(x, labels, **kw)
    for f in ("clbest", "cvpredbest", "folds", "vect_acc", "vect_score", "proposal_size",
              "active_classes", "flags", "counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert a.accbest == b.accbest and a.scorebest == b.scorebest


@needs_ref
def test_pls_matrix_vs_reference(orc):
    x, _ = datasets.low_rank(n=800, d=30, seed=3)
    gi, gd = orc.exact_knn(x, 20, threads=8)
    kw = dict(runs=3, cycles=8, landmarks=600, splitting=12, graph_neighbors=20, folds=5, knn_k=10,
              threads=3, materialize=1, classifier=1, components=4)
    a = ref.kodama_matrix_graph_data(x, gi, gd, 0, seed=77, **kw)
    b = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=77, **kw)
    for f in ("res", "acc", "v", "hashes", "run_counters", "cycle_diag", "knn_idx", "knn_dist", "pls_counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


@needs_ref
@pytest.mark.parametrize("n,d,stratified,maxc,fixc", [(300, 20, True, 5, 0), (500, 40, False, 5, 5),
                                                     (400, 10, False, 4, 0), (250, 80, True, 6, 6)])
def test_plsdacv_vs_reference(orc, n, d, stratified, maxc, fixc):
    x, lab = _low_rank_noisy(n, d, seed=n + d)
    kw = dict(folds=10, stratified=stratified, max_components=maxc, fixed_components=fixc, cv_seed=7, da=True)
    a = ref.plsldacv(x, lab, **kw)
    b = orc.plsldacv(x, lab, **kw)
    for u, v in zip(a[:4], b[:4]):
        assert np.array_equal(u, v)


@needs_ref
@pytest.mark.parametrize("classifier", [0, 1])
@pytest.mark.parametrize("inputs", ["start", "constrain", "fixed", "all"])
def test_semi_matrix_vs_reference(orc, classifier, inputs):
    x, y = datasets.gaussian_mixture(n=1500, d=12, seed=8)
    gi, gd = orc.exact_knn(x, 20, threads=8)
    rng = np.random.default_rng(3)
    n = len(x)
    start = (y % 5 + 1).astype(np.int32)
    flip = rng.random(n) < 0.3
    start[flip] = rng.integers(1, 6, int(flip.sum()))
    con = (rng.integers(0, 600, n) * 3 + 7).astype(np.int32)
    fix = (rng.random(n) < 0.1).astype(np.int32)
    extra = dict(starting=start if inputs in ("start", "all") else None,
                 constrain=con if inputs in ("constrain", "all") else None,
                 fixed=fix if inputs in ("fixed", "all") else None)
    kw = dict(runs=4, cycles=10, landmarks=1000, splitting=20, graph_neighbors=20, folds=5, knn_k=10, threads=4,
              materialize=1, classifier=classifier, components=4)
    a = ref.kodama_matrix_graph_data(x, gi, gd, 0, seed=11, **extra, **kw)
    b = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=11, **extra, **kw)
    for f in ("res", "acc", "v", "hashes", "run_counters", "cycle_diag", "knn_idx", "knn_dist", "pls_counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def _clustered(n, d, seed):
    rng = np.random.default_rng(seed)
    sizes = [n // 3, n // 3, n - 2 * (n // 3)]
    centres = rng.standard_normal((3, d)) * 1.5
    x = (rng.standard_normal((n, d)) + np.repeat(centres, sizes, axis=0)).astype(np.float32)
    return x, np.repeat([1, 2, 3], sizes).astype(np.int32)


@needs_ref
@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("stratified", [False, True])
def test_knncv_vs_reference(orc, metric, stratified):
    # small folds: the reference's HNSW search is exact here
    x, y = _clustered(300, 10, 3)
    a, fa, _ = ref.knncv(x, y, k=10, folds=10, stratified=stratified, metric=metric, cv_seed=5)
    b, fb, _ = orc.knncv(x, y, k=10, folds=10, stratified=stratified, metric=metric, cv_seed=5)
    assert np.array_equal(fa, fb) and np.array_equal(a, b)


@needs_ref
@pytest.mark.parametrize("metric", [0, 2])
@pytest.mark.parametrize("constrained", [False, True])
def test_core_knn_vs_reference(orc, metric, constrained):
    x, _ = _clustered(600, 20, 4)
    rng = np.random.default_rng(9)
    init = rng.integers(1, 7, 600).astype(np.int32)
    con = (np.arange(600) // 3 * 7 + 5).astype(np.int32)[rng.permutation(600)] if constrained else None
    fix = (rng.random(600) < 0.1).astype(np.int32) if constrained else None
    kw = dict(metric=metric, constrain=con, fixed=fix, cycles=15, k=10, folds=5, seed=4, cv_seed=6,
              evolutionary=constrained, guarded=constrained, absorption=constrained)
    a = ref.core_knn(x, init, **kw)
    b = orc.core_knn(x, init, **kw)
    for f in ("clbest", "cvpredbest", "folds", "vect_acc", "vect_score", "proposal_size",
              "active_classes", "flags", "counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
