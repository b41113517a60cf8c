"""CUDA path vs the CPU restatement (itself pinned to the reference), bit for bit.

Integer results (labels, indices, counters, hashes) and every double that the
reference computes (accuracies, scores) must be identical."""

import numpy as np
import pytest

from kodama_gb300 import datasets

pytestmark = pytest.mark.gpu


def _matrix_kw(**kw):
    base = dict(runs=4, cycles=10, landmarks=10000, splitting=0, graph_neighbors=50, folds=10,
                knn_k=10, seed=1234)
    base.update(kw)
    return base


def _oracle_matrix(orc, x, gi, gd, base, kw):
    return orc.kodama_matrix_graph_data(
        x, gi, gd, base, seed=kw["seed"], runs=kw["runs"], cycles=kw["cycles"],
        landmarks=kw["landmarks"], splitting=kw["splitting"], graph_neighbors=kw["graph_neighbors"],
        folds=kw["folds"], knn_k=kw["knn_k"], threads=4, materialize=1)


def _assert_matrix_equal(gpu, ref):
    assert np.array_equal(gpu.run_hashes, ref.hashes), "landmark / initial-label / fold hashes"
    assert np.array_equal(gpu.run_counters, ref.run_counters), "per-run counters"
    assert np.array_equal(gpu.cycle_diag, ref.cycle_diag), "per-cycle diagnostics"
    assert np.array_equal(gpu.acc, ref.acc), "best CV accuracy per run"
    assert np.array_equal(gpu.v, ref.v), "accuracy trace"
    assert np.array_equal(gpu.res, ref.res), "label matrix"
    assert np.array_equal(gpu.knn_idx, ref.knn_idx), "corrected graph indices"
    assert np.array_equal(gpu.knn_dist, ref.knn_dist), "corrected graph distances"


@pytest.mark.parametrize("K", [10, 50])
def test_knn_graph_spirals(kg, orc, K):
    x = datasets.spirals()[0].astype(np.float32)
    gi, gd = kg.knn_graph(x, K)
    ri, rd = orc.exact_knn(x, K, threads=4)
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)


def test_knn_graph_mixture(kg, orc):
    x, _ = datasets.gaussian_mixture(n=3000, d=50, seed=11)
    gi, gd = kg.knn_graph(x, 30)
    ri, rd = orc.exact_knn(x, 30, threads=8)
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)


def test_matrix_graph_data_spirals(kg, orc):
    x = datasets.spirals()[0].astype(np.float32)
    gi, gd = orc.exact_knn(x, 50, threads=4)
    kw = _matrix_kw()
    gpu = kg.KODAMA_matrix(x, graph=(gi + 1, gd), index_base=1, materialize_graph=True, **kw)
    ref = _oracle_matrix(orc, x, gi + 1, gd, 1, kw)
    _assert_matrix_equal(gpu, ref)


def test_matrix_raw_spirals(kg, orc):
    x = datasets.spirals()[0].astype(np.float32)
    kw = _matrix_kw(runs=6, cycles=20)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, **kw)
    gi, gd = orc.exact_knn(x, 50, threads=4)
    ref = _oracle_matrix(orc, x, gi, gd, 0, kw)
    _assert_matrix_equal(gpu, ref)


def test_matrix_raw_mixture(kg, orc):
    x, _ = datasets.gaussian_mixture(n=4000, d=50, seed=21)
    kw = _matrix_kw(runs=5, cycles=25, graph_neighbors=30, knn_k=30, splitting=40)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, **kw)
    gi, gd = orc.exact_knn(x, 30, threads=8)
    ref = _oracle_matrix(orc, x, gi, gd, 0, kw)
    _assert_matrix_equal(gpu, ref)


@pytest.mark.parametrize("d", [72, 100, 128, 160, 200])
def test_matrix_raw_high_dim(kg, orc, d):
    # tensor-core graph (d <= 128) and k-means (d <= 256) with 16-coordinate k-steps up to 8 / 16
    x, _ = datasets.gaussian_mixture(n=2500, d=d, clusters=9, mean_scale=3.0, seed=d)
    kw = _matrix_kw(runs=3, cycles=8, graph_neighbors=30, knn_k=10, splitting=100)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, **kw)
    gi, gd = orc.exact_knn(x, 30, threads=8)
    ref = _oracle_matrix(orc, x, gi, gd, 0, kw)
    _assert_matrix_equal(gpu, ref)


@pytest.mark.parametrize("d,splitting", [(50, 300), (100, 200), (20, 320)])
def test_matrix_raw_many_clusters(kg, orc, d, splitting):
    # more than 128 centroids: the exact assignment; the atlas and the landmark k-means differ in k
    x, _ = datasets.gaussian_mixture(n=4000, d=d, clusters=25, mean_scale=3.0, seed=d + splitting)
    kw = _matrix_kw(runs=3, cycles=6, graph_neighbors=30, knn_k=10, splitting=splitting)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, **kw)
    gi, gd = orc.exact_knn(x, 30, threads=8)
    ref = _oracle_matrix(orc, x, gi, gd, 0, kw)
    _assert_matrix_equal(gpu, ref)


@pytest.mark.parametrize("mode", [
    dict(evolutionary_search=False, guarded_diversity=False, many_to_one_absorption=False, stratified=True),
    dict(evolutionary_search=True, guarded_diversity=True, many_to_one_absorption=True, stratified=False),
    dict(evolutionary_search=True, guarded_diversity=True, many_to_one_absorption=True, stratified=True,
         adaptive_proposal_size=False),
])
def test_core_knn_graph_batch(kg, orc, mode):
    x, _ = datasets.gaussian_mixture(n=2000, d=20, seed=5)
    gi, gd = orc.exact_knn(x, 40, threads=8)
    rng = np.random.default_rng(3)
    problems = 4
    labels = np.stack([rng.integers(1, 2 + 3 * p, 2000) for p in range(problems)]).astype(np.int32) * 3 - 5
    seeds = np.arange(10, 10 + problems, dtype=np.uint64)
    cv_seeds = np.arange(100, 100 + problems, dtype=np.uint64)
    out = kg.CoreKNNGraph_batch(gi, gd, labels, seeds, cv_seeds, cycles=25, k=10, folds=7, index_base=0,
                                metric="euclidean", **mode)
    omode = dict(evolutionary=mode["evolutionary_search"], guarded=mode["guarded_diversity"],
                 absorption=mode["many_to_one_absorption"], stratified=mode["stratified"],
                 adaptive=mode.get("adaptive_proposal_size", True))
    for p in range(problems):
        r = orc.core_knn_graph(gi, gd, labels[p], index_base=0, cycles=25, k=10, folds=7,
                               seed=int(seeds[p]), cv_seed=int(cv_seeds[p]), **omode)
        g = out[p]
        assert np.array_equal(g.fold_assignments, r.folds)
        assert np.array_equal(g.clbest, r.clbest)
        assert np.array_equal(g.cvpredbest, r.cvpredbest)
        assert np.array_equal(g.vect_acc, r.vect_acc)
        assert np.array_equal(g.vect_score, r.vect_score)
        assert np.array_equal(g.proposal_size, r.proposal_size)
        assert np.array_equal(g.active_classes, r.active_classes)
        assert np.array_equal(g.flags, r.flags)
        assert g.accbest == r.accbest and g.scorebest == r.scorebest
        assert np.array_equal(g.counters[:16], r.counters) and not g.counters[16:].any()


def test_dissimilarity_inplace(kg, orc):
    rng = np.random.default_rng(9)
    n, K, M = 3000, 20, 30
    x, _ = datasets.gaussian_mixture(n=n, d=10, seed=9)
    gi, gd = orc.exact_knn(x, K, threads=8)
    gi1 = (gi + 1).astype(np.int32)
    gi1[rng.random(gi1.shape) < 0.02] = -1
    res = rng.integers(0, 6, (M, n)).astype(np.int32)
    ri, rd = orc.dissimilarity(gi1, gd, res)
    a, b = gi1.copy(), gd.copy()
    kg.KODAMADissimilarityInPlace(a, b, res)
    assert np.array_equal(a, ri)
    assert np.array_equal(b, rd)


def test_matrix_first_run_shard(kg):
    x = datasets.spirals()[0].astype(np.float32)
    kw = _matrix_kw(cycles=12)
    kw.pop("runs")
    full = kg.KODAMA_matrix(x, runs=6, **kw)
    part = kg.KODAMA_matrix(x, runs=3, first_run=3, **kw)
    assert np.array_equal(part.res, full.res[2:5])
    assert np.array_equal(part.acc, full.acc[2:5])
    assert np.array_equal(part.run_hashes, full.run_hashes[2:5])
    assert np.array_equal(part.run_counters, full.run_counters[2:5])
