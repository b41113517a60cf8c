"""The cosine and inner-product metrics on the GPU against the CPU restatement
(itself pinned to the reference for these metrics in test_oracle_pins.py).

* the exact graph under each metric (KODAMAGraph / kgb_knn_graph_metric);
* KODAMA.matrix from raw data with KODAMAMatrixOptions::metric: the graph of
  that metric, its distances clamped at zero as the graph-input path clamps
  them, and the vote score 1 - d (core.cpp:672-677);
* CoreKNNGraph with KNNOptions' default cosine metric;
* the resident graph handle built under a metric;
* an unknown metric is an error, not a silent Euclidean run.
"""

import numpy as np
import pytest

from kodama_gb300 import datasets

pytestmark = pytest.mark.gpu

METRICS = {"cosine": 0, "inner_product": 1}


def _data():
    # overlapping clusters near unit norm: the inner-product graph holds
    # negative and positive reported distances, and count ties in the vote
    # are frequent enough for the score rule to matter
    x, _ = datasets.gaussian_mixture(n=1800, d=12, clusters=6, mean_scale=1.0, seed=8)
    return (x * 0.2).astype(np.float32)


@pytest.mark.parametrize("metric", list(METRICS))
def test_metric_graph(kg, orc, metric):
    x = _data()
    gi, gd = kg.knn_graph(x, 30, metric=metric)
    ri, rd = orc.exact_knn_metric(x, 30, METRICS[metric], threads=8)
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)


@pytest.mark.parametrize("metric", list(METRICS))
def test_metric_graph_wide(kg, orc, metric):
    x, _ = datasets.gaussian_mixture(n=3000, d=50, seed=13)
    gi, gd = kg.knn_graph(x, 30, metric=metric)
    ri, rd = orc.exact_knn_metric(x, 30, METRICS[metric], threads=8)
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)


@pytest.mark.parametrize("metric", list(METRICS))
def test_metric_matrix_raw(kg, orc, metric):
    x = _data()
    kw = dict(runs=5, cycles=12, landmarks=10000, splitting=20, graph_neighbors=30, folds=10, knn_k=4, seed=99)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, metric=metric, **kw)
    gi, gd = orc.exact_knn_metric(x, 30, METRICS[metric], threads=8)
    ref = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=kw.pop("seed"), threads=8, materialize=1,
                                       metric=METRICS[metric], **kw)
    assert np.array_equal(gpu.run_hashes, ref.hashes)
    assert np.array_equal(gpu.run_counters, ref.run_counters)
    assert np.array_equal(gpu.cycle_diag, ref.cycle_diag)
    assert np.array_equal(gpu.acc, ref.acc)
    assert np.array_equal(gpu.v, ref.v)
    assert np.array_equal(gpu.res, ref.res)
    assert np.array_equal(gpu.knn_idx, ref.knn_idx)
    assert np.array_equal(gpu.knn_dist, ref.knn_dist)


def test_core_knn_graph_cosine_default(kg, orc):
    x, _ = datasets.gaussian_mixture(n=1200, d=16, seed=6)
    gi, gd = orc.exact_knn_metric(x, 25, 0, threads=8)
    labels = np.random.default_rng(3).integers(1, 6, 1200).astype(np.int32)
    kw = dict(cycles=15, k=10, folds=5, seed=3, cv_seed=4, stratified=False)
    g = kg.CoreKNNGraph(gi, gd, labels, index_base=0, evolutionary_search=True, guarded_diversity=True,
                        many_to_one_absorption=True, **kw)
    r = orc.core_knn_graph(gi, gd, labels, index_base=0, evolutionary=True, guarded=True, absorption=True,
                           metric=0, **kw)
    assert np.array_equal(g.clbest, r.clbest)
    assert np.array_equal(g.cvpredbest, r.cvpredbest)
    assert np.array_equal(g.vect_acc, r.vect_acc)
    assert np.array_equal(g.vect_score, r.vect_score)
    assert np.array_equal(g.counters[:16], r.counters)


def test_metric_graph_handle(kg):
    x = _data()
    kw = dict(runs=4, cycles=10, landmarks=10000, splitting=20, graph_neighbors=30, folds=10, knn_k=4, seed=5,
              materialize_graph=True, metric="inner_product")
    direct = kg.KODAMA_matrix(x, **kw)
    with kg.KODAMAGraph(x, neighbors=30, metric="inner_product") as g:
        gi, gd = g.graph()
        assert (gd < 0).any(), "the handle keeps the reported distances as KODAMAGraph does"
        via = g.matrix(**kw)
    assert np.array_equal(direct.res, via.res)
    assert np.array_equal(direct.v, via.v)
    assert np.array_equal(direct.knn_idx, via.knn_idx)
    assert np.array_equal(direct.knn_dist, via.knn_dist)


def test_unknown_metric_rejected(kg):
    x = _data()
    with pytest.raises(Exception, match="metric"):
        kg.KODAMA_matrix(x, runs=2, cycles=2, metric=7)
