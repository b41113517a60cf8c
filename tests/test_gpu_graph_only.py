"""KODAMA.matrix from a graph alone (kgb_kodama_matrix_from_graph): the
graph's Laplacian features (host) then the graph-input path on the device,
against the CPU restatement of that path on the same features."""

import numpy as np
import pytest

from kodama_gb300 import datasets

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("base,classifier", [(0, "knn"), (1, "knn"), (0, "pls")])
def test_matrix_from_graph_matches_oracle(kg, orc, base, classifier):
    x, _ = datasets.gaussian_mixture(n=2000, d=16, clusters=7, mean_scale=3.0, seed=62)
    gi, gd = orc.exact_knn(x, 20, threads=8)
    g_in = gi + 1 if base == 1 else gi
    kw = dict(runs=3, cycles=8, splitting=20, graph_neighbors=20, folds=5, knn_k=10, components=6, seed=5)
    r = kg.KODAMA_matrix(None, graph=(g_in, gd), graph_only=True, index_base=base, materialize_graph=True,
                         classifier=classifier, feature_components=0, feature_steps=3, **kw)
    f = kg.KODAMA_graph_features(g_in, gd, index_base=base, components=6, steps=3, seed=5)
    o = orc.kodama_matrix_graph_data(f, g_in, gd, base, seed=5, runs=3, cycles=8, landmarks=10000, splitting=20,
                                     graph_neighbors=20, folds=5, knn_k=10, threads=4, materialize=1,
                                     classifier=1 if classifier == "pls" else 0, components=6)
    assert np.array_equal(r.run_hashes, o.hashes)
    assert np.array_equal(r.run_counters, o.run_counters)
    assert np.array_equal(r.acc, o.acc) and np.array_equal(r.v, o.v)
    assert np.array_equal(r.res, o.res)
    assert np.array_equal(r.knn_idx, o.knn_idx) and np.array_equal(r.knn_dist, o.knn_dist)
