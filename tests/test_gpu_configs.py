"""Bit-exact parity at the benchmark configurations themselves.

Each test runs one full KODAMA.matrix call on the GPU through the C ABI and
the CPU restatement (pinned to the reference core) on the same exact graph,
at the workload's own sizes, and compares every output field bit for bit:
labels, best accuracies, accuracy traces, per-run landmark / initial-label /
fold hashes, run counters, per-cycle diagnostics, PLS coarsening counters and
the corrected graph.

* spirals: N=1000, d=10, M=20, Tcycle=20, knn.k=10, K=50, 10 folds (L=750);
* mixture: N=20000, d=50, M=100, Tcycle=100, K=30, knn.k=30, 10 folds,
  splitting=50, landmarks=10000 -- the workload bench.py times;
* PLS-LDA: N=10000, d=200, ncomp=5, M=50, Tcycle=50, 10 folds (L=7500);
* PCA-like mixture: N=100000, d=50, M=100, Tcycle=100, K=30, knn.k=30: the
  device graph is checked row for row against the exact search on 4000
  sampled rows, then the matrix against the restatement fed that graph.
"""

import os

import numpy as np
import pytest

from kodama_gb300 import datasets

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _oracle(orc, x, gi, gd, kw, classifier=0):
    kw = dict(kw)
    seed = kw.pop("seed")
    return orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=seed, threads=THREADS, materialize=1,
                                        classifier=classifier, **kw)


def _assert_equal(gpu, ref, pls=False):
    assert np.array_equal(gpu.run_hashes, ref.hashes), "landmark / initial-label / fold hashes"
    assert np.array_equal(gpu.run_counters, ref.run_counters), "per-run counters"
    assert np.array_equal(gpu.cycle_diag, ref.cycle_diag), "per-cycle diagnostics"
    assert np.array_equal(gpu.acc, ref.acc), "best CV accuracy per run"
    assert np.array_equal(gpu.v, ref.v), "accuracy trace"
    assert np.array_equal(gpu.res, ref.res), "label matrix"
    assert np.array_equal(gpu.knn_idx, ref.knn_idx), "corrected graph indices"
    assert np.array_equal(gpu.knn_dist, ref.knn_dist), "corrected graph distances"
    if pls:
        assert np.array_equal(gpu.pls_counters, ref.pls_counters), "PLS coarsening counters"


def test_config_spirals(kg, orc):
    x = datasets.spirals()[0].astype(np.float32)
    kw = dict(runs=20, cycles=20, landmarks=10000, splitting=0, graph_neighbors=50, folds=10, knn_k=10, seed=1234)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, **kw)
    assert gpu.effective_landmarks == 750
    gi, gd = orc.exact_knn(x, 50, threads=THREADS)
    assert np.array_equal(kg.knn_graph(x, 50)[0], gi)
    _assert_equal(gpu, _oracle(orc, x, gi, gd, kw))


def test_config_mixture_20k(kg, orc):
    x, _ = datasets.gaussian_mixture(n=20000, d=50, seed=2)
    kw = dict(runs=100, cycles=100, landmarks=10000, splitting=50, graph_neighbors=30, folds=10, knn_k=30,
              seed=1234)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, **kw)
    assert gpu.effective_landmarks == 10000
    gi, gd = orc.exact_knn(x, 30, threads=THREADS)
    dgi, dgd = kg.knn_graph(x, 30)
    assert np.array_equal(dgi, gi) and np.array_equal(dgd, gd), "device exact graph"
    _assert_equal(gpu, _oracle(orc, x, gi, gd, kw))


def test_config_pls_low_rank(kg, orc):
    x, _ = datasets.low_rank(n=10000, d=200, seed=3)
    kw = dict(runs=50, cycles=50, landmarks=10000, splitting=0, graph_neighbors=30, folds=10, knn_k=30,
              seed=1234, components=5)
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, classifier="pls", **kw)
    assert gpu.effective_landmarks == 7500
    gi, gd = orc.exact_knn(x, 30, threads=THREADS)
    _assert_equal(gpu, _oracle(orc, x, gi, gd, kw, classifier=1), pls=True)


def test_config_pca_mixture_100k(kg, orc):
    x, _ = datasets.pca_mixture(n=100000, d=50, seed=5)
    kw = dict(runs=100, cycles=100, landmarks=10000, splitting=0, graph_neighbors=30, folds=10, knn_k=30,
              seed=1234)
    gi, gd = kg.knn_graph(x, 30)
    rows = np.random.default_rng(5).choice(x.shape[0], 4000, replace=False).astype(np.int32)
    ri, rd = orc.exact_knn_rows(x, 30, rows, threads=THREADS)
    assert np.array_equal(gi[rows], ri) and np.array_equal(gd[rows], rd), "device exact graph (sampled rows)"
    gpu = kg.KODAMA_matrix(x, materialize_graph=True, **kw)
    _assert_equal(gpu, _oracle(orc, x, gi, gd, kw))
