"""The CPU restatement must be at least as fast as the reference's own CPU core.

The restatement (oracle/kodama_oracle.cpp, oracle/pls_oracle.cpp) is what the
benchmark times as the CPU baseline on the GPU host, where the reference
sources are absent.  A port slower than the reference would overstate the
GPU's speed-up, so this test times both on the same graph and the same sample
of the benchmark workloads (all host threads, best of two) and fails if the
port takes more than 1.1x the reference's time.  Skipped where the reference
core (oracle/_ref) was not built."""

import os
import time

import numpy as np
import pytest

from kodama_gb300 import datasets

SLACK = 1.1


def _ref():
    from oracle import ref
    if not ref.available():
        pytest.skip("reference core (oracle/_ref) not built")
    return ref


def _best_of(fn, repeats=2):
    best = float("inf")
    out = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        out = fn()
        best = min(best, time.perf_counter() - t0)
    return best, out


def _compare(orc, ref, x, gi, gd, kw):
    threads = os.cpu_count() or 1
    run = lambda lib: lib.kodama_matrix_graph_data(x, gi, gd, 0, seed=1234, threads=threads, materialize=0, **kw)
    t_ref, r_ref = _best_of(lambda: run(ref))
    t_orc, r_orc = _best_of(lambda: run(orc))
    assert np.array_equal(r_orc.res, r_ref.res) and np.array_equal(r_orc.acc, r_ref.acc)
    print(f"reference {t_ref:.3f} s, port {t_orc:.3f} s on {threads} threads")
    assert t_orc <= SLACK * t_ref, f"port {t_orc:.3f} s > {SLACK} x reference {t_ref:.3f} s"


def test_port_speed_knn_matrix(orc):
    """KODAMA.matrix kNN, N=20000, d=50, 16 of the 100 runs, Tcycle=100."""
    ref = _ref()
    x, _ = datasets.gaussian_mixture(n=20000, d=50, seed=2)
    x = np.ascontiguousarray(x, np.float32)
    gi, gd = orc.exact_knn(x, 30, threads=os.cpu_count() or 1)
    _compare(orc, ref, x, gi, gd, dict(runs=16, cycles=100, landmarks=10000, splitting=50, graph_neighbors=30,
                                       folds=10, knn_k=30))


def test_port_speed_pls_matrix(orc):
    """KODAMA.matrix PLS-LDA, N=10000, d=200, ncomp=5, 8 of the 50 runs, Tcycle=20."""
    ref = _ref()
    x, _ = datasets.low_rank(n=10000, d=200, seed=3)
    x = np.ascontiguousarray(x, np.float32)
    gi, gd = orc.exact_knn(x, 30, threads=os.cpu_count() or 1)
    _compare(orc, ref, x, gi, gd, dict(runs=8, cycles=20, landmarks=10000, splitting=0, graph_neighbors=30,
                                       folds=10, knn_k=30, components=5, classifier=1))
