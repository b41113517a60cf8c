"""The learned relabelling proposal: its network's forward pass and gradients
on the GPU against the CPU restatement in oracle/mlp_oracle.py, training, and
its use inside KODAMA.matrix."""

import numpy as np
import pytest

from kodama_gb300 import datasets
from oracle import mlp_oracle as M


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.PARAMS, np.float32)
    p[M.W1:M.B1] = rng.uniform(-0.8, 0.8, M.B1 - M.W1)
    p[M.B1:M.W2] = rng.uniform(-0.1, 0.1, M.W2 - M.B1)
    p[M.W2:M.B2] = rng.uniform(-0.3, 0.3, M.B2 - M.W2)
    p[M.B2:M.W3] = rng.uniform(-0.1, 0.1, M.W3 - M.B2)
    p[M.W3:M.B3] = rng.uniform(-0.3, 0.3, M.B3 - M.W3)
    return p


def _rows(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 8)).astype(np.float32)
    y = (x[:, 1] + 0.3 * rng.standard_normal(n) > x[:, 0]).astype(np.uint8)
    return x, y


def test_oracle_backprop_matches_finite_differences():
    # without bfloat16 rounding the network is smooth almost everywhere
    p = _params(1).astype(np.float64)
    x, y = _rows(64, 2)
    g, _ = M.gradient(p.astype(np.float32), x, y, rounding=False)
    rng = np.random.default_rng(3)
    for e in rng.choice(M.PARAMS, 40, replace=False):
        eps = 1e-2
        hi, lo = p.copy(), p.copy()
        hi[e] += eps
        lo[e] -= eps
        lh = M.gradient(hi.astype(np.float32), x, y, rounding=False)[1]
        ll = M.gradient(lo.astype(np.float32), x, y, rounding=False)[1]
        fd = (lh - ll) / (float(np.float32(hi[e])) - float(np.float32(lo[e])))
        assert abs(fd - g[e]) <= 2e-3 * max(1.0, abs(g[e])) + 2e-4, e


@pytest.mark.gpu
def test_gradient_matches_oracle(kg):
    p = _params(4)
    x, y = _rows(3000, 5)
    g, loss = kg.proposal_gradient(p, x, y)
    go, lo = M.gradient(p, x, y)
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    cos = float(g @ go / (np.linalg.norm(g) * np.linalg.norm(go)))
    assert rel < 2e-2 and cos > 0.999, (rel, cos)
    assert abs(loss - lo) < 1e-3


@pytest.mark.gpu
def test_predict_matches_oracle(kg):
    p = _params(6)
    x, _ = _rows(2000, 7)
    z = kg.proposal_predict(p, x)
    zo, _ = M.forward(p, x)
    assert np.max(np.abs(z - zo)) < 2e-2 * max(1.0, np.max(np.abs(zo)))


@pytest.mark.gpu
def test_training_reduces_loss(kg):
    x, y = _rows(20000, 8)
    w, losses = kg.train_proposal(x, y, epochs=8, batch=1024, learning_rate=3e-3, seed=2)
    assert losses[-1] < losses[0] and losses[-1] < 0.45
    w2, losses2 = kg.train_proposal(x, y, epochs=8, batch=1024, learning_rate=3e-3, seed=2)
    assert np.array_equal(w, w2) and np.array_equal(losses, losses2)  # deterministic


@pytest.mark.gpu
def test_snapshot_leaves_plain_run_unchanged(kg):
    x, _ = datasets.gaussian_mixture(n=3000, d=20, seed=9)
    kw = dict(runs=4, cycles=12, landmarks=2000, splitting=20, graph_neighbors=20, folds=5, knn_k=10, seed=5)
    a = kg.KODAMA_matrix(x, **kw)
    b = kg.KODAMA_matrix(x, snapshot_cycle=4, **kw)
    assert np.array_equal(a.res, b.res) and np.array_equal(a.acc, b.acc)
    assert b.snapshot_features.shape == (4, 2000, 8)
    assert (b.snapshot_flags & 1).any()


def test_default_weights_ship():
    from kodama_gb300 import proposal_training as PT
    w = PT.load_default()
    assert w.shape == (M.PARAMS,) and np.isfinite(w).all()


@pytest.mark.gpu
def test_trained_network_gains_over_plain(kg):
    # shipped weights, trained on plain-run moves of other workloads; at equal
    # cycle counts the learned proposal reaches a higher mean final CV accuracy
    from kodama_gb300 import proposal_training as PT
    w = PT.load_default()
    x, _ = datasets.gaussian_mixture(n=6000, d=30, seed=13)
    kw = dict(runs=16, landmarks=4000, splitting=30, graph_neighbors=20, knn_k=20, folds=10, seed=5)
    for T in (8, 12):
        plain = kg.KODAMA_matrix(x, cycles=T, **kw)
        learned = kg.KODAMA_matrix(x, cycles=T, proposal_weights=w, **kw)
        assert learned.acc.mean() > plain.acc.mean() + 0.01, (T, plain.acc.mean(), learned.acc.mean())
        assert (learned.acc > plain.acc).sum() > kw["runs"] // 2
