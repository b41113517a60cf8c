"""FP64 restatement of one PLS-LDA cross-validation (TEST INFRASTRUCTURE ONLY).

The GPU path computes PLS-LDA in the reference's float32 arithmetic, bit for
bit (its predictions equal the CPU restatement's, which equal the
reference's).  This module states the error of that arithmetic against the
same computation in float64: per fold the standardisation
(train_center_scale_float, plscv.cpp:669-698), the centred label
cross-product (:700-731), SIMPLS with two power refreshes per component from
the same float32 start vector (fit_pls_components_from_crossprod_float,
:816-955; the Gram form is the same algebra), the LDA from the score
statistics with the same ridge grid (fit_lda_from_score_statistics_float,
:1419-1487) and the validation predictions; all in numpy float64.  The
comparison reports the labels the two disagree on and the float64 relative
margin of the LDA discriminant (best - second) / max(|best|, |second|) at
those rows, the quantity the contract on PLS-LDA labels is stated in."""

from __future__ import annotations

import ctypes

import numpy as np

FLT_MIN = float(np.finfo(np.float32).tiny)
RIDGES = (1e-8, 1e-6, 1e-5, 1e-4, 1e-3, 1e-2)


def start_vector(L, p: int) -> np.ndarray:
    out = np.zeros(p, np.float32)
    L.pls_start(p, out.ctypes.data_as(ctypes.c_void_p))
    return out.astype(np.float64)


def _simpls(zt: np.ndarray, s: np.ndarray, max_components: int, start: np.ndarray) -> np.ndarray:
    n, p = zt.shape
    max_rank = min(max_components, p, max(1, n - 1))
    s = s.copy()
    weights, basis, prev = [], [], None
    for _ in range(max_rank):
        w = start.copy() if prev is None else prev.copy()

        def refresh(v):
            for _ in range(2):
                v = s @ (s.T @ v)
            return v

        w = refresh(w)
        nrm = float(np.linalg.norm(w))
        if prev is None and (not np.isfinite(nrm) or nrm <= 1e-10):
            col = int(np.argmax((s * s).sum(0)))
            if float((s[:, col] ** 2).sum()) > 1e-20:
                w = refresh(s[:, col].copy())
                nrm = float(np.linalg.norm(w))
        if not np.isfinite(nrm) or nrm <= 1e-10:
            break
        w = w / nrm
        t = zt @ w
        tn = float(np.linalg.norm(t))
        if not np.isfinite(tn) or tn <= 1e-10:
            break
        t, w = t / tn, w / tn
        ld = zt.T @ t
        prev = w.copy()
        for v in basis:
            ld = ld - float(v @ ld) * v
        ln = float(np.linalg.norm(ld))
        if not np.isfinite(ln) or ln <= 1e-10:
            break
        ld = ld / ln
        weights.append(w)
        basis.append(ld)
        s = s - np.outer(ld, s.T @ ld)
    return np.stack(weights, axis=1) if weights else np.zeros((p, 0))


def fold_fp64(x: np.ndarray, labels: np.ndarray, train: np.ndarray, val: np.ndarray, components: int,
              start: np.ndarray, center: bool = True, scale: bool = True):
    """Float64 predictions and relative LDA margins of the validation rows."""
    xt = x[train].astype(np.float64)
    n = xt.shape[0]
    mean = xt.mean(0) if center else np.zeros(x.shape[1])
    sd = np.ones(x.shape[1])
    if scale:
        d = xt - mean
        sd = np.sqrt((d * d).sum(0) / max(1.0, n - 1.0))
        sd[~(np.isfinite(sd) & (sd > 0))] = 1.0
    zt = (xt - mean) / sd
    zv = (x[val].astype(np.float64) - mean) / sd
    y = labels[train]
    classes = np.unique(y)
    m = len(classes)
    if m <= 1:
        return np.full(len(val), classes[0] if m else 0), np.full(len(val), np.inf)
    onehot = (y[:, None] == classes[None, :]).astype(np.float64)
    counts = onehot.sum(0)
    cross = zt.T @ onehot - np.outer(zt.sum(0), counts / n)
    w = _simpls(zt, cross, components, start)
    if w.shape[1] == 0:
        # DegeneratePLSFit: the most frequent training label
        return np.full(len(val), classes[int(np.argmax(counts))]), np.full(len(val), np.inf)
    t = zt @ w
    mu = (onehot.T @ t) / np.maximum(counts, 1.0)[:, None]
    pooled = (t.T @ t - (mu * counts[:, None]).T @ mu) / max(1, n - m)
    trace = float(np.trace(pooled))
    ridge_scale = trace / max(1, w.shape[1]) if np.isfinite(trace) and trace > 0 else 1.0
    lin = None
    for ridge in RIDGES:
        cov = pooled + ridge * ridge_scale * np.eye(w.shape[1])
        try:
            c = np.linalg.cholesky(cov)
        except np.linalg.LinAlgError:
            continue
        lin = np.linalg.solve(c.T, np.linalg.solve(c, mu.T))
        break
    if lin is None:
        raise RuntimeError("float64 PLS-LDA Cholesky factorization failed")
    const = -0.5 * (mu * lin.T).sum(1) + np.log(np.maximum(counts / n, FLT_MIN))
    disc = const[None, :] + (zv @ w) @ lin
    order = np.argsort(-disc, axis=1, kind="stable")
    best = disc[np.arange(len(val)), order[:, 0]]
    second = disc[np.arange(len(val)), order[:, 1]]
    rel = (best - second) / np.maximum(np.maximum(np.abs(best), np.abs(second)), 1e-300)
    return classes[order[:, 0]], rel


def compare(L, x: np.ndarray, labels: np.ndarray, folds: np.ndarray, float_pred: np.ndarray, components: int) -> dict:
    """Float64 restatement against the float32 predictions of one CV run."""
    x = np.ascontiguousarray(x, np.float32)
    start = start_vector(L, x.shape[1])
    pred64 = np.zeros_like(float_pred)
    rel = np.zeros(len(labels))
    for f in np.unique(folds):
        val = np.flatnonzero(folds == f)
        train = np.flatnonzero(folds != f)
        p, r = fold_fp64(x, labels, train, val, components, start)
        pred64[val] = p
        rel[val] = r
    diff = pred64 != float_pred
    return {"rows": int(len(labels)), "label_mismatches": int(diff.sum()),
            "mismatch_fraction": float(diff.mean()),
            "max_rel_margin_at_mismatch": float(rel[diff].max()) if diff.any() else None,
            "min_rel_margin": float(rel.min()),
            "mismatches_below_1e-5_rel_margin": bool((rel[diff] < 1e-5).all()) if diff.any() else True,
            "accuracy_float32": float((float_pred == labels).mean()),
            "accuracy_float64": float((pred64 == labels).mean())}
