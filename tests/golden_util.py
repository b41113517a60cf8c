"""Replay of the cases in tests/golden/golden.json (made from the reference's
own CPU core by tests/golden/make_golden.py) through any implementation with
the oracle's calling convention."""

import hashlib
import json
import os

import numpy as np

from kodama_gb300 import datasets

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cases():
    with open(os.path.join(HERE, "golden", "golden.json")) as f:
        return json.load(f)["cases"]


def pls_inputs(spec):
    """Low-rank PLS workload of a case spec: (x, labels) with optional label noise."""
    x, y = datasets.low_rank(n=spec["n"], d=spec["d"], seed=spec["seed"])
    rng = np.random.default_rng(spec["seed"] + 1000)
    labels = y.copy()
    flip = rng.random(len(y)) < spec.get("flip", 0.0)
    labels[flip] = rng.integers(1, 9, int(flip.sum()))
    if spec.get("random_labels"):
        labels = rng.integers(1, spec["random_labels"] + 1, len(y)).astype(np.int32)
    return x, labels.astype(np.int32)


def knn_inputs(spec):
    """Mixture workload of a KNNCV / CoreKNN case spec: (x, labels, constrain,
    fixed) -- the cluster labels with a fraction replaced, or random start
    labels; constrain groups of `groups_of` rows; a `fixed_frac` of fixed rows."""
    x, y = datasets.gaussian_mixture(n=spec["n"], d=spec["d"], seed=spec["seed"])
    rng = np.random.default_rng(spec["seed"] + 2000)
    labels = (y + 1).astype(np.int32)
    flip = rng.random(len(y)) < spec.get("flip", 0.0)
    labels[flip] = rng.integers(1, 9, int(flip.sum()))
    if spec.get("random_labels"):
        labels = rng.integers(1, spec["random_labels"] + 1, len(y)).astype(np.int32)
    con = fix = None
    if spec.get("groups_of"):
        g = spec["groups_of"]
        con = (np.arange(len(y)) // g * 7 + 5).astype(np.int32)[rng.permutation(len(y))]
    if spec.get("fixed_frac"):
        fix = (rng.random(len(y)) < spec["fixed_frac"]).astype(np.int32)
    return np.ascontiguousarray(x, np.float32), labels.astype(np.int32), con, fix


def semi_inputs(spec):
    """Semi-supervised KODAMA.matrix case: (x, starting_labels, constrain,
    fixed) from knn_inputs(spec), the start labels mapped to 3*label - 7 (so
    they are neither positive nor consecutive); each of the three is kept
    only where the spec asks for it (use_start, groups_of, fixed_frac)."""
    x, labels, con, fix = knn_inputs(spec)
    start = (labels * 3 - 7).astype(np.int32) if spec.get("use_start") else None
    return x, start, con, fix


def check_knncv(case, pred, folds):
    assert sha(folds) == case["folds_sha256"], "folds"
    assert np.asarray(pred)[:32].tolist() == case["predicted_head"], "predictions head"
    assert sha(pred) == case["predicted_sha256"], "predictions"


def inputs(case):
    if "input" in case:
        return pls_inputs(case["input"])[0]
    name = case["name"]
    if name.startswith("spirals"):
        return datasets.spirals()[0].astype(np.float32)
    if name.startswith("mixture"):
        return datasets.gaussian_mixture(n=3000, d=50, seed=21)[0]
    return datasets.gaussian_mixture(n=2000, d=20, seed=5)[0]


def core_labels():
    rng = np.random.default_rng(3)
    return (rng.integers(1, 9, 2000) * 3 - 5).astype(np.int32)


def check_matrix(case, r):
    """r: object with res, acc, v, hashes/run_hashes, run_counters, cycle_diag, knn_idx, knn_dist."""
    hashes = getattr(r, "run_hashes", None)
    if hashes is None:
        hashes = r.hashes
    assert [[int(v) for v in row] for row in hashes] == case["hashes"], "per-run hashes"
    assert np.asarray(r.run_counters).tolist() == case["run_counters"], "run counters"
    assert sha(r.cycle_diag) == case["cycle_diag_sha256"], "cycle diagnostics"
    assert np.asarray(r.acc).tolist() == case["acc"], "accuracies"
    assert sha(r.v) == case["v_sha256"], "accuracy trace"
    assert np.asarray(r.res)[:, :16].tolist() == case["res_head"], "label matrix head"
    assert sha(r.res) == case["res_sha256"], "label matrix"
    assert sha(r.knn_idx) == case["knn_idx_sha256"], "corrected graph indices"
    assert sha(r.knn_dist) == case["knn_dist_sha256"], "corrected graph distances"


def check_core(case, r, folds_attr="folds"):
    assert sha(getattr(r, folds_attr)) == case["folds_sha256"], "folds"
    assert sha(r.clbest) == case["clbest_sha256"], "clbest"
    assert sha(r.cvpredbest) == case["cvpredbest_sha256"], "cvpredbest"
    assert np.asarray(r.vect_acc).tolist() == case["vect_acc"], "vect_acc"
    assert np.asarray(r.vect_score).tolist() == case["vect_score"], "vect_score"
    assert np.asarray(r.proposal_size).tolist() == case["proposal_size"], "proposal sizes"
    assert np.asarray(r.active_classes).tolist() == case["active_classes"], "active classes"
    assert np.asarray(r.flags).tolist() == case["flags"], "accept flags"
    assert r.accbest == case["accbest"] and r.scorebest == case["scorebest"], "best scalars"
    got = np.asarray(r.counters).tolist()
    want = case["counters"]
    # the kNN core has no PLS coarsening: counters beyond the recorded ones are zero
    assert got[:len(want)] == want and not any(got[len(want):]), "counters"


def check_pls_matrix(case, r):
    check_matrix(case, r)
    assert np.asarray(r.pls_counters).tolist() == case["pls_counters"], "PLS coarsening counters"
