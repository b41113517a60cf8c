"""Error of the float32 PLS-LDA arithmetic (which the GPU reproduces bit for
bit) against an FP64 restatement of the same cross-validation
(oracle/pls_fp64.py): predicted labels may differ only where the float64 LDA
margin is below 1e-5 relative, and the float64 restatement must reach the
same accuracy."""

import numpy as np
import pytest

from kodama_gb300 import datasets


@pytest.mark.parametrize("noise", [0.0, 0.25])
def test_plslda_float32_vs_fp64(orc, noise):
    from oracle import pls_fp64
    x, y = datasets.low_rank(n=3000, d=60, seed=11)
    x = np.ascontiguousarray(x, np.float32)
    rng = np.random.default_rng(5)
    lab = y.copy()
    flip = rng.random(len(y)) < noise
    lab[flip] = rng.integers(1, 9, int(flip.sum()))
    pred, folds, _, _, _ = orc.plsldacv(x, lab, folds=10, stratified=False, max_components=5, fixed_components=5,
                                        threads=4, cv_seed=3)
    rep = pls_fp64.compare(orc._LIB, x, lab, folds, pred, 5)
    assert rep["mismatches_below_1e-5_rel_margin"], rep
    assert rep["mismatch_fraction"] <= 1e-3, rep
    assert abs(rep["accuracy_float32"] - rep["accuracy_float64"]) <= 1e-3, rep
