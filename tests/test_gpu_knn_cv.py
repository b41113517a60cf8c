"""Raw-data fold-wise kNN on the GPU (KNNCV, CoreKNN) and CoreKNNGraph with
constraints and fixed rows, against the CPU restatement in oracle/."""

import numpy as np
import pytest

from kodama_gb300 import datasets


def _data(n, d, seed, classes=4):
    x, y = datasets.gaussian_mixture(n=n, d=d, seed=seed)
    rng = np.random.default_rng(seed)
    labels = (y % classes + 1).astype(np.int32)
    flip = rng.random(n) < 0.25
    labels[flip] = rng.integers(1, classes + 1, int(flip.sum()))
    return np.ascontiguousarray(x, np.float32), labels


@pytest.mark.gpu
@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("n,d,k,folds,stratified", [(1500, 20, 10, 10, True), (997, 70, 7, 5, False),
                                                      (400, 3, 25, 4, True)])
def test_knncv_matches_oracle(kg, orc, metric, n, d, k, folds, stratified):
    x, y = _data(n, d, n + d)
    a = kg.KNNCV(x, y, k=k, folds=folds, stratified=stratified, metric=metric, seed=11)
    b, fb, _ = orc.knncv(x, y, k=k, folds=folds, stratified=stratified, metric=metric, cv_seed=11)
    assert np.array_equal(a.fold_assignments, fb)
    assert np.array_equal(a.predicted_labels, b)
    assert a.global_accuracy == float(np.mean(b == y))
    assert sum(f.n_validation for f in a.folds) == n


@pytest.mark.gpu
def test_knncv_constrained_and_small_training_folds(kg, orc):
    # k larger than some folds' training sets: every remaining row votes
    x, y = _data(30, 5, 3)
    con = (np.arange(30) // 4).astype(np.int32)
    a = kg.KNNCV(x, y, constrain=con, k=40, folds=3, metric="euclidean", seed=2)
    b, fb, _ = orc.knncv(x, y, constrain=con, k=40, folds=3, metric=2, cv_seed=2)
    assert np.array_equal(a.fold_assignments, fb) and np.array_equal(a.predicted_labels, b)


@pytest.mark.gpu
def test_knncv_errors(kg):
    x, y = _data(50, 4, 1)
    with pytest.raises(RuntimeError, match="no training samples"):
        kg.KNNCV(x, y, constrain=np.zeros(50, np.int32), folds=5)
    with pytest.raises(ValueError, match="k must be positive"):
        kg.KNNCV(x, y, k=0)
    with pytest.raises(ValueError):
        kg.KNNCV(x, y, metric="manhattan")


@pytest.mark.gpu
@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("evolutionary", [False, True])
def test_core_knn_matches_oracle(kg, orc, metric, evolutionary):
    x, _ = _data(1200, 24, 5)
    rng = np.random.default_rng(metric + 10 * evolutionary)
    init = rng.integers(1, 9, 1200).astype(np.int32)
    kw = dict(cycles=25, k=30, folds=10, stratified=not evolutionary, seed=7, cv_seed=8)
    a = kg.CoreKNN(x, init, metric=metric, evolutionary_search=evolutionary, guarded_diversity=evolutionary,
                   many_to_one_absorption=evolutionary, **kw)
    b = orc.core_knn(x, init, metric=metric, evolutionary=evolutionary, guarded=evolutionary,
                     absorption=evolutionary, **kw)
    for f, g in (("clbest", "clbest"), ("cvpredbest", "cvpredbest"), ("fold_assignments", "folds"),
                 ("vect_acc", "vect_acc"), ("vect_score", "vect_score"), ("proposal_size", "proposal_size"),
                 ("active_classes", "active_classes"), ("flags", "flags")):
        assert np.array_equal(getattr(a, f), getattr(b, g)), f
    assert np.array_equal(a.counters[:16], b.counters) and not a.counters[16:].any()
    assert a.accbest == b.accbest and a.scorebest == b.scorebest


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
def test_constrained_fixed_core_matches_oracle(kg, orc, graph):
    x, _ = _data(900, 12, 6)
    rng = np.random.default_rng(4)
    init = rng.integers(1, 6, 900).astype(np.int32)
    con = rng.integers(0, 350, 900).astype(np.int32)
    fix = (rng.random(900) < 0.12).astype(np.int32)
    kw = dict(cycles=20, k=10, folds=5, stratified=True, seed=3, cv_seed=5)
    ev = dict(evolutionary_search=True, guarded_diversity=True, many_to_one_absorption=True)
    if graph:
        gi, gd = kg.knn_graph(x, 25)
        a = kg.CoreKNNGraph(gi, gd, init, index_base=0, constrain=con, fixed=fix, metric="euclidean", **kw, **ev)
        b = orc.core_knn_graph(gi, gd, init, index_base=0, constrain=con, fixed=fix, evolutionary=True,
                               guarded=True, absorption=True, **kw)
    else:
        a = kg.CoreKNN(x, init, metric="euclidean", constrain=con, fixed=fix, **kw, **ev)
        b = orc.core_knn(x, init, metric=2, constrain=con, fixed=fix, evolutionary=True, guarded=True,
                         absorption=True, **kw)
    assert np.array_equal(a.fold_assignments, b.folds)
    assert np.array_equal(a.clbest, b.clbest) and np.array_equal(a.vect_score, b.vect_score)
    assert np.array_equal(a.counters[:16], b.counters)
    # fixed rows keep their labels
    assert np.array_equal(a.clbest[fix == 1], init[fix == 1])
