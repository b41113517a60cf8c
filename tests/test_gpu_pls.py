"""PLS-LDA on the GPU against the CPU restatement (oracle) and the reference's
recorded outputs (tests/golden).  Every comparison is exact: the CUDA path
replays the reference's float32 / double accumulation order, so labels,
accuracies and scores must be bit-identical."""

import numpy as np
import pytest

import golden_util as G
from kodama_gb300 import datasets

pytestmark = pytest.mark.gpu


def _noisy(n, d, seed, flip=0.3):
    x, y = datasets.low_rank(n=n, d=d, seed=seed)
    rng = np.random.default_rng(seed)
    lab = y.copy()
    f = rng.random(n) < flip
    lab[f] = rng.integers(1, 9, int(f.sum()))
    return x, lab.astype(np.int32)


@pytest.mark.parametrize("n,d,stratified,maxc,fixc", [(300, 20, True, 5, 0), (500, 40, False, 5, 5),
                                                       (200, 300, False, 4, 4), (120, 10, True, 12, 0),
                                                       (2000, 60, False, 8, 0), (300, 600, False, 4, 0),
                                                       (240, 1100, True, 3, 0)])
def test_plsldacv_matches_oracle(kg, orc, n, d, stratified, maxc, fixc):
    x, lab = _noisy(n, d, seed=n + d)
    kw = dict(folds=10, stratified=stratified, max_components=maxc, fixed_components=fixc, cv_seed=7)
    pred, folds, sel, abc, _ = orc.plsldacv(x, lab, **kw)
    g = kg.PLSLDACV(x, lab, **kw)
    assert np.array_equal(g.fold_assignments, folds)
    assert np.array_equal(g.predicted_labels, pred)
    assert g.selected_components == sel
    assert np.array_equal(g.accuracy_by_components, abc)


def test_plsldacv_degenerate_and_single_class_folds(kg, orc):
    # labels that make some folds single-class and one class tiny
    x, _ = datasets.low_rank(n=60, d=8, seed=4)
    lab = np.ones(60, np.int32)
    lab[:3] = 2
    kw = dict(folds=5, stratified=False, max_components=3, fixed_components=0, cv_seed=3)
    pred, folds, sel, abc, _ = orc.plsldacv(x, lab, **kw)
    g = kg.PLSLDACV(x, lab, **kw)
    assert np.array_equal(g.predicted_labels, pred) and g.selected_components == sel


@pytest.mark.parametrize("n,d,stratified,maxc,fixc", [(300, 20, True, 5, 0), (500, 40, False, 5, 5),
                                                     (800, 60, True, 8, 3), (400, 10, False, 4, 0),
                                                     (250, 80, True, 6, 6)])
def test_plsdacv_matches_oracle(kg, orc, n, d, stratified, maxc, fixc):
    x, lab = _noisy(n, d, seed=n + d, flip=0.3)
    kw = dict(folds=10, stratified=stratified, max_components=maxc, fixed_components=fixc, cv_seed=7)
    pred, folds, sel, abc, _ = orc.plsldacv(x, lab, da=True, **kw)
    g = kg.PLSDACV(x, lab, **kw)
    assert np.array_equal(g.fold_assignments, folds)
    assert np.array_equal(g.predicted_labels, pred) and g.selected_components == sel
    assert np.array_equal(g.accuracy_by_components[:maxc], abc[:maxc])


@pytest.mark.parametrize("n,nt,d,comp", [(400, 300, 30, 5), (150, 500, 200, 4), (1000, 1000, 50, 10),
                                         (200, 150, 700, 3)])
def test_plsldapredict_matches_oracle(kg, orc, n, nt, d, comp):
    x, lab = _noisy(n + nt, d, seed=nt + d, flip=0.2)
    want = orc.plsldapredict(x[:n], lab[:n], x[n:], components=comp)
    got = kg.PLSLDAPredict(x[:n], lab[:n], x[n:], max_components=comp, fixed_components=comp)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("coarsening,constrained,stratified", [(True, False, False), (False, False, False),
                                                               (True, True, False), (True, False, True),
                                                               (False, True, True)])
def test_core_plslda_matches_oracle(kg, orc, coarsening, constrained, stratified):
    x, _ = datasets.low_rank(n=600, d=30, seed=5)
    rng = np.random.default_rng(6)
    labels = rng.integers(1, 12, 600).astype(np.int32)
    con = np.arange(1, 601, dtype=np.int32) if not constrained else rng.integers(0, 300, 600).astype(np.int32)
    fix = (rng.random(600) < 0.05).astype(np.int32) if constrained else None
    kw = dict(cycles=15, folds=5, stratified=stratified, evolutionary=True, guarded=True, absorption=True,
              coarsening=coarsening, seed=11, cv_seed=12)
    a = orc.core_plslda(x, labels, constrain=con, fixed=fix, components=4, **kw)
    b = kg.CorePLSLDA(x, labels, constrain=con, fixed=fix, cycles=15, folds=5, stratified=stratified,
                      max_components=4, fixed_components=4, evolutionary_search=True,
                      guarded_diversity=True, many_to_one_absorption=True,
                      auto_class_coarsening=coarsening, seed=11, cv_seed=12)
    assert np.array_equal(b.fold_assignments, a.folds)
    assert np.array_equal(b.clbest, a.clbest)
    assert np.array_equal(b.cvpredbest, a.cvpredbest)
    assert np.array_equal(b.vect_acc, a.vect_acc)
    assert np.array_equal(b.vect_score, a.vect_score)
    assert np.array_equal(b.proposal_size, a.proposal_size)
    assert np.array_equal(b.active_classes, a.active_classes)
    assert np.array_equal(b.flags, a.flags)
    assert np.array_equal(b.counters, a.counters)
    assert b.accbest == a.accbest and b.scorebest == a.scorebest


@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "plsldacv"], ids=lambda c: c["name"])
def test_gpu_plsldacv_golden(kg, case):
    x, labels = G.pls_inputs(case["input"])
    o = case["options"]
    fn = kg.PLSDACV if o.get("da") else kg.PLSLDACV
    r = fn(x, labels, folds=o["folds"], stratified=o["stratified"], max_components=o["max_components"],
           fixed_components=o["fixed_components"], cv_seed=o["cv_seed"])
    assert r.predicted_labels[:32].tolist() == case["predicted_head"]
    assert G.sha(r.predicted_labels) == case["predicted_sha256"]
    assert G.sha(r.fold_assignments) == case["folds_sha256"]
    assert r.selected_components == case["selected_components"]
    assert r.accuracy_by_components.tolist() == case["accuracy_by_components"]


@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "plsldapredict"], ids=lambda c: c["name"])
def test_gpu_plsldapredict_golden(kg, case):
    x, labels = G.pls_inputs(case["input"])
    t, c = case["n_train"], case["options"]["components"]
    pred = kg.PLSLDAPredict(x[:t], labels[:t], x[t:], max_components=c, fixed_components=c)
    assert pred[:32].tolist() == case["predicted_head"] and G.sha(pred) == case["predicted_sha256"]


@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "core_plslda"], ids=lambda c: c["name"])
def test_gpu_core_plslda_golden(kg, case):
    x, labels = G.pls_inputs(case["input"])
    o = case["options"]
    n = len(labels)
    r = kg.CorePLSLDA(x, labels, constrain=np.arange(1, n + 1, dtype=np.int32), cycles=o["cycles"],
                      folds=o["folds"], stratified=o["stratified"], max_components=o["components"],
                      fixed_components=o["components"], evolutionary_search=o["evolutionary"],
                      guarded_diversity=o["guarded"], many_to_one_absorption=o["absorption"],
                      auto_class_coarsening=o["coarsening"], seed=o["seed"], cv_seed=o["cv_seed"])
    G.check_core(case, r, folds_attr="fold_assignments")


def test_pls_matrix_matches_oracle(kg, orc):
    x, _ = datasets.low_rank(n=900, d=30, seed=3)
    gi, gd = orc.exact_knn(x, 20, threads=8)
    kw = dict(runs=3, cycles=8, landmarks=600, splitting=12, graph_neighbors=20, folds=5, knn_k=10,
              components=4)
    a = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=77, threads=3, materialize=1, classifier=1, **kw)
    b = kg.KODAMA_matrix(x, graph=(gi, gd), index_base=0, seed=77, materialize_graph=True,
                         classifier="pls", **kw)
    for f in ("res", "acc", "v", "run_counters", "cycle_diag", "knn_idx", "knn_dist", "pls_counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert np.array_equal(a.hashes, b.run_hashes)


def test_pls_matrix_many_slices_matches_oracle(kg, orc):
    # 16 runs x 10 folds = 160 slices (more than the SMs) and 150 initial
    # clusters: the Gram-less first evaluation keeps the label cross-product
    # in global memory, the Gram evaluations in shared memory
    x, _ = datasets.low_rank(n=800, d=100, seed=5)
    gi, gd = orc.exact_knn(x, 20, threads=8)
    kw = dict(runs=16, cycles=4, landmarks=600, splitting=150, graph_neighbors=20, folds=10, knn_k=10,
              components=4)
    a = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=91, threads=8, materialize=1, classifier=1, **kw)
    b = kg.KODAMA_matrix(x, graph=(gi, gd), index_base=0, seed=91, materialize_graph=True,
                         classifier="pls", **kw)
    for f in ("res", "acc", "v", "run_counters", "cycle_diag", "pls_counters"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert np.array_equal(a.hashes, b.run_hashes)


@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "kodama_matrix" and "input" in c],
                         ids=lambda c: c["name"])
def test_gpu_pls_matrix_golden(kg, case):
    x = G.inputs(case)
    o = dict(case["options"])
    o.pop("classifier")
    r = kg.KODAMA_matrix(x, materialize_graph=True, classifier="pls", **o)
    G.check_pls_matrix(case, r)
