"""The CPU restatement and the CUDA path against the reference's recorded
outputs (tests/golden/golden.json)."""

import numpy as np
import pytest

import golden_util as G


def _matrix_args(case):
    o = dict(case["options"])
    return o


@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "kodama_matrix"], ids=lambda c: c["name"])
def test_oracle_matrix_golden(orc, case):
    x = G.inputs(case)
    gi, gd = orc.exact_knn(x, case["K"], threads=8)
    assert G.sha(gi) + ":" + G.sha(gd) == case["graph_sha256"], "canonical exact graph"
    g_in = gi + 1 if case["index_base"] == 1 else gi
    r = orc.kodama_matrix_graph_data(x, g_in, gd, case["index_base"], threads=8, materialize=1, **case["options"])
    if "pls_counters" in case:
        G.check_pls_matrix(case, r)
    else:
        G.check_matrix(case, r)


@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "core_knn_graph"], ids=lambda c: c["name"])
def test_oracle_core_golden(orc, case):
    x = G.inputs(case)
    labels = G.core_labels()
    assert G.sha(labels) == case["labels_sha256"]
    gi, gd = orc.exact_knn(x, case["K"], threads=8)
    r = orc.core_knn_graph(gi, gd, labels, index_base=0, **case["options"])
    G.check_core(case, r)


def _cases(kind):
    return [c for c in G.cases() if c["kind"] == kind]


def _core_kw(o):
    return dict(cycles=o["cycles"], k=o["k"], folds=o["folds"], stratified=o["stratified"],
                evolutionary=o["evolutionary"], guarded=o["guarded"], absorption=o["absorption"],
                seed=o["seed"], cv_seed=o["cv_seed"])


@pytest.mark.parametrize("case", _cases("knncv"), ids=lambda c: c["name"])
def test_oracle_knncv_golden(orc, case):
    x, labels, _, _ = G.knn_inputs(case["input"])
    assert G.sha(labels) == case["labels_sha256"]
    pred, folds, _ = orc.knncv(x, labels, **case["options"])
    G.check_knncv(case, pred, folds)


@pytest.mark.parametrize("case", _cases("core_knn"), ids=lambda c: c["name"])
def test_oracle_core_knn_golden(orc, case):
    x, labels, con, fix = G.knn_inputs(case["input"])
    assert G.sha(labels) == case["labels_sha256"]
    o = case["options"]
    r = orc.core_knn(x, labels, metric=o["metric"], constrain=con, fixed=fix, **_core_kw(o))
    G.check_core(case, r)


@pytest.mark.parametrize("case", _cases("core_knn_graph_input"), ids=lambda c: c["name"])
def test_oracle_core_graph_input_golden(orc, case):
    x, labels, con, fix = G.knn_inputs(case["input"])
    gi, gd = orc.exact_knn(x, case["K"], threads=8)
    assert G.sha(gi) + ":" + G.sha(gd) == case["graph_sha256"], "canonical exact graph"
    r = orc.core_knn_graph(gi, gd, labels, index_base=0, constrain=con, fixed=fix, **_core_kw(case["options"]))
    G.check_core(case, r)


@pytest.mark.parametrize("case", _cases("plsldacv"), ids=lambda c: c["name"])
def test_oracle_plsldacv_golden(orc, case):
    x, labels = G.pls_inputs(case["input"])
    assert G.sha(labels) == case["labels_sha256"]
    pred, folds, sel, abc, _ = orc.plsldacv(x, labels, **case["options"])
    assert pred[:32].tolist() == case["predicted_head"]
    assert G.sha(pred) == case["predicted_sha256"] and G.sha(folds) == case["folds_sha256"]
    assert sel == case["selected_components"] and abc.tolist() == case["accuracy_by_components"]


@pytest.mark.parametrize("case", _cases("plsldapredict"), ids=lambda c: c["name"])
def test_oracle_plsldapredict_golden(orc, case):
    x, labels = G.pls_inputs(case["input"])
    t = case["n_train"]
    pred = orc.plsldapredict(x[:t], labels[:t], x[t:], **case["options"])
    assert pred[:32].tolist() == case["predicted_head"] and G.sha(pred) == case["predicted_sha256"]


@pytest.mark.parametrize("case", _cases("core_plslda"), ids=lambda c: c["name"])
def test_oracle_core_plslda_golden(orc, case):
    x, labels = G.pls_inputs(case["input"])
    assert G.sha(labels) == case["labels_sha256"]
    n = len(labels)
    r = orc.core_plslda(x, labels, constrain=np.arange(1, n + 1, dtype=np.int32), **case["options"])
    G.check_core(case, r)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "kodama_matrix" and "input" not in c],
                         ids=lambda c: c["name"])
def test_gpu_matrix_golden(kg, case):
    x = G.inputs(case)
    o = dict(case["options"])
    r = kg.KODAMA_matrix(x, materialize_graph=True, **o)
    gi, gd = kg.knn_graph(x, case["K"])
    assert G.sha(gi) + ":" + G.sha(gd) == case["graph_sha256"], "device exact graph"
    G.check_matrix(case, r)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in G.cases() if c["kind"] == "core_knn_graph"], ids=lambda c: c["name"])
def test_gpu_core_golden(kg, case):
    x = G.inputs(case)
    labels = G.core_labels()
    gi, gd = kg.knn_graph(x, case["K"])
    o = case["options"]
    out = kg.CoreKNNGraph_batch(gi, gd, labels[None, :], np.array([o["seed"]], np.uint64),
                                np.array([o["cv_seed"]], np.uint64), cycles=o["cycles"], k=o["k"],
                                folds=o["folds"], stratified=o["stratified"],
                                evolutionary_search=o["evolutionary"], guarded_diversity=o["guarded"],
                                many_to_one_absorption=o["absorption"], index_base=0, metric="euclidean")
    G.check_core(case, out[0], folds_attr="fold_assignments")


def _gpu_core_kw(o):
    return dict(cycles=o["cycles"], k=o["k"], folds=o["folds"], stratified=o["stratified"],
                evolutionary_search=o["evolutionary"], guarded_diversity=o["guarded"],
                many_to_one_absorption=o["absorption"], seed=o["seed"], cv_seed=o["cv_seed"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases("knncv"), ids=lambda c: c["name"])
def test_gpu_knncv_golden(kg, case):
    x, labels, _, _ = G.knn_inputs(case["input"])
    o = case["options"]
    r = kg.KNNCV(x, labels, k=o["k"], folds=o["folds"], stratified=o["stratified"], metric=o["metric"],
                 seed=o["cv_seed"])
    G.check_knncv(case, r.predicted_labels, r.fold_assignments)


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases("core_knn"), ids=lambda c: c["name"])
def test_gpu_core_knn_golden(kg, case):
    x, labels, con, fix = G.knn_inputs(case["input"])
    o = case["options"]
    r = kg.CoreKNN(x, labels, metric=o["metric"], constrain=con, fixed=fix, **_gpu_core_kw(o))
    G.check_core(case, r, folds_attr="fold_assignments")


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases("core_knn_graph_input"), ids=lambda c: c["name"])
def test_gpu_core_graph_input_golden(kg, case):
    x, labels, con, fix = G.knn_inputs(case["input"])
    gi, gd = kg.knn_graph(x, case["K"])
    assert G.sha(gi) + ":" + G.sha(gd) == case["graph_sha256"], "exact graph"
    r = kg.CoreKNNGraph(gi, gd, labels, index_base=0, constrain=con, fixed=fix, metric="euclidean",
                        **_gpu_core_kw(case["options"]))
    G.check_core(case, r, folds_attr="fold_assignments")


@pytest.mark.parametrize("case", _cases("kodama_matrix_semi"), ids=lambda c: c["name"])
def test_oracle_semi_matrix_golden(orc, case):
    x, start, con, fix = G.semi_inputs(case["input"])
    gi, gd = orc.exact_knn(x, case["K"], threads=8)
    assert G.sha(gi) + ":" + G.sha(gd) == case["graph_sha256"], "canonical exact graph"
    r = orc.kodama_matrix_graph_data(x, gi, gd, 0, threads=8, materialize=1, starting=start, constrain=con,
                                     fixed=fix, **case["options"])
    G.check_pls_matrix(case, r)


@pytest.mark.gpu
@pytest.mark.parametrize("raw", [False, True], ids=["graph_input", "raw_data"])
@pytest.mark.parametrize("case", _cases("kodama_matrix_semi"), ids=lambda c: c["name"])
def test_gpu_semi_matrix_golden(kg, case, raw):
    x, start, con, fix = G.semi_inputs(case["input"])
    graph = None
    if not raw:
        graph = kg.knn_graph(x, case["K"])
        assert G.sha(graph[0]) + ":" + G.sha(graph[1]) == case["graph_sha256"], "exact graph"
    r = kg.KODAMA_matrix(x, graph, index_base=0, materialize_graph=True, starting_labels=start, constrain=con,
                         fixed=fix, **case["options"])
    G.check_pls_matrix(case, r)
