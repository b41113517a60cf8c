"""Generate tests/golden/*.json from the reference's own CPU core.

Runs oracle/_ref/libkodama_ref.so (the reference compiled from its sources by
oracle/build_ref.sh) on seeded synthetic inputs and records its outputs:
small arrays in full, large arrays as SHA-256 of their little-endian bytes.
The neighbour graphs fed to the reference are the canonical exact graphs
(float32, coordinate order, index tie-break), whose SHA-256 is recorded too.

Usage (where the reference checkout exists):  python tests/golden/make_golden.py
"""

from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

sys.path.insert(0, os.path.join(ROOT, "tests"))

from golden_util import knn_inputs, semi_inputs  # noqa: E402
from kodama_gb300 import datasets  # noqa: E402
from oracle import oracle, ref  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def matrix_case(name, x, K, index_base, **kw):
    gi, gd = oracle.exact_knn(x, K, threads=8)
    g_in = gi + 1 if index_base == 1 else gi
    r = ref.kodama_matrix_graph_data(x, g_in, gd, index_base, threads=8, materialize=1, **kw)
    return {
        "kind": "kodama_matrix", "name": name, "K": K, "index_base": index_base, "options": kw,
        "graph_sha256": sha(gi) + ":" + sha(gd),
        "acc": r.acc.tolist(), "v_sha256": sha(r.v), "res_sha256": sha(r.res),
        "hashes": [[int(v) for v in row] for row in r.hashes], "run_counters": r.run_counters.tolist(),
        "cycle_diag_sha256": sha(r.cycle_diag), "knn_idx_sha256": sha(r.knn_idx),
        "knn_dist_sha256": sha(r.knn_dist), "res_head": r.res[:, :16].tolist(),
    }


def core_case(name, x, K, labels, **kw):
    gi, gd = oracle.exact_knn(x, K, threads=8)
    r = ref.core_knn_graph(gi, gd, labels, index_base=0, **kw)
    kw_json = {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
    return {
        "kind": "core_knn_graph", "name": name, "K": K, "options": kw_json, "labels_sha256": sha(labels),
        "graph_sha256": sha(gi) + ":" + sha(gd),
        "clbest_sha256": sha(r.clbest), "cvpredbest_sha256": sha(r.cvpredbest), "folds_sha256": sha(r.folds),
        "vect_acc": r.vect_acc.tolist(), "vect_score": r.vect_score.tolist(),
        "proposal_size": r.proposal_size.tolist(), "active_classes": r.active_classes.tolist(),
        "flags": r.flags.tolist(), "accbest": r.accbest, "scorebest": r.scorebest,
        "counters": r.counters.tolist(),
    }


def pls_inputs(spec):
    x, y = datasets.low_rank(n=spec["n"], d=spec["d"], seed=spec["seed"])
    rng = np.random.default_rng(spec["seed"] + 1000)
    labels = y.copy()
    flip = rng.random(len(y)) < spec.get("flip", 0.0)
    labels[flip] = rng.integers(1, 9, int(flip.sum()))
    if spec.get("random_labels"):
        labels = rng.integers(1, spec["random_labels"] + 1, len(y)).astype(np.int32)
    return x, labels.astype(np.int32)


def plsldacv_case(name, spec, **kw):
    x, labels = pls_inputs(spec)
    pred, folds, sel, abc, _ = ref.plsldacv(x, labels, **kw)
    return {"kind": "plsldacv", "name": name, "input": spec, "options": kw, "labels_sha256": sha(labels),
            "predicted_sha256": sha(pred), "folds_sha256": sha(folds), "selected_components": sel,
            "accuracy_by_components": abc.tolist(), "predicted_head": pred[:32].tolist()}


def plsldapredict_case(name, spec, n_train, **kw):
    x, labels = pls_inputs(spec)
    pred = ref.plsldapredict(x[:n_train], labels[:n_train], x[n_train:], **kw)
    return {"kind": "plsldapredict", "name": name, "input": spec, "n_train": n_train, "options": kw,
            "predicted_sha256": sha(pred), "predicted_head": pred[:32].tolist()}


def core_plslda_case(name, spec, **kw):
    x, labels = pls_inputs(spec)
    n = len(labels)
    r = ref.core_plslda(x, labels, constrain=np.arange(1, n + 1, dtype=np.int32), **kw)
    return {
        "kind": "core_plslda", "name": name, "input": spec, "options": kw, "labels_sha256": sha(labels),
        "clbest_sha256": sha(r.clbest), "cvpredbest_sha256": sha(r.cvpredbest), "folds_sha256": sha(r.folds),
        "vect_acc": r.vect_acc.tolist(), "vect_score": r.vect_score.tolist(),
        "proposal_size": r.proposal_size.tolist(), "active_classes": r.active_classes.tolist(),
        "flags": r.flags.tolist(), "accbest": r.accbest, "scorebest": r.scorebest,
        "counters": r.counters.tolist(),
    }


def pls_matrix_case(name, spec, K, **kw):
    x, _ = pls_inputs(spec)
    case = matrix_case(name, x, K, 0, classifier=1, **kw)
    r = ref.kodama_matrix_graph_data(x, *oracle.exact_knn(x, K, threads=8), 0, threads=8, materialize=1,
                                     classifier=1, **kw)
    case["input"] = spec
    case["pls_counters"] = r.pls_counters.tolist()
    return case


def knncv_case(name, spec, **kw):
    x, labels, con, _ = knn_inputs(spec)
    if con is not None:
        raise ValueError("the reference shim of KNNCV takes no constraint")
    pred, folds, _ = ref.knncv(x, labels, threads=8, **kw)
    return {"kind": "knncv", "name": name, "input": spec, "options": kw, "labels_sha256": sha(labels),
            "predicted_sha256": sha(pred), "folds_sha256": sha(folds), "predicted_head": pred[:32].tolist()}


def core_knn_case(name, spec, **kw):
    x, labels, con, fix = knn_inputs(spec)
    r = ref.core_knn(x, labels, constrain=con, fixed=fix, **kw)
    return {
        "kind": "core_knn", "name": name, "input": spec, "options": kw, "labels_sha256": sha(labels),
        "clbest_sha256": sha(r.clbest), "cvpredbest_sha256": sha(r.cvpredbest), "folds_sha256": sha(r.folds),
        "vect_acc": r.vect_acc.tolist(), "vect_score": r.vect_score.tolist(),
        "proposal_size": r.proposal_size.tolist(), "active_classes": r.active_classes.tolist(),
        "flags": r.flags.tolist(), "accbest": r.accbest, "scorebest": r.scorebest,
        "counters": r.counters.tolist(),
    }


def core_graph_case(name, spec, K, **kw):
    """CoreKNNGraph on the canonical exact graph of knn_inputs(spec), with its
    constraint / fixed flags."""
    x, labels, con, fix = knn_inputs(spec)
    gi, gd = oracle.exact_knn(x, K, threads=8)
    r = ref.core_knn_graph(gi, gd, labels, index_base=0, constrain=con, fixed=fix, **kw)
    return {
        "kind": "core_knn_graph_input", "name": name, "input": spec, "K": K, "options": kw,
        "graph_sha256": sha(gi) + ":" + sha(gd), "labels_sha256": sha(labels),
        "clbest_sha256": sha(r.clbest), "cvpredbest_sha256": sha(r.cvpredbest), "folds_sha256": sha(r.folds),
        "vect_acc": r.vect_acc.tolist(), "vect_score": r.vect_score.tolist(),
        "proposal_size": r.proposal_size.tolist(), "active_classes": r.active_classes.tolist(),
        "flags": r.flags.tolist(), "accbest": r.accbest, "scorebest": r.scorebest,
        "counters": r.counters.tolist(),
    }


def semi_matrix_case(name, spec, K, **kw):
    """KODAMAMatrixFromGraphData with starting labels / constraint / fixed
    flags of semi_inputs(spec), on the canonical exact graph."""
    x, start, con, fix = semi_inputs(spec)
    gi, gd = oracle.exact_knn(x, K, threads=8)
    r = ref.kodama_matrix_graph_data(x, gi, gd, 0, threads=8, materialize=1, starting=start, constrain=con,
                                     fixed=fix, **kw)
    return {
        "kind": "kodama_matrix_semi", "name": name, "input": spec, "K": K, "index_base": 0, "options": kw,
        "graph_sha256": sha(gi) + ":" + sha(gd),
        "acc": r.acc.tolist(), "v_sha256": sha(r.v), "res_sha256": sha(r.res),
        "hashes": [[int(v) for v in row] for row in r.hashes], "run_counters": r.run_counters.tolist(),
        "cycle_diag_sha256": sha(r.cycle_diag), "knn_idx_sha256": sha(r.knn_idx),
        "knn_dist_sha256": sha(r.knn_dist), "res_head": r.res[:, :16].tolist(),
        "pls_counters": r.pls_counters.tolist(),
    }


def main():
    if not ref.available():
        raise SystemExit("build oracle/_ref first (oracle/build_ref.sh)")
    if not oracle.available():
        oracle.build()
    cases = []
    xs = datasets.spirals()[0].astype(np.float32)
    cases.append(matrix_case("spirals_N1000_M20_T20", xs, 50, 1, seed=1234, runs=20, cycles=20,
                             landmarks=10000, splitting=0, graph_neighbors=50, folds=10, knn_k=10))
    xg, _ = datasets.gaussian_mixture(n=3000, d=50, seed=21)
    cases.append(matrix_case("mixture_N3000_d50_M6_T30", xg, 30, 0, seed=7, runs=6, cycles=30,
                             landmarks=10000, splitting=40, graph_neighbors=30, folds=10, knn_k=30))
    xc, _ = datasets.gaussian_mixture(n=2000, d=20, seed=5)
    rng = np.random.default_rng(3)
    labels = (rng.integers(1, 9, 2000) * 3 - 5).astype(np.int32)
    cases.append(core_case("core_evolutionary", xc, 40, labels, cycles=25, k=10, folds=7, seed=5, cv_seed=11,
                           evolutionary=True, guarded=True, absorption=True, stratified=False))
    cases.append(core_case("core_greedy_stratified", xc, 40, labels, cycles=25, k=10, folds=7, seed=5,
                           cv_seed=11, evolutionary=False, guarded=False, absorption=False, stratified=True))
    cases.append(plsldacv_case("plsldacv_stratified", dict(n=1200, d=60, seed=31, flip=0.3),
                               folds=10, stratified=True, max_components=6, fixed_components=0, cv_seed=7))
    cases.append(plsldacv_case("plsldacv_fixed5", dict(n=1000, d=80, seed=32, flip=0.4),
                               folds=8, stratified=False, max_components=5, fixed_components=5, cv_seed=9))
    cases.append(plsldacv_case("plsdacv_stratified", dict(n=1100, d=60, seed=37, flip=0.3),
                               folds=10, stratified=True, max_components=6, fixed_components=0, cv_seed=8, da=True))
    cases.append(plsldacv_case("plsdacv_fixed4", dict(n=900, d=30, seed=38, flip=0.4),
                               folds=8, stratified=False, max_components=4, fixed_components=4, cv_seed=9, da=True))
    cases.append(plsldapredict_case("plsldapredict_c5", dict(n=1500, d=50, seed=33, flip=0.2), 1000,
                                    components=5))
    cases.append(core_plslda_case("core_plslda_evolutionary", dict(n=900, d=40, seed=34, random_labels=10),
                                  cycles=20, folds=5, stratified=False, components=5, evolutionary=True,
                                  guarded=True, absorption=True, coarsening=True, seed=13, cv_seed=14))
    cases.append(core_plslda_case("core_plslda_stratified", dict(n=700, d=30, seed=36, random_labels=6),
                                  cycles=12, folds=5, stratified=True, components=4, evolutionary=True,
                                  guarded=True, absorption=True, coarsening=False, seed=15, cv_seed=16))
    cases.append(pls_matrix_case("pls_matrix_N1500_d50_M4_T12", dict(n=1500, d=50, seed=35), 20,
                                 seed=99, runs=4, cycles=12, landmarks=10000, splitting=20,
                                 graph_neighbors=20, folds=5, knn_k=10, components=5))
    cases.append(knncv_case("knncv_cosine_stratified", dict(n=900, d=20, seed=41, flip=0.2),
                            k=10, folds=10, stratified=True, metric=0, cv_seed=3))
    cases.append(knncv_case("knncv_euclidean", dict(n=700, d=12, seed=42, flip=0.3),
                            k=7, folds=5, stratified=False, metric=2, cv_seed=4))
    cases.append(knncv_case("knncv_inner_product", dict(n=600, d=24, seed=44, flip=0.1),
                            k=15, folds=8, stratified=True, metric=1, cv_seed=5))
    cases.append(core_knn_case("core_knn_cosine_evolutionary", dict(n=800, d=16, seed=43, random_labels=6),
                               metric=0, cycles=20, k=10, folds=5, stratified=True, evolutionary=True,
                               guarded=True, absorption=True, seed=4, cv_seed=6))
    cases.append(core_knn_case("core_knn_euclidean_constrained_fixed",
                               dict(n=800, d=16, seed=45, random_labels=6, groups_of=3, fixed_frac=0.1),
                               metric=2, cycles=20, k=30, folds=10, stratified=False, evolutionary=False,
                               guarded=False, absorption=False, seed=7, cv_seed=8))
    cases.append(core_graph_case("core_graph_constrained_fixed",
                                 dict(n=900, d=16, seed=46, random_labels=7, groups_of=2, fixed_frac=0.15),
                                 30, cycles=20, k=10, folds=5, stratified=True, evolutionary=True, guarded=True,
                                 absorption=True, seed=9, cv_seed=10))
    semi_kw = dict(runs=4, cycles=12, landmarks=1000, splitting=20, graph_neighbors=20, folds=5, knn_k=10)
    cases.append(semi_matrix_case("semi_knn_start_constrain_fixed",
                                  dict(n=1500, d=12, seed=47, flip=0.3, use_start=True, groups_of=3,
                                       fixed_frac=0.1), 20, seed=11, **semi_kw))
    cases.append(semi_matrix_case("semi_knn_constrain", dict(n=1300, d=10, seed=48, groups_of=2), 20,
                                  seed=12, **semi_kw))
    cases.append(semi_matrix_case("semi_knn_start_fixed", dict(n=1200, d=16, seed=49, flip=0.4, use_start=True,
                                                               fixed_frac=0.2), 20, seed=13, **semi_kw))
    cases.append(semi_matrix_case("semi_pls_start_constrain",
                                  dict(n=1400, d=14, seed=50, flip=0.3, use_start=True, groups_of=2), 20,
                                  seed=14, classifier=1, components=4, **semi_kw))
    cases.append(semi_matrix_case("semi_pls_fixed", dict(n=1100, d=12, seed=51, fixed_frac=0.15), 20, seed=15,
                                  classifier=1, components=4, **semi_kw))
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases")


if __name__ == "__main__":
    main()
