#!/usr/bin/env python
"""Benchmark: KODAMA.matrix label evolution on one GB300 (and its CPU baseline).

Workload (one "step" = one full KODAMA.matrix call): N=20000 points, d=50,
12-cluster Gaussian mixture (synthetic, seed 2), M=100 runs x Tcycle=100,
exact kNN graph K=30, knn.k=30, 10 folds, splitting=50, landmarks=10000
(L=10000 per run), kNN classifier, default evolution policy.

value  : device seconds per step (CUDA events on the library's stream), input
         matrix already resident in HBM, label matrix left in HBM;
e2e    : seconds per step through the public host-buffer C-ABI call
         (pinned host input copied in, label matrix + traces copied out);
roofline: the persistent evolution kernel (the dominant kernel) against
         the measured HBM copy bandwidth;
learned: the learned relabelling proposal (shipped weights) at the smallest
         cycle count reaching the plain run's mean final CV accuracy, timed
         the same way, with the Spearman correlation of its dissimilarities;
cpu_baseline / --impl reference: the CPU restatement of the reference
         algorithm (oracle/, all host threads) on the whole workload, exact
         graph and all M=100 runs, nothing extrapolated; its result is also
         compared field by field with the timed GPU result
         (parity_vs_oracle), outside the timed region.

Launch: python bench.py [--gpus N --steps K --warmup W] [--impl reference]
(N>1 under torchrun: the M=100 runs of the one job are split across the
ranks, the label blocks all-gathered over NCCL and the proximity applied on
rank 0; strong scaling.  --sharded runs that path at N=1 too).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "KODAMA.matrix wall-s at N=20k,d=50,M=100: learned vs plain GPU at equal CV acc"
WORKLOAD = dict(n=20000, d=50, runs=100, cycles=100, graph_neighbors=30, knn_k=30, folds=10,
                splitting=50, landmarks=10000, seed=1234)
# --workload pls: the PLS-LDA configuration (CorePLSLDA inside KODAMA.matrix)
PLS_METRIC = "KODAMA.matrix PLS-LDA wall-s at N=10k,d=200,ncomp=5,F=10,M=50,Tcycle=50"
PLS_WORKLOAD = dict(n=10000, d=200, runs=50, cycles=50, graph_neighbors=30, knn_k=30, folds=10,
                    splitting=0, landmarks=10000, seed=1234, components=5)
# --workload batch: 256 independent KODAMA.matrix problems of uneven size
# (datasets.uneven_batch: N log-uniform in [500, 20000], d in {10, 50, 100},
# Gaussian mixtures of 3-20 clusters, half kNN k=10, half PLS-LDA ncomp=5),
# M=50 runs x Tcycle=50 each, in one captured CUDA graph
BATCH_METRIC = "256-problem uneven KODAMA.matrix batch wall-s (M=50, Tcycle=50 each, one captured CUDA graph)"
BATCH_KW = dict(runs=50, cycles=50, knn_k=10, components=5, graph_neighbors=30, folds=10, seed=1234)
# DRAM bytes (read + write) of one evolution-kernel launch, scaled from the
# ncu capture of the full bench-size launch (dram__bytes_read.sum +
# dram__bytes_write.sum; None until captured).
EVOLVE_TRAFFIC_BYTES = 598524416


CONFIG_DESC = ("KODAMA.matrix kNN N=20000 d=50 (12-cluster Gaussian mixture), M=100 runs, "
               "Tcycle=100, exact graph K=30, knn.k=30, folds=10, splitting=50, landmarks=10000")
DATA_DESC = "synthetic gaussian_mixture(seed=2)"


def _use_config5():
    """--workload learned100k: the learned-vs-plain comparison at N=100000,
    d=50 (PCA-like mixture of 30 clusters, sigma_i = 10 / i along random
    orthonormal axes, Dirichlet(0.5) sizes, seed 5), K=30, M=100, Tcycle=100,
    kNN classifier, default splitting (300 above N=40000)."""
    global METRIC, WORKLOAD, CONFIG_DESC, DATA_DESC
    METRIC = "KODAMA.matrix wall-s at N=100k,d=50,M=100: learned vs plain GPU at equal CV acc"
    WORKLOAD = dict(n=100000, d=50, runs=100, cycles=100, graph_neighbors=30, knn_k=30, folds=10,
                    splitting=0, landmarks=10000, seed=1234)
    CONFIG_DESC = ("KODAMA.matrix kNN N=100000 d=50 (30-cluster PCA-like mixture), M=100 runs, Tcycle=100, "
                   "exact graph K=30, knn.k=30, folds=10, default splitting (300), landmarks=10000")
    DATA_DESC = "synthetic pca_mixture(seed=5)"


def _config(extra=None):
    c = {"workload": CONFIG_DESC,
         "global_batch": WORKLOAD["runs"], "seq_len": WORKLOAD["cycles"],
         "parallelism": "replicas", "l2": "flushed between steps (512 MB write)",
         "data": DATA_DESC}
    if extra:
        c.update(extra)
    return c


def _data():
    from kodama_gb300 import datasets
    if WORKLOAD["n"] == 100000:
        x, _ = datasets.pca_mixture(n=WORKLOAD["n"], d=WORKLOAD["d"], seed=5)
    else:
        x, _ = datasets.gaussian_mixture(n=WORKLOAD["n"], d=WORKLOAD["d"], seed=2)
    return np.ascontiguousarray(x, np.float32)


def _matrix_kw():
    return dict(runs=WORKLOAD["runs"], cycles=WORKLOAD["cycles"], landmarks=WORKLOAD["landmarks"],
                splitting=WORKLOAD["splitting"], graph_neighbors=WORKLOAD["graph_neighbors"],
                folds=WORKLOAD["folds"], knn_k=WORKLOAD["knn_k"], seed=WORKLOAD["seed"])


def _peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def evolve_bytes_per_launch(L, w, runs, cycles):
    """Algorithmic bytes of one evolution-kernel launch: per CV evaluation of a
    run, the L x k' neighbour table (2-byte ids + 4-byte scores) is streamed
    once and L 2-byte labels read and L 2-byte predictions written; M*(T+1)
    evaluations."""
    return runs * (cycles + 1) * (L * w * (2 + 4) + L * 2 * 2)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        self.device_index = device_index
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        if not self.lines:
            return None
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(x, threads=None):
    """The CPU restatement of the whole workload on all host threads: the
    exact graph, then the full KODAMA.matrix call (all M runs), timed with
    nothing extrapolated.  Returns (baseline dict, the restatement's result),
    the result serving as the parity check of the GPU run."""
    from oracle import oracle
    if not oracle.available():
        oracle.build()
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    gi, gd = oracle.exact_knn(x, WORKLOAD["graph_neighbors"], threads=threads)
    t_graph = time.perf_counter() - t0
    kw = _matrix_kw()
    t1 = time.perf_counter()
    r = oracle.kodama_matrix_graph_data(x, gi, gd, 0, seed=kw.pop("seed"), threads=threads, materialize=0, **kw)
    t_matrix = time.perf_counter() - t1
    total = t_graph + t_matrix
    return ({"value": round(total, 4), "unit": "s", "cores": threads, "kind": "port",
             "sample": f"the whole workload: exact graph (N={x.shape[0]}) + KODAMA.matrix with all "
                       f"{WORKLOAD['runs']} runs, nothing extrapolated",
             "stages_s": {"graph": round(t_graph, 3), "atlas": round(float(r.timings[4]), 3),
                          "runs": round(float(r.timings[2]), 3)}}, r)


def _parity(gpu_res, gpu_acc, gpu_v, gpu_hashes, gpu_counters, ref):
    """Field-by-field bit equality of a GPU KODAMA.matrix result with the CPU
    restatement's on the same workload."""
    checks = {"res": np.array_equal(gpu_res, ref.res), "acc": np.array_equal(gpu_acc, ref.acc),
              "v": np.array_equal(gpu_v, ref.v), "run_hashes": np.array_equal(gpu_hashes, ref.hashes),
              "run_counters": np.array_equal(gpu_counters, ref.run_counters)}
    return {"bit_exact": all(checks.values()), "fields": checks}


def _pls_data():
    from kodama_gb300 import datasets
    x, _ = datasets.low_rank(n=PLS_WORKLOAD["n"], d=PLS_WORKLOAD["d"], seed=3)
    return np.ascontiguousarray(x, np.float32)


def _pls_kw():
    w = PLS_WORKLOAD
    return dict(runs=w["runs"], cycles=w["cycles"], landmarks=w["landmarks"], splitting=w["splitting"],
                graph_neighbors=w["graph_neighbors"], folds=w["folds"], knn_k=w["knn_k"], seed=w["seed"],
                components=w["components"])


def _pls_config(extra=None):
    c = {"workload": "KODAMA.matrix PLS-LDA N=10000 d=200 (low-rank X=ZW+E, 8 classes), M=50 runs, "
                     "Tcycle=50, ncomp=5, folds=10, landmarks=10000 (L=7500), splitting=100",
         "global_batch": PLS_WORKLOAD["runs"], "seq_len": PLS_WORKLOAD["cycles"],
         "parallelism": "replicas", "l2": "flushed between steps (512 MB write)",
         "data": "synthetic low_rank(seed=3)"}
    if extra:
        c.update(extra)
    return c


def pls_cpu_baseline(x, threads=None):
    """The CPU restatement of the whole PLS-LDA workload on all host threads:
    exact graph plus the full KODAMA.matrix call (all M runs), nothing
    extrapolated.  Returns (baseline dict, the restatement's result)."""
    from oracle import oracle
    if not oracle.available():
        oracle.build()
    threads = threads or os.cpu_count() or 1
    w = PLS_WORKLOAD
    t0 = time.perf_counter()
    gi, gd = oracle.exact_knn(x, w["graph_neighbors"], threads=threads)
    t_graph = time.perf_counter() - t0
    kw = _pls_kw()
    seed = kw.pop("seed")
    t1 = time.perf_counter()
    r = oracle.kodama_matrix_graph_data(x, gi, gd, 0, seed=seed, threads=threads, materialize=0,
                                        classifier=1, **kw)
    t_matrix = time.perf_counter() - t1
    return ({"value": round(t_graph + t_matrix, 4), "unit": "s", "cores": threads, "kind": "port",
             "sample": f"the whole workload: exact graph + KODAMA.matrix PLS-LDA with all {w['runs']} runs, "
                       "nothing extrapolated",
             "stages_s": {"graph": round(t_graph, 3), "atlas": round(float(r.timings[4]), 3),
                          "runs": round(float(r.timings[2]), 3)},
             "mean_final_cv_acc": round(float(np.mean(r.acc)), 6)}, r)


def pls_fp64_check(x):
    """The float32 PLS-LDA arithmetic (reproduced bit for bit on the GPU)
    against an FP64 restatement of one 10-fold PLSLDACV on the workload's
    data (5 components, the 8 classes of the generator, and the same labels
    with 20% of them redrawn): label disagreements and the float64 relative
    LDA margin where they occur (oracle/pls_fp64.py)."""
    from kodama_gb300 import datasets
    from oracle import oracle, pls_fp64
    _, y = datasets.low_rank(n=PLS_WORKLOAD["n"], d=PLS_WORKLOAD["d"], seed=3)
    rng = np.random.default_rng(0)
    out = {}
    for name, noise in (("true_classes", 0.0), ("labels_20pct_redrawn", 0.2)):
        lab = y.copy()
        flip = rng.random(len(y)) < noise
        lab[flip] = rng.integers(1, 9, int(flip.sum()))
        pred, folds, _, _, _ = oracle.plsldacv(x, lab, folds=PLS_WORKLOAD["folds"], stratified=False,
                                               max_components=PLS_WORKLOAD["components"],
                                               fixed_components=PLS_WORKLOAD["components"],
                                               threads=os.cpu_count() or 1, cv_seed=7)
        out[name] = pls_fp64.compare(oracle._LIB, x, lab, folds, pred, PLS_WORKLOAD["components"])
    return out


def run_gpu_pls(args):
    import torch

    import kodama_gb300 as kg
    from kodama_gb300 import build as kbuild

    kbuild.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    x = _pls_data()
    kw = _pls_kw()
    w = PLS_WORKLOAD
    n, runs, cycles = w["n"], w["runs"], w["cycles"]
    x_dev = torch.from_numpy(x).to(f"cuda:{local}")
    res_dev = torch.empty((runs, n), dtype=torch.int32, device=f"cuda:{local}")
    x_pin = torch.from_numpy(x).pin_memory()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    for _ in range(args.warmup):
        kg.KODAMA_matrix(x_dev, res_out=res_dev, device=local, classifier="pls", **kw)
    spans, evo, accs = [], [], []
    launches0 = kg.launch_count()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            r = kg.KODAMA_matrix(x_dev, res_out=res_dev, device=local, classifier="pls", **kw)
            spans.append(r.kernel_ms["device_span"] / 1000.0)
            evo.append(r.kernel_ms["evolution"] / 1000.0)
            accs.append(float(r.acc.mean()))
        torch.cuda.synchronize()
    launches = (kg.launch_count() - launches0) // max(1, args.steps)
    e2e = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kg.KODAMA_matrix(x_pin.numpy(), device=local, classifier="pls", **kw)
        e2e.append(time.perf_counter() - t0)
    value = float(np.mean(spans))
    L = int(np.ceil(0.75 * n)) if w["landmarks"] >= n else w["landmarks"]
    F, p = w["folds"], w["d"]
    # one evaluation streams, per (run, fold), the standardised training rows
    # twice (cross-product, scores) and the validation rows once
    nt = L - L // F
    bytes_eval = runs * F * (2 * nt + (L - nt)) * p * 4
    evo_s = float(np.mean(evo))
    peak, peak_kind = _peaks()
    achieved = bytes_eval * (cycles + 1) / evo_s / 1e9
    line = {"metric": PLS_METRIC, "value": round(value, 5), "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
            "config": _pls_config(),
            "e2e": {"value": round(float(np.mean(e2e)), 5), "unit": "s", "h2d_bytes_per_step": x.nbytes,
                    "d2h_bytes_per_step": runs * n * 4 + runs * cycles * 8},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "kernel": "PLS evolution span (eval_kernel x (T+1) + evolution steps + Gram)",
                         "algorithmic_bytes_per_eval": bytes_eval, "traffic": None},
            "gpu_launches": int(launches), "clocks": clocks.summary(),
            "stage_ms": {k: round(v, 3) for k, v in r.kernel_ms.items()},
            "mean_final_cv_acc": round(float(np.mean(accs)), 6)}
    if not args.no_cpu_baseline:
        line["cpu_baseline"], ref = pls_cpu_baseline(x)
        line["parity_vs_oracle"] = _parity(res_dev.cpu().numpy(), r.acc, r.v, r.run_hashes, r.run_counters, ref)
        line["fp64_check"] = pls_fp64_check(x)
    print(json.dumps(line))
    if "parity_vs_oracle" in line and not line["parity_vs_oracle"]["bit_exact"]:
        sys.exit("GPU result differs from the CPU restatement on the timed workload")


def _batch_config(extra=None):
    c = {"workload": "256 independent KODAMA.matrix problems: N log-uniform [500, 20000], d in {10, 50, 100}, "
                     "Gaussian mixtures of 3-20 clusters (means ~ N(0, 9 I)), even problems kNN (knn.k=10), odd "
                     "PLS-LDA (ncomp=5); M=50 runs x Tcycle=50 each, exact graph K=30, folds=10, default "
                     "landmarks/splitting; one captured CUDA graph, schedule autotuned",
         "global_batch": 256 * BATCH_KW["runs"], "seq_len": BATCH_KW["cycles"], "parallelism": "replicas",
         "l2": "inputs (1.6 M rows) larger than L2", "data": "synthetic uneven_batch(seed=4)"}
    if extra:
        c.update(extra)
    return c


def _batch_cost(n, d, L, cls, runs, cycles):
    # the library's own dealing estimate (api.cu batch_cost), used to scale
    # the CPU sample to the whole batch
    graph = n * n * d * 1e-9
    evolve = runs * (cycles + 1) * L * ((d + 20.0) * 2e-9 if cls == "pls" else 4e-9)
    return graph + evolve + runs * L * d * 1e-8


def batch_cpu_baseline(problems, threads=None):
    """The CPU restatement on a bounded sample of the batch: per classifier
    the three problems nearest that classifier's median cost, each timed as the
    exact graph, the atlas and min(threads, 16) runs (run waves scaled to
    M=50); the per-classifier seconds-per-cost ratio then prices every
    problem of the batch."""
    from oracle import oracle
    if not oracle.available():
        oracle.build()
    threads = threads or os.cpu_count() or 1
    kw = dict(BATCH_KW)
    seed = kw.pop("seed")
    runs = kw["runs"]
    costs = []
    for pr in problems:
        n, d = pr["x"].shape
        L = int(np.ceil(0.75 * n)) if 10000 >= n else 10000
        costs.append(_batch_cost(n, d, L, pr["classifier"], runs, kw["cycles"]))
    ratio, timed = {}, []
    for cls in ("knn", "pls"):
        idx = [i for i, pr in enumerate(problems) if pr["classifier"] == cls]
        med = float(np.median([costs[i] for i in idx]))
        pick = sorted(idx, key=lambda i: abs(costs[i] - med))[:3]
        tsum, csum = 0.0, 0.0
        for i in pick:
            x = np.ascontiguousarray(problems[i]["x"], np.float32)
            sample_runs = min(threads, 16)
            t0 = time.perf_counter()
            gi, gd = oracle.exact_knn(x, kw["graph_neighbors"], threads=threads)
            t_graph = time.perf_counter() - t0
            r = oracle.kodama_matrix_graph_data(
                x, gi, gd, 0, seed=seed, threads=threads, materialize=0, classifier=1 if cls == "pls" else 0,
                runs=sample_runs, cycles=kw["cycles"], graph_neighbors=kw["graph_neighbors"], folds=kw["folds"],
                knn_k=kw["knn_k"], components=kw["components"], landmarks=10000, splitting=0)
            t_atlas, t_runs = float(r.timings[4]), float(r.timings[2])
            waves = -(-runs // threads) / -(-sample_runs // threads)
            t = t_graph + t_atlas + t_runs * waves
            timed.append({"problem": i, "classifier": cls, "n": int(x.shape[0]), "d": int(x.shape[1]),
                          "seconds": round(t, 3)})
            tsum += t
            csum += costs[i]
        ratio[cls] = tsum / csum
    total = sum(ratio[pr["classifier"]] * c for pr, c in zip(problems, costs))
    return {"value": round(total, 3), "unit": "s", "cores": threads, "kind": "port",
            "sample": "3 kNN + 3 PLS-LDA problems nearest their classifier's median cost, each graph + atlas + "
                      f"min(threads,16) runs (waves scaled to M={runs}); batch priced by seconds per cost unit",
            "timed": timed}


def run_gpu_batch(args):
    import torch

    import kodama_gb300 as kg
    from kodama_gb300 import build as kbuild
    from kodama_gb300 import datasets

    kbuild.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    problems = datasets.uneven_batch()
    kw = dict(BATCH_KW)
    t0 = time.perf_counter()
    res, rep = kg.KODAMA_matrix_batch(problems, device=local, **kw)
    first_call = time.perf_counter() - t0
    tune_s = rep.tune_ms / 1000.0 if rep.rebuilt else 0.0
    for _ in range(max(0, args.warmup - 1)):
        kg.KODAMA_matrix_batch(problems, device=local, **kw)
    dev, e2e, accs = [], [], []
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res, rep = kg.KODAMA_matrix_batch(problems, device=local, **kw)
            e2e.append(time.perf_counter() - t0)
            dev.append(rep.device_ms / 1000.0)
            accs.append(float(np.mean([r.acc.mean() for r in res])))
        torch.cuda.synchronize()
    value = float(np.mean(dev))
    runs, cycles = kw["runs"], kw["cycles"]
    h2d = int(sum(p["x"].nbytes for p in problems))
    d2h = int(sum(runs * p["x"].shape[0] * 4 + runs * cycles * (8 + 20) + runs * 72 for p in problems))
    # algorithmic bytes of the evolution of every problem: kNN vote tables
    # per CV evaluation, PLS standardised rows streamed per evaluation
    algo = 0
    for p in problems:
        n, d = p["x"].shape
        L = int(np.ceil(0.75 * n)) if 10000 >= n else 10000
        if p["classifier"] == "knn":
            algo += evolve_bytes_per_launch(L, min(kw["knn_k"], kw["graph_neighbors"]), runs, cycles)
        else:
            F = kw["folds"]
            nt = L - L // F
            algo += runs * F * (2 * nt + (L - nt)) * d * 4 * (cycles + 1)
    peak, peak_kind = _peaks()
    achieved = algo / value / 1e9
    line = {"metric": BATCH_METRIC, "value": round(value, 4), "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 2), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/f32/f64", "data": "synthetic",
            "config": _batch_config({"lanes": rep.lanes, "order": "longest first" if rep.order == 1 else "round robin"}),
            "e2e": {"value": round(float(np.mean(e2e)), 4), "unit": "s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "kernel": "whole batch graph (evolution traffic of all 256 problems over the graph time; "
                                   "the PLS eval_kernel dominates and is issue-bound)",
                         "algorithmic_bytes_per_launch": int(algo), "traffic": None},
            "gpu_launches": int(rep.kernel_nodes), "graph_nodes": int(rep.graph_nodes),
            "clocks": clocks.summary(),
            "first_call_s": round(first_call, 2), "autotune_s": round(tune_s, 2),
            "mean_final_cv_acc": round(float(np.mean(accs)), 6)}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = batch_cpu_baseline(problems)
    print(json.dumps(line))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload == "batch":
        from kodama_gb300 import datasets
        problems = datasets.uneven_batch()
        vals, last = [], None
        for _ in range(args.steps):
            last = batch_cpu_baseline(problems)
            vals.append(last["value"])
        v = float(np.mean(vals))
        print(json.dumps({"metric": BATCH_METRIC, "value": round(v, 3), "unit": "s", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": 0, "ms_per_step": round(v * 1000, 1),
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                          "dtype": "int32/f32/f64", "data": "synthetic", "config": _batch_config(),
                          "impl": "reference", "cpu_baseline": dict(last, value=round(v, 3)),
                          "e2e": {"value": round(v, 3), "unit": "s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    pls = args.workload == "pls"
    x = _pls_data() if pls else _data()
    base = pls_cpu_baseline if pls else cpu_baseline
    for _ in range(args.warmup):
        base(x)
    vals = []
    last = None
    for _ in range(args.steps):
        last, _ = base(x)
        vals.append(last["value"])
    v = float(np.mean(vals))
    line = {"metric": PLS_METRIC if pls else METRIC, "value": round(v, 4), "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(v * 1000, 2),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32/f64" if pls else "int32/f64", "data": "synthetic",
            "config": _pls_config() if pls else _config(), "impl": "reference",
            "cpu_baseline": dict(last, value=round(v, 4)),
            "e2e": {"value": round(v, 4), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# cycle counts tried for the learned proposal, smallest first: the first whose
# mean final CV accuracy reaches the plain Tcycle=100 run's is timed
LEARNED_LADDER = (30, 40, 50, 60, 70, 80, 90, 100)


def _spearman(a, b):
    from scipy.stats import spearmanr
    m = np.isfinite(a) & np.isfinite(b)
    return float(spearmanr(a[m], b[m]).correlation)


def learned_comparison(kg, x, x_dev, res_dev, local, kw, flush, plain_acc, plain_value, plain_evo, steps):
    """The learned proposal (shipped weights) against the plain runs: the
    smallest ladder cycle count reaching the plain mean final CV accuracy,
    timed like the plain step, and the Spearman correlation of its
    dissimilarity graph with the plain one (beside the plain seed-to-seed
    correlation)."""
    import torch

    from kodama_gb300 import proposal_training as PT

    w = PT.load_default()
    ladder, chosen = [], None
    for T in LEARNED_LADDER:
        r = kg.KODAMA_matrix(x_dev, res_out=res_dev, device=local, proposal_weights=w, **dict(kw, cycles=T))
        ladder.append([T, round(float(r.acc.mean()), 6)])
        if r.acc.mean() >= plain_acc:
            chosen = T
            break
    T = chosen if chosen is not None else LEARNED_LADDER[-1]
    lkw = dict(kw, cycles=T)
    spans, evo, accs = [], [], []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        r = kg.KODAMA_matrix(x_dev, res_out=res_dev, device=local, proposal_weights=w, **lkw)
        spans.append(r.kernel_ms["device_span"] / 1000.0)
        evo.append(r.kernel_ms["evolution"])
        accs.append(float(r.acc.mean()))
    plain_g = kg.KODAMA_matrix(x, device=local, materialize_graph=True, **kw)
    plain_g2 = kg.KODAMA_matrix(x, device=local, materialize_graph=True, **dict(kw, seed=kw["seed"] + 7919))
    learned_g = kg.KODAMA_matrix(x, device=local, materialize_graph=True, proposal_weights=w, **lkw)
    value = float(np.mean(spans))
    return {"weights": "kodama_gb300/proposal_default.npy (plain-run moves on spirals N=1000, "
                       "mixture N=20000 seed 7, low-rank N=10000 seed 3; not the benchmark data)",
            "proposal": "Gumbel top-k sampling from the network's softmax, as many relabellings as the plain "
                        "draw; every move judged by the exact CV accuracy",
            "cycles": T, "reached_plain_acc": chosen is not None, "ladder": ladder,
            "value": round(value, 5), "unit": "s", "ratio_vs_plain": round(value / plain_value, 4),
            "mean_final_cv_acc": round(float(np.mean(accs)), 6), "plain_mean_final_cv_acc": round(plain_acc, 6),
            "evolution_ms": round(float(np.mean(evo)), 3), "plain_evolution_ms": round(plain_evo, 3),
            "evolution_ratio_vs_plain": round(float(np.mean(evo)) / plain_evo, 4),
            "spearman_vs_plain": round(_spearman(learned_g.knn_dist.ravel(), plain_g.knn_dist.ravel()), 4),
            "spearman_plain_other_seed": round(_spearman(plain_g2.knn_dist.ravel(), plain_g.knn_dist.ravel()), 4)}


def run_gpu_sharded(args):
    """The headline job on N GPUs of one node with its M runs split across the
    ranks (strong scaling: the job is fixed, N grows).  Per step and rank:
    KODAMA.matrix on its block of runs (first_run, count; the rank builds the
    exact graph itself, runs draw only from seed + run id), an NCCL all_gather
    of the label blocks (device tensors padded to the largest block), and on
    rank 0 the co-label proximity of the graph over all M label rows on the
    device (kgb_dissimilarity_inplace_device).  Timed between barriers, the
    maximum over ranks.  With --sharded it also runs at N=1 (one rank), which
    is how the path is exercised on a single GPU; there the result is
    compared with the single-call job and the CPU restatement."""
    import torch
    import torch.distributed as dist

    import kodama_gb300 as kg
    from kodama_gb300 import build as kbuild
    from kodama_gb300.distributed import shard

    kbuild.build()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29541")
        dist.init_process_group("nccl", rank=rank, world_size=world)
    dev = f"cuda:{local}"
    x = _data()
    kw = _matrix_kw()
    n, M, T = WORKLOAD["n"], WORKLOAD["runs"], WORKLOAD["cycles"]
    counts = [shard(M, world, r)[1] for r in range(world)]
    first, count = shard(M, world, rank)
    cap = max(max(counts), 1)
    block_kw = {k: v for k, v in kw.items() if k != "runs"}
    x_dev = torch.from_numpy(x).to(dev)
    x_pin = torch.from_numpy(x).pin_memory()
    blk = torch.zeros((cap, n), dtype=torch.int32, device=dev)
    gathered = [torch.empty_like(blk) for _ in range(world)]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def job(xin):
        """One job; rank 0 returns (full label matrix, corrected graph) on the device."""
        r = None
        if count > 0:
            r = kg.KODAMA_matrix(xin, res_out=blk[:count], device=local, runs=count, first_run=first,
                                 apply_dissimilarity=False, materialize_graph=rank == 0, **block_kw)
        dist.all_gather(gathered, blk)
        if rank != 0:
            return None, r
        full = torch.cat([g[:c] for g, c in zip(gathered, counts)]).contiguous()
        gi = torch.from_numpy(r.knn_idx).to(dev)
        gd = torch.from_numpy(r.knn_dist).to(dev)
        kg.KODAMADissimilarityInPlace_device(gi, gd, full, device=local)
        return (full, gi, gd), r

    def timed(xfn, steps, d2h):
        out, times, last = None, [], None
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            dist.barrier()
            t0 = time.perf_counter()
            out, last = job(xfn())
            if rank == 0 and d2h:
                # end to end: the label matrix and the corrected graph come back to the host
                for t in out:
                    t.cpu()
            torch.cuda.synchronize()
            dist.barrier()
            t = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            times.append(float(t))
        return out, last, float(np.mean(times))

    def dev_input():
        return x_dev

    def host_input():
        return x_pin.to(dev, non_blocking=True)

    for _ in range(args.warmup):
        job(x_dev)
    launches0 = kg.launch_count()
    with ClockSampler(local) as clocks:
        out, last, value = timed(dev_input, args.steps, False)
    launches = (kg.launch_count() - launches0) // max(1, args.steps)
    _, _, e2e_v = timed(host_input, args.steps, True)
    if rank != 0:
        dist.barrier()
        dist.destroy_process_group()
        return
    full, gi, gd = out
    res_host = full.cpu().numpy()
    line = {"metric": METRIC, "value": round(value, 5), "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 3), "higher_is_better": False,
            "scaling": "strong", "vs_baseline": None, "dtype": "int32/f64", "data": "synthetic",
            "config": _config({"parallelism": f"the {M} runs split over {world} GPU(s) ({counts} runs), "
                                              "label blocks all-gathered over NCCL, proximity on rank 0"}),
            "e2e": {"value": round(e2e_v, 5), "unit": "s", "h2d_bytes_per_step": world * x.nbytes + gi.numel() * 8,
                    "d2h_bytes_per_step": M * n * 4 + gi.numel() * 8},
            "gpu_launches": int(launches), "clocks": clocks.summary(),
            "stage_ms_rank0": {k: round(v, 3) for k, v in last.kernel_ms.items()} if last is not None else None}
    if world == 1:
        # the sharded job equals the single-call job, labels and corrected graph
        ref_call = kg.KODAMA_matrix(x, device=local, materialize_graph=True, **kw)
        line["matches_single_call"] = bool(np.array_equal(res_host, ref_call.res) and
                                           np.array_equal(gi.cpu().numpy(), ref_call.knn_idx) and
                                           np.array_equal(gd.cpu().numpy(), ref_call.knn_dist))
        if not args.no_cpu_baseline:
            line["cpu_baseline"], ref = cpu_baseline(x)
            line["parity_vs_oracle"] = {"bit_exact": bool(np.array_equal(res_host, ref.res))}
    print(json.dumps(line))
    dist.barrier()
    dist.destroy_process_group()


def run_gpu(args):
    import torch

    import kodama_gb300 as kg
    from kodama_gb300 import build as kbuild

    kbuild.build()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    x = _data()
    kw = _matrix_kw()
    n, runs, cycles = WORKLOAD["n"], WORKLOAD["runs"], WORKLOAD["cycles"]
    x_dev = torch.from_numpy(x).to(f"cuda:{local}")
    res_dev = torch.empty((runs, n), dtype=torch.int32, device=f"cuda:{local}")
    x_pin = torch.from_numpy(x).pin_memory()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        kg.KODAMA_matrix(x_dev, res_out=res_dev, device=local, **kw)
    kg.KODAMA_matrix(x_pin.numpy(), device=local, **kw)

    # device-resident timing
    spans, evo, walls, accs = [], [], [], []
    launches0 = kg.launch_count()
    barrier()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = kg.KODAMA_matrix(x_dev, res_out=res_dev, device=local, **kw)
            walls.append(time.perf_counter() - t0)
            spans.append(r.kernel_ms["device_span"] / 1000.0)
            evo.append(r.kernel_ms["evolution"] / 1000.0)
            accs.append(float(r.acc.mean()))
        barrier()
    launches = (kg.launch_count() - launches0) // max(1, args.steps)
    value = float(np.mean(spans))
    stage_ms = {k: round(v, 3) for k, v in r.kernel_ms.items()}
    timed_res = res_dev.cpu().numpy()   # the timed call's label matrix, for the parity check

    # end-to-end through the host-buffer C-ABI call
    e2e = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        re = kg.KODAMA_matrix(x_pin.numpy(), device=local, **kw)
        e2e.append(time.perf_counter() - t0)
    e2e_v = float(np.mean(e2e))
    same = bool(np.array_equal(re.acc, r.acc))

    if dist is not None:
        t = torch.tensor([value, e2e_v], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        value, e2e_v = float(t[0]), float(t[1])
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    L = min(WORKLOAD["landmarks"], n - 1)
    w = min(WORKLOAD["knn_k"], WORKLOAD["graph_neighbors"])
    evo_s = float(np.mean(evo))
    bytes_launch = evolve_bytes_per_launch(L, w, runs, cycles)
    peak, peak_kind = _peaks()
    achieved = bytes_launch / evo_s / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "kernel": "evolve_kernel (persistent, one CTA per run)",
                "algorithmic_bytes_per_launch": bytes_launch,
                "launch_ms": round(evo_s * 1000, 3),
                "traffic": EVOLVE_TRAFFIC_BYTES if WORKLOAD["n"] == 20000 else None}
    h2d = x.nbytes
    d2h = runs * n * 4 + runs * 8 + runs * cycles * 8 + runs * 3 * 8 + runs * 8 * 4 + runs * cycles * 5 * 4
    line = {"metric": METRIC, "value": round(value, 5), "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/f64", "data": "synthetic",
            "config": _config({"parallelism": f"replicas{world}"}),
            "e2e": {"value": round(e2e_v, 5), "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roofline,
            "gpu_launches": int(launches),
            "clocks": clocks.summary(),
            "stage_ms": stage_ms,
            "host_wall_s": round(float(np.mean(walls)), 5),
            "mean_final_cv_acc": round(float(np.mean(accs)), 6),
            "e2e_matches_resident": same}
    if world == 1 and not args.no_learned:
        line["learned"] = learned_comparison(kg, x, x_dev, res_dev, local, kw, flush, float(np.mean(accs)), value,
                                             evo_s * 1000.0, args.steps)
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"], ref = cpu_baseline(x)
        line["parity_vs_oracle"] = _parity(timed_res, r.acc, r.v, r.run_hashes, r.run_counters, ref)
    print(json.dumps(line))
    if "parity_vs_oracle" in line and not line["parity_vs_oracle"]["bit_exact"]:
        sys.exit("GPU result differs from the CPU restatement on the timed workload")
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-proposal comparison")
    ap.add_argument("--sharded", action="store_true",
                    help="split the runs across ranks even at N=1 (the N>1 path always does)")
    ap.add_argument("--workload", default="knn", choices=["knn", "pls", "batch", "learned100k"],
                    help="knn: the headline configuration; pls: the PLS-LDA configuration; batch: 256 uneven "
                         "problems in one captured CUDA graph; learned100k: learned vs plain at N=100000")
    args = ap.parse_args()
    if args.workload == "learned100k":
        _use_config5()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "pls":
        run_gpu_pls(args)
    elif args.workload == "batch":
        run_gpu_batch(args)
    elif args.workload == "knn" and (args.sharded or int(os.environ.get("WORLD_SIZE", "1")) > 1):
        run_gpu_sharded(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
