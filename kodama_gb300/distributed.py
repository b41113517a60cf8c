"""Runs of one KODAMA.matrix job sharded across ranks (one GPU per rank).

The M runs are independent: run r draws only from seed + r
(kodama_matrix.cpp:2897, :3113).  Rank k computes a contiguous block of runs
(`first_run` = its first run id) on its own device; the label rows, traces and
per-run diagnostics are gathered in run order; the co-label proximity of the
graph then uses all M label rows on every rank.  There is no other exchange.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def shard(runs: int, world: int, rank: int) -> tuple[int, int]:
    """(first run id, number of runs) of `rank`: contiguous, balanced blocks."""
    lo = rank * runs // world
    hi = (rank + 1) * runs // world
    return lo + 1, hi - lo


@dataclass
class ShardedResult:
    res: np.ndarray
    acc: np.ndarray
    v: np.ndarray
    run_hashes: np.ndarray
    run_counters: np.ndarray
    cycle_diag: np.ndarray
    knn_idx: np.ndarray | None
    knn_dist: np.ndarray | None


def _gather(dist, arr: np.ndarray, counts: list[int], device) -> np.ndarray:
    """all_gather of the ranks' run blocks (first dimension counts[rank]) in
    rank order: each block is padded to the largest, exchanged as a tensor
    (NCCL or gloo), then trimmed.  64-bit unsigned values travel as int64."""
    import torch

    cap = max(max(counts), 1)
    unsigned = arr.dtype == np.uint64
    a = arr.view(np.int64) if unsigned else arr
    pad = np.zeros((cap,) + a.shape[1:], dtype=a.dtype)
    pad[: len(a)] = a
    t = torch.from_numpy(pad).to(device)
    outs = [torch.empty_like(t) for _ in counts]
    dist.all_gather(outs, t)
    out = np.concatenate([o.cpu().numpy()[:c] for o, c in zip(outs, counts)], axis=0)
    return out.view(np.uint64) if unsigned else out


def kodama_matrix_sharded(x, *, runs, graph, matrix_fn, dissimilarity_fn, dist, device="cpu",
                          **options) -> ShardedResult:
    """One KODAMA.matrix job over all ranks of `dist` (torch.distributed).

    graph: (zero-based indices, distances) of the exact graph, shared by all
    ranks.  matrix_fn(x, graph, first_run=..., runs=..., **options) computes
    a block of runs; dissimilarity_fn(idx1, dist, res) applies the proximity
    correction to a one-based graph.  `device` holds the exchanged tensors
    ("cuda:<i>" with NCCL, "cpu" with gloo).  A rank whose block is empty
    (more ranks than runs) computes nothing but still takes part in every
    exchange.
    """
    world, rank = dist.get_world_size(), dist.get_rank()
    counts = [shard(runs, world, r)[1] for r in range(world)]
    first, count = shard(runs, world, rank)
    n = x.shape[0]
    cycles = int(options.get("cycles", 20))
    if count > 0:
        part = matrix_fn(x, graph, first_run=first, runs=count, **options)
        blocks = (part.res, part.acc, part.v, part.run_hashes, part.run_counters, part.cycle_diag)
    else:
        blocks = (np.zeros((0, n), np.int32), np.zeros(0, np.float64), np.zeros((0, cycles), np.float64),
                  np.zeros((0, 3), np.uint64), np.zeros((0, 8), np.int32), np.zeros((0, cycles, 5), np.int32))
    res, acc, v, hashes, counters, diag = (_gather(dist, np.ascontiguousarray(b), counts, device) for b in blocks)
    gi, gd = graph
    idx1 = np.where(gi >= 0, gi + 1, gi).astype(np.int32)
    kidx, kdist = dissimilarity_fn(idx1, gd.astype(np.float32), res)
    return ShardedResult(res, acc, v, hashes, counters, diag, kidx, kdist)
