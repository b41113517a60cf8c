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


def _gather(dist, arr: np.ndarray) -> np.ndarray:
    """all_gather of variable-length first dimension (gloo/nccl agnostic via objects)."""
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, arr)
    return np.concatenate([o for o in out if o is not None and len(o)], axis=0)


def kodama_matrix_sharded(x, *, runs, graph, matrix_fn, dissimilarity_fn, dist, **options) -> ShardedResult:
    """One KODAMA.matrix job over all ranks of `dist` (torch.distributed).

    graph: (zero-based indices, distances) of the exact graph, shared by all
    ranks.  matrix_fn(x, graph, first_run=..., runs=..., **options) computes
    a block of runs; dissimilarity_fn(idx1, dist, res) applies the proximity
    correction to a one-based graph.
    """
    world, rank = dist.get_world_size(), dist.get_rank()
    first, count = shard(runs, world, rank)
    part = matrix_fn(x, graph, first_run=first, runs=count, **options)
    res = _gather(dist, part.res)
    acc = _gather(dist, part.acc)
    v = _gather(dist, part.v)
    hashes = _gather(dist, part.run_hashes)
    counters = _gather(dist, part.run_counters)
    diag = _gather(dist, part.cycle_diag)
    gi, gd = graph
    idx1 = np.where(gi >= 0, gi + 1, gi).astype(np.int32)
    kidx, kdist = dissimilarity_fn(idx1, gd.astype(np.float32), res)
    return ShardedResult(res, acc, v, hashes, counters, diag, kidx, kdist)
