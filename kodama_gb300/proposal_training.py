"""Training data and default weights of the learned relabelling proposal.

The network is trained on the moves the plain method itself makes: a plain
KODAMA.matrix run records, at the start of a chosen cycle, the features of
every landmark and whether its label differs from its CV prediction (a
candidate move); the target of a candidate is whether the run's final best
labelling took that move (best label == the prediction at the snapshot).
Every candidate move is still accepted or rejected by the exact CV accuracy
when the network proposes it.

``python -m kodama_gb300.proposal_training [--out PATH]`` regenerates the
shipped weights (``proposal_default.npy``) on the GPU: snapshots of plain runs
on three synthetic workloads that are not the benchmark's data -- the
interleaved spirals (N=1000, d=10), a 12-cluster Gaussian mixture (N=20000,
d=50, seed 7) and the low-rank PLS workload (N=10000, d=200, seed 3) -- then
30 epochs of Adam.  Deterministic on a given GPU model.
"""

from __future__ import annotations

import argparse
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "proposal_default.npy")

# cycles whose starting states are recorded (of Tcycle = 100)
_SNAPSHOT_CYCLES = (0, 2, 5, 10, 20, 35, 50)


def _workloads():
    from . import datasets
    xs, _ = datasets.spirals()
    xm, _ = datasets.gaussian_mixture(n=20000, d=50, seed=7)
    xl, _ = datasets.low_rank(n=10000, d=200, seed=3)
    return [
        (xs.astype(np.float32), dict(runs=20, landmarks=10000, splitting=0, graph_neighbors=50, folds=10,
                                     knn_k=10)),
        (xm, dict(runs=20, landmarks=10000, splitting=50, graph_neighbors=30, folds=10, knn_k=30)),
        (xl, dict(runs=10, landmarks=10000, splitting=50, graph_neighbors=30, folds=10, knn_k=30)),
    ]


def collect_snapshots(x, *, cycles=100, snapshot_cycles=_SNAPSHOT_CYCLES, seed=77, device=0, **matrix_kw):
    """Candidate moves of plain runs: (features n x 8 float32, targets n uint8)."""
    from . import KODAMA_matrix
    feats, targets = [], []
    for c in snapshot_cycles:
        if c >= cycles:
            continue
        r = KODAMA_matrix(x, cycles=cycles, seed=seed, snapshot_cycle=c, device=device, **matrix_kw)
        cand = (r.snapshot_flags & 1).astype(bool)
        feats.append(r.snapshot_features[cand])
        targets.append(((r.snapshot_flags[cand] >> 1) & 1).astype(np.uint8))
    return np.concatenate(feats), np.concatenate(targets)


def train_default(device=0, epochs=30, batch=4096, learning_rate=2e-3, seed=1):
    """The default weights: (weights, loss per epoch, training rows)."""
    from . import train_proposal
    feats, targets = [], []
    for x, kw in _workloads():
        f, t = collect_snapshots(x, device=device, **kw)
        feats.append(f)
        targets.append(t)
    f = np.concatenate(feats)
    t = np.concatenate(targets)
    w, losses = train_proposal(f, t, epochs=epochs, batch=batch, learning_rate=learning_rate, seed=seed,
                               device=device)
    return w, losses, len(f)


def load_default() -> np.ndarray:
    """The shipped default weights (4801 float32)."""
    w = np.load(DEFAULT_WEIGHTS)
    if w.dtype != np.float32 or w.shape != (4801,):
        raise ValueError(f"{DEFAULT_WEIGHTS} does not hold 4801 float32 weights")
    return w


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args()
    w, losses, rows = train_default(device=args.device)
    np.save(args.out, w)
    print(f"wrote {args.out}: {rows} candidate moves, loss {losses[0]:.4f} -> {losses[-1]:.4f}")


if __name__ == "__main__":
    main()
