"""Seeded synthetic workloads with the shapes the KODAMA.matrix hot path is
measured on.  No public dataset is used: every matrix is regenerated from its
seed with numpy's PCG64 generator, so tests, the bench and the CPU baseline
all see the same bytes.

* ``spirals``          N=1000, d=10: three interleaved Archimedean spirals
                       (333/333/334 points) plus 8 N(0,1) noise columns.
* ``gaussian_mixture`` N=20000, d=50: 12 isotropic unit-variance clusters with
                       means ~ N(0, 4^2 I) and Dirichlet(1) proportions.
* ``low_rank``         N=10000, d=200: X = Z W + E with 8 classes taken as the
                       nearest of 8 random centres in Z (PLS-LDA workload).
* ``pca_mixture``      N=100000, d=50: 30 clusters along a decaying spectrum.
"""

from __future__ import annotations

import numpy as np


def spirals(n: int = 1000, seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    sizes = [n // 3, n // 3, n - 2 * (n // 3)]
    rows, labels = [], []
    for arm, size in enumerate(sizes):
        t = rng.uniform(0.0, 4.0 * np.pi, size)
        rot = arm * 2.0 * np.pi / 3.0
        x = t * np.cos(t + rot) + rng.normal(0.0, 0.3, size)
        y = t * np.sin(t + rot) + rng.normal(0.0, 0.3, size)
        rows.append(np.stack([x, y], axis=1))
        labels.append(np.full(size, arm + 1, dtype=np.int32))
    xy = np.concatenate(rows)
    noise = rng.normal(0.0, 1.0, (n, 8))
    return np.concatenate([xy, noise], axis=1).astype(np.float64), np.concatenate(labels)


def gaussian_mixture(
    n: int = 20000, d: int = 50, clusters: int = 12, mean_scale: float = 4.0,
    alpha: float = 1.0, seed: int = 2,
) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    props = rng.dirichlet(np.full(clusters, alpha))
    counts = rng.multinomial(n, props)
    means = rng.normal(0.0, mean_scale, (clusters, d))
    x = np.empty((n, d), dtype=np.float32)
    y = np.empty(n, dtype=np.int32)
    pos = 0
    for c, cnt in enumerate(counts):
        x[pos:pos + cnt] = means[c] + rng.normal(0.0, 1.0, (cnt, d))
        y[pos:pos + cnt] = c + 1
        pos += cnt
    order = rng.permutation(n)
    return x[order], y[order]


def low_rank(n: int = 10000, d: int = 200, rank: int = 10, classes: int = 8,
             seed: int = 3) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    z = rng.normal(0.0, 1.0, (n, rank))
    w = rng.normal(0.0, 1.0, (rank, d))
    e = rng.normal(0.0, 0.5, (n, d))
    centres = rng.normal(0.0, 1.0, (classes, rank))
    d2 = ((z[:, None, :] - centres[None, :, :]) ** 2).sum(-1)
    y = (np.argmin(d2, axis=1) + 1).astype(np.int32)
    return (z @ w + e).astype(np.float32), y


def pca_mixture(n: int = 100000, d: int = 50, clusters: int = 30, seed: int = 5
                ) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    props = rng.dirichlet(np.full(clusters, 0.5))
    counts = rng.multinomial(n, props)
    q, _ = np.linalg.qr(rng.normal(size=(d, d)))
    sigma = 10.0 * np.arange(1, d + 1, dtype=np.float64) ** -1.0
    means = (rng.normal(0.0, 1.0, (clusters, d)) * sigma) @ q.T * 3.0
    x = np.empty((n, d), dtype=np.float32)
    y = np.empty(n, dtype=np.int32)
    pos = 0
    for c, cnt in enumerate(counts):
        x[pos:pos + cnt] = means[c] + (rng.normal(0.0, 1.0, (cnt, d)) * sigma) @ q.T
        y[pos:pos + cnt] = c + 1
        pos += cnt
    order = rng.permutation(n)
    return x[order], y[order]


def uneven_batch(count: int = 256, seed: int = 4) -> list[dict]:
    """Independent KODAMA.matrix problems of uneven size: problem i draws, from
    its own generator seeded seed + i, N log-uniform in [500, 20000],
    d uniform in {10, 50, 100} and a Gaussian mixture of 3-20 clusters with
    means ~ N(0, 3^2 I) and unit covariance; even problems use the kNN
    classifier, odd ones PLS-LDA.  Returns dicts with x (float32), classifier."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        n = int(round(float(np.exp(rng.uniform(np.log(500.0), np.log(20000.0))))))
        d = int(rng.choice([10, 50, 100]))
        clusters = int(rng.integers(3, 21))
        x, _ = gaussian_mixture(n=n, d=d, clusters=clusters, mean_scale=3.0, seed=int(rng.integers(1 << 31)))
        out.append({"x": x, "classifier": "knn" if i % 2 == 0 else "pls"})
    return out

