"""The tensor-core candidate search of the exact graph (knn_tc.cu): identical
to the canonical brute force and to the CPU restatement on every shape, on
data made of ties and duplicates, far from the origin, and with non-finite
values (which send every row to the brute force)."""

import numpy as np
import pytest

from kodama_gb300 import datasets


def _same(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,K", [(300, 3, 1), (1000, 10, 50), (2500, 16, 30), (3000, 17, 10), (4000, 33, 96),
                                   (6000, 50, 30), (5000, 64, 20), (20000, 50, 30), (3000, 65, 30),
                                   (4000, 100, 30), (2500, 128, 64), (12000, 100, 30), (3000, 129, 30),
                                   (4000, 160, 30), (2500, 200, 64), (3000, 256, 96), (10000, 200, 30)])
def test_tensor_search_matches_oracle(kg, orc, n, d, K):
    x, _ = datasets.gaussian_mixture(n=n, d=d, seed=n + d)
    t = kg.knn_graph(x, K, method="tensor", return_fallback=True)
    b = kg.knn_graph(x, K, method="brute_force")
    assert _same(t[:2], b)
    if n <= 6000:
        assert _same(t[:2], orc.exact_knn(x, K, threads=8))
    # the certificate holds for almost every row (distances concentrate above
    # d = 128, so more rows land within 2 delta of their K-th distance)
    assert t[2] <= (n // 50 if d <= 128 else n // 20), t[2]


@pytest.mark.gpu
@pytest.mark.parametrize("d", [90, 200])
def test_tensor_search_low_rank(kg, orc, d):
    # low-rank data with noise: many near-equal distances in a few directions
    x, _ = datasets.low_rank(n=4000, d=d, seed=d)
    t = kg.knn_graph(x, 30, method="tensor", return_fallback=True)
    assert _same(t[:2], kg.knn_graph(x, 30, method="brute_force"))
    assert _same(t[:2], orc.exact_knn(x, 30, threads=8))


@pytest.mark.gpu
def test_tensor_search_ties_and_duplicates(kg):
    rng = np.random.default_rng(5)
    x = rng.integers(-3, 4, (3000, 8)).astype(np.float32)  # many equal distances
    x[1000:1300] = x[0:300]                                  # exact duplicates
    t = kg.knn_graph(x, 25, method="tensor", return_fallback=True)
    assert _same(t[:2], kg.knn_graph(x, 25, method="brute_force"))


@pytest.mark.gpu
def test_tensor_search_far_from_origin(kg):
    x, _ = datasets.gaussian_mixture(n=4000, d=24, seed=3)
    x = x + np.float32(500.0)
    t = kg.knn_graph(x, 30, method="tensor", return_fallback=True)
    assert _same(t[:2], kg.knn_graph(x, 30, method="brute_force"))


@pytest.mark.gpu
def test_tensor_search_non_finite_falls_back(kg):
    x, _ = datasets.gaussian_mixture(n=2000, d=12, seed=4)
    x[17, 3] = np.inf
    t = kg.knn_graph(x, 10, method="tensor", return_fallback=True)
    assert t[2] == 2000
    assert _same(t[:2], kg.knn_graph(x, 10, method="brute_force"))


@pytest.mark.gpu
def test_tensor_search_limits(kg):
    x, _ = datasets.gaussian_mixture(n=500, d=257, seed=1)
    with pytest.raises(ValueError, match="tensor-core"):
        kg.knn_graph(x, 10, method="tensor")
    idx, _ = kg.knn_graph(x, 10)  # auto: the brute force
    assert idx.shape == (500, 10)
