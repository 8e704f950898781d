"""The seeded synthetic workloads that stand in for the reference's datasets
(MNIST and the configurations of the benchmark): each follows its stated law,
is a function of its seed, and the torch (device-side) generators used at full
size draw the same law as the numpy ones (checked here on the CPU device)."""
import numpy as np
import pytest

from sdbscan_gb300 import datasets as ds


def test_cfg2_law_nonnegative_unit_rows_ten_components():
    X, y = ds.cfg2_mnist_like(4000, 784, seed=5)
    assert X.dtype == np.float32 and X.shape == (4000, 784)
    assert (X >= 0).all()
    np.testing.assert_allclose(np.linalg.norm(X, axis=1), 1.0, atol=1e-5)
    assert set(np.unique(y)) == set(range(10))
    # about 20 % of a prototype's pixels are on; 10 % of a point's pixels redrawn
    assert 0.17 < float((X > 0).mean()) < 0.23
    X2, y2 = ds.cfg2_mnist_like(4000, 784, seed=5)
    np.testing.assert_array_equal(X, X2)
    np.testing.assert_array_equal(y, y2)
    # within-component pairs are close in cosine distance, across components far
    a, b = X[y == 0][:50], X[y == 1][:50]
    assert float(np.median(1 - a @ a.T)) < 0.3 < float(np.median(1 - a @ b.T))


def test_cfg2_torch_generator_draws_the_same_law():
    torch = pytest.importorskip("torch")
    Xt, yt = ds.cfg2_mnist_like_torch(4000, 784, seed=5, device="cpu", chunk=1000)
    X = Xt.numpy()
    assert X.shape == (4000, 784) and (X >= 0).all()
    np.testing.assert_allclose(np.linalg.norm(X, axis=1), 1.0, atol=1e-5)
    assert len(torch.unique(yt)) == 10
    assert 0.17 < float((X > 0).mean()) < 0.23
    Xn, _ = ds.cfg2_mnist_like(4000, 784, seed=5)
    assert abs(float(X[X > 0].mean()) - float(Xn[Xn > 0].mean())) < 0.01


def test_cfg1_cfg5_unit_rows_and_noise_share():
    X, y = ds.cfg1_cosine(5000, 128, seed=3)
    np.testing.assert_allclose(np.linalg.norm(X, axis=1), 1.0, atol=1e-5)
    assert 0.03 < float((y == -1).mean()) < 0.07 and len(np.unique(y[y >= 0])) == 20
    sets = ds.cfg5_batch(64, seed=5007, n_lo=20, n_hi=200)  # the full batch's d and cluster draws, small n
    assert len(sets) == 64
    assert all(20 <= s[0].shape[0] <= 200 and s[0].shape[1] in (64, 128, 256) for s in sets)
    assert all(len(np.unique(s[1][s[1] >= 0])) <= 40 for s in sets)


def test_cfg3_cfg4_laws():
    X, y = ds.cfg3_aniso_l2(3000, 32, n_comp=5, scale=0.5, seed=7)
    assert X.shape == (3000, 32) and len(np.unique(y)) == 5
    Xu, _ = ds.cfg3_aniso_l2(3000, 32, n_comp=5, scale=1.0, seed=7)
    np.testing.assert_allclose(X, 0.5 * Xu, rtol=1e-6, atol=1e-6)
    H, _ = ds.cfg4_dirichlet(2000, 64, n_comp=6, seed=9)
    assert (H >= 0).all()
    np.testing.assert_allclose(H.sum(axis=1), 1.0, atol=1e-5)
    assert H[H > 0].min() >= 1e-9 * 0.5  # entries below 1e-9 are zeroed
