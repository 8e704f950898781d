"""Seeded synthetic stand-ins for the five benchmark workloads.

No dataset ships with the reference (its scripts read a private MNIST copy),
so every workload is generated from a fixed seed with the shapes, sizes and
value distributions of the benchmark configurations.  All generators return
float32 arrays of shape (n, d), C-contiguous: row p is point p, which is the
reference's d x n column-major layout (src/Utilities.cpp:69-76).

Data seeds default to 1000*cfg + 7.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = [
    "cfg2_mnist_like_torch", "vmf_mixture_torch", "cfg5_batch_torch",
    "vmf_mixture", "cfg1_cosine", "cfg2_mnist_like", "cfg3_aniso_l2", "cfg4_dirichlet", "cfg5_batch",
    "CONFIGS",
]


def _unit_rows(a: np.ndarray) -> np.ndarray:
    return a / np.linalg.norm(a, axis=1, keepdims=True)


def vmf_mixture(n: int, d: int, n_clusters: int, sigma: float, noise_frac: float, seed: int,
                normalise: bool = True, chunk: int = 1 << 18) -> tuple[np.ndarray, np.ndarray]:
    """Unit-norm Gaussian centres; point = centre + N(0, sigma^2 I), then
    L2-normalised; a `noise_frac` share are uniform on the sphere (label -1)."""
    rng = np.random.default_rng(seed)
    centres = _unit_rows(rng.standard_normal((n_clusters, d))).astype(np.float32)
    X = np.empty((n, d), np.float32)
    y = rng.integers(0, n_clusters, n).astype(np.int32)
    is_noise = rng.random(n) < noise_frac
    y[is_noise] = -1
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        yy = y[s:e]
        blk = rng.standard_normal((e - s, d), dtype=np.float32)
        cl = yy >= 0
        blk[cl] = centres[yy[cl]] + np.float32(sigma) * blk[cl]
        if normalise:
            blk /= np.linalg.norm(blk, axis=1, keepdims=True)
        X[s:e] = blk
    return X, y


def cfg1_cosine(n: int = 50_000, d: int = 128, literal: bool = False, seed: int = 1007):
    """Config 1: 20 vMF-like clusters + 5% uniform noise, Cosine.

    literal=True uses per-coordinate sigma 0.15 (which, at d=128, puts almost
    every pair beyond eps=0.15, i.e. an all-noise clustering); the default
    uses noise of norm 0.15 (sigma = 0.15/sqrt(d)), a meaningful clustering."""
    sigma = 0.15 if literal else 0.15 / math.sqrt(d)
    return vmf_mixture(n, d, 20, sigma, 0.05, seed)


def cfg2_mnist_like(n: int = 1_000_000, d: int = 784, n_comp: int = 10, seed: int = 2007,
                    chunk: int = 1 << 16) -> tuple[np.ndarray, np.ndarray]:
    """Config 2: nonnegative values in [0,1]; each of 10 prototypes is a
    Bernoulli(0.2) mask times Uniform(0.3,1); a point copies its prototype and
    redraws 10% of its pixels from the same mask-times-uniform law; rows are
    L2-normalised."""
    rng = np.random.default_rng(seed)
    protos = ((rng.random((n_comp, d)) < 0.2) * rng.uniform(0.3, 1.0, (n_comp, d))).astype(np.float32)
    y = rng.integers(0, n_comp, n).astype(np.int32)
    X = np.empty((n, d), np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        u = rng.random((3, e - s, d), dtype=np.float32)
        fresh = np.where(u[1] < 0.2, np.float32(0.3) + np.float32(0.7) * u[2], np.float32(0.0))
        blk = np.where(u[0] < 0.1, fresh, protos[y[s:e]])
        blk[:, 0] += np.float32(1e-3)  # keeps every row nonzero
        X[s:e] = blk / np.sqrt(np.einsum("ij,ij->i", blk, blk))[:, None]
    return X, y


def cfg3_aniso_l2(n: int = 1_000_000, d: int = 256, n_comp: int = 50, scale: float = 1.0, seed: int = 3007,
                  chunk: int = 1 << 16) -> tuple[np.ndarray, np.ndarray]:
    """Config 3: 50 anisotropic Gaussians in R^256 with seeded rotations and
    eigenvalues Uniform(0.1, 2); centres N(0, 5^2 I).  `scale` multiplies the
    whole dataset (scale < 1 gives the scaled-data variant where eps=0.3 is
    meaningful)."""
    rng = np.random.default_rng(seed)
    centres = (5.0 * rng.standard_normal((n_comp, d))).astype(np.float32)
    factors = []
    for _ in range(n_comp):
        q, _r = np.linalg.qr(rng.standard_normal((d, d)))
        ev = rng.uniform(0.1, 2.0, d)
        factors.append((q * np.sqrt(ev)[None, :]).astype(np.float32))  # cov = Q diag(ev) Q^T
    factors = np.stack(factors)
    y = rng.integers(0, n_comp, n).astype(np.int32)
    X = np.empty((n, d), np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        z = rng.standard_normal((e - s, d), dtype=np.float32)
        yy = y[s:e]
        out = np.empty((e - s, d), np.float32)
        for c in np.unique(yy):  # point = factor_c z + centre_c, one GEMM per component
            rows = np.nonzero(yy == c)[0]
            out[rows] = z[rows] @ factors[c].T + centres[c]
        X[s:e] = (out * scale).astype(np.float32)
    return X, y


def cfg4_dirichlet(n: int = 500_000, d: int = 512, n_comp: int = 30, alpha: float = 0.1, conc: float = 200.0,
                   seed: int = 4007, chunk: int = 1 << 16, zero_below: float = 1e-9) -> tuple[np.ndarray, np.ndarray]:
    """Config 4: nonnegative histograms.  30 prototypes ~ Dirichlet(alpha=0.1);
    a point ~ Dirichlet(conc * prototype + alpha/10).  Entries below
    zero_below (1e-9: less than one count in a billion) are set to 0 and the
    row renormalised: the Dirichlet's tiny shape parameters otherwise give
    entries near 1e-30 whose pairwise products fall into float32's subnormal
    range.  zero_below = 0 keeps the raw law (tiny entries included)."""
    rng = np.random.default_rng(seed)
    protos = rng.dirichlet(np.full(d, alpha), n_comp)
    y = rng.integers(0, n_comp, n).astype(np.int32)
    X = np.empty((n, d), np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        a = conc * protos[y[s:e]] + alpha / 10.0
        g = rng.standard_gamma(a)
        g /= g.sum(axis=1, keepdims=True)
        if zero_below > 0:
            g[g < zero_below] = 0.0
            g /= g.sum(axis=1, keepdims=True)
        X[s:e] = g.astype(np.float32)
    return X, y


def cfg5_batch(n_sets: int = 64, seed: int = 5007, n_lo: int = 2_000, n_hi: int = 200_000):
    """Config 5: `n_sets` independent unit-norm vMF-style mixtures, n
    log-uniform in [n_lo, n_hi], d in {64, 128, 256}, 5-40 clusters each."""
    rng = np.random.default_rng(seed)
    sets = []
    for i in range(n_sets):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        d = int(rng.choice([64, 128, 256]))
        c = int(rng.integers(5, 41))
        X, y = vmf_mixture(n, d, c, 0.15 / math.sqrt(d), 0.05, seed * 100 + i)
        sets.append((X, y))
    return sets


# Benchmark configurations: data generator + set_params / fit arguments.
CONFIGS = {
    1: dict(name="cfg1_cosine_50Kx128", gen=cfg1_cosine, distance="Cosine", n_proj=1024, topK=5, topM=50,
            eps=0.15, minPts=20),
    2: dict(name="cfg2_cosine_1Mx784", gen=cfg2_mnist_like, distance="Cosine", n_proj=1024, topK=10, topM=50,
            eps=0.25, minPts=50),
    3: dict(name="cfg3_l2_rff_1Mx256", gen=cfg3_aniso_l2, distance="L2", n_proj=1024, topK=10, topM=100,
            eps=0.3, minPts=30, ker_n_features=1024),
    4: dict(name="cfg4_chi2_soptics_500Kx512", gen=cfg4_dirichlet, distance="Chi2", n_proj=1024, topK=10, topM=50,
            eps=0.17, minPts=50, ker_n_features=1024),
}


def cfg2_mnist_like_torch(n: int = 1_000_000, d: int = 784, n_comp: int = 10, seed: int = 2007,
                          device: str = "cuda", chunk: int = 1 << 17):
    """The config-2 law of cfg2_mnist_like, drawn on the GPU with torch (for
    the full-size benchmark, where numpy generation would take minutes).
    Returns a (n, d) float32 tensor on `device` and the component labels."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    protos = ((torch.rand(n_comp, d, generator=g, device=device) < 0.2).float() *
              (0.3 + 0.7 * torch.rand(n_comp, d, generator=g, device=device)))
    y = torch.randint(0, n_comp, (n,), generator=g, device=device)
    X = torch.empty(n, d, dtype=torch.float32, device=device)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        u = torch.rand(3, e - s, d, generator=g, device=device)
        fresh = torch.where(u[1] < 0.2, 0.3 + 0.7 * u[2], torch.zeros((), device=device))
        blk = torch.where(u[0] < 0.1, fresh, protos[y[s:e]])
        blk[:, 0] += 1e-3
        X[s:e] = blk / blk.norm(dim=1, keepdim=True)
    return X, y


def vmf_mixture_torch(n: int, d: int, n_clusters: int, sigma: float, noise_frac: float, seed: int,
                      device: str = "cuda"):
    """vmf_mixture's law drawn on the GPU with torch; (n, d) float32 tensor."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    centres = torch.randn(n_clusters, d, generator=g, device=device)
    centres = centres / centres.norm(dim=1, keepdim=True)
    y = torch.randint(0, n_clusters, (n,), generator=g, device=device)
    noise = torch.rand(n, generator=g, device=device) < noise_frac
    z = torch.randn(n, d, generator=g, device=device)
    X = torch.where(noise[:, None], z, centres[y] + sigma * z)
    X = X / X.norm(dim=1, keepdim=True)
    return X.contiguous(), torch.where(noise, torch.full_like(y, -1), y)


def cfg5_batch_torch(n_sets: int = 64, seed: int = 5007, n_lo: int = 2_000, n_hi: int = 200_000,
                     device: str = "cuda"):
    """cfg5_batch's sets (same sizes, dims and cluster counts, from the same
    numpy seed) with the points drawn on the GPU."""
    rng = np.random.default_rng(seed)
    sets = []
    for i in range(n_sets):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        d = int(rng.choice([64, 128, 256]))
        c = int(rng.integers(5, 41))
        X, y = vmf_mixture_torch(n, d, c, 0.15 / math.sqrt(d), 0.05, seed * 100 + i, device=device)
        sets.append((X, y))
    return sets
