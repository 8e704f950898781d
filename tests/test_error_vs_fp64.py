"""Error of the FP32 path against an FP64 evaluation of the same mathematics.

The engine's plain FP32 projections, distances and core distances are
bit-identical to the oracle's (tests/test_gpu_parity.py), so the oracle's
error against FP64 is the engine's.  Reachability values are such FP32
distances (a core distance or a pair distance, src/sDbscan.cpp:1660-1690) and
carry the same error.  Bounds asserted here, as relative errors:
  - projections: 1e-5 of the projection vector's norm (three 1024-point
    FWHT rounds of FP32 adds);
  - Cosine distance 1 - x.y: 2e-6 absolute (784 sequential fmaf, unit rows);
  - L2 distance: 1e-5 relative;  Chi2 distance: 1e-5 absolute.
"""
import numpy as np

from oracle.oracle import fht_dim
from sdbscan_gb300 import datasets


def _fwht64(v):
    v = v.copy()
    n = v.shape[1]
    h = 1
    while h < n:
        v = v.reshape(v.shape[0], -1, 2, h)
        a, b = v[:, :, 0, :].copy(), v[:, :, 1, :].copy()
        v[:, :, 0, :], v[:, :, 1, :] = a + b, a - b
        v = v.reshape(v.shape[0], n)
        h *= 2
    return v


def test_projection_error_vs_fp64(port):
    X, _ = datasets.cfg2_mnist_like(1500, 196, seed=61)
    n, d = X.shape
    nproj = 1024
    fd = fht_dim(nproj, d)
    bits = port.hd3_bits(3 * fd, 7).astype(np.float64)
    Xt, rc = port.transform(X, "Cosine")
    assert rc == 0
    P32 = port.project(Xt, "Cosine", d, 0.4, np.zeros(1, np.float32), bits.astype(np.uint8), fd, nproj)
    x64 = X.astype(np.float64)
    x64 /= np.linalg.norm(x64, axis=1, keepdims=True)
    v = np.zeros((n, fd))
    v[:, :d] = x64
    for r in range(3):
        v *= np.where(bits[r * fd:(r + 1) * fd] > 0, 1.0, -1.0)[None, :]
        v = _fwht64(v)
    P64 = v[:, :nproj]
    rel = np.abs(P32 - P64) / np.linalg.norm(P64, axis=1, keepdims=True)
    print(f"projection error vs FP64: max {rel.max():.2e}, median {np.median(rel):.2e} of the row norm")
    assert rel.max() < 1e-5


def test_distance_error_vs_fp64(port):
    rng = np.random.default_rng(5)
    Xc, _ = datasets.cfg2_mnist_like(400, 784, seed=62)
    Xc, _ = port.transform(Xc, "Cosine")
    Xl, _ = datasets.cfg3_aniso_l2(400, 256, n_comp=5, seed=63)
    Xh, _ = datasets.cfg4_dirichlet(400, 512, n_comp=5, seed=64)
    Xh, _ = port.transform(Xh, "Chi2")
    worst = {}
    for name, X in (("Cosine", Xc), ("L2", Xl), ("Chi2", Xh)):
        errs = []
        for _ in range(300):
            i, j = rng.integers(0, X.shape[0], 2)
            a, b = X[i].astype(np.float64), X[j].astype(np.float64)
            f32 = port.distance(X[i], X[j], name)
            if name == "Cosine":
                f64 = 1.0 - a @ b
                errs.append(abs(f32 - f64))
            elif name == "L2":
                f64 = np.sqrt(((a - b) ** 2).sum())
                errs.append(abs(f32 - f64) / max(f64, 1e-30))
            else:
                m = (a > 0) & (b > 0)
                f64 = 1.0 - 2.0 * (a[m] * b[m] / (a[m] + b[m])).sum()
                errs.append(abs(f32 - f64))
        worst[name] = max(errs)
    print("distance error vs FP64:", {k: f"{v:.2e}" for k, v in worst.items()})
    assert worst["Cosine"] < 2e-6 and worst["L2"] < 1e-5 and worst["Chi2"] < 1e-5
