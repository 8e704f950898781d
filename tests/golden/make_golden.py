"""Generates the golden fixtures in this folder from the reference itself.

Runs the reference's unmodified sDbscan class (built by ``make -C oracle ref``
from the reference sources against the shim headers in ``oracle/shim``) with
one thread on small seeded inputs, and stores inputs and outputs as
compressed ``.npz`` files.  Run on the development machine where the
reference sources exist:

    python tests/golden/make_golden.py [fixture names...]

The fixtures are what pins the oracle (and through it the GPU engine) to the
reference on machines where the reference cannot be built.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Ref, build_ref  # noqa: E402
from sdbscan_gb300 import datasets as ds  # noqa: E402


def cases():
    """(name, X, params, eps, minPts, optics)."""
    X1, _ = ds.cfg1_cosine(2000, 32, seed=11)
    yield "cosine_vmf_2000x32", X1, dict(n_proj=256, topK=5, topM=20, distance="Cosine"), 0.15, 10, False
    X2, _ = ds.cfg1_cosine(1500, 100, seed=12)  # d not a power of two, d < fhtDim
    yield "cosine_d100_1500", X2, dict(n_proj=128, topK=4, topM=25, distance="Cosine"), 0.15, 8, False
    X3, _ = ds.cfg2_mnist_like(2000, 196, seed=13)
    yield "cosine_mnistlike_2000x196", X3, dict(n_proj=256, topK=10, topM=30, distance="Cosine"), 0.25, 20, False
    yield "cosine_optics_2000x32", X1, dict(n_proj=256, topK=5, topM=20, distance="Cosine"), 0.2, 10, True
    # the raw Dirichlet law: entries down to ~1e-30, products in float32's subnormal range
    X4, _ = ds.cfg4_dirichlet(1500, 64, n_comp=5, seed=14, zero_below=0.0)
    yield "chi2_ker512_1500x64", X4, dict(n_proj=256, topK=5, topM=20, distance="Chi2", ker_n_features=512), 0.3, 10, False
    yield "chi2_optics_ker1024_1500x64", X4, dict(n_proj=1024, topK=5, topM=20, distance="Chi2",
                                                   ker_n_features=1024), 0.3, 10, True
    X5, _ = ds.cfg3_aniso_l2(1500, 16, n_comp=5, scale=0.1, seed=15)
    yield "l2_rff_1500x16", X5, dict(n_proj=256, topK=5, topM=20, distance="L2", ker_n_features=256,
                                      ker_sigma=0.5), 0.6, 10, False
    yield "l1_rff_1500x16", X5, dict(n_proj=256, topK=5, topM=20, distance="L1", ker_n_features=256,
                                      ker_sigma=0.5), 2.0, 10, False
    yield "js_ker512_1500x64", X4, dict(n_proj=256, topK=5, topM=20, distance="JS", ker_n_features=512), 0.3, 10, False
    # edge cases
    rng = np.random.default_rng(16)
    base = rng.standard_normal((40, 24)).astype(np.float32)
    Xd = np.repeat(base, 25, axis=0)  # every point has 24 exact duplicates: massive ties
    yield "cosine_duplicates_1000x24", Xd, dict(n_proj=64, topK=3, topM=30, distance="Cosine"), 0.05, 5, False
    X6, _ = ds.cfg1_cosine(800, 16, seed=17)
    yield "cosine_all_noise_800x16", X6, dict(n_proj=64, topK=2, topM=10, distance="Cosine"), 1e-6, 5, False
    X7 = (np.ones((500, 8)) + 1e-3 * rng.standard_normal((500, 8))).astype(np.float32)
    yield "cosine_single_cluster_500x8", X7, dict(n_proj=32, topK=2, topM=40, distance="Cosine"), 0.01, 5, False
    X8, _ = ds.cfg1_cosine(60, 12, seed=18)  # m close to n
    yield "cosine_tiny_60x12", X8, dict(n_proj=16, topK=1, topM=50, distance="Cosine"), 0.3, 3, False
    X9, _ = ds.cfg1_cosine(3000, 64, seed=19)
    yield "cosine_k1_m1_3000x64", X9, dict(n_proj=1024, topK=1, topM=1, distance="Cosine"), 0.2, 2, False
    # sDbscan-1NN noise labelling; samplingProb = 1 takes every core point, so
    # the reference's unseeded rand() is never consulted
    yield "cosine_noise1nn_2000x32", X1, dict(n_proj=256, topK=5, topM=20, distance="Cosine", clusterNoise=1,
                                               samplingProb=1.0), 0.12, 12, False
    # rotation vectors longer than 2048 (the shared-memory projection path)
    X11, _ = ds.cfg1_cosine(600, 2100, seed=25)
    yield "cosine_d2100_fht4096_600", X11, dict(n_proj=256, topK=5, topM=20, distance="Cosine"), 0.15, 8, False
    X4z, _ = ds.cfg4_dirichlet(1500, 64, n_comp=5, seed=14)  # entries below 1e-9 zeroed
    yield "chi2_ker4096_1500x64", X4z, dict(n_proj=256, topK=5, topM=20, distance="Chi2", ker_n_features=4096), \
        0.3, 10, False
    X10, _ = ds.cfg4_dirichlet(1500, 64, n_comp=5, conc=10, seed=24)  # wider histograms: a third left as noise
    yield "chi2_noise1nn_1500x64", X10, dict(n_proj=256, topK=5, topM=20, distance="Chi2", ker_n_features=512,
                                              clusterNoise=1, samplingProb=1.0), 0.2, 12, False


def sng_cases():
    """sngDbscan fixtures: (name, X, distance, samplingProb, eps, minPts).  The
    reference seeds every point's generator with random_seed (7 here), so its
    neighbourhoods are reproducible."""
    X1, _ = ds.cfg1_cosine(2000, 32, seed=11)
    yield "sng_cosine_2000x32", X1, "Cosine", 0.05, 0.15, 10
    yield "sng_cosine_p001_2000x32", X1, "Cosine", 0.01, 0.15, 3
    X6, _ = ds.cfg1_cosine(800, 16, seed=17)
    yield "sng_cosine_exact_800x16", X6, "Cosine", 1.0, 0.08, 8
    X5, _ = ds.cfg3_aniso_l2(1500, 16, n_comp=5, scale=0.1, seed=15)
    yield "sng_l2_1500x16", X5, "L2", 0.1, 0.5, 10
    X10, _ = ds.cfg4_dirichlet(1500, 64, n_comp=5, conc=10, seed=24)
    yield "sng_chi2_1500x64", X10, "Chi2", 0.2, 0.2, 15


def main_sng(only=(), out_dir=HERE):
    for name, X, dist, prob, eps, minPts in sng_cases():
        if only and name not in only:
            continue
        n, d = X.shape
        r = Ref(n, d)
        r.set_sngParams(dist, prob, 0, False, 1, 7)
        r.fit_sngDbscan(X, eps, minPts)
        off, idx = r.neighbors()
        out = dict(X=X, labels=r.labels_, n_clusters=np.int32(r.n_clusters_), core=r.core(),
                   core_degree=np.diff(off).astype(np.int32))
        meta = dict(distance=dist, samplingProb=prob, eps=eps, minPts=minPts, random_seed=7, n_threads=1)
        out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **out)
        print(name, "n_clusters", r.n_clusters_, "cores", int(out["core"].sum()))


def main(only=(), out_dir=HERE):
    """Writes every fixture, or only the named ones, into out_dir."""
    if build_ref() is None:
        sys.exit("the reference sources are not available here; fixtures cannot be regenerated")
    main_sng(only, out_dir)
    for name, X, params, eps, minPts, optics in cases():
        if only and name not in only:
            continue
        n, d = X.shape
        r = Ref(n, d)
        r.set_params(**params, n_threads=1, random_seed=7)
        if optics:
            r.fit_sOptics(X, eps, minPts)
        else:
            r.fit_sDbscan(X, eps, minPts)
        out = dict(X=X, bits=r.bits(), R=r.R(), topK=r.topK(), topM=r.topM(), core=r.core())
        out["proj_head"] = r.projections()[: min(n, 64)]
        if optics:
            off, idx, dd = r.neighbor_dist()
            out.update(ordering=r.ordering_, reachability=r.reachability_, core_dist=r.core_dist(),
                       degree=np.diff(off).astype(np.int32))
        else:
            off, idx = r.neighbors()
            out.update(labels=r.labels_, n_clusters=np.int32(r.n_clusters_),
                       core_degree=np.diff(off).astype(np.int32))
        meta = dict(params, eps=eps, minPts=minPts, optics=optics, random_seed=7, n_threads=1)
        out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **out)
        print(name, "n_clusters" if not optics else "ordering", r.n_clusters_ if not optics else len(r.ordering_),
              "cores", int(out["core"].sum()))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
