"""The oracle restatement against the reference's own outputs.

The golden fixtures were produced by the reference itself (its unmodified
sources, one thread, seed 7; see tests/golden/make_golden.py).  Every stage of
the oracle must reproduce them bit for bit: sign bits, random Fourier matrix,
projections, top-k / top-m index matrices, core flags, neighbourhood sizes,
labels, n_clusters_, core distances, and - with the reference's neighbour-list
order (one thread) - the sOPTICS ordering and reachability.
"""
import glob
import json
import os

import numpy as np
import pytest

from oracle.oracle import fht_dim

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith("sng_"))  # sngDbscan fixtures: tests/test_sng*.py


def _load(path):
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_fixture(port, path):
    z, meta = _load(path)
    X = z["X"]
    n, d = X.shape
    dist = meta["distance"]
    ker = d if dist == "Cosine" else meta.get("ker_n_features", 1024)
    nproj, k, m = meta["n_proj"], meta["topK"], meta["topM"]
    fd = fht_dim(nproj, ker)
    bits = port.hd3_bits(3 * fd, meta["random_seed"])
    np.testing.assert_array_equal(bits, z["bits"])
    R = port._R(dist, ker, d, meta.get("ker_sigma", 1.0), meta["random_seed"])
    if R is not None:
        np.testing.assert_array_equal(R, z["R"])
    Xt, rc = port.transform(X, dist)
    assert rc == 0
    P = port.project(Xt, dist, ker, 0.4, R, bits, fd, nproj)
    np.testing.assert_array_equal(P[: z["proj_head"].shape[0]], z["proj_head"])
    topK = port.topk(P, k)
    topM = port.topm(P, m)
    np.testing.assert_array_equal(topK, z["topK"])
    np.testing.assert_array_equal(topM, z["topM"])
    port.L.orc_set_threads(1)
    core, deg, off, idx, dd = port.find_core(Xt, dist, topK, topM, meta["eps"], meta["minPts"],
                                             with_dist=True, ref_order=meta["optics"])
    port.L.orc_set_threads(0)
    np.testing.assert_array_equal(core, z["core"])
    if meta["optics"]:
        np.testing.assert_array_equal(deg, z["degree"])
        cd = port.core_dist(n, meta["minPts"], core)
        np.testing.assert_array_equal(cd, z["core_dist"])
        order, reach = port.form_optics(core, cd, off, idx, dd, tie_mode=0)
        np.testing.assert_array_equal(order, z["ordering"])
        np.testing.assert_array_equal(reach, z["reachability"])
        # the canonical tie order is a permutation with the same core set
        order1, reach1 = port.form_optics(core, cd, off, idx, dd, tie_mode=1)
        assert sorted(order1.tolist()) == list(range(n))
    else:
        np.testing.assert_array_equal(deg[core == 1], z["core_degree"][core == 1])
        labels, ncl = port.form_cluster(core, off, idx)
        if meta.get("clusterNoise", 0) == 1:  # sDbscan-1NN (samplingProb 1: every core point)
            labels = port.label_noise(P, topK, core, labels, meta["samplingProb"], meta["random_seed"])
        np.testing.assert_array_equal(labels, z["labels"])
        assert ncl == int(z["n_clusters"])
    port.graph_free()


def test_whole_fit_matches_reference_fixture(port):
    """orc_fit_sdbscan (the CPU baseline) reproduces a fixture end to end."""
    z, meta = _load(os.path.join(os.path.dirname(__file__), "golden", "cosine_vmf_2000x32.npz"))
    labels, ncl, core, _ = port.fit_sdbscan(z["X"], meta["eps"], meta["minPts"], n_proj=meta["n_proj"],
                                            topK=meta["topK"], topM=meta["topM"], seed=7, threads=4)
    np.testing.assert_array_equal(labels, z["labels"])
    np.testing.assert_array_equal(core, z["core"])
    assert ncl == int(z["n_clusters"])


def test_transform_rejects_like_reference(port):
    """Chi2/JS reject negative values and zero-sum columns (src/Utilities.h:308-324)."""
    X = np.abs(np.random.default_rng(0).standard_normal((10, 4))).astype(np.float32)
    assert port.transform(X, "Chi2")[1] == 0
    Xn = X.copy()
    Xn[3, 1] = -1e-3
    assert port.transform(Xn, "Chi2")[1] == 1
    Xz = X.copy()
    Xz[5] = 0
    assert port.transform(Xz, "JS")[1] == 2


def test_oracle_sweep_equals_separate_fits(port):
    """The index-once eps sweep (test_sDbscan, src/sDbscan.cpp:980-1039) gives
    each eps the labels of a separate fit_sDbscan."""
    from sdbscan_gb300 import datasets
    X, _ = datasets.cfg2_mnist_like(3000, 64, seed=3)
    eps = [0.15, 0.25, 0.35]
    labels, ncl, _ = port.fit_sdbscan_sweep(X, eps, 20, n_proj=256, topK=5, topM=30, seed=4)
    for i, e in enumerate(eps):
        l1, n1, _, _ = port.fit_sdbscan(X, e, 20, n_proj=256, topK=5, topM=30, seed=4)
        np.testing.assert_array_equal(labels[i], l1)
        assert ncl[i] == n1


@pytest.mark.parametrize("name", ["cosine_noise1nn_2000x32", "chi2_noise1nn_1500x64"])
def test_whole_fit_noise_labelling_matches_reference(port, name):
    """fit_sDbscan with clusterNoise = 1 (labelNoise, src/sDbscan.cpp:648-807):
    noise points take the labels the reference's sDbscan-1NN gives them."""
    z, meta = _load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    labels, ncl, core, _ = port.fit_sdbscan(z["X"], meta["eps"], meta["minPts"], dist=meta["distance"],
                                            n_proj=meta["n_proj"], topK=meta["topK"], topM=meta["topM"],
                                            ker=meta.get("ker_n_features", 1024), seed=7, threads=4,
                                            clusterNoise=1, samplingProb=meta["samplingProb"])
    np.testing.assert_array_equal(labels, z["labels"])
    assert ncl == int(z["n_clusters"])


def test_oracle_rejects_chi2_js_with_fewer_kernel_features_than_dimensions(port):
    """embedChi2 / embedJS fill n_features slots of a ker_n_features-long
    vector (src/Utilities.h:140-145); with ker_n_features < n_features the
    reference overruns it (undefined behaviour), so the oracle, like the
    engine, refuses those parameters; ker_n_features = n_features runs."""
    from sdbscan_gb300 import datasets as ds
    X = ds.cfg4_dirichlet(300, 130, n_comp=3, seed=2)[0]
    for dist in ("Chi2", "JS"):
        with pytest.raises(ValueError, match="ker_n_features"):
            port.fit_sdbscan(X, 0.3, 5, dist=dist, n_proj=64, topK=3, topM=10, ker=64, seed=1)
        with pytest.raises(ValueError, match="ker_n_features"):
            port.fit_soptics(X, 0.3, 5, dist=dist, n_proj=64, topK=3, topM=10, ker=64, seed=1)
        port.fit_sdbscan(X, 0.3, 5, dist=dist, n_proj=64, topK=3, topM=10, ker=130, seed=1)
