"""sngDbscan / sngOptics (src/sDbscan.cpp:416-504, 1131-1304, 1484-1583,
1846-1923): the oracle restatement against the reference's own outputs.

The sng fixtures were produced by the reference itself (seeded: every point's
generator gets random_seed 7, src/sDbscan.cpp:437-440; see
tests/golden/make_golden.py).  The oracle restates sng_findCorePoints point by
point and must reproduce labels, n_clusters_, core flags and the core points'
neighbourhood sizes (repeats counted) exactly.  sngOptics seeds each point
from std::random_device in the reference, so its restatement (the engine's
shared seeded sample) is checked for its own invariants here.  The
block-sampled rule (each block of consecutive points draws its own sample) is
checked against the reference's unreproducible runs in law: core counts.
"""
import glob
import json
import os

import numpy as np
import pytest

SNG = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sng_*.npz")))


def _load(path):
    z = np.load(path)
    return z, json.loads(bytes(z["meta"]).decode())


@pytest.mark.parametrize("path", SNG, ids=[os.path.basename(p)[:-4] for p in SNG])
def test_oracle_sngdbscan_matches_reference_fixture(port, path):
    z, meta = _load(path)
    labels, ncl, core, deg, _ = port.fit_sngdbscan(z["X"], meta["eps"], meta["minPts"], dist=meta["distance"],
                                                   samplingProb=meta["samplingProb"], seed=meta["random_seed"],
                                                   threads=4)
    np.testing.assert_array_equal(core, z["core"])
    np.testing.assert_array_equal(deg[core == 1], z["core_degree"][z["core"] == 1])
    assert np.all(z["core_degree"][z["core"] == 0] == 0)  # non-core lists are cleared (src/sDbscan.cpp:495)
    np.testing.assert_array_equal(labels, z["labels"])
    assert ncl == int(z["n_clusters"])


def test_fixtures_cover_sampled_exact_and_distances():
    metas = [_load(p)[1] for p in SNG]
    assert {m["distance"] for m in metas} >= {"Cosine", "L2", "Chi2"}
    assert any(m["samplingProb"] >= 1.0 for m in metas) and any(m["samplingProb"] < 1.0 for m in metas)
    for p in SNG:
        z, _ = _load(p)
        assert 0 < int(z["core"].sum()) < z["core"].shape[0]  # neither all noise nor all core


def test_oracle_sngoptics_invariants(port):
    """Ordering is a permutation; every core point's core distance is its
    (minPts-1)-th smallest neighbour distance, so it is <= eps; points never
    reached keep -2^31 (src/sDbscan.cpp:1590); the first point of the ordering
    is point 0."""
    from sdbscan_gb300 import datasets
    X, _ = datasets.cfg1_cosine(1500, 24, seed=5)
    eps, minPts = 0.2, 8
    o, r, c, cd, deg, _ = port.fit_sngoptics(X, eps, minPts, samplingProb=0.1, seed=3, threads=4)
    assert np.array_equal(np.sort(o), np.arange(1500)) and o[0] == 0
    assert np.all(c == (deg >= minPts - 1))
    assert np.all(cd[c == 1] <= eps) and np.all(cd[c == 1] >= 0) and np.all(cd[c == 0] == 0)
    reached = r != np.float32(-2147483648.0)
    assert reached.sum() > 0 and np.all(r[reached] >= 0)


def _mnist_like():
    from sdbscan_gb300 import datasets
    return datasets.cfg2_mnist_like(4000, 64, seed=41)[0]


def test_block_rule_is_deterministic_and_exact_mode_unchanged(port):
    """The block-sampled rule is a function of the seed; at samplingProb >= 1
    it is the reference's exact DBSCAN, the point-by-point oracle's result."""
    X = _mnist_like()[:1500]
    a = port.fit_sngdbscan_blocks(X, 0.2, 10, samplingProb=0.05, seed=9, block_rows=32, threads=4)
    b = port.fit_sngdbscan_blocks(X, 0.2, 10, samplingProb=0.05, seed=9, block_rows=32, threads=2)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    c = port.fit_sngdbscan_blocks(X, 0.2, 10, samplingProb=0.05, seed=10, block_rows=32, threads=4)
    assert not np.array_equal(a[3], c[3])
    e1 = port.fit_sngdbscan_blocks(X, 0.15, 10, samplingProb=1.0, seed=9, block_rows=32, threads=4)
    l2, n2, c2, d2, _ = port.fit_sngdbscan(X, 0.15, 10, samplingProb=1.0, seed=9, threads=4)
    np.testing.assert_array_equal(e1[0], l2)
    np.testing.assert_array_equal(e1[3], d2)
    o1 = port.fit_sngoptics_blocks(X, 0.2, 10, samplingProb=0.05, seed=9, block_rows=32, threads=4)
    o2 = port.fit_sngoptics_blocks(X, 0.2, 10, samplingProb=0.05, seed=9, block_rows=32, threads=1)
    for u, v in zip(o1, o2):
        np.testing.assert_array_equal(u, v)
    assert sorted(o1[0].tolist()) == list(range(X.shape[0]))


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "libsdbscan_ref.so")), reason="reference library not built here")
def test_block_rule_keeps_the_reference_statistics(port):
    """The reference's sngOptics (std::random_device per point) and its
    unseeded sngDbscan (a clock seed per point) sample independently per
    point.  Three runs of each against three seeds of the rules: the
    block-sampled rule (32-point blocks) finds the reference's number of core
    points within 2 %; one sample shared by all points finds at least 5 %
    fewer (the deviation the block rule removes)."""
    from oracle.oracle import Ref
    X = _mnist_like()
    n, d = X.shape
    eps, minPts, prob = 0.2, 10, 0.05

    def ref_cores(optics):
        out = []
        for _ in range(3):
            r = Ref(n, d)
            r.set_sngParams(distance="Cosine", samplingProb=prob, n_threads=4, random_seed=-1)
            (r.fit_sngOptics if optics else r.fit_sngDbscan)(X, eps, minPts)
            out.append(int(r.core().sum()))
        return float(np.mean(out))

    ref_o, ref_d = ref_cores(True), ref_cores(False)
    blk_o = np.mean([port.fit_sngoptics_blocks(X, eps, minPts, samplingProb=prob, seed=s, block_rows=32,
                                               threads=4)[2].sum() for s in range(3)])
    blk_d = np.mean([port.fit_sngdbscan_blocks(X, eps, minPts, samplingProb=prob, seed=s, block_rows=32,
                                               threads=4)[2].sum() for s in range(3)])
    shr_o = np.mean([port.fit_sngoptics(X, eps, minPts, samplingProb=prob, seed=s, threads=4)[2].sum()
                     for s in range(3)])
    shr_d = np.mean([port.fit_sngdbscan(X, eps, minPts, samplingProb=prob, seed=s, threads=4)[2].sum()
                     for s in range(3)])
    assert abs(blk_o - ref_o) < 0.02 * ref_o, (blk_o, ref_o)
    assert abs(blk_d - ref_d) < 0.02 * ref_d, (blk_d, ref_d)
    assert shr_o < 0.95 * ref_o and shr_d < 0.95 * ref_d, (shr_o, shr_d, ref_o, ref_d)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "libsdbscan_ref.so")), reason="reference library not built here")
@pytest.mark.parametrize("case", range(20))
def test_random_sngdbscan_configurations_match_reference(port, case):
    """Seeded random sngDbscan configurations (all distances, 2-900 points,
    samplingProb from 0.001 to 1.5, i.e. sampled and exact): labels,
    n_clusters_ and core flags equal the reference's, one thread."""
    from oracle.oracle import Ref
    from sdbscan_gb300 import datasets as ds
    rng = np.random.default_rng(5000 + case)
    dist = str(rng.choice(["Cosine", "L1", "L2", "Chi2", "JS"]))
    n, d = int(rng.integers(2, 900)), int(rng.choice([3, 8, 17, 32, 65]))
    prob = float(rng.choice([0.001, 0.01, 0.05, 0.3, 0.9, 1.0, 1.5]))
    minPts, seed = int(rng.integers(2, 20)), int(rng.integers(0, 1000))
    if dist == "Cosine":
        X, eps = ds.cfg1_cosine(n, d, seed=seed)[0], float(rng.uniform(0.02, 0.4))
    elif dist in ("L1", "L2"):
        X, eps = ds.cfg3_aniso_l2(n, d, n_comp=4, scale=0.1, seed=seed)[0], float(rng.uniform(0.2, 3.0))
    else:
        X, eps = ds.cfg4_dirichlet(n, d, n_comp=4, conc=10, seed=seed)[0], float(rng.uniform(0.05, 0.5))
    r = Ref(n, d)
    r.set_sngParams(distance=dist, samplingProb=prob, n_threads=1, random_seed=seed)
    r.fit_sngDbscan(X, eps, minPts)
    labels, ncl, core, _, _ = port.fit_sngdbscan(X, eps, minPts, dist=dist, samplingProb=prob, seed=seed, threads=1)
    np.testing.assert_array_equal(core, r.core())
    np.testing.assert_array_equal(labels, r.labels_)
    assert ncl == r.n_clusters_
