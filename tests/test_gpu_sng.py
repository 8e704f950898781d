"""sngDbscan / sngOptics on the GPU (src/sDbscan.cpp:416-504, 1131-1304,
1484-1583, 1846-1923) through the C ABI and the drop-in module.

Parity bar: bit-exact.  sngDbscan with a seed >= 0 must give the reference's
labels, n_clusters_, core flags and core neighbourhood sizes (golden
fixtures made by the reference itself) and the oracle's neighbourhood sizes
for every point; sngOptics must give the oracle's ordering, reachability,
core flags, core distances and neighbourhood sizes under the same sampling
rule (per 32-point block by default, as the reference's per-point
std::random_device samples are independent; or one shared seeded sample).
"""
import glob
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SNG = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sng_*.npz")))


def _load(path):
    z = np.load(path)
    return z, json.loads(bytes(z["meta"]).decode())


def _sng_engine(X, distance, prob, seed):
    from sdbscan_gb300 import capi
    eng = capi.Engine(*X.shape)
    eng.set_sng_params(distance=distance, samplingProb=prob, random_seed=seed)
    return eng


@pytest.mark.parametrize("path", SNG, ids=[os.path.basename(p)[:-4] for p in SNG])
def test_fit_sngdbscan_matches_reference(path):
    z, meta = _load(path)
    X = z["X"]
    eng = _sng_engine(X, meta["distance"], meta["samplingProb"], meta["random_seed"])
    eng.fit_sngdbscan(X, meta["eps"], meta["minPts"])
    labels, ncl = eng.labels()
    core, deg = eng.core()
    np.testing.assert_array_equal(core, z["core"])
    np.testing.assert_array_equal(deg[core == 1], z["core_degree"][z["core"] == 1])
    np.testing.assert_array_equal(labels, z["labels"])
    assert ncl == int(z["n_clusters"])
    eng.close()


CASES = [
    # (name, distance, samplingProb, eps, minPts, seed)
    ("cosine_p002", "Cosine", 0.02, 0.15, 6, 1),
    ("cosine_p05_many_extra_draws", "Cosine", 0.5, 0.12, 40, 2),
    ("cosine_exact", "Cosine", 1.0, 0.1, 10, 3),
    ("l1_p01", "L1", 0.1, 2.0, 10, 4),
    ("l2_p01", "L2", 0.1, 0.5, 10, 5),
    ("chi2_p01", "Chi2", 0.1, 0.2, 10, 6),
    ("js_p01", "JS", 0.1, 0.2, 10, 7),
    ("cosine_p0_no_sample", "Cosine", 0.0, 0.2, 5, 8),
]


def _data(distance, n=2500):
    from sdbscan_gb300 import datasets
    if distance == "Cosine":
        return datasets.cfg1_cosine(n, 40, seed=61)[0]
    if distance in ("L1", "L2"):
        return datasets.cfg3_aniso_l2(n, 16, n_comp=5, scale=0.1, seed=62)[0]
    return datasets.cfg4_dirichlet(n, 64, n_comp=5, conc=10, seed=63)[0]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fit_sngdbscan_matches_oracle(port, case):
    _, distance, prob, eps, minPts, seed = case
    X = _data(distance)
    eng = _sng_engine(X, distance, prob, seed)
    eng.fit_sngdbscan(X, eps, minPts)
    labels, ncl = eng.labels()
    core, deg = eng.core()
    l2, n2, c2, d2, _ = port.fit_sngdbscan(X, eps, minPts, dist=distance, samplingProb=prob, seed=seed, threads=8)
    np.testing.assert_array_equal(deg, d2)
    np.testing.assert_array_equal(core, c2)
    np.testing.assert_array_equal(labels, l2)
    assert ncl == n2
    if prob == 0.0:
        assert np.all(labels == -1) and ncl == 2
    eng.close()


@pytest.mark.parametrize("prob,eps,minPts", [(0.05, 0.2, 20), (1.0, 0.15, 50), (0.3, 0.25, 100)])
def test_sngdbscan_bf16_screening_is_exact(port, prob, eps, minPts):
    """BF16 precision (Cosine): the block on the tensor cores, pairs within
    the margin re-decided in FP32 -- degrees, core flags and labels equal the
    oracle's, with pairs actually re-decided and no fallback.  MNIST-like data
    (thousands of pairs within 0.009 of eps; well-separated vMF clusters have
    none)."""
    from sdbscan_gb300 import capi, datasets
    X = datasets.cfg2_mnist_like(5000, 196, seed=13)[0]
    eng = _sng_engine(X, "Cosine", prob, 21)
    eng.set_precision(capi.PREC_BF16)
    eng.fit_sngdbscan(X, eps, minPts)
    labels, ncl = eng.labels()
    core, deg = eng.core()
    c = eng.counters()
    l2, n2, c2, d2, _ = port.fit_sngdbscan(X, eps, minPts, samplingProb=prob, seed=21, threads=8)
    np.testing.assert_array_equal(deg, d2)
    np.testing.assert_array_equal(core, c2)
    np.testing.assert_array_equal(labels, l2)
    assert ncl == n2
    assert c["rechecked"] > 0 and c["fallbacks"] == 0
    labels_sw, _ = eng.fit_sngdbscan_sweep(X, [eps, eps + 0.05], minPts)
    np.testing.assert_array_equal(labels_sw[0], l2)
    eng.close()


def test_sngdbscan_sweep_equals_separate_fits(port):
    """test_sngDbscan (src/sDbscan.cpp:1192-1240): one transform and sample,
    each eps's labels equal a separate fit (and the oracle's)."""
    X = _data("Cosine", 3000)
    eps = [0.2, 0.1, 0.15]
    eng = _sng_engine(X, "Cosine", 0.05, 11)
    labels, ncl = eng.fit_sngdbscan_sweep(X, eps, 8)
    for i, e in enumerate(eps):
        eng.fit_sngdbscan(X, e, 8)
        l1, n1 = eng.labels()
        np.testing.assert_array_equal(labels[i], l1)
        assert ncl[i] == n1
        lo, no, _, _, _ = port.fit_sngdbscan(X, e, 8, samplingProb=0.05, seed=11, threads=8)
        np.testing.assert_array_equal(labels[i], lo)
    eng.close()


OPTICS = [
    ("cosine_p01", "Cosine", 0.1, 0.2, 8, 1),
    ("l2_p02", "L2", 0.2, 0.6, 10, 2),
    ("chi2_p01", "Chi2", 0.1, 0.25, 6, 3),
    ("cosine_p15_more_draws_than_points", "Cosine", 1.5, 0.15, 12, 4),
]


@pytest.mark.parametrize("mode", ["blocks", "shared"])
@pytest.mark.parametrize("case", OPTICS, ids=[c[0] for c in OPTICS])
def test_fit_sngoptics_matches_oracle(port, case, mode):
    """sngOptics under both sampling rules: per 32-point block (the default:
    the reference samples every point independently) against the oracle's
    orc_fit_sngoptics_blocks, and one shared sample (sdb_set_sng_sampling 1)
    against orc_fit_sngoptics -- neighbourhood sizes, core flags, core
    distances, ordering and reachability bit for bit."""
    _, distance, prob, eps, minPts, seed = case
    X = _data(distance, 2000)
    eng = _sng_engine(X, distance, prob, seed)
    if mode == "shared":
        eng.set_sng_sampling(1)
    eng.fit_sngoptics(X, eps, minPts)
    ordering, reach = eng.optics()
    core, deg = eng.core()
    cd = eng.core_dist()
    if mode == "shared":
        o2, r2, c2, cd2, d2, _ = port.fit_sngoptics(X, eps, minPts, dist=distance, samplingProb=prob, seed=seed,
                                                    threads=8)
    else:
        o2, r2, c2, cd2, d2 = port.fit_sngoptics_blocks(X, eps, minPts, dist=distance, samplingProb=prob,
                                                        seed=seed, block_rows=32, threads=8)
    assert c2.sum() > 0
    np.testing.assert_array_equal(deg, d2)
    np.testing.assert_array_equal(core, c2)
    np.testing.assert_array_equal(cd, cd2)
    np.testing.assert_array_equal(ordering, o2)
    np.testing.assert_array_equal(reach, r2)
    eng.close()


def test_sng_single_point():
    """One point: sampled sngDbscan cannot draw another point (the reference's
    draw loop, src/sDbscan.cpp:449-465, never ends), so it is rejected; the
    exact mode and sngOptics (which skips self draws) give one noise point."""
    from sdbscan_gb300 import capi
    X = np.ones((1, 8), np.float32)
    eng = _sng_engine(X, "Cosine", 0.5, 3)
    with pytest.raises(capi.SdbError) as e:
        eng.fit_sngdbscan(X, 0.1, 2)
    assert e.value.status == 1
    eng.set_sng_params(distance="Cosine", samplingProb=1.0, random_seed=3)
    eng.fit_sngdbscan(X, 0.1, 2)
    labels, ncl = eng.labels()
    assert labels.tolist() == [-1] and ncl == 2
    eng.set_sng_params(distance="Cosine", samplingProb=0.5, random_seed=3)
    eng.fit_sngoptics(X, 0.1, 2)
    ordering, reach = eng.optics()
    assert ordering.tolist() == [0] and reach[0] == np.float32(-2147483648.0)
    eng.close()


def test_sng_state_and_argument_errors():
    from sdbscan_gb300 import capi
    X = _data("Cosine", 500)
    eng = capi.Engine(*X.shape)
    with pytest.raises(capi.SdbError) as e:
        eng.fit_sngdbscan(X, 0.1, 5)  # no set_sngParams yet
    assert e.value.status == 5
    eng.set_sng_params(distance="Cosine", samplingProb=0.1, random_seed=1)
    with pytest.raises(capi.SdbError) as e:
        eng.fit_sngoptics(X, 0.1, 1)  # nth_element at minPts - 2
    assert e.value.status == 1
    eng.fit_sngdbscan(X, 0.1, 5)
    with pytest.raises(capi.SdbError) as e:
        eng.topk()  # no index after an sng fit
    assert e.value.status == 5
    with pytest.raises(capi.SdbError) as e:
        eng.core_dist()
    assert e.value.status == 5
    eng.close()


def test_pybind_sng_dropin(tmp_path):
    """set_sngParams / fit_sngDbscan / test_sngDbscan / fit_sngOptics through
    the drop-in module (python/python_wrapper.cpp:26-27, :56-64): the C ABI's
    results, and one labels file per eps named as src/sDbscan.cpp:1232-1236."""
    from sdbscan_gb300 import capi
    from sdbscan_gb300 import sDbscan as mod
    z, meta = _load(os.path.join(os.path.dirname(__file__), "golden", "sng_cosine_2000x32.npz"))
    X = z["X"]
    dbs = mod.sDbscan(X.shape[0], X.shape[1])
    prefix = str(tmp_path / "sng")
    dbs.set_sngParams(distance="Cosine", samplingProb=meta["samplingProb"], random_seed=7, output=prefix)
    dbs.fit_sngDbscan(np.asfortranarray(X.T), meta["eps"], meta["minPts"])
    np.testing.assert_array_equal(np.asarray(dbs.labels_), z["labels"])
    assert dbs.n_clusters_ == int(z["n_clusters"])
    dbs.test_sngDbscan(np.asfortranarray(X.T), 0.1, 0.05, 2, meta["minPts"])
    eng = _sng_engine(X, "Cosine", meta["samplingProb"], 7)
    for i in range(2):
        e = np.float32(np.float64(np.float32(0.1)) + 1.0 * i * np.float64(np.float32(0.05)))
        eng.fit_sngdbscan(X, float(e), meta["minPts"])
        want, _ = eng.labels()
        f = f"{prefix}_Cosine_Eps_{int(round(1000 * float(e)))}_MinPts_{meta['minPts']}_Prob_50"
        np.testing.assert_array_equal(np.loadtxt(f, dtype=np.int32), want)
    dbs.fit_sngOptics(np.asfortranarray(X.T), 0.2, 10)
    eng.fit_sngoptics(X, 0.2, 10)
    o, r = eng.optics()
    np.testing.assert_array_equal(np.asarray(dbs.ordering_), o)
    np.testing.assert_array_equal(np.asarray(dbs.reachability_, dtype=np.float32), r)
    eng.close()


BLOCKS = [
    ("cosine_p05", "Cosine", 0.05, 0.2, 10, 7),
    ("l2_p10", "L2", 0.1, 0.6, 10, 8),
    ("chi2_p05", "Chi2", 0.05, 0.25, 6, 9),
    ("js_p02", "JS", 0.02, 0.3, 4, 10),
    ("cosine_p0", "Cosine", 0.0, 0.2, 5, 11),
]


@pytest.mark.parametrize("case", BLOCKS, ids=[c[0] for c in BLOCKS])
def test_fit_sngdbscan_blocks_matches_oracle(port, case):
    """Independent samples per 32-point block (sdb_set_sng_sampling 2, the
    rule of random_seed < 0): neighbourhood sizes with repeats, core flags,
    labels and n_clusters_ equal the oracle's restatement of the rule
    (orc_fit_sngdbscan_blocks) for the same seed, bit for bit."""
    _, distance, prob, eps, minPts, seed = case
    X = _data(distance, 3000)
    eng = _sng_engine(X, distance, prob, seed)
    eng.set_sng_sampling(2)
    eng.fit_sngdbscan(X, eps, minPts)
    labels, ncl = eng.labels()
    core, deg = eng.core()
    l2, n2, c2, d2 = port.fit_sngdbscan_blocks(X, eps, minPts, dist=distance, samplingProb=prob, seed=seed,
                                               block_rows=32, threads=8)
    np.testing.assert_array_equal(deg, d2)
    np.testing.assert_array_equal(core, c2)
    np.testing.assert_array_equal(labels, l2)
    assert ncl == n2
    if prob > 0:
        assert core.sum() > 0
    # sweeps: every eps equals a separate fit
    lab_sw, ncl_sw = eng.fit_sngdbscan_sweep(X, [eps, 0.8 * eps], minPts)
    np.testing.assert_array_equal(lab_sw[0], l2)
    l3, n3, _, _ = port.fit_sngdbscan_blocks(X, 0.8 * np.float32(eps), minPts, dist=distance, samplingProb=prob,
                                             seed=seed, block_rows=32, threads=8)
    np.testing.assert_array_equal(lab_sw[1], l3)
    eng.close()


def test_unseeded_sngdbscan_draws_per_block():
    """random_seed < 0 takes the block rule (independent samples, the
    reference's law for clock-seeded points): about S forward and S reverse
    draws per point, so the mean neighbourhood size (repeats counted) is
    about twice the forward passes -- far above one shared sample's, where
    only the sampled points get reverse draws."""
    from sdbscan_gb300 import capi, datasets
    X = datasets.cfg2_mnist_like(4000, 64, seed=12)[0]
    degs = {}
    for mode in (1, 0):
        eng = capi.Engine(*X.shape)
        eng.set_sng_params(distance="Cosine", samplingProb=0.05, random_seed=-1)
        eng.set_sng_sampling(mode)
        eng.fit_sngdbscan(X, 0.2, 10)
        degs[mode] = eng.core()
        eng.close()
    # same law of forward passes; the block rule adds the reverse ones for every point
    assert degs[0][0].sum() > 1.05 * degs[1][0].sum()
