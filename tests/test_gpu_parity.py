"""GPU engine against the reference (golden fixtures) and the oracle, through
the C ABI.

Bar: bit-exact core flags, labels, n_clusters_, top-k / top-m index matrices
(except where a boundary tie is counted), bit-exact projections for the
Cosine and Chi2 paths.  The L1/L2 random-Fourier and JS paths use CUDA's
cosf/sinf/logf, which may differ from glibc's in the last place: projections
there are held to a relative tolerance of 1e-5 of the vector norm and the
clustering to agreement on >= 99.5% of points.
"""
import glob
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith("sng_"))  # sngDbscan fixtures: tests/test_sng*.py
EXACT_DISTS = ("Cosine", "Chi2")


def _fixture(path):
    z = np.load(path)
    return z, json.loads(bytes(z["meta"]).decode())


def _engine(X, meta):
    from sdbscan_gb300 import capi
    eng = capi.Engine(*X.shape)
    kw = dict(n_proj=meta["n_proj"], topK=meta["topK"], topM=meta["topM"], distance=meta["distance"],
              random_seed=meta["random_seed"])
    if "ker_n_features" in meta:
        kw["ker_n_features"] = meta["ker_n_features"]
    if "ker_sigma" in meta:
        kw["ker_sigma"] = meta["ker_sigma"]
    for key in ("clusterNoise", "samplingProb"):
        if key in meta:
            kw[key] = meta[key]
    eng.set_params(**kw)
    return eng


def _rows_equal_as_sets(a, b):
    return all(set(x) == set(y) for x, y in zip(a.tolist(), b.tolist()))


DBSCAN_FIXTURES = [p for p in GOLDEN if not _fixture(p)[1]["optics"]]


def _oracle_canonical(port, X, meta):
    """The oracle's fit of a fixture with the engine's tie rule at the top-k /
    top-m boundaries (smallest index kept): top-k, top-m, core flags,
    neighbourhood sizes, labels (with sDbscan-1NN when the fixture asks for
    it) and n_clusters_."""
    from oracle.oracle import fht_dim
    n, d = X.shape
    dist = meta["distance"]
    ker = d if dist == "Cosine" else meta.get("ker_n_features", 1024)
    fd = fht_dim(meta["n_proj"], ker)
    bits = port.hd3_bits(3 * fd, meta["random_seed"])
    R = port._R(dist, ker, d, meta.get("ker_sigma", 1.0), meta["random_seed"])
    Xt, rc = port.transform(X, dist)
    assert rc == 0
    P = port.project(Xt, dist, ker, 0.4, R, bits, fd, meta["n_proj"])
    tK, tM = port.topk_canon(P, meta["topK"]), port.topm_canon(P, meta["topM"])
    core, deg, labels, ncl = port.core_cluster_lean(Xt, dist, tK, tM, meta["eps"], meta["minPts"])
    if meta.get("clusterNoise", 0) == 1:
        labels = port.label_noise(P, tK, core, labels, meta.get("samplingProb", 0.01), meta["random_seed"])
    return tK, tM, core, deg, labels, ncl


def _sorted_rows(a):
    return np.sort(np.asarray(a), axis=1)


@pytest.mark.parametrize("path", DBSCAN_FIXTURES, ids=[os.path.basename(p)[:-4] for p in DBSCAN_FIXTURES])
def test_fit_sdbscan_matches_reference(port, path):
    z, meta = _fixture(path)
    X = z["X"]
    eng = _engine(X, meta)
    eng.fit_sdbscan(X, meta["eps"], meta["minPts"])
    labels, ncl = eng.labels()
    core, deg = eng.core()
    topK, topM = eng.topk(), eng.topm()
    P = eng.projections()[: z["proj_head"].shape[0]]
    c = eng.counters()
    exact = meta["distance"] in EXACT_DISTS
    if meta["distance"] == "Chi2" and meta.get("ker_n_features", 1024) // X.shape[1] >= 3:
        exact = False  # cos/sin/log components of the Chi2 embedding
    if exact:
        np.testing.assert_array_equal(P, z["proj_head"])
    else:
        scale = np.linalg.norm(z["proj_head"], axis=1, keepdims=True)
        assert np.max(np.abs(P - z["proj_head"]) / scale) < 1e-5
    # Index sets must match; inside a row, points with equal projection values
    # may come in a different order (the reference's heap order), which no
    # later stage depends on.
    if exact and c["topk_ties"] == 0:
        assert _rows_equal_as_sets(topK, z["topK"])
    if exact and c["topm_ties"] == 0:
        assert _rows_equal_as_sets(topM, z["topM"])
    if exact:
        # bit-exact against the oracle with the engine's tie rule, ties or not
        oK, oM, ocore, odeg, olabels, oncl = _oracle_canonical(port, X, meta)
        np.testing.assert_array_equal(_sorted_rows(topK), _sorted_rows(oK))
        np.testing.assert_array_equal(_sorted_rows(topM), _sorted_rows(oM))
        np.testing.assert_array_equal(core, ocore)
        np.testing.assert_array_equal(deg, odeg)
        np.testing.assert_array_equal(labels, olabels)
        assert ncl == oncl
    if exact and c["topk_ties"] == 0 and c["topm_ties"] == 0:
        np.testing.assert_array_equal(core, z["core"])
        np.testing.assert_array_equal(deg[core == 1], z["core_degree"][core == 1])
        np.testing.assert_array_equal(labels, z["labels"])
        assert ncl == int(z["n_clusters"])
    else:
        from tests._metrics import adjusted_rand_score
        agree = np.mean(core == z["core"])
        assert agree >= 0.995, agree
        assert adjusted_rand_score(z["labels"], labels) >= 0.99


@pytest.mark.parametrize("n,d,nproj,k,m,eps,minPts", [
    (20000, 128, 1024, 5, 50, 0.15, 20),
    (12000, 784, 1024, 10, 50, 0.25, 50),
    (9000, 100, 512, 7, 70, 0.2, 15),
])
def test_fit_sdbscan_matches_oracle(port, n, d, nproj, k, m, eps, minPts):
    from sdbscan_gb300 import capi, datasets
    if d == 784:
        X, _ = datasets.cfg2_mnist_like(n, d, seed=31)
    else:
        X, _ = datasets.cfg1_cosine(n, d, seed=32)
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=nproj, topK=k, topM=m, distance="Cosine", random_seed=11)
    eng.fit_sdbscan(X, eps, minPts)
    labels, ncl = eng.labels()
    core, deg = eng.core()
    Xt, _ = port.transform(X, "Cosine")
    from oracle.oracle import fht_dim
    fd = fht_dim(nproj, d)
    bits = port.hd3_bits(3 * fd, 11)
    P = port.project(Xt, "Cosine", d, 0.4, None, bits, fd, nproj)
    np.testing.assert_array_equal(eng.projections(), P)
    tK, tM = port.topk(P, k), port.topm(P, m)
    c = eng.counters()
    if c["topk_ties"] == 0:
        assert _rows_equal_as_sets(eng.topk(), tK)
    if c["topm_ties"] == 0:
        assert _rows_equal_as_sets(eng.topm(), tM)
    ocore, odeg, off, idx, _ = port.find_core(Xt, "Cosine", tK, tM, eps, minPts, with_dist=False)
    np.testing.assert_array_equal(deg, odeg)
    np.testing.assert_array_equal(core, ocore)
    olabels, oncl = port.form_cluster(ocore, off, idx)
    port.graph_free()
    np.testing.assert_array_equal(labels, olabels)
    assert ncl == oncl


def test_repeat_fits_are_identical():
    from sdbscan_gb300 import capi, datasets
    X, _ = datasets.cfg1_cosine(30000, 64, seed=41)
    eng = capi.Engine(*X.shape)
    eng.set_params(n_proj=1024, topK=5, topM=50, distance="Cosine", random_seed=3)
    eng.fit_sdbscan(X, 0.15, 20)
    a = eng.labels()
    eng.fit_sdbscan(X, 0.15, 20)
    b = eng.labels()
    np.testing.assert_array_equal(a[0], b[0])
    assert a[1] == b[1]


def test_errors_follow_reference_checks():
    from sdbscan_gb300 import capi
    rng = np.random.default_rng(5)
    X = np.abs(rng.standard_normal((500, 16))).astype(np.float32)
    eng = capi.Engine(*X.shape)
    eng.set_params(n_proj=64, topK=3, topM=10, distance="Chi2", ker_n_features=64, random_seed=1)
    eng.fit_sdbscan(X, 0.3, 5)
    Xn = X.copy()
    Xn[7, 3] = -0.5
    with pytest.raises(capi.SdbError) as e:
        eng.fit_sdbscan(Xn, 0.3, 5)
    assert e.value.status == 3  # SDB_ERR_NEGATIVE (src/Utilities.h:308-312)
    Xz = X.copy()
    Xz[9] = 0
    with pytest.raises(capi.SdbError) as e:
        eng.fit_sdbscan(Xz, 0.3, 5)
    assert e.value.status == 4  # SDB_ERR_ZERO_POINT (:318-325)
    with pytest.raises(capi.SdbError):
        eng.labels() if False else eng.set_params(n_proj=64, topK=3, topM=600, distance="Cosine")
    eng2 = capi.Engine(*X.shape)
    with pytest.raises(capi.SdbError) as e:
        eng2.labels()
    assert e.value.status == 5  # SDB_ERR_STATE
    with pytest.raises(capi.SdbError) as e:  # embedChi2 fills n_features slots of ker_n_features
        eng2.set_params(n_proj=64, topK=3, topM=10, distance="Chi2", ker_n_features=8)
    assert e.value.status == 1  # SDB_ERR_ARG


def test_pybind_dropin_matches_capi():
    """The drop-in module (reference names, X as (d, n)) gives the C ABI's result."""
    from sdbscan_gb300 import capi, datasets
    from sdbscan_gb300 import sDbscan as mod
    X, _ = datasets.cfg1_cosine(5000, 32, seed=51)
    dbs = mod.sDbscan(X.shape[0], X.shape[1])
    dbs.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", random_seed=9)
    dbs.fit_sDbscan(np.asfortranarray(X.T), 0.15, 10)
    eng = capi.Engine(*X.shape)
    eng.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", random_seed=9)
    eng.fit_sdbscan(X, 0.15, 10)
    labels, ncl = eng.labels()
    np.testing.assert_array_equal(np.asarray(dbs.labels_), labels)
    assert dbs.n_clusters_ == ncl


def test_load_fit_from_text_matches_in_memory_fit(tmp_path):
    """load_fit_sDbscan / load_fit_sOptics (src/sDbscan.cpp:903-966,
    :1777-1837): the data read from a text file (one point per line) gives the
    in-memory fits' results."""
    from sdbscan_gb300 import datasets
    from sdbscan_gb300 import sDbscan as mod
    X, _ = datasets.cfg1_cosine(3000, 24, seed=52)
    path = tmp_path / "points.txt"
    np.savetxt(path, X, fmt="%.9g")
    Xr = np.loadtxt(path, dtype=np.float64).astype(np.float32)  # the values the file holds
    a = mod.sDbscan(X.shape[0], X.shape[1])
    a.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", random_seed=9)
    a.load_fit_sDbscan(str(path), 0.15, 10)
    b = mod.sDbscan(X.shape[0], X.shape[1])
    b.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", random_seed=9)
    b.fit_sDbscan(np.asfortranarray(Xr.T), 0.15, 10)
    np.testing.assert_array_equal(np.asarray(a.labels_), np.asarray(b.labels_))
    a.load_fit_sOptics(str(path), 0.2, 10)
    b.fit_sOptics(np.asfortranarray(Xr.T), 0.2, 10)
    np.testing.assert_array_equal(np.asarray(a.ordering_), np.asarray(b.ordering_))
    np.testing.assert_array_equal(np.asarray(a.reachability_), np.asarray(b.reachability_))


def test_test_sdbscan_writes_each_eps(tmp_path):
    """test_sDbscan (src/sDbscan.cpp:980-1039) through the drop-in module: one
    labels file per eps + i rangeEps, each equal to a separate fit at that eps,
    and labels_ holding the last."""
    from sdbscan_gb300 import datasets
    from sdbscan_gb300 import sDbscan as mod
    X, _ = datasets.cfg1_cosine(4000, 32, seed=53)
    prefix = str(tmp_path / "run")
    a = mod.sDbscan(X.shape[0], X.shape[1])
    a.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", random_seed=9, output=prefix)
    a.test_sDbscan(np.asfortranarray(X.T), 0.1, 0.05, 3, 10)
    b = mod.sDbscan(X.shape[0], X.shape[1])
    b.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", random_seed=9)
    for i in range(3):
        e = np.float32(np.float64(np.float32(0.1)) + 1.0 * i * np.float64(np.float32(0.05)))  # the module's float math
        b.fit_sDbscan(np.asfortranarray(X.T), float(e), 10)
        f = f"{prefix}_Cosine_Eps_{int(round(1000 * float(e)))}_MinPts_10_KerFeatures_32_NumProj_256_TopM_20_TopK_5"
        np.testing.assert_array_equal(np.loadtxt(f, dtype=np.int32), np.asarray(b.labels_))
    np.testing.assert_array_equal(np.asarray(a.labels_), np.asarray(b.labels_))
    assert a.n_clusters_ == b.n_clusters_


OPTICS_FIXTURES = [p for p in GOLDEN if _fixture(p)[1]["optics"]]


@pytest.mark.parametrize("path", OPTICS_FIXTURES, ids=[os.path.basename(p)[:-4] for p in OPTICS_FIXTURES])
def test_fit_soptics_matches_reference(port, path):
    """Core flags, neighbourhood sizes and core distances equal the
    reference's; the ordering equals the oracle's with the canonical tie order
    (reachability, then point id), and reachability agrees with it exactly."""
    z, meta = _fixture(path)
    X = z["X"]
    eng = _engine(X, meta)
    eng.fit_soptics(X, meta["eps"], meta["minPts"])
    order, reach = eng.optics()
    core, deg = eng.core()
    cd = eng.core_dist()
    exact = meta["distance"] == "Cosine" or meta.get("ker_n_features", 1024) // X.shape[1] < 3
    if exact:
        np.testing.assert_array_equal(core, z["core"])
        np.testing.assert_array_equal(deg, z["degree"])
        np.testing.assert_array_equal(cd, z["core_dist"])
    assert sorted(order.tolist()) == list(range(X.shape[0]))
    # canonical ordering from the oracle on the same data and parameters
    from oracle.oracle import fht_dim
    dist = meta["distance"]
    ker = X.shape[1] if dist == "Cosine" else meta.get("ker_n_features", 1024)
    o_order, o_reach, o_core, o_cd, _ = port.fit_soptics(X, meta["eps"], meta["minPts"], dist=dist,
                                                         n_proj=meta["n_proj"], topK=meta["topK"],
                                                         topM=meta["topM"], ker=ker, seed=meta["random_seed"],
                                                         threads=4, tie_mode=1)
    if exact:
        np.testing.assert_array_equal(order, o_order)
        np.testing.assert_array_equal(reach, o_reach)


@pytest.mark.parametrize("n,d,k,m,eps,minPts", [(8000, 64, 5, 30, 0.2, 10), (6000, 196, 10, 50, 0.25, 30),
                                                (5000, 30, 5, 20, 0.02, 10)])  # d % 4 != 0
def test_fit_soptics_matches_oracle(port, n, d, k, m, eps, minPts):
    from sdbscan_gb300 import capi, datasets
    if d == 196:
        X, _ = datasets.cfg2_mnist_like(n, d, seed=61)
    else:
        X, _ = datasets.cfg1_cosine(n, d, seed=62)
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=512, topK=k, topM=m, distance="Cosine", random_seed=13)
    eng.fit_soptics(X, eps, minPts)
    order, reach = eng.optics()
    core, deg = eng.core()
    o_order, o_reach, o_core, o_cd, _ = port.fit_soptics(X, eps, minPts, n_proj=512, topK=k, topM=m, seed=13,
                                                         threads=4, tie_mode=1)
    np.testing.assert_array_equal(core, o_core)
    np.testing.assert_array_equal(eng.core_dist(), o_cd)
    np.testing.assert_array_equal(order, o_order)
    np.testing.assert_array_equal(reach, o_reach)


@pytest.mark.parametrize("gen,n,d,k,m,eps,minPts", [
    ("vmf", 3000, 64, 5, 20, 0.15, 10),
    ("vmf", 30000, 128, 5, 50, 0.15, 20),
    ("mnist", 20000, 784, 10, 50, 0.25, 50),
    ("vmf", 6000, 30, 5, 20, 0.02, 10),     # d % 4 != 0: rows staged element-wise, BF16 rows end mid-chunk
    ("mnist", 8000, 100, 8, 40, 0.25, 20),  # d % 8 == 4: the BF16 row's last 8-value store is partly padding
    ("mnist", 8000, 196, 6, 100, 0.25, 20),  # topM 100: two 64-column candidate tiles per list
    ("vmf", 5000, 64, 31, 70, 0.15, 10),     # topK 31 (62 slots per point) with two candidate tiles
])
def test_bf16_screening_equals_plain(gen, n, d, k, m, eps, minPts):
    """BF16 tensor-core screening with FP32 re-decision near eps gives the
    plain FP32 path's eps decisions, hence identical core flags,
    neighbourhood sizes, labels and n_clusters_."""
    from sdbscan_gb300 import capi, datasets
    if gen == "mnist":
        X, _ = datasets.cfg2_mnist_like(n, d, seed=71)
    else:
        X, _ = datasets.cfg1_cosine(n, d, seed=72)
    res = {}
    for prec in (capi.PREC_FP32, capi.PREC_BF16):
        eng = capi.Engine(n, d)
        eng.set_params(n_proj=1024, topK=k, topM=m, distance="Cosine", random_seed=17, precision=prec)
        eng.fit_sdbscan(X, eps, minPts)
        res[prec] = (eng.labels(), eng.core(), eng.counters())
    (l32, c32, k32), (l16, c16, k16) = res[capi.PREC_FP32], res[capi.PREC_BF16]
    assert k16["fallbacks"] == 0
    if gen == "mnist":  # distances spread across eps there, so some pairs are re-decided
        assert k16["rechecked"] > 0
    assert k16["pairs"] == k32["pairs"]
    np.testing.assert_array_equal(c16[0], c32[0])
    np.testing.assert_array_equal(c16[1], c32[1])
    np.testing.assert_array_equal(l16[0], l32[0])
    assert l16[1] == l32[1]


@pytest.mark.parametrize("n,d,ker,sigma,eps", [(12000, 32, 256, 1.5, 0.55), (16000, 192, 512, 6.0, 1.72)])
def test_bf16_l2_screening_is_exact_on_its_candidates(port, n, d, ker, sigma, eps):
    """L2 in BF16 mode: the split-BF16 tensor-core screening with exact FP32
    re-decision inside the per-pair band gives, on the fit's own candidate
    sets (its top-k / top-m, which the BF16 embedding GEMM shapes), exactly
    the oracle's neighbourhood sizes, core flags and labels."""
    from sdbscan_gb300 import capi, datasets
    X = datasets.cfg3_aniso_l2(n, d, n_comp=8, scale=0.1, seed=97)[0]
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=512, topK=5, topM=40, distance="L2", ker_n_features=ker, ker_sigma=sigma, random_seed=4,
                   precision=capi.PREC_BF16)
    eng.fit_sdbscan(X, eps, 10)
    c = eng.counters()
    assert c["fallbacks"] == 0
    assert c["rechecked"] > 0  # pairs fell inside the band and were re-decided
    tK, tM = eng.topk(), eng.topm()
    Xt, rc = port.transform(X, "L2")
    assert rc == 0
    ocore, odeg, olabels, oncl = port.core_cluster_lean(Xt, "L2", tK, tM, eps, 10)
    core, deg = eng.core()
    labels, ncl = eng.labels()
    np.testing.assert_array_equal(deg, odeg)
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(labels, olabels)
    assert ncl == oncl
    assert 0 < ocore.sum() < n


def _ragged_case(dist, d, seed):
    """Data, kernel width sigma and an eps for the ragged-dimension L1 / L2
    cases: sigma = the median pairwise distance of 200 points, eps = the
    median distance to the 20th nearest of 200 sampled points."""
    from sdbscan_gb300 import datasets
    X = datasets.cfg3_aniso_l2(6000, d, n_comp=8, scale=0.1, seed=seed)[0]
    S = X[:200].astype(np.float64)
    diff = S[:, None, :] - X[None, :, :].astype(np.float64)
    D = np.abs(diff).sum(-1) if dist == "L1" else np.sqrt((diff ** 2).sum(-1))
    sigma = float(np.median(D[:, :200][np.triu_indices(200, 1)]))
    eps = float(np.median(np.sort(D, axis=1)[:, 20]))
    return X, sigma, eps


@pytest.mark.parametrize("dist,d,nproj,ker", [("L2", 30, 512, 256), ("L1", 19, 256, 256), ("L2", 17, 1024, 1024)])
def test_rff_ragged_dims(port, dist, d, nproj, ker):
    """L1 / L2 with d not a multiple of 4: the transformed rows are padded to
    a multiple of 4 and the projection kernel stages them through shared
    memory, the last d % 4 elements included.  Projections agree with the
    oracle's to 1e-5 of the row norm (CUDA's cosf / sinf), and on the fit's
    own top-k / top-m the neighbourhood sizes, core flags, labels and
    n_clusters_ equal the oracle's bit for bit."""
    from oracle.oracle import fht_dim
    from sdbscan_gb300 import capi
    X, sigma, eps = _ragged_case(dist, d, seed=61 + d)
    n = X.shape[0]
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=nproj, topK=5, topM=40, distance=dist, ker_n_features=ker, ker_sigma=sigma,
                   random_seed=8)
    eng.fit_sdbscan(X, eps, 10)
    tK, tM = eng.topk(), eng.topm()
    core, deg = eng.core()
    labels, ncl = eng.labels()
    P = eng.projections()
    eng.close()
    Xt, rc = port.transform(X, dist)
    assert rc == 0
    fd = fht_dim(nproj, ker)
    oP = port.project(Xt, dist, ker, 0.4, port._R(dist, ker, d, sigma, 8), port.hd3_bits(3 * fd, 8), fd, nproj)
    scale = np.linalg.norm(oP, axis=1, keepdims=True)
    assert np.max(np.abs(P - oP) / scale) < 1e-5
    ocore, odeg, olabels, oncl = port.core_cluster_lean(Xt, dist, tK, tM, eps, 10)
    np.testing.assert_array_equal(deg, odeg)
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(labels, olabels)
    assert ncl == oncl
    assert 0 < ocore.sum() < n


def _maxima_case(dist, n, d, seed):
    """Data and eps for the engine-maxima cases: eps = the median distance to
    the 15th nearest of 100 sampled points, on the transformed rows."""
    from sdbscan_gb300 import datasets
    if dist == "Chi2":
        X = datasets.cfg2_mnist_like(n, d, n_comp=6, seed=seed)[0]
        T = X / X.sum(1, keepdims=True)
        S = T[:100].astype(np.float64)
        D = np.empty((100, n))
        for i in range(100):
            a, b = S[i][None, :], T.astype(np.float64)
            both = (a > 0) & (b > 0)
            D[i] = 1.0 - 2.0 * np.where(both, a * b / np.where(both, a + b, 1.0), 0.0).sum(1)
    else:
        X = (datasets.cfg2_mnist_like(n, d, n_comp=6, seed=seed)[0] if d > 256
             else datasets.cfg1_cosine(n, d, seed=seed)[0])
        T = X / np.linalg.norm(X, axis=1, keepdims=True)
        D = 1.0 - T[:100].astype(np.float64) @ T.astype(np.float64).T
    return X, float(np.median(np.sort(D, axis=1)[:, 15]))


@pytest.mark.parametrize("dist,n,d,nproj,ker,k,m", [
    ("Cosine", 3000, 1500, 256, None, 5, 20),   # 2048-point rotations from d: the register kernel's widest form
    ("Cosine", 4000, 64, 2048, None, 31, 100),  # n_proj 2048 and topK 31 (the engine's maxima), two mask words
    ("Chi2", 2000, 1024, 256, 2048, 5, 20),     # 2048-point rotations from the Chi2 embedding (square roots only)
])
def test_engine_maxima_match_oracle(port, dist, n, d, nproj, ker, k, m):
    """The widest register projection kernel (2048-element rotation vectors,
    64 per lane), the largest n_proj and topK, and top-m lists over two mask
    words: projections bit-exact against the oracle, top-k / top-m sets equal
    to the oracle's under the engine's tie rule, and neighbourhood sizes, core
    flags, labels and n_clusters_ bit-exact."""
    from oracle.oracle import fht_dim
    from sdbscan_gb300 import capi
    X, eps = _maxima_case(dist, n, d, seed=nproj + d)
    kw = dict(ker_n_features=ker) if ker else {}
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=nproj, topK=k, topM=m, distance=dist, random_seed=13, **kw)
    eng.fit_sdbscan(X, eps, 10)
    P, tK, tM = eng.projections(), eng.topk(), eng.topm()
    core, deg = eng.core()
    labels, ncl = eng.labels()
    eng.close()
    Xt, rc = port.transform(X, dist)
    assert rc == 0
    kk = ker or d
    fd = fht_dim(nproj, kk)
    assert fd == 2048
    oP = port.project(Xt, dist, kk, 0.4, None, port.hd3_bits(3 * fd, 13), fd, nproj)
    np.testing.assert_array_equal(P, oP)
    oK, oM = port.topk_canon(oP, k), port.topm_canon(oP, m)
    np.testing.assert_array_equal(_sorted_rows(tK), _sorted_rows(oK))
    np.testing.assert_array_equal(_sorted_rows(tM), _sorted_rows(oM))
    ocore, odeg, olabels, oncl = port.core_cluster_lean(Xt, dist, oK, oM, eps, 10)
    np.testing.assert_array_equal(deg, odeg)
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(labels, olabels)
    assert ncl == oncl
    assert 0 < ocore.sum() < n


@pytest.mark.parametrize("dist,d", [("Chi2", 30), ("Chi2", 61), ("Cosine", 30), ("Cosine", 45)])
def test_ragged_dims_bit_exact(port, dist, d):
    """Cosine and Chi2 with d not a multiple of 4: rows staged element by
    element, Xt written from the staged row with its padding zeroed, and for
    Chi2 the embedding's row buffer padded to a multiple of 4, with
    ker_n_features = the next multiple of 32 (square-root terms only).
    Projections bit-exact, top-k / top-m sets equal to the oracle's under the
    engine's tie rule, sizes, core flags, labels and n_clusters_ bit-exact."""
    from oracle.oracle import fht_dim
    from sdbscan_gb300 import capi, datasets
    n, nproj, k, m = 5000, 256, 5, 20
    ker = (d + 31) // 32 * 32 if dist == "Chi2" else d
    X = datasets.cfg2_mnist_like(n, d, n_comp=6, seed=90 + d)[0]
    Xt, rc = port.transform(X, dist)
    assert rc == 0
    fd = fht_dim(nproj, ker)
    oP = port.project(Xt, dist, ker, 0.4, None, port.hd3_bits(3 * fd, 21), fd, nproj)
    oK, oM = port.topk_canon(oP, k), port.topm_canon(oP, m)
    # eps: the median distance to the 15th nearest of 100 sampled points
    S, T = Xt[:100].astype(np.float64), Xt.astype(np.float64)
    if dist == "Chi2":
        D = np.empty((100, n))
        for i in range(100):
            a, b = S[i][None, :], T
            both = (a > 0) & (b > 0)
            D[i] = 1.0 - 2.0 * np.where(both, a * b / np.where(both, a + b, 1.0), 0.0).sum(1)
    else:
        D = 1.0 - S @ T.T
    eps = float(np.median(np.sort(D, axis=1)[:, 15]))
    eng = capi.Engine(n, d)
    kw = dict(ker_n_features=ker) if dist == "Chi2" else {}
    eng.set_params(n_proj=nproj, topK=k, topM=m, distance=dist, random_seed=21, **kw)
    eng.fit_sdbscan(X, eps, 10)
    np.testing.assert_array_equal(eng.projections(), oP)
    np.testing.assert_array_equal(_sorted_rows(eng.topk()), _sorted_rows(oK))
    np.testing.assert_array_equal(_sorted_rows(eng.topm()), _sorted_rows(oM))
    core, deg = eng.core()
    labels, ncl = eng.labels()
    eng.close()
    ocore, odeg, olabels, oncl = port.core_cluster_lean(Xt, dist, oK, oM, eps, 10)
    np.testing.assert_array_equal(deg, odeg)
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(labels, olabels)
    assert ncl == oncl
    assert 0 < ocore.sum() < n


@pytest.mark.parametrize("precision", [0, 1])
def test_eps_sweep_equals_separate_fits(precision):
    """test_sDbscan's pattern (index and distances once, then per eps) gives
    the labels of separate plain fit_sDbscan calls at each eps, also when the
    sweep's distances are BF16-screened (exact re-decision near every eps)."""
    from sdbscan_gb300 import capi, datasets
    X, _ = datasets.cfg2_mnist_like(8000, 196, seed=81)
    eps_list = [0.25, 0.15, 0.3, 0.2, 0.25]  # unsorted, with a repeat: rounds run in ascending eps
    eng = capi.Engine(*X.shape)
    eng.set_params(n_proj=512, topK=8, topM=40, distance="Cosine", random_seed=19, precision=precision)
    labels, ncl = eng.fit_sdbscan_sweep(X, eps_list, 20)
    if precision:
        assert eng.counters()["rechecked"] > 0 and eng.counters()["fallbacks"] == 0
    eng.set_params(n_proj=512, topK=8, topM=40, distance="Cosine", random_seed=19)
    for i, e in enumerate(eps_list):
        eng.fit_sdbscan(X, e, 20)
        l1, n1 = eng.labels()
        np.testing.assert_array_equal(labels[i], l1)
        assert ncl[i] == n1


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_graph_equals_sweeps(precision):
    """The CUDA-graph batch gives, for every set and eps, the plain sweep's
    labels, with plain or BF16-screened distances."""
    import torch
    from sdbscan_gb300 import capi, datasets
    sets = datasets.cfg5_batch_torch(n_sets=5, seed=91, n_lo=2000, n_hi=12000)
    eps_list = [0.05, 0.1, 0.2, 0.3]
    ptrs = [(X.data_ptr(), X.shape[0], X.shape[1]) for X, _ in sets]
    b = capi.Batch(ptrs, eps_list, 20, n_proj=1024, topK=5, topM=50, distance="Cosine", random_seed=23,
                   precision=precision)
    b.run()
    b.run()
    for i, (X, _) in enumerate(sets):
        eng = capi.Engine(*X.shape)
        eng.set_params(n_proj=1024, topK=5, topM=50, distance="Cosine", random_seed=23)
        labels, ncl = eng.fit_sdbscan_sweep(X.cpu().numpy(), eps_list, 20)
        for j in range(len(eps_list)):
            lb, nb = b.labels(i, j)
            np.testing.assert_array_equal(lb, labels[j])
            assert nb == ncl[j]
    assert b.lanes() >= 1
    # the autotuner picked a plain tile shape per set, or (BF16) the tensor-core screening (0)
    assert all(v in ((1, 2, 3) if precision == 0 else (0, 1, 2, 3)) for v in b.tile_variants())
    b.close()
    torch.cuda.synchronize()


def test_bf16_rff_embedding_on_tensor_cores():
    """BF16 mode for L2: the random-Fourier embedding GEMM runs on the tcgen05
    tensor cores (BF16 operands, FP32 accumulation).  Against the plain FP32
    embedding: projections within 2e-3 of each point's projection norm (BF16
    rounding of X and R perturbs v = R x by ~2^-8 relative, and cos/sin and
    the orthogonal rotation keep that scale), labels at ARI >= 0.99, and the
    tensor-core kernel did not fall back."""
    import torch
    from sdbscan_gb300 import capi, datasets
    from tests._metrics import adjusted_rand_score
    X, _ = datasets.cfg3_aniso_l2(20000, 64, n_comp=10, seed=33)
    Xt = torch.from_numpy(X).cuda()
    dist = lambda a, b: (a.pow(2).sum(1)[:, None] + b.pow(2).sum(1)[None, :] - 2 * a @ b.T).clamp_min(0).sqrt()
    sigma = float(dist(Xt[:2000], Xt[:2000])[torch.triu_indices(2000, 2000, 1).unbind()].median())
    eps = float(torch.sort(dist(Xt[:500], Xt), dim=1).values[:, 30].median())  # median 30-NN distance
    out = {}
    for prec in (0, 1):
        eng = capi.Engine(*X.shape)
        eng.set_params(n_proj=1024, topK=10, topM=100, distance="L2", ker_n_features=1024, ker_sigma=sigma,
                       random_seed=5, precision=prec)
        eng.fit_sdbscan(X, eps, 30)
        out[prec] = (eng.labels()[0], eng.projections(), eng.counters())
    assert out[1][2]["fallbacks"] == 0
    P0, P1 = out[0][1], out[1][1]
    rel = np.abs(P1 - P0) / np.linalg.norm(P0, axis=1, keepdims=True)
    assert rel.max() < 2e-3, rel.max()
    assert adjusted_rand_score(out[0][0], out[1][0]) >= 0.99


def test_noise_labelling_sampled_matches_oracle(port):
    """clusterNoise = 1 with sampling (samplingProb n < #cores): the engine and
    the oracle draw the same cores (seeded rule) and label every noise point
    the same way; no noise point is left when a cluster exists."""
    from sdbscan_gb300 import capi, datasets
    X, _ = datasets.cfg2_mnist_like(12000, 64, seed=77)
    kw = dict(n_proj=512, topK=6, topM=40, distance="Cosine", random_seed=31)
    eps, minPts, sp = 0.08, 25, 0.02
    eng = capi.Engine(*X.shape)
    eng.set_params(clusterNoise=0, **kw)
    eng.fit_sdbscan(X, eps, minPts)
    plain, _ = eng.labels()
    core, _ = eng.core()
    assert (plain == -1).sum() > 500 and core.sum() > sp * X.shape[0]  # sampling is exercised
    eng.set_params(clusterNoise=1, samplingProb=sp, **kw)
    eng.fit_sdbscan(X, eps, minPts)
    labels, ncl = eng.labels()
    want, ncl_o, _, _ = port.fit_sdbscan(X, eps, minPts, dist="Cosine", n_proj=512, topK=6, topM=40, seed=31,
                                         clusterNoise=1, samplingProb=sp)
    np.testing.assert_array_equal(labels, want)
    assert ncl == ncl_o
    np.testing.assert_array_equal(labels[plain >= 0], plain[plain >= 0])
    assert (labels == -1).sum() == 0
    # no core point at all: nothing to join (the reference reads labels_[-1]
    # here, src/sDbscan.cpp:798-805); every point stays noise, as in the oracle
    eng.fit_sdbscan(X, -1.0, minPts)  # no pair is within a negative eps
    labels, ncl = eng.labels()
    assert eng.core()[0].sum() == 0 and (labels == -1).all() and ncl == 2


@pytest.mark.parametrize("dist,m,optics", [("Cosine", 50, False), ("Cosine", 70, False), ("L2", 50, False),
                                           ("Chi2", 50, True)])
def test_every_distance_tile_shape_gives_the_same_bits(dist, m, optics):
    """The plain distance kernel's tile shapes (sdb_set_tile_variant 1-5:
    one CTA per tile with 64 or 50 columns, and the persistent
    warp-specialised kernel with 4 or 6 stages) compute the same sequential
    fmaf chains, so neighbourhood sizes, core flags and labels -- and for
    sOPTICS every stored distance, hence the ordering and reachability -- are
    identical to the default shape's."""
    from sdbscan_gb300 import capi, datasets
    if dist == "Chi2":
        X = datasets.cfg4_dirichlet(8000, 96, seed=61)[0]
        eps, minPts, kw = 0.3, 10, dict(ker_n_features=1024)
    elif dist == "L2":
        X = datasets.cfg3_aniso_l2(8000, 32, n_comp=8, scale=0.1, seed=62)[0]
        eps, minPts, kw = 0.9, 10, dict(ker_n_features=256, ker_sigma=1.5)
    else:
        X = datasets.cfg1_cosine(12000, 64, seed=63)[0]
        eps, minPts, kw = 0.15, 15, {}
    eng = capi.Engine(*X.shape)
    eng.set_params(n_proj=512, topK=6, topM=m, distance=dist, random_seed=8, **kw)
    ref = None
    for v in range(6):
        eng.set_tile_variant(v)
        if optics:
            eng.fit_soptics(X, eps, minPts)
            out = eng.optics() + eng.core() + (eng.core_dist(),)
        else:
            eng.fit_sdbscan(X, eps, minPts)
            out = eng.labels() + eng.core()
        assert eng.counters()["pairs"] > 0
        if ref is None:
            ref = out
            continue
        for a_, b_ in zip(out, ref):
            np.testing.assert_array_equal(np.asarray(a_), np.asarray(b_), err_msg=f"variant {v}")
