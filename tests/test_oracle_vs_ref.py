"""Direct oracle-vs-reference comparison where the reference library exists
(the development machine); skipped elsewhere."""
import os

import numpy as np
import pytest

from oracle.oracle import REF_SO, Ref
from sdbscan_gb300 import datasets as ds

pytestmark = pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")


def _data(dist, n=3000):
    if dist in ("Chi2", "JS"):
        return ds.cfg4_dirichlet(n, 64, n_comp=6, seed=21)[0]
    if dist in ("L1", "L2"):
        return ds.cfg3_aniso_l2(n, 16, n_comp=6, scale=0.1, seed=21)[0]
    return ds.cfg1_cosine(n, 48, seed=21)[0]


@pytest.mark.parametrize("dist,eps,ker", [("Cosine", 0.15, 1024), ("Chi2", 0.3, 512), ("L2", 0.6, 256),
                                          ("L1", 1.5, 256), ("JS", 0.02, 512)])
def test_multithreaded_fit_labels(port, dist, eps, ker):
    X = _data(dist)
    n, d = X.shape
    r = Ref(n, d)
    r.set_params(n_proj=256, topK=5, topM=20, distance=dist, ker_n_features=ker, ker_sigma=0.5, n_threads=4,
                 random_seed=3)
    r.fit_sDbscan(X, eps, 10)
    labels, ncl, core, _ = port.fit_sdbscan(X, eps, 10, dist=dist, n_proj=256, topK=5, topM=20, ker=ker, sigma=0.5,
                                            seed=3, threads=4)
    np.testing.assert_array_equal(core, r.core())
    np.testing.assert_array_equal(labels, r.labels_)
    assert ncl == r.n_clusters_


@pytest.mark.parametrize("dist,eps,ker", [("Cosine", 0.016, 1024), ("Chi2", 0.03, 1024)])
def test_multithreaded_soptics_core_distances(port, dist, eps, ker):
    """fit_sOptics with 4 threads: core flags and core distances do not
    depend on the order in which threads fill the neighbour lists
    (src/sDbscan.cpp:1428-1446), so they equal the oracle's; the ordering is a
    permutation of the points (its tie order is thread-dependent)."""
    X = _data(dist, 2500)
    n, d = X.shape
    r = Ref(n, d)
    r.set_params(n_proj=256, topK=5, topM=20, distance=dist, ker_n_features=ker, n_threads=4, random_seed=5)
    r.fit_sOptics(X, eps, 10)
    order, reach, core, cd, _ = port.fit_soptics(X, eps, 10, dist=dist, n_proj=256, topK=5, topM=20, ker=ker,
                                                 seed=5, threads=4)
    np.testing.assert_array_equal(core, r.core())
    np.testing.assert_array_equal(cd, r.core_dist())
    assert sorted(r.ordering_.tolist()) == list(range(n))
    np.testing.assert_array_equal(np.sort(order), np.arange(n))


@pytest.mark.parametrize("dist,prob,eps", [("Cosine", 0.05, 0.15), ("L2", 0.1, 0.6), ("Cosine", 1.0, 0.1)])
def test_multithreaded_sngdbscan(port, dist, prob, eps):
    """fit_sngDbscan with 4 threads and a fixed seed (every point draws the
    same sequence, src/sDbscan.cpp:437-455): labels, n_clusters_ and core flags
    equal the oracle's point-by-point restatement."""
    X = _data(dist, 2000)
    n, d = X.shape
    r = Ref(n, d)
    r.set_sngParams(distance=dist, samplingProb=prob, n_threads=4, random_seed=11)
    r.fit_sngDbscan(X, eps, 10)
    labels, ncl, core, _, _ = port.fit_sngdbscan(X, eps, 10, dist=dist, samplingProb=prob, seed=11, threads=4)
    np.testing.assert_array_equal(core, r.core())
    np.testing.assert_array_equal(labels, r.labels_)
    assert ncl == r.n_clusters_


def test_noise_labelling_with_partial_core_sampling_same_law(port):
    """sDbscan-1NN with fewer sampled cores than cores (src/sDbscan.cpp:683-706):
    the reference keeps each core with probability fProb through the unseeded
    rand(); the engine's rule keeps it iff a hash of (seed, point) falls below
    fProb.  Same law: no point stays noise, and the labels given to the former
    noise points agree between a reference run and a run of the rule as often
    as two reference runs agree with each other."""
    from oracle.oracle import fht_dim
    X = ds.cfg1_cosine(3000, 48, seed=21)[0]
    n, d = X.shape
    eps, prob = 0.15, 0.02
    refs = []
    for _ in range(4):
        r = Ref(n, d)
        r.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", clusterNoise=1, samplingProb=prob,
                     n_threads=4, random_seed=3)
        r.fit_sDbscan(X, eps, 10)
        refs.append(r.labels_.copy())
    base, _, core, _ = port.fit_sdbscan(X, eps, 10, n_proj=256, topK=5, topM=20, seed=3, threads=4)
    noise = base == -1
    assert 50 < noise.sum() < 500
    Xt, _ = port.transform(X, "Cosine")
    fd = fht_dim(256, d)
    P = port.project(Xt, "Cosine", d, 0.4, None, port.hd3_bits(3 * fd, 3), fd, 256)
    topK = port.topk(P, 5)
    ours = [port.label_noise(P, topK, core, base, prob, 1000 + s) for s in range(4)]
    for lab in refs + ours:
        assert (lab != -1).all()
        np.testing.assert_array_equal(lab[~noise], base[~noise])

    def agree(a, b):
        return float(np.mean(a[noise] == b[noise]))

    rr = np.mean([agree(refs[i], refs[j]) for i in range(4) for j in range(i + 1, 4)])
    oo = np.mean([agree(ours[i], ours[j]) for i in range(4) for j in range(i + 1, 4)])
    ro = np.mean([agree(a, b) for a in refs for b in ours])
    assert abs(ro - rr) < 0.1 and abs(oo - rr) < 0.1, (rr, oo, ro)


def test_reference_sweep_files_equal_oracle_sweep(port, tmp_path):
    """The reference's own test_sDbscan (src/sDbscan.cpp:980-1039): index once,
    then for eps + i * rangeEps (computed in double, stored as float) one labels
    file named <output>_<dist>_Eps_<round(1000 eps)>_MinPts_.._KerFeatures_..
    _NumProj_.._TopM_.._TopK_..; every file equals the oracle's sweep."""
    X = ds.cfg2_mnist_like(2500, 64, seed=41)[0]
    n, d = X.shape
    eps0, step, nt, minPts = 0.06, 0.03, 4, 10
    r = Ref(n, d)
    r.set_params(n_proj=256, topK=5, topM=20, distance="Cosine", n_threads=4, random_seed=6)
    prefix = tmp_path / "ref"
    r.test_sDbscan(X, eps0, step, nt, minPts, prefix)
    eps = [np.float32(np.float64(np.float32(eps0)) + 1.0 * i * np.float64(np.float32(step))) for i in range(nt)]
    labels, ncl, _ = port.fit_sdbscan_sweep(X, eps, minPts, n_proj=256, topK=5, topM=20, seed=6, threads=4)
    for i, e in enumerate(eps):
        f = (f"{prefix}_Cosine_Eps_{int(round(1000 * float(e)))}_MinPts_{minPts}_KerFeatures_{d}"
             f"_NumProj_256_TopM_20_TopK_5")
        np.testing.assert_array_equal(np.loadtxt(f, dtype=np.int32), labels[i])
    assert len(set(map(int, ncl))) > 1  # the eps values give different clusterings


_FIXTURES = sorted(os.path.basename(p)[:-4] for p in
                   __import__("glob").glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("name", _FIXTURES)
def test_golden_fixture_regenerates_bit_identically(name, tmp_path):
    """tests/golden/make_golden.py, run again with the reference, writes the
    committed fixture bit for bit (the fixtures are reproducible from the
    committed script)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.main((name,), str(tmp_path))
    new = np.load(tmp_path / f"{name}.npz")
    old = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    assert sorted(new.files) == sorted(old.files)
    for k in old.files:
        np.testing.assert_array_equal(new[k], old[k], err_msg=k)


def _random_params(case):
    """A seeded random parameter set within the reference's preconditions:
    distance, n, d, n_proj, topK, topM, ker_n_features, minPts, eps, fit
    (True = sOPTICS) and seed.  Cheap: no data is drawn."""
    rng = np.random.default_rng(1000 + case)
    dist = str(rng.choice(["Cosine", "L1", "L2", "Chi2", "JS"]))
    n = int(rng.integers(50, 1200))
    d = int(rng.choice([3, 8, 17, 32, 65, 130]))
    n_proj = int(rng.choice([16, 64, 100, 256, 512]))
    k = int(rng.integers(1, min(12, n_proj) + 1))
    m = int(rng.integers(1, min(60, n) + 1))
    ker = d if dist == "Cosine" else int(rng.choice([64, 128, 256, 512]))
    if dist in ("Chi2", "JS") and ker < d:
        ker = int(2 ** np.ceil(np.log2(d)))
    minPts = int(rng.integers(2, 20))
    seed = int(rng.integers(0, 1000))
    lo, hi = {"Cosine": (0.02, 0.4), "L1": (0.2, 3.0), "L2": (0.2, 3.0)}.get(dist, (0.05, 0.5))
    eps = float(rng.uniform(lo, hi))
    return dist, n, d, n_proj, k, m, ker, minPts, eps, bool(rng.integers(0, 2)), seed


def _random_config(case):
    """_random_params with the data drawn from the distance's law."""
    dist, n, d, n_proj, k, m, ker, minPts, eps, optics, seed = _random_params(case)
    if dist == "Cosine":
        X = ds.cfg1_cosine(n, d, seed=seed)[0]
    elif dist in ("L1", "L2"):
        X = ds.cfg3_aniso_l2(n, d, n_comp=4, scale=0.1, seed=seed)[0]
    else:
        X = ds.cfg4_dirichlet(n, d, n_comp=4, conc=10, seed=seed)[0]
    return dist, X, n_proj, k, m, ker, minPts, eps, optics, seed


@pytest.mark.parametrize("case", range(30))
def test_random_configurations_match_reference(port, case):
    """Seeded random configurations over every distance and both fits, one
    thread: sDBSCAN labels, core flags and n_clusters_, or sOPTICS core flags
    and core distances, equal the reference's."""
    dist, X, n_proj, k, m, ker, minPts, eps, optics, seed = _random_config(case)
    n, d = X.shape
    r = Ref(n, d)
    r.set_params(n_proj=n_proj, topK=k, topM=m, distance=dist, ker_n_features=ker, ker_sigma=0.7, n_threads=1,
                 random_seed=seed)
    kw = dict(dist=dist, n_proj=n_proj, topK=k, topM=m, ker=ker, sigma=0.7, seed=seed, threads=1)
    if optics:
        r.fit_sOptics(X, eps, minPts)
        _, _, core, cd, _ = port.fit_soptics(X, eps, minPts, **kw)
        np.testing.assert_array_equal(core, r.core())
        np.testing.assert_array_equal(cd, r.core_dist())
    else:
        r.fit_sDbscan(X, eps, minPts)
        labels, ncl, core, _ = port.fit_sdbscan(X, eps, minPts, **kw)
        np.testing.assert_array_equal(core, r.core())
        np.testing.assert_array_equal(labels, r.labels_)
        assert ncl == r.n_clusters_


@pytest.mark.parametrize("case", range(15))
def test_random_noise_labelling_configurations_match_reference(port, case):
    """sDbscan-1NN (clusterNoise = 1) with every core sampled, seeded random
    configurations: labels equal the reference's.  Where there is no core
    point the reference reads labels_[-1] (undefined); the oracle keeps every
    point as noise."""
    rng = np.random.default_rng(3000 + case)
    dist = str(rng.choice(["Cosine", "L1", "L2", "Chi2", "JS"]))
    n, d = int(rng.integers(50, 1500)), int(rng.choice([8, 17, 32, 65]))
    n_proj = int(rng.choice([16, 64, 256]))
    k, m = int(rng.integers(1, min(10, n_proj) + 1)), int(rng.integers(1, min(50, n) + 1))
    ker = d if dist == "Cosine" else int(rng.choice([64, 128, 256]))
    if dist in ("Chi2", "JS") and ker < d:
        ker = 128
    minPts, seed = int(rng.integers(2, 20)), int(rng.integers(0, 1000))
    if dist == "Cosine":
        X, eps = ds.cfg1_cosine(n, d, seed=seed)[0], float(rng.uniform(0.02, 0.3))
    elif dist in ("L1", "L2"):
        X, eps = ds.cfg3_aniso_l2(n, d, n_comp=4, scale=0.1, seed=seed)[0], float(rng.uniform(0.2, 2.0))
    else:
        X, eps = ds.cfg4_dirichlet(n, d, n_comp=4, conc=10, seed=seed)[0], float(rng.uniform(0.05, 0.4))
    kw = dict(dist=dist, n_proj=n_proj, topK=k, topM=m, ker=ker, sigma=0.7, seed=seed, threads=1)
    labels, ncl, core, _ = port.fit_sdbscan(X, eps, minPts, clusterNoise=1, samplingProb=1.0, **kw)
    if core.sum() == 0:
        assert (labels == -1).all() and ncl == 2
        return
    r = Ref(n, d)
    r.set_params(n_proj=n_proj, topK=k, topM=m, distance=dist, ker_n_features=ker, ker_sigma=0.7, clusterNoise=1,
                 samplingProb=1.0, n_threads=1, random_seed=seed)
    r.fit_sDbscan(X, eps, minPts)
    np.testing.assert_array_equal(labels, r.labels_)
    assert ncl == r.n_clusters_


@pytest.mark.parametrize("case", [c for c in range(60) if _random_params(c)[9]][:15])
def test_random_soptics_ordering_matches_reference(port, case):
    """sOPTICS ordering and reachability on seeded random configurations, one
    thread: the oracle's stages, with the neighbour lists in the reference's
    own order and the reference's value-only heap ties (tie_mode 0), give the
    reference's ordering_ and reachability_ bit for bit."""
    from oracle.oracle import fht_dim
    dist, X, n_proj, k, m, ker, minPts, eps, _, seed = _random_config(case)
    n, d = X.shape
    r = Ref(n, d)
    r.set_params(n_proj=n_proj, topK=k, topM=m, distance=dist, ker_n_features=ker, ker_sigma=0.7, n_threads=1,
                 random_seed=seed)
    r.fit_sOptics(X, eps, minPts)
    fd = fht_dim(n_proj, ker)
    Xt, _ = port.transform(X, dist)
    P = port.project(Xt, dist, ker, 0.4, port._R(dist, ker, d, 0.7, seed), port.hd3_bits(3 * fd, seed), fd, n_proj)
    port.L.orc_set_threads(1)
    try:
        core, _, off, idx, dd = port.find_core(Xt, dist, port.topk(P, k), port.topm(P, m), eps, minPts,
                                               with_dist=True, ref_order=True)
    finally:
        port.L.orc_set_threads(0)
    order, reach = port.form_optics(core, port.core_dist(n, minPts, core), off, idx, dd, tie_mode=0)
    port.graph_free()
    np.testing.assert_array_equal(order, r.ordering_)
    np.testing.assert_array_equal(reach, r.reachability_)


def test_text_loader_parses_like_the_reference(tmp_path):
    """sdb_load_txt against the reference's own loadtxtData (fscanf "%f",
    src/Utilities.cpp:60-95) on long decimal strings (near-halfway roundings),
    exponents down to the subnormal range and past it, signs and odd spacing:
    every float32 is the same."""
    from oracle.oracle import ref_load_txt
    from sdbscan_gb300 import capi
    try:
        capi.load()
    except Exception as e:
        pytest.skip(f"engine library not built here: {e}")
    rng = np.random.default_rng(8)
    n, d = 400, 9
    toks = []
    for i in range(n * d):
        kind = i % 6
        if kind == 0:
            toks.append(f"{rng.standard_normal():.25f}")
        elif kind == 1:
            toks.append(f"{rng.standard_normal():.20e}")
        elif kind == 2:
            toks.append(f"{rng.random() * 1e-39:.30e}")  # subnormal float32 range
        elif kind == 3:
            toks.append(f"{rng.random() * 1e-47:.10e}")  # below the smallest subnormal
        elif kind == 4:
            toks.append(str(int(rng.integers(-10**6, 10**6))))
        else:
            toks.append(f"+{rng.random() * 10 ** int(rng.integers(-8, 8)):.17g}")
    path = tmp_path / "data.txt"
    with open(path, "w") as f:
        for r in range(n):
            f.write(("  " if r % 2 else "\t").join(toks[r * d:(r + 1) * d]) + (" \n" if r % 3 else "\n"))
    want = ref_load_txt(path, n, d)
    got = capi.load_txt(path, n, d)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
