"""The engine against the oracle at the benchmark configurations' own sizes.

Each case runs the configuration bench.py measures (same data law, seed,
parameters and random_seed = 42) through the C ABI, and the oracle's stages
on the same data on all host cores:
  - config 2, 1M x 784 Cosine sDBSCAN (the headline): projections bit-exact;
    top-k / top-m index sets per row; neighbourhood sizes, core flags, labels
    and n_clusters_ bit-exact;
  - config 1, 50K x 128 Cosine sDBSCAN: the same bar;
  - config 3, 1M x 256 L2 through the random-Fourier embedding (FP32 and the
    split-BF16 tensor-core embedding): projections within 1e-5 (FP32) or
    2e-3 (BF16) of the row norm, core flags >= 99.5 % equal, labels ARI >=
    0.99 against the oracle's own run (CUDA's cosf / sinf are not glibc's);
  - config 4, 500K x 512 Chi2 sOPTICS: projections, core flags, sizes, core
    distances, ordering and reachability bit-exact, the ordering in the
    canonical tie order (equal reachabilities pop by point id).
Ties: the oracle's selections here break boundary ties by the smallest index
(orc_topk_canon / orc_topm_canon, the engine's rule), so the whole pipeline is
compared bit for bit through any tie.  The reference's heap selections are
run too: the rows where they differ from the canonical sets must be rows where
the engine counted a boundary tie.  The neighbourhoods are built by the
oracle's large-n construction (orc_core_cluster_lean / orc_find_core_lean),
which tests/test_oracle_lean.py pins to the point-by-point restatement.
"""
import os
import sys
import time

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

pytestmark = pytest.mark.gpu


def _mem_available_gb():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


def _need_host_memory(gb):
    have = _mem_available_gb()
    if have < gb:
        pytest.skip(f"needs {gb} GB of free host memory for the oracle, {have:.0f} GB available")


def _cfg(i):
    import bench
    return dict(bench.WORKLOADS[i])


def _sorted_rows(a):
    return np.sort(np.asarray(a), axis=1)


def _engine_fit(cfg, X_dev, kp, precision=0):
    from sdbscan_gb300 import capi
    n, d = X_dev.shape
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=cfg["n_proj"], topK=cfg["topK"], topM=cfg["topM"], distance=cfg["distance"],
                   random_seed=42, precision=precision, **kp)
    if cfg["fit"] == "soptics":
        eng.fit_soptics_device(X_dev.data_ptr(), cfg["eps"], cfg["minPts"])
    else:
        eng.fit_sdbscan_device(X_dev.data_ptr(), cfg["eps"], cfg["minPts"])
    return eng


def _oracle_index(port, Xh, cfg, kp):
    """Transform, projections and the canonical top-k / top-m of the oracle."""
    from oracle.oracle import fht_dim
    n, d = Xh.shape
    dist = cfg["distance"]
    ker = d if dist == "Cosine" else kp.get("ker_n_features", 1024)
    fd = fht_dim(cfg["n_proj"], ker)
    bits = port.hd3_bits(3 * fd, 42)
    R = port._R(dist, ker, d, kp.get("ker_sigma", 1.0), 42)
    Xt, rc = port.transform(Xh, dist)
    assert rc == 0
    P = port.project(Xt, dist, ker, 0.4, R, bits, fd, cfg["n_proj"])
    return Xt, P


def _check_selections(eng, port, P, cfg, exact=True):
    """Canonical top-k / top-m of the oracle's projections; with exact
    projections they must equal the engine's sets row for row."""
    k, m = cfg["topK"], cfg["topM"]
    tK, tM = port.topk_canon(P, k), port.topm_canon(P, m)
    if exact:
        np.testing.assert_array_equal(_sorted_rows(eng.topk()), _sorted_rows(tK))
        np.testing.assert_array_equal(_sorted_rows(eng.topm()), _sorted_rows(tM))
        # the reference's heap rule differs from the canonical one only at
        # boundary ties, which the engine counts
        c = eng.counters()
        hK, hM = port.topk(P, k), port.topm(P, m)
        dk = int(np.sum(np.any(_sorted_rows(hK[:, :k]) != _sorted_rows(tK[:, :k]), axis=1)) +
                 np.sum(np.any(_sorted_rows(hK[:, k:]) != _sorted_rows(tK[:, k:]), axis=1)))
        dm = int(np.sum(np.any(_sorted_rows(hM[:, :m]) != _sorted_rows(tM[:, :m]), axis=1)) +
                 np.sum(np.any(_sorted_rows(hM[:, m:]) != _sorted_rows(tM[:, m:]), axis=1)))
        print(f"boundary ties: top-k {c['topk_ties']} counted, {dk} rows differ from the heap rule; "
              f"top-m {c['topm_ties']} counted, {dm} rows differ")
        assert dk <= c["topk_ties"] and dm <= c["topm_ties"]
    return tK, tM


def _dbscan_exact(cfg, X_dev, kp=None):
    import torch

    from oracle.oracle import Port, build_port
    kp = kp or {}
    build_port()
    port = Port()
    t0 = time.time()
    eng = _engine_fit(cfg, X_dev, kp)
    labels, ncl = eng.labels()
    core, deg = eng.core()
    Peng = eng.projections()
    Xh = X_dev.cpu().numpy()
    torch.cuda.synchronize()
    t1 = time.time()
    Xt, P = _oracle_index(port, Xh, cfg, kp)
    assert np.array_equal(Peng, P), "projections differ from the oracle"
    del Peng
    tK, tM = _check_selections(eng, port, P, cfg)
    del P
    ocore, odeg, olabels, oncl = port.core_cluster_lean(Xt, cfg["distance"], tK, tM, cfg["eps"], cfg["minPts"])
    t2 = time.time()
    print(f"{cfg['workload']}: engine + download {t1 - t0:.1f} s, oracle {t2 - t1:.1f} s; "
          f"{int(ocore.sum())} core points, {oncl - 1} clusters")
    np.testing.assert_array_equal(deg, odeg)
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(labels, olabels)
    assert ncl == oncl
    assert ocore.sum() > 0 and oncl > 2  # a clustering with several clusters, not a vacuous one
    eng.close()


def test_cfg2_1Mx784_cosine_bit_exact():
    _need_host_memory(48)
    import torch

    from sdbscan_gb300 import datasets
    cfg = _cfg(2)
    X, _ = datasets.cfg2_mnist_like_torch(cfg["n"], cfg["d"], seed=cfg["seed"], device="cuda")
    torch.cuda.synchronize()
    _dbscan_exact(cfg, X)


def test_cfg1_50Kx128_cosine_bit_exact():
    import torch

    from sdbscan_gb300 import datasets
    cfg = _cfg(1)
    X = torch.from_numpy(datasets.cfg1_cosine(cfg["n"], cfg["d"], seed=cfg["seed"])[0]).cuda()
    _dbscan_exact(cfg, X)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32", "bf16"])
def test_cfg3_1Mx256_l2_rff(precision):
    _need_host_memory(32)
    import torch

    import bench
    from oracle.oracle import Port, build_port
    from sdbscan_gb300 import datasets
    from tests._metrics import adjusted_rand_score
    cfg = _cfg(3)
    Xh = datasets.cfg3_aniso_l2(cfg["n"], cfg["d"], seed=cfg["seed"], scale=cfg["scale"])[0]
    X = torch.from_numpy(Xh).cuda()
    kp = bench._kernel_params(cfg, X)
    eng = _engine_fit(cfg, X, kp, precision)
    labels, ncl = eng.labels()
    core, _ = eng.core()
    Peng = eng.projections()
    if precision == 1:
        assert eng.counters()["fallbacks"] == 0
    build_port()
    port = Port()
    Xt, P = _oracle_index(port, Xh, cfg, kp)
    scale = np.linalg.norm(P, axis=1, keepdims=True)
    err = float(np.max(np.abs(Peng - P) / scale))
    print(f"config 3 ({'BF16' if precision else 'FP32'}): projection error {err:.3g} of the row norm")
    assert err < (2e-3 if precision else 1e-5)
    del Peng
    tK, tM = _check_selections(eng, port, P, cfg, exact=False)
    del P
    ocore, _odeg, olabels, oncl = port.core_cluster_lean(Xt, "L2", tK, tM, cfg["eps"], cfg["minPts"])
    agree = float(np.mean(core == ocore))
    ari = adjusted_rand_score(olabels, labels)
    print(f"config 3: core agreement {agree:.5f}, ARI {ari:.5f}, clusters {ncl - 1} vs {oncl - 1}")
    assert ocore.sum() > 1000
    assert agree >= 0.995
    assert ari >= 0.99
    eng.close()


def test_cfg4_500Kx512_chi2_soptics_bit_exact():
    _need_host_memory(32)
    import torch

    from oracle.oracle import Port, build_port
    from sdbscan_gb300 import datasets
    cfg = _cfg(4)
    Xh = datasets.cfg4_dirichlet(cfg["n"], cfg["d"], seed=cfg["seed"])[0]
    X = torch.from_numpy(Xh).cuda()
    kp = {"ker_n_features": cfg["ker_n_features"]}
    eng = _engine_fit(cfg, X, kp)
    order, reach = eng.optics()
    core, deg = eng.core()
    cd = eng.core_dist()
    Peng = eng.projections()
    build_port()
    port = Port()
    Xt, P = _oracle_index(port, Xh, cfg, kp)
    assert np.array_equal(Peng, P), "projections differ from the oracle"
    del Peng
    tK, tM = _check_selections(eng, port, P, cfg)
    del P
    ocore, odeg, off, idx, dd = port.find_core(Xt, "Chi2", tK, tM, cfg["eps"], cfg["minPts"], with_dist=True,
                                               lean=True)
    ocd = port.core_dist(cfg["n"], cfg["minPts"], ocore)
    oorder, oreach = port.form_optics(ocore, ocd, off, idx, dd, tie_mode=1)
    port.graph_free()
    print(f"config 4: {int(ocore.sum())} core points, {int(np.sum(oreach > -1e9))} points reached")
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(deg, odeg)
    np.testing.assert_array_equal(cd, ocd)
    np.testing.assert_array_equal(order, oorder)
    np.testing.assert_array_equal(reach, oreach)
    assert 0 < ocore.sum() < len(ocore)
    eng.close()
