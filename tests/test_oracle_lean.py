"""The oracle's large-n checkers against its reference-pinned stages.

Two additions let the GPU engine be checked at the configurations' own sizes
(a million points):
  - orc_topk_canon / orc_topm_canon: the selections with ties at the
    boundary broken by the smallest index (the engine's rule).  Without a
    boundary tie they equal the reference's heap selections (orc_topk /
    orc_topm, pinned to the reference's fixtures) as sets; with ties they
    equal a lexicographic (value, index) sort.
  - orc_core_cluster_lean: core flags, neighbourhood sizes, labels and
    n_clusters_ of orc_find_core + orc_form_cluster without the per-pair
    pushes under a global lock.  It must equal them exactly, for every
    distance.
  - orc_find_core_lean: the same construction leaving orc_find_core's
    sorted neighbour graph with distances, for the sOPTICS stages (core
    distances, ordering, reachability).
"""
import numpy as np
import pytest

from oracle.oracle import fht_dim


def _sets(a):
    return [frozenset(r) for r in a.tolist()]


def _lexsort_top(vals, k):
    """k largest by (value desc, index asc) per row of vals."""
    n = vals.shape[1]
    out = []
    for row in vals:
        order = np.lexsort((np.arange(n), -row.astype(np.float64)))
        out.append(frozenset(order[:k].tolist()))
    return out


def test_canonical_selections_break_ties_by_smallest_index(port):
    rng = np.random.default_rng(3)
    # values on a coarse grid: many exact ties at every boundary
    P = rng.integers(-6, 7, size=(400, 64)).astype(np.float32) / 4
    k, m = 5, 20
    tK = port.topk_canon(P, k)
    tM = port.topm_canon(P, m)
    assert _sets(tK[:, :k]) == _lexsort_top(P, k)
    assert _sets(tK[:, k:]) == _lexsort_top(-P, k)
    assert _sets(tM[:, :m]) == _lexsort_top(P.T, m)
    assert _sets(tM[:, m:]) == _lexsort_top(-P.T, m)
    # rows in (value, index) order, most extreme first
    for p in range(0, 400, 37):
        v = P[p, tK[p, :k]]
        assert np.all(np.diff(v) <= 0)


def test_canonical_selections_equal_heap_selections_without_ties(port):
    rng = np.random.default_rng(4)
    P = rng.standard_normal((3000, 128)).astype(np.float32)
    for k in (1, 7):
        assert _sets(port.topk_canon(P, k)) == _sets(port.topk(P, k))
    for m in (1, 30):
        assert _sets(port.topm_canon(P, m)) == _sets(port.topm(P, m))


@pytest.mark.parametrize("dist,n,d,nproj,k,m,eps,minPts", [
    ("Cosine", 3000, 32, 256, 5, 40, 0.15, 10),
    ("Cosine", 2500, 100, 128, 3, 60, 0.3, 25),
    ("L2", 2000, 16, 256, 4, 30, 1.2, 8),
    ("L1", 1500, 16, 128, 4, 30, 3.0, 8),
    ("Chi2", 1500, 64, 512, 5, 40, 0.3, 12),
    ("JS", 1200, 64, 512, 5, 40, 0.3, 12),
    ("Cosine", 800, 16, 64, 3, 20, 0.001, 5),  # all noise: n_clusters_ = 2
])
def test_lean_core_cluster_equals_find_core(port, dist, n, d, nproj, k, m, eps, minPts):
    from sdbscan_gb300 import datasets
    if dist in ("Chi2", "JS"):
        X = datasets.cfg4_dirichlet(n, d, seed=12)[0]
    elif dist == "Cosine":
        X = datasets.cfg1_cosine(n, d, seed=13)[0]
    else:
        X = datasets.cfg3_aniso_l2(n, d, seed=14, scale=0.1)[0]
    ker = d if dist == "Cosine" else 512
    fd = fht_dim(nproj, ker)
    bits = port.hd3_bits(3 * fd, 9)
    R = port._R(dist, ker, d, 1.0, 9)
    Xt, rc = port.transform(X, dist)
    assert rc == 0
    P = port.project(Xt, dist, ker, 0.4, R, bits, fd, nproj)
    tK, tM = port.topk(P, k), port.topm(P, m)
    core, deg, off, idx, _ = port.find_core(Xt, dist, tK, tM, eps, minPts, with_dist=False)
    labels, ncl = port.form_cluster(core, off, idx)
    port.graph_free()
    lcore, ldeg, llabels, lncl = port.core_cluster_lean(Xt, dist, tK, tM, eps, minPts)
    assert core.sum() > 0 or eps < 0.01
    np.testing.assert_array_equal(ldeg, deg)
    np.testing.assert_array_equal(lcore, core)
    np.testing.assert_array_equal(llabels, labels)
    assert lncl == ncl
    # the graph with distances, and the sOPTICS outputs built on it
    core, deg, off, idx, dd = port.find_core(Xt, dist, tK, tM, eps, minPts, with_dist=True)
    cd = port.core_dist(n, minPts, core)
    order, reach = port.form_optics(core, cd, off, idx, dd, tie_mode=1)
    port.graph_free()
    lcore, ldeg, loff, lidx, ldd = port.find_core(Xt, dist, tK, tM, eps, minPts, with_dist=True, lean=True)
    lcd = port.core_dist(n, minPts, lcore)
    lorder, lreach = port.form_optics(lcore, lcd, loff, lidx, ldd, tie_mode=1)
    port.graph_free()
    for a, b in ((lcore, core), (ldeg, deg), (loff, off), (lidx, idx), (ldd, dd), (lcd, cd), (lorder, order),
                 (lreach, reach)):
        np.testing.assert_array_equal(a, b)
