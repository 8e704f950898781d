"""sngDbscan / sngOptics (src/sDbscan.cpp:416-504, 1131-1304, 1484-1583,
1846-1923): the oracle restatement against the reference's own outputs.

The sng fixtures were produced by the reference itself (seeded: every point's
generator gets random_seed 7, src/sDbscan.cpp:437-440; see
tests/golden/make_golden.py).  The oracle restates sng_findCorePoints point by
point and must reproduce labels, n_clusters_, core flags and the core points'
neighbourhood sizes (repeats counted) exactly.  sngOptics seeds each point
from std::random_device in the reference, so its restatement (the engine's
shared seeded sample) is checked for its own invariants here.
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
