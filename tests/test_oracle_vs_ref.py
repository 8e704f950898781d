"""Direct oracle-vs-reference comparison where the reference library exists
(the development machine); skipped elsewhere."""
import os

import numpy as np
import pytest

from oracle.oracle import REF_SO, Ref
from sdbscan_gb300 import datasets as ds

pytestmark = pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")


@pytest.mark.parametrize("dist,eps,ker", [("Cosine", 0.15, 1024), ("Chi2", 0.3, 512), ("L2", 0.6, 256)])
def test_multithreaded_fit_labels(port, dist, eps, ker):
    if dist == "Chi2":
        X, _ = ds.cfg4_dirichlet(3000, 64, n_comp=6, seed=21)
    elif dist == "L2":
        X, _ = ds.cfg3_aniso_l2(3000, 16, n_comp=6, scale=0.1, seed=21)
    else:
        X, _ = ds.cfg1_cosine(3000, 48, seed=21)
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
