"""sdb_topm_noalloc, the allocation-free top-m entry point, against the
top-m the regular fit computes (sdb_fit_sdbscan + sdb_get_topm).

It serves callers that cannot allocate device memory while they run (a
serving loop whose pool owns the GPU's memory, work issued during stream
capture), so it takes its scratch from a fixed __device__ array.  Each case
calls it twice in a row through the C ABI on the fit's own projections; both
calls must reproduce the fit's top-m matrix exactly (index output, so the
tolerance is zero) -- the second call shows that what the first call left in
the shared array does not leak into the next result.  The cases cover the
float4 row reads (n_proj % 4 == 0) and the scalar reads (n_proj = 1022), a
set smaller than the chunk count (one point per chunk), and heavy ties: 600
copies of one point give lists whose candidates overflow the 512 slots, which
the exact whole-column select resolves.  This file is named to be collected
last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(case):
    from sdbscan_gb300 import datasets
    if case == "ties":
        X, _ = datasets.cfg1_cosine(3000, 32, seed=78)
        X[1000:1600] = X[7]  # 600 identical points: equal projections on every vector
        return X
    if case == "small":
        X, _ = datasets.cfg1_cosine(300, 48, seed=79)
        return X
    X, _ = datasets.cfg1_cosine(30000, 96, seed=77)
    return X


@pytest.mark.parametrize("case,nproj,m", [("base", 1024, 50), ("base", 1022, 50), ("small", 1024, 50),
                                          ("ties", 256, 50)])
def test_topm_noalloc_matches_fit_twice(case, nproj, m):
    import torch

    from sdbscan_gb300 import capi
    X = _data(case)
    n, d = X.shape
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=nproj, topK=5, topM=m, distance="Cosine", random_seed=5)
    eng.fit_sdbscan(X, 0.15, 20)
    want = eng.topm()
    if case == "ties":
        assert eng.counters()["topm_ties"] > 0
    proj = torch.from_numpy(eng.projections()).cuda()
    eng.close()
    for call in range(2):
        out = torch.full((nproj, 2 * m), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        capi.topm_noalloc(proj.data_ptr(), n, nproj, m, out.data_ptr(), 0)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got, want, err_msg=f"call {call}")


def test_topm_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    from sdbscan_gb300 import capi
    proj = torch.zeros((100, 2048), dtype=torch.float32, device="cuda")
    out = torch.zeros((2048, 20), dtype=torch.int32, device="cuda")
    with pytest.raises(capi.SdbError) as e:
        capi.topm_noalloc(proj.data_ptr(), 100, 2048, 10, out.data_ptr(), 0)
    assert e.value.status == 1
    with pytest.raises(capi.SdbError):
        capi.topm_noalloc(proj.data_ptr(), 100, 1024, 65, out.data_ptr(), 0)
