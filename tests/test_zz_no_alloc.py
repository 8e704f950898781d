"""sdb_topm_noalloc, the allocation-free top-m entry point, against the
top-m the regular fit computes (sdb_fit_sdbscan + sdb_get_topm).

It serves callers that cannot allocate device memory while they run (a
serving loop whose pool owns the GPU's memory, work issued during stream
capture), so it takes its scratch from a fixed __device__ array.  The test
calls it twice in a row through the C ABI on the fit's own projections; both
calls must reproduce the fit's top-m matrix exactly (index output, so the
tolerance is zero) -- the second call shows that what the first call left in
the shared array does not leak into the next result.  This file is named to
be collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_topm_noalloc_matches_fit_twice():
    import torch

    from sdbscan_gb300 import capi, datasets
    X, _ = datasets.cfg1_cosine(30000, 96, seed=77)
    n, d = X.shape
    nproj, m = 1024, 50
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=nproj, topK=5, topM=m, distance="Cosine", random_seed=5)
    eng.fit_sdbscan(X, 0.15, 20)
    want = eng.topm()
    proj = torch.from_numpy(eng.projections()).cuda()
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
