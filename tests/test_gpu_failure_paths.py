"""Failure paths of the engine, made to run without a GPU fault.

sdb_set_debug_limits (off by default) gives three controls:
  - stall_spins: each tensor-core kernel and the persistent plain distance
    kernel waits once per launch on a barrier that nothing completes, and gives
    up after that many polls -- a bounded wait that runs out, standing in for a
    producer that stopped.  The kernel must then stop its roles, wait for the
    copies and MMAs it has in flight, free its tensor memory and raise its
    flag; nothing hangs and the context stays usable.
  - queue_cap: the BF16 re-decision queue overflows.
  - device_bytes_cap: the next fit cannot allocate.
Each case checks the outcome the engine promises: the BF16 stages fall back to
their FP32 kernels with labels identical to the plain fit (and the fallback
counter rises), the persistent plain kernel fails the fit with
SDB_ERR_INTERNAL, an allocation over the cap gives SDB_ERR_NOMEM -- and in
every case the next fit with the limits off is correct.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STALL = 1 << 12  # polls of the never-completed barrier


def _cosine(n=12000, d=196, seed=91):
    """MNIST-like nonnegative rows: many pairs fall within the BF16 margin of
    eps = 0.25 (well-separated vMF clusters have none), so the re-decision
    queue is in use."""
    from sdbscan_gb300 import datasets
    return datasets.cfg2_mnist_like(n, d, seed=seed)[0]


def _fit(X, precision=0, variant=0, **limits):
    from sdbscan_gb300 import capi
    eng = capi.Engine(*X.shape)
    eng.set_params(n_proj=512, topK=5, topM=40, distance="Cosine", random_seed=4, precision=precision)
    if variant:
        eng.set_tile_variant(variant)
    if limits:
        eng.set_debug_limits(**limits)
    return eng


def test_bf16_screening_stall_falls_back_to_fp32():
    X = _cosine()
    plain = _fit(X)
    plain.fit_sdbscan(X, 0.25, 20)
    want = plain.labels()
    eng = _fit(X, precision=1, stall_spins=STALL)
    eng.fit_sdbscan(X, 0.25, 20)
    assert eng.counters()["fallbacks"] == 1
    got = eng.labels()
    np.testing.assert_array_equal(got[0], want[0])
    assert got[1] == want[1]
    np.testing.assert_array_equal(eng.core()[1], plain.core()[1])
    eng.set_debug_limits()  # off again: screening runs and succeeds
    eng.fit_sdbscan(X, 0.25, 20)
    assert eng.counters()["fallbacks"] == 1 and eng.counters()["rechecked"] > 0
    np.testing.assert_array_equal(eng.labels()[0], want[0])


def test_bf16_queue_overflow_falls_back_to_fp32():
    X = _cosine(seed=92)
    plain = _fit(X)
    plain.fit_sdbscan(X, 0.25, 20)
    eng = _fit(X, precision=1)
    eng.fit_sdbscan(X, 0.25, 20)
    assert eng.counters()["rechecked"] > 4  # pairs near eps exist
    eng.set_debug_limits(queue_cap=4)
    eng.fit_sdbscan(X, 0.25, 20)
    assert eng.counters()["fallbacks"] == 1
    np.testing.assert_array_equal(eng.labels()[0], plain.labels()[0])
    np.testing.assert_array_equal(eng.core()[1], plain.core()[1])


def test_bf16_embedding_stall_falls_back_to_fp32():
    """L2, BF16 mode: the tensor-core random-Fourier embedding and the
    tensor-core distance screening both stall, the FP32 embedding and the
    plain distance kernel replace them, and the fit equals a plain FP32 fit bit
    for bit (both use the FP32 embedding then)."""
    from sdbscan_gb300 import capi, datasets
    X = datasets.cfg3_aniso_l2(8000, 32, n_comp=8, scale=0.1, seed=93)[0]
    out = {}
    for prec, lim in ((0, 0), (1, STALL)):
        eng = capi.Engine(*X.shape)
        eng.set_params(n_proj=512, topK=5, topM=40, distance="L2", ker_n_features=256, ker_sigma=1.5,
                       random_seed=4, precision=prec)
        eng.set_debug_limits(stall_spins=lim)
        eng.fit_sdbscan(X, 0.9, 10)
        out[prec] = (eng.labels(), eng.projections(), eng.counters()["fallbacks"])
    assert out[1][2] == 2  # the embedding and the screening
    np.testing.assert_array_equal(out[1][1], out[0][1])
    np.testing.assert_array_equal(out[1][0][0], out[0][0][0])


def test_bf16_sng_block_stall_falls_back_to_fp32():
    from sdbscan_gb300 import capi
    X = _cosine(6000, 64, seed=94)
    res = {}
    for prec, lim in ((0, 0), (1, STALL)):
        eng = capi.Engine(*X.shape)
        eng.set_sng_params(distance="Cosine", samplingProb=0.1, random_seed=6)
        eng.set_precision(prec)
        eng.set_debug_limits(stall_spins=lim)
        eng.fit_sngdbscan(X, 0.25, 10)
        res[prec] = (eng.labels(), eng.core(), eng.counters()["fallbacks"])
    assert res[1][2] == 1
    np.testing.assert_array_equal(res[1][0][0], res[0][0][0])
    np.testing.assert_array_equal(res[1][1][1], res[0][1][1])


@pytest.mark.parametrize("variant", [4, 5])
def test_persistent_plain_kernel_stall_fails_the_fit_cleanly(variant):
    from sdbscan_gb300 import capi
    X = _cosine(seed=95)
    ref = _fit(X)
    ref.fit_sdbscan(X, 0.25, 20)
    eng = _fit(X, variant=variant, stall_spins=STALL)
    with pytest.raises(capi.SdbError) as e:
        eng.fit_sdbscan(X, 0.25, 20)
    assert e.value.status == 7  # SDB_ERR_INTERNAL
    eng.set_debug_limits()
    eng.fit_sdbscan(X, 0.25, 20)
    np.testing.assert_array_equal(eng.labels()[0], ref.labels()[0])


def test_device_memory_cap_gives_nomem_and_the_engine_recovers():
    from sdbscan_gb300 import capi
    X = _cosine(seed=96)
    eng = _fit(X, device_bytes_cap=1 << 20)
    with pytest.raises(capi.SdbError) as e:
        eng.fit_sdbscan(X, 0.25, 20)
    assert e.value.status == 6  # SDB_ERR_NOMEM
    with pytest.raises(capi.SdbError):
        eng.labels()  # no result from the failed fit
    eng.set_debug_limits()
    eng.fit_sdbscan(X, 0.25, 20)
    ref = _fit(X)
    ref.fit_sdbscan(X, 0.25, 20)
    np.testing.assert_array_equal(eng.labels()[0], ref.labels()[0])
