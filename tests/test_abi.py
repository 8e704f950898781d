"""The C ABI library loads and exports every entry point declared in
include/*.h (no compute call: this runs without a GPU)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(sdb_[a-z0-9_]+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib():
    from sdbscan_gb300 import _build
    _build.build_lib()
    from sdbscan_gb300 import capi
    return capi.load()


def test_every_declared_symbol_is_exported(lib):
    declared = _declared()
    assert {"sdb_engine_create", "sdb_fit_sdbscan", "sdb_fit_soptics", "sdb_get_labels"} <= declared
    for name in sorted(declared):
        assert hasattr(lib, name), name
    from sdbscan_gb300 import capi
    assert declared == set(capi.EXPORTS) | (declared - set(capi.EXPORTS))
    assert set(capi.EXPORTS) <= declared


def test_params_default_matches_python_binding(lib):
    """sdb_params_default gives python/python_wrapper.cpp:17-24's defaults."""
    from sdbscan_gb300 import capi
    p = capi.SdbParams()
    lib.sdb_params_default(ctypes.byref(p))
    assert (p.n_proj, p.topK, p.topM, p.distance, p.ker_n_features) == (1024, 10, 50, 0, 1024)
    assert abs(p.ker_sigma - 1.0) < 1e-7 and abs(p.ker_intervalSampling - 0.4) < 1e-7
    assert (p.clusterNoise, p.verbose, p.n_threads, p.random_seed, p.precision) == (0, 0, -1, -1, 0)


def test_null_engine_is_rejected(lib):
    assert lib.sdb_set_params(None, None) == 1
    assert lib.sdb_fit_sdbscan(None, None, ctypes.c_float(0.1), 5) == 1
    assert lib.sdb_last_error(None) == b"null engine"
    assert lib.sdb_set_debug_limits(None, 0, 0, 0) == 1


def test_load_txt_parses_like_fscanf(tmp_path):
    """sdb_load_txt (loadtxtData, src/Utilities.cpp:57-95): n lines of d
    numbers, float32 values exactly those written (shortest round-trip
    decimal strings), odd whitespace accepted; short or missing files raise."""
    from sdbscan_gb300 import capi
    rng = np.random.default_rng(3)
    X = (rng.standard_normal((700, 13)) * 10.0 ** rng.integers(-6, 6, (700, 13))).astype(np.float32)
    X[0, 0], X[1, 1] = 0.0, -1.5
    path = tmp_path / "data.txt"
    with open(path, "w") as f:
        for i, row in enumerate(X):
            sep = "\t" if i % 3 == 0 else " "
            f.write(sep.join(np.format_float_positional(v, unique=True, trim="-") if i % 2 else
                             np.format_float_scientific(v, unique=True) for v in row) + "\n")
    np.testing.assert_array_equal(capi.load_txt(path, 700, 13), X)
    with pytest.raises(capi.SdbError):
        capi.load_txt(path, 701, 13)
    with pytest.raises(capi.SdbError):
        capi.load_txt(tmp_path / "missing.txt", 2, 2)


# The reference binding's names (python/python_wrapper.cpp:14-65): every
# method and result member a caller of the reference module uses.
REFERENCE_MODULE_NAMES = (
    "set_params", "set_sngParams", "clear", "set_topM", "set_threads", "set_clusterNoise", "set_topK",
    "set_kernel_params", "fit_sDbscan", "load_fit_sDbscan", "test_sDbscan", "load_test_sDbscan", "fit_sOptics",
    "load_fit_sOptics", "fit_sngDbscan", "test_sngDbscan", "load_test_sngDbscan", "fit_sngOptics",
    "load_fit_sngOptics", "labels_", "n_clusters_", "ordering_", "reachability_")


def test_dropin_module_has_every_reference_name():
    """The pybind module `sDbscan` (importable without a GPU) exposes the
    reference binding's class with all of its methods and result members."""
    import importlib
    try:
        mod = importlib.import_module("sdbscan_gb300.sDbscan")
    except ImportError as e:
        pytest.skip(f"drop-in module not built here: {e}")
    missing = [n for n in REFERENCE_MODULE_NAMES if not hasattr(mod.sDbscan, n)]
    assert not missing, missing


# Keyword names and defaults of the reference binding (python/python_wrapper.cpp:15-51).
REFERENCE_SIGNATURES = {
    "set_params": [("n_proj", "1024"), ("topK", "10"), ("topM", "50"), ("distance", "'Cosine'"),
                   ("ker_n_features", "1024"), ("ker_sigma", "1.0"), ("ker_intervalSampling", "0.4"),
                   ("clusterNoise", "0"), ("samplingProb", "0.01"), ("verbose", "False"), ("output", "''"),
                   ("n_threads", "-1"), ("random_seed", "-1")],
    "set_sngParams": [("distance", "'Cosine'"), ("samplingProb", "0.01"), ("clusterNoise", "0"),
                      ("verbose", "False"), ("output", "''"), ("n_threads", "-1"), ("random_seed", "-1")],
    "set_kernel_params": [("distance", "'L2'"), ("ker_n_features", "1024"), ("ker_sigma", "1.0"),
                          ("ker_intervalSampling", "0.4")],
    "set_topM": [("topM", None)], "set_topK": [("topK", None)], "set_threads": [("n_threads", None)],
    "set_clusterNoise": [("clusterNoise", None)],
    "fit_sDbscan": [("X", None), ("eps", None), ("minPts", None)],
    "fit_sOptics": [("X", None), ("eps", None), ("minPts", None)],
    "fit_sngDbscan": [("X", None), ("eps", None), ("minPts", None)],
    "fit_sngOptics": [("X", None), ("eps", None), ("minPts", None)],
    "load_fit_sDbscan": [("dataset", None), ("eps", None), ("minPts", None)],
    "load_fit_sOptics": [("dataset", None), ("eps", None), ("minPts", None)],
    "load_fit_sngOptics": [("dataset", None), ("eps", None), ("minPts", None)],
    "test_sDbscan": [("X", None), ("eps", None), ("rangeEps", None), ("n_tests", None), ("minPts", None)],
    "test_sngDbscan": [("X", None), ("eps", None), ("rangeEps", None), ("n_tests", None), ("minPts", None)],
    "load_test_sDbscan": [("dataset", None), ("eps", None), ("rangeEps", None), ("n_tests", None), ("minPts", None)],
    "load_test_sngDbscan": [("dataset", None), ("eps", None), ("rangeEps", None), ("n_tests", None),
                            ("minPts", None)],
}


def _doc_params(doc):
    """(name, default) pairs of a pybind11 signature line, self dropped."""
    import re
    sig = doc.strip().splitlines()[0]
    body = sig[sig.index("(") + 1: sig.rindex(")")]
    while "[" in body:  # drop bracketed type arguments (they hold commas)
        body = re.sub(r"\[[^\[\]]*\]", "", body)
    out = []
    for part in body.split(", "):
        name = part.split(":")[0].strip()
        default = part.split(" = ", 1)[1].strip() if " = " in part else None
        if name != "self":
            out.append((name, default))
    return out


def test_dropin_keywords_and_defaults_match_reference():
    import importlib
    try:
        mod = importlib.import_module("sdbscan_gb300.sDbscan")
    except ImportError as e:
        pytest.skip(f"drop-in module not built here: {e}")
    for name, want in REFERENCE_SIGNATURES.items():
        assert _doc_params(getattr(mod.sDbscan, name).__doc__) == want, name
    init = _doc_params(mod.sDbscan.__init__.__doc__)
    assert [n for n, _ in init[:2]] == ["n_points", "n_features"]  # python_wrapper.cpp:16


def test_no_cpu_fallback_without_a_gpu():
    """Without a usable CUDA device the engine refuses to start: the C ABI
    returns SDB_ERR_CUDA and both bindings raise; nothing computes on the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sdbscan_gb300 import capi
    with pytest.raises(capi.SdbError) as e:
        capi.Engine(10, 4)
    assert e.value.status == 2
    import importlib
    try:
        mod = importlib.import_module("sdbscan_gb300.sDbscan")
    except ImportError as err:
        pytest.skip(f"drop-in module not built here: {err}")
    with pytest.raises(RuntimeError):
        mod.sDbscan(10, 4)


def test_topm_noalloc_rejects_misaligned_rows(lib):
    """sdb_topm_noalloc reads rows of a multiple of 4 projections as 16-byte
    vectors; a base that is not 16-byte aligned is refused on the host before
    anything is launched (the pointer below is never dereferenced)."""
    vp = ctypes.c_void_p
    assert lib.sdb_topm_noalloc(vp(0x10004), 1000, 1024, 50, vp(0x20000), None) == 1
    assert lib.sdb_topm_noalloc(vp(0x10008), 1000, 512, 50, vp(0x20000), None) == 1
