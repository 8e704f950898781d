"""ctypes binding of the engine's C ABI (include/sdbscan_gb300.h).

This is how the tests and bench.py drive the engine: through the same C
entry points a foreign-language caller binds.  Importing this module loads
``libsdbscan_gb300.so`` from the package folder and fails loudly if it is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsdbscan_gb300.so")

DISTANCES = {"Cosine": 0, "L1": 1, "L2": 2, "Chi2": 3, "JS": 4}
PREC_FP32, PREC_BF16 = 0, 1
STATUS = {0: "SDB_OK", 1: "SDB_ERR_ARG", 2: "SDB_ERR_CUDA", 3: "SDB_ERR_NEGATIVE", 4: "SDB_ERR_ZERO_POINT",
          5: "SDB_ERR_STATE", 6: "SDB_ERR_NOMEM", 7: "SDB_ERR_INTERNAL"}
EXPORTS = ["sdb_params_default", "sdb_engine_create", "sdb_engine_destroy", "sdb_set_params", "sdb_fit_sdbscan",
           "sdb_fit_sdbscan_device", "sdb_fit_soptics", "sdb_fit_soptics_device", "sdb_get_labels", "sdb_get_optics",
           "sdb_clear", "sdb_get_topk", "sdb_get_topm", "sdb_get_core", "sdb_get_core_dist", "sdb_get_projections",
           "sdb_get_counters", "sdb_get_stage_ms", "sdb_engine_stream", "sdb_last_error", "sdb_topm_noalloc",
           "sdb_fit_sdbscan_sweep", "sdb_batch_create", "sdb_batch_run", "sdb_batch_labels", "sdb_batch_lanes",
           "sdb_batch_destroy", "sdb_batch_last_error", "sdb_load_txt",
           "sdb_batch_tile_variant", "sdb_set_sng_params", "sdb_fit_sngdbscan", "sdb_fit_sngdbscan_device",
           "sdb_fit_sngdbscan_sweep", "sdb_fit_sngoptics", "sdb_fit_sngoptics_device", "sdb_set_precision",
           "sdb_set_tile_variant", "sdb_set_debug_limits", "sdb_set_sng_sampling"]


class SdbParams(ctypes.Structure):
    _fields_ = [("n_proj", ctypes.c_int32), ("topK", ctypes.c_int32), ("topM", ctypes.c_int32),
                ("distance", ctypes.c_int32), ("ker_n_features", ctypes.c_int32), ("ker_sigma", ctypes.c_float),
                ("ker_intervalSampling", ctypes.c_float), ("clusterNoise", ctypes.c_int32),
                ("samplingProb", ctypes.c_float), ("verbose", ctypes.c_int32), ("n_threads", ctypes.c_int32),
                ("random_seed", ctypes.c_int32), ("precision", ctypes.c_int32)]


class SdbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_LIB = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the engine library (building it first if the sources are newer)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(the engine has no CPU fallback)")
    L = ctypes.CDLL(path)
    vp, i32, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_float
    L.sdb_params_default.argtypes = [ctypes.POINTER(SdbParams)]
    L.sdb_engine_create.argtypes = [i32, i32, i32, ctypes.POINTER(vp)]
    L.sdb_engine_destroy.argtypes = [vp]
    L.sdb_set_params.argtypes = [vp, ctypes.POINTER(SdbParams)]
    for f in ("sdb_fit_sdbscan", "sdb_fit_sdbscan_device", "sdb_fit_soptics", "sdb_fit_soptics_device",
              "sdb_fit_sngdbscan", "sdb_fit_sngdbscan_device", "sdb_fit_sngoptics", "sdb_fit_sngoptics_device"):
        getattr(L, f).argtypes = [vp, vp, f32, i32]
    L.sdb_get_labels.argtypes = [vp, vp, vp]
    L.sdb_get_optics.argtypes = [vp, vp, vp]
    L.sdb_clear.argtypes = [vp]
    for f in ("sdb_get_topk", "sdb_get_topm", "sdb_get_core_dist", "sdb_get_projections"):
        getattr(L, f).argtypes = [vp, vp]
    L.sdb_get_core.argtypes = [vp, vp, vp]
    L.sdb_get_counters.argtypes = [vp, vp, i32]
    L.sdb_get_stage_ms.argtypes = [vp, vp, i32]
    L.sdb_engine_stream.argtypes = [vp]
    L.sdb_engine_stream.restype = vp
    L.sdb_last_error.argtypes = [vp]
    L.sdb_last_error.restype = ctypes.c_char_p
    L.sdb_topm_noalloc.argtypes = [vp, i32, i32, i32, vp, vp]
    L.sdb_fit_sdbscan_sweep.argtypes = [vp, vp, vp, i32, i32, vp, vp]
    L.sdb_fit_sngdbscan_sweep.argtypes = [vp, vp, vp, i32, i32, vp, vp]
    L.sdb_set_sng_params.argtypes = [vp, i32, f32, i32, i32, i32, i32]
    L.sdb_set_precision.argtypes = [vp, i32]
    L.sdb_set_tile_variant.argtypes = [vp, i32]
    L.sdb_set_debug_limits.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
    L.sdb_set_sng_sampling.argtypes = [vp, i32]
    L.sdb_batch_create.argtypes = [i32, vp, vp, vp, ctypes.POINTER(SdbParams), vp, i32, i32, i32,
                                   ctypes.POINTER(vp)]
    L.sdb_batch_run.argtypes = [vp, ctypes.POINTER(f32)]
    L.sdb_batch_labels.argtypes = [vp, i32, i32, vp, vp]
    L.sdb_batch_lanes.argtypes = [vp]
    L.sdb_batch_lanes.restype = i32
    L.sdb_batch_destroy.argtypes = [vp]
    L.sdb_batch_last_error.argtypes = [vp]
    L.sdb_batch_last_error.restype = ctypes.c_char_p
    L.sdb_load_txt.argtypes = [ctypes.c_char_p, i32, i32, vp]
    L.sdb_batch_tile_variant.argtypes = [vp, i32]
    L.sdb_batch_tile_variant.restype = i32
    _LIB = L
    return L


def _ptr(a: np.ndarray | None):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Engine:
    """One engine = one reference `sDbscan(n_points, n_features)` object."""

    def __init__(self, n_points: int, n_features: int, device: int = 0):
        self.L = load()
        self.n, self.d = int(n_points), int(n_features)
        h = ctypes.c_void_p()
        s = self.L.sdb_engine_create(self.n, self.d, device, ctypes.byref(h))
        if s != 0:
            raise SdbError(s, "sdb_engine_create failed (no usable CUDA device?)")
        self.h = h
        self.params = SdbParams()
        self.L.sdb_params_default(ctypes.byref(self.params))

    def close(self):
        if getattr(self, "h", None):
            self.L.sdb_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s: int):
        if s != 0:
            raise SdbError(s, self.L.sdb_last_error(self.h).decode())

    # set_params with the reference binding's keyword names (python/python_wrapper.cpp:17-24)
    def set_params(self, n_proj=1024, topK=10, topM=50, distance="Cosine", ker_n_features=1024, ker_sigma=1.0,
                   ker_intervalSampling=0.4, clusterNoise=0, samplingProb=0.01, verbose=False, output="",
                   n_threads=-1, random_seed=-1, precision=PREC_FP32):
        p = self.params
        p.n_proj, p.topK, p.topM = n_proj, topK, topM
        p.distance = DISTANCES[distance]
        p.ker_n_features, p.ker_sigma, p.ker_intervalSampling = ker_n_features, ker_sigma, ker_intervalSampling
        p.clusterNoise, p.samplingProb, p.verbose = clusterNoise, samplingProb, int(bool(verbose))
        p.n_threads, p.random_seed, p.precision = n_threads, random_seed, precision
        self._check(self.L.sdb_set_params(self.h, ctypes.byref(p)))

    # fits -----------------------------------------------------------------------
    def fit_sdbscan(self, X: np.ndarray, eps: float, minPts: int):
        """X: (n, d) C-contiguous float32 = d x n column-major."""
        X = self._host(X)
        self._check(self.L.sdb_fit_sdbscan(self.h, _ptr(X), ctypes.c_float(eps), minPts))

    def fit_sdbscan_device(self, x_dev_ptr: int, eps: float, minPts: int):
        self._check(self.L.sdb_fit_sdbscan_device(self.h, ctypes.c_void_p(x_dev_ptr), ctypes.c_float(eps), minPts))

    def fit_sdbscan_sweep(self, X: np.ndarray, eps_list, minPts: int):
        """test_sDbscan: index and distances once, labels for every eps.
        Returns (labels [n_eps, n], n_clusters [n_eps])."""
        X = self._host(X)
        eps = np.ascontiguousarray(eps_list, dtype=np.float32)
        labels = np.empty((eps.shape[0], self.n), np.int32)
        ncl = np.empty(eps.shape[0], np.int32)
        self._check(self.L.sdb_fit_sdbscan_sweep(self.h, _ptr(X), _ptr(eps), eps.shape[0], minPts, _ptr(labels),
                                                 _ptr(ncl)))
        return labels, ncl

    def fit_soptics(self, X: np.ndarray, eps: float, minPts: int):
        X = self._host(X)
        self._check(self.L.sdb_fit_soptics(self.h, _ptr(X), ctypes.c_float(eps), minPts))

    def fit_soptics_device(self, x_dev_ptr: int, eps: float, minPts: int):
        self._check(self.L.sdb_fit_soptics_device(self.h, ctypes.c_void_p(x_dev_ptr), ctypes.c_float(eps), minPts))

    # sngDbscan / sngOptics (src/sDbscan.h:127-139, :190-201) ----------------------
    def set_sng_params(self, distance="Cosine", samplingProb=0.01, clusterNoise=0, verbose=False, output="",
                       n_threads=-1, random_seed=-1):
        p = self.params
        self._check(self.L.sdb_set_sng_params(self.h, DISTANCES[distance], ctypes.c_float(samplingProb),
                                              clusterNoise, int(bool(verbose)), n_threads, random_seed))
        p.distance, p.samplingProb, p.verbose = DISTANCES[distance], samplingProb, int(bool(verbose))
        p.n_threads, p.random_seed = n_threads, random_seed
        if clusterNoise > 0:
            p.clusterNoise = 2

    def set_precision(self, precision: int):
        """PREC_FP32 or PREC_BF16 alone (no index parameter checks)."""
        self._check(self.L.sdb_set_precision(self.h, precision))
        self.params.precision = precision

    def set_tile_variant(self, variant: int):
        """Tile shape of the plain FP32 distance kernel (0 = by topM; see the header)."""
        self._check(self.L.sdb_set_tile_variant(self.h, variant))

    def set_sng_sampling(self, mode: int):
        """sdb_set_sng_sampling: 0 by seed, 1 shared sample, 2 per-block samples."""
        self._check(self.L.sdb_set_sng_sampling(self.h, mode))

    def set_debug_limits(self, stall_spins: int = 0, queue_cap: int = 0, device_bytes_cap: int = 0):
        """sdb_set_debug_limits: the failure-path test controls (0 = off)."""
        self._check(self.L.sdb_set_debug_limits(self.h, stall_spins, queue_cap, device_bytes_cap))

    def fit_sngdbscan(self, X: np.ndarray, eps: float, minPts: int):
        X = self._host(X)
        self.params.clusterNoise = 0
        self._check(self.L.sdb_fit_sngdbscan(self.h, _ptr(X), ctypes.c_float(eps), minPts))

    def fit_sngdbscan_device(self, x_dev_ptr: int, eps: float, minPts: int):
        self.params.clusterNoise = 0
        self._check(self.L.sdb_fit_sngdbscan_device(self.h, ctypes.c_void_p(x_dev_ptr), ctypes.c_float(eps), minPts))

    def fit_sngdbscan_sweep(self, X: np.ndarray, eps_list, minPts: int):
        """test_sngDbscan: one transform and sample, labels for every eps.
        Returns (labels [n_eps, n], n_clusters [n_eps])."""
        X = self._host(X)
        eps = np.ascontiguousarray(eps_list, dtype=np.float32)
        labels = np.empty((eps.shape[0], self.n), np.int32)
        ncl = np.empty(eps.shape[0], np.int32)
        self._check(self.L.sdb_fit_sngdbscan_sweep(self.h, _ptr(X), _ptr(eps), eps.shape[0], minPts, _ptr(labels),
                                                   _ptr(ncl)))
        return labels, ncl

    def fit_sngoptics(self, X: np.ndarray, eps: float, minPts: int):
        X = self._host(X)
        self._check(self.L.sdb_fit_sngoptics(self.h, _ptr(X), ctypes.c_float(eps), minPts))

    def fit_sngoptics_device(self, x_dev_ptr: int, eps: float, minPts: int):
        self._check(self.L.sdb_fit_sngoptics_device(self.h, ctypes.c_void_p(x_dev_ptr), ctypes.c_float(eps), minPts))

    def _host(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        if X.shape != (self.n, self.d):
            raise ValueError(f"X must be (n_points, n_features) = ({self.n}, {self.d}), got {X.shape}")
        return X

    # results ---------------------------------------------------------------------
    def labels(self) -> tuple[np.ndarray, int]:
        out = np.empty(self.n, np.int32)
        nc = ctypes.c_int32()
        self._check(self.L.sdb_get_labels(self.h, _ptr(out), ctypes.byref(nc)))
        return out, nc.value

    def optics(self) -> tuple[np.ndarray, np.ndarray]:
        order = np.empty(self.n, np.int32)
        reach = np.empty(self.n, np.float32)
        self._check(self.L.sdb_get_optics(self.h, _ptr(order), _ptr(reach)))
        return order, reach

    def topk(self) -> np.ndarray:
        out = np.empty((self.n, 2 * self.params.topK), np.int32)
        self._check(self.L.sdb_get_topk(self.h, _ptr(out)))
        return out

    def topm(self) -> np.ndarray:
        out = np.empty((self.params.n_proj, 2 * self.params.topM), np.int32)
        self._check(self.L.sdb_get_topm(self.h, _ptr(out)))
        return out

    def core(self) -> tuple[np.ndarray, np.ndarray]:
        core = np.empty(self.n, np.uint8)
        deg = np.empty(self.n, np.int32)
        self._check(self.L.sdb_get_core(self.h, _ptr(core), _ptr(deg)))
        return core, deg

    def core_dist(self) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self._check(self.L.sdb_get_core_dist(self.h, _ptr(out)))
        return out

    def projections(self) -> np.ndarray:
        out = np.empty((self.n, self.params.n_proj), np.float32)
        self._check(self.L.sdb_get_projections(self.h, _ptr(out)))
        return out

    def counters(self) -> dict:
        out = np.zeros(8, np.int64)
        self._check(self.L.sdb_get_counters(self.h, _ptr(out), 8))
        return dict(topk_ties=int(out[0]), topm_ties=int(out[1]), launches=int(out[2]), pairs=int(out[3]),
                    rechecked=int(out[4]), fallbacks=int(out[5]), sng_sampled=int(out[6]), sng_extra=int(out[7]))

    def stage_ms(self) -> dict:
        out = np.zeros(9, np.float32)
        self._check(self.L.sdb_get_stage_ms(self.h, _ptr(out), 9))
        names = ["upload", "project", "topm", "index", "distances", "core", "cluster", "readback", "total"]
        return dict(zip(names, out.tolist()))

    def stream(self) -> int:
        return int(self.L.sdb_engine_stream(self.h) or 0)


def load_txt(path: str, n_points: int, n_features: int) -> np.ndarray:
    """sdb_load_txt: n_points lines of n_features numbers -> (n_points, n_features)
    float32 (= the d x n column-major matrix the fits take), parsed like fscanf "%f"."""
    L = load()
    out = np.empty((n_points, n_features), np.float32)
    s = L.sdb_load_txt(str(path).encode(), n_points, n_features, _ptr(out))
    if s != 0:
        raise SdbError(s, f"sdb_load_txt: {path} is missing or holds fewer than {n_points * n_features} numbers")
    return out


def topm_noalloc(proj_dev_ptr: int, n_points: int, n_proj: int, topM: int, out_dev_ptr: int, stream: int = 0) -> None:
    """sdb_topm_noalloc: top-m selection on device projections, no device
    allocation (scratch is a fixed __device__ array in the library)."""
    L = load()
    s = L.sdb_topm_noalloc(ctypes.c_void_p(proj_dev_ptr), n_points, n_proj, topM, ctypes.c_void_p(out_dev_ptr),
                           ctypes.c_void_p(stream) if stream else None)
    if s != 0:
        raise SdbError(s, "sdb_topm_noalloc failed")


class Batch:
    """sdb_batch_*: many datasets, one eps sweep each, replayed as one CUDA graph.
    X_device: list of (data_ptr, n, d) of device-resident (n, d) float32 rows."""

    def __init__(self, X_device, eps_list, minPts: int, device: int = 0, **params):
        self.L = load()
        p = SdbParams()
        self.L.sdb_params_default(ctypes.byref(p))
        for k_, v_ in params.items():
            setattr(p, k_, DISTANCES[v_] if k_ == "distance" else v_)
        self.ns = len(X_device)
        self.sizes = [int(n) for _, n, _ in X_device]
        n_arr = (ctypes.c_int32 * self.ns)(*[int(n) for _, n, _ in X_device])
        d_arr = (ctypes.c_int32 * self.ns)(*[int(d) for _, _, d in X_device])
        x_arr = (ctypes.c_void_p * self.ns)(*[int(ptr) for ptr, _, _ in X_device])
        self.eps = np.ascontiguousarray(eps_list, dtype=np.float32)
        h = ctypes.c_void_p()
        s = self.L.sdb_batch_create(self.ns, n_arr, d_arr, x_arr, ctypes.byref(p), _ptr(self.eps),
                                    self.eps.shape[0], minPts, device, ctypes.byref(h))
        self.h = h
        if s != 0:
            msg = self.L.sdb_batch_last_error(h).decode() if h.value else ""
            self.close()
            raise SdbError(s, "sdb_batch_create: " + msg)

    def run(self) -> float:
        ms = ctypes.c_float()
        s = self.L.sdb_batch_run(self.h, ctypes.byref(ms))
        if s != 0:
            raise SdbError(s, self.L.sdb_batch_last_error(self.h).decode())
        return ms.value

    def labels(self, set_index: int, eps_index: int):
        out = np.empty(self.sizes[set_index], np.int32)
        nc = ctypes.c_int32()
        s = self.L.sdb_batch_labels(self.h, set_index, eps_index, _ptr(out), ctypes.byref(nc))
        if s != 0:
            raise SdbError(s, self.L.sdb_batch_last_error(self.h).decode())
        return out, nc.value

    def lanes(self) -> int:
        return int(self.L.sdb_batch_lanes(self.h))

    def tile_variants(self) -> list[int]:
        """Per set, the distance tile shape the autotuner kept (see sdb_batch_tile_variant)."""
        return [int(self.L.sdb_batch_tile_variant(self.h, i)) for i in range(self.ns)]

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.sdb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
