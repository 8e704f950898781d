"""ORACLE — test infrastructure, not product code.

ctypes bindings for the two CPU checkers built by ``oracle/Makefile``:

* ``Port``  (``oracle/_build/liboracle.so``): the from-scratch restatement of
  the reference algorithm (``oracle/sdbscan_oracle.cpp``).  Portable; builds
  wherever gcc and OpenMP exist.
* ``Ref``   (``oracle/_ref/libsdbscan_ref.so``): the reference's own unmodified
  sources compiled against the shim headers.  Exists only where the reference
  sources were available at build time (x86-64 development machine).

Only tests, ``__graft_entry__.smoke()`` and the CPU baseline of ``bench.py``
import this module.  Arrays follow the reference's layout: data is d x n
column-major, i.e. a C-contiguous numpy array of shape (n, d), one point per
row.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsdbscan_ref.so")
DIST_CODES = {"Cosine": 0, "L1": 1, "L2": 2, "Chi2": 3, "JS": 4}

_vp = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_i64 = ctypes.c_int64


def _p(a):
    return a.ctypes.data_as(_vp) if a is not None else None


def build_port(quiet: bool = True) -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return PORT_SO


def build_ref(quiet: bool = True) -> str | None:
    """Builds oracle/_ref when the reference sources are present; else None."""
    # SDBSCAN_REF_SRC, else a checkout of the reference next to this repository
    src = os.environ.get("SDBSCAN_REF_SRC") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "src")
    if not os.path.isfile(os.path.join(src, "sDbscan.cpp")):
        return None
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        return None  # the reference's FFHT is x86 inline assembly
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={src}"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return REF_SO


def _fit_error(code: int) -> str:
    """Message for a negative return of the oracle's whole-fit entry points."""
    return {1: "transformData: negative input value (Chi2/JS)",
            2: "transformData: a point sums to zero (Chi2/JS)",
            3: "ker_n_features must be >= n_features for Chi2/JS (the reference overruns its embedding)",
            }.get(code, f"rejected (code {code})")


def fht_dim(n_proj: int, ker: int) -> int:
    """fhtDim = 2^ceil(log2(max(n_proj, ker)))  (src/sDbscan.h:107)."""
    import math
    return 1 << int(math.ceil(math.log2(max(n_proj, ker))))


class Port:
    """The oracle restatement (oracle/sdbscan_oracle.cpp)."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build_port()
        L = ctypes.CDLL(path)
        self.L = L
        L.orc_transform.restype = _i
        L.orc_form_cluster.restype = _i
        L.orc_neighbors_total.restype = _i64
        L.orc_form_optics.restype = _i64
        L.orc_fit_sdbscan.restype = _i
        L.orc_fit_soptics.restype = _i
        L.orc_fit_sdbscan_sweep.restype = _i
        L.orc_fit_sngdbscan.restype = _i
        L.orc_fit_sngoptics.restype = _i
        L.orc_distance.restype = _f
        L.orc_core_cluster_lean.restype = _i

    def set_timing_mode(self, on: bool) -> None:
        """Cosine / L1 / L2 distances with vectorisable partial sums, at the
        speed of the reference's Eigen build, for the CPU baseline's timed
        legs only (the last bits leave the numerical contract).  The setting
        belongs to the loaded library, so it holds for every Port of the
        process until it is switched off."""
        self.L.orc_set_timing_mode(_i(1 if on else 0))

    # RNG -------------------------------------------------------------------
    def hd3_bits(self, nbits: int, seed: int) -> np.ndarray:
        out = np.zeros(nbits, np.uint8)
        self.L.orc_hd3_bits(_i(nbits), _i(seed), _p(out))
        return out

    def gauss(self, rows, cols, mean, std, seed) -> np.ndarray:
        out = np.zeros(rows * cols, np.float32)
        self.L.orc_gauss(_i(rows), _i(cols), _f(mean), _f(std), _i(seed), _p(out))
        return out  # column-major rows x cols

    def cauchy(self, rows, cols, x0, gamma, seed) -> np.ndarray:
        out = np.zeros(rows * cols, np.float32)
        self.L.orc_cauchy(_i(rows), _i(cols), _f(x0), _f(gamma), _i(seed), _p(out))
        return out

    # stages ------------------------------------------------------------------
    def transform(self, X: np.ndarray, dist: str) -> tuple[np.ndarray, int]:
        Xc = np.ascontiguousarray(X, np.float32).copy()
        n, d = Xc.shape
        rc = self.L.orc_transform(_p(Xc), _i(n), _i(d), _i(DIST_CODES[dist]))
        return Xc, rc

    def project(self, Xt, dist, ker, L, R, bits, fhtdim, nproj) -> np.ndarray:
        n, d = Xt.shape
        out = np.zeros((n, nproj), np.float32)
        self.L.orc_project(_p(Xt), _i(n), _i(d), _i(DIST_CODES[dist]), _i(ker), _f(L), _p(R), _p(bits),
                           _i(fhtdim), _i(nproj), _p(out))
        return out

    def topk(self, P: np.ndarray, k: int) -> np.ndarray:
        n, nproj = P.shape
        out = np.zeros((n, 2 * k), np.int32)
        self.L.orc_topk(_p(np.ascontiguousarray(P)), _i(n), _i(nproj), _i(k), _p(out))
        return out

    def topm(self, P: np.ndarray, m: int) -> np.ndarray:
        n, nproj = P.shape
        out = np.zeros((nproj, 2 * m), np.int32)
        self.L.orc_topm(_p(np.ascontiguousarray(P)), _i(n), _i(nproj), _i(m), _p(out))
        return out

    def topk_canon(self, P: np.ndarray, k: int) -> np.ndarray:
        """Per-point top-k with ties at the boundary broken by the smallest
        index (the engine's rule), rows in (value, index) order."""
        n, nproj = P.shape
        out = np.zeros((n, 2 * k), np.int32)
        self.L.orc_topk_canon(_p(np.ascontiguousarray(P)), _i(n), _i(nproj), _i(k), _p(out))
        return out

    def topm_canon(self, P: np.ndarray, m: int) -> np.ndarray:
        """Per-vector top-m with the engine's smallest-index tie rule."""
        n, nproj = P.shape
        out = np.zeros((nproj, 2 * m), np.int32)
        self.L.orc_topm_canon(_p(np.ascontiguousarray(P)), _i(n), _i(nproj), _i(m), _p(out))
        return out

    def core_cluster_lean(self, Xt, dist, topK, topM, eps, minPts):
        """Core flags, neighbourhood sizes, labels and n_clusters_ of
        find_core + form_cluster, through the oracle's lock-free large-n
        restatement.  Returns (core, degree, labels, n_clusters)."""
        n, d = Xt.shape
        k = topK.shape[1] // 2
        m = topM.shape[1] // 2
        core = np.zeros(n, np.uint8)
        deg = np.zeros(n, np.int32)
        labels = np.zeros(n, np.int32)
        ncl = self.L.orc_core_cluster_lean(_p(np.ascontiguousarray(Xt, np.float32)), _i(n), _i(d),
                                           _i(DIST_CODES[dist]), _p(np.ascontiguousarray(topK, np.int32)), _i(k),
                                           _p(np.ascontiguousarray(topM, np.int32)), _i(m), _f(eps), _i(minPts),
                                           _p(core), _p(deg), _p(labels))
        return core, deg, labels, int(ncl)

    def find_core(self, Xt, dist, topK, topM, eps, minPts, with_dist=True, ref_order=False, lean=False):
        """Returns core (u8), degree (i32), CSR (off, idx, dist) of the
        de-duplicated symmetric neighbourhoods of every point: sorted by id,
        or (ref_order=True, run with one thread) in the reference's order.
        lean=True builds the same sorted graph through the large-n
        construction (orc_find_core_lean)."""
        n, d = Xt.shape
        k = topK.shape[1] // 2
        m = topM.shape[1] // 2
        core = np.zeros(n, np.uint8)
        deg = np.zeros(n, np.int32)
        Xt = np.ascontiguousarray(Xt, np.float32)
        if lean:
            assert not ref_order
            self.L.orc_find_core_lean(_p(Xt), _i(n), _i(d), _i(DIST_CODES[dist]),
                                      _p(np.ascontiguousarray(topK, np.int32)), _i(k),
                                      _p(np.ascontiguousarray(topM, np.int32)), _i(m), _f(eps), _i(minPts),
                                      _i(1 if with_dist else 0), _p(core), _p(deg))
        else:
            self.L.orc_find_core(_p(Xt), _i(n), _i(d), _i(DIST_CODES[dist]), _p(np.ascontiguousarray(topK)), _i(k),
                                 _p(np.ascontiguousarray(topM)), _i(m), _f(eps), _i(minPts), _i(1 if with_dist else 0),
                                 _i(1 if ref_order else 0), _p(core), _p(deg))
        tot = self.L.orc_neighbors_total(_i(n))
        off = np.zeros(n + 1, np.int64)
        idx = np.zeros(tot, np.int32)
        dd = np.zeros(tot, np.float32) if with_dist else None
        self.L.orc_neighbors_export(_i(n), _p(off), _p(idx), _p(dd))
        return core, deg, off, idx, dd

    def core_dist(self, n, minPts, core) -> np.ndarray:
        out = np.zeros(n, np.float32)
        self.L.orc_core_dist(_i(n), _i(minPts), _p(core), _p(out))
        return out

    def graph_free(self):
        self.L.orc_graph_free()

    def form_cluster(self, core, off, idx) -> tuple[np.ndarray, int]:
        n = core.shape[0]
        labels = np.zeros(n, np.int32)
        ncl = self.L.orc_form_cluster(_i(n), _p(core), _p(off), _p(idx), _p(labels))
        return labels, ncl

    def form_optics(self, core, coreDist, off, idx, dist, tie_mode=1):
        n = core.shape[0]
        order = np.zeros(n, np.int32)
        reach = np.zeros(n, np.float32)
        no = self.L.orc_form_optics(_i(n), _p(core), _p(coreDist), _p(off), _p(idx), _p(dist), _i(tie_mode),
                                    _p(order), _p(reach))
        return order[:no], reach

    def distance(self, x, y, dist) -> float:
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        return float(self.L.orc_distance(_p(x), _p(y), _i(x.shape[0]), _i(DIST_CODES[dist])))

    # whole fits ----------------------------------------------------------------
    def fit_sdbscan(self, X, eps, minPts, *, dist="Cosine", n_proj=1024, topK=10, topM=50, ker=1024,
                    sigma=1.0, L=0.4, seed=42, threads=-1, clusterNoise=0, samplingProb=0.01):
        """The reference's fit_sDbscan restated (src/sDbscan.cpp:830-890), with its
        sDbscan-1NN noise labelling for clusterNoise = 1 (seeded sampling)."""
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        ker = d if dist == "Cosine" else ker
        fd = fht_dim(n_proj, ker)
        bits = self.hd3_bits(3 * fd, seed)
        R = self._R(dist, ker, d, sigma, seed)
        labels = np.zeros(n, np.int32)
        core = np.zeros(n, np.uint8)
        times = np.zeros(5, np.float64)
        ncl = self.L.orc_fit_sdbscan(_p(X), _i(n), _i(d), _i(DIST_CODES[dist]), _i(n_proj), _i(topK), _i(topM),
                                     _i(ker), _f(L), _p(R), _p(bits), _i(fd), _f(eps), _i(minPts), _i(threads),
                                     _i(clusterNoise), _f(samplingProb), ctypes.c_uint32(seed & 0xFFFFFFFF),
                                     _p(labels), _p(core), _p(times))
        if ncl < 0:
            raise ValueError(_fit_error(-ncl))
        return labels, ncl, core, times

    def fit_sngdbscan(self, X, eps, minPts, *, dist="Cosine", samplingProb=0.01, seed=42, threads=-1):
        """The reference's fit_sngDbscan restated point by point
        (src/sDbscan.cpp:416-504, 1131-1179).  Returns (labels, n_clusters,
        core, degree, times)."""
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        if seed < 0:
            raise ValueError("the oracle needs a seed >= 0 (a clock seed cannot be reproduced)")
        labels = np.zeros(n, np.int32)
        core = np.zeros(n, np.uint8)
        deg = np.zeros(n, np.int32)
        times = np.zeros(5, np.float64)
        ncl = self.L.orc_fit_sngdbscan(_p(X), _i(n), _i(d), _i(DIST_CODES[dist]), _f(samplingProb), _i(seed),
                                       _f(eps), _i(minPts), _i(threads), _p(labels), _p(core), _p(deg), _p(times))
        if ncl < 0:
            raise ValueError(_fit_error(-ncl))
        return labels, ncl, core, deg, times

    def fit_sngoptics(self, X, eps, minPts, *, dist="Cosine", samplingProb=0.01, seed=42, threads=-1):
        """sngOptics with the engine's shared seeded sample (src/sDbscan.cpp:1484-1583,
        1846-1880).  Returns (ordering, reachability, core, core_dist, degree, times)."""
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        ordering = np.zeros(n, np.int32)
        reach = np.zeros(n, np.float32)
        core = np.zeros(n, np.uint8)
        cd = np.zeros(n, np.float32)
        deg = np.zeros(n, np.int32)
        times = np.zeros(5, np.float64)
        r = self.L.orc_fit_sngoptics(_p(X), _i(n), _i(d), _i(DIST_CODES[dist]), _f(samplingProb), _i(seed),
                                     _f(eps), _i(minPts), _i(threads), _p(ordering), _p(reach), _p(core), _p(cd),
                                     _p(deg), _p(times))
        if r < 0:
            raise ValueError(_fit_error(-r))
        return ordering, reach, core, cd, deg, times

    def fit_sngdbscan_blocks(self, X, eps, minPts, *, dist="Cosine", samplingProb=0.01, seed=42, block_rows=32,
                             threads=-1):
        """sngDbscan under the block-sampled rule (each block of block_rows
        points draws its own sample; block_rows = 1 is the reference's
        independent per-point sampling in law).  Returns (labels, n_clusters,
        core, degree)."""
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        labels = np.zeros(n, np.int32)
        core = np.zeros(n, np.uint8)
        deg = np.zeros(n, np.int32)
        ncl = self.L.orc_fit_sngdbscan_blocks(_p(X), _i(n), _i(d), _i(DIST_CODES[dist]), _f(samplingProb),
                                              ctypes.c_uint32(seed & 0xFFFFFFFF), _i(block_rows), _f(eps),
                                              _i(minPts), _i(threads), _p(labels), _p(core), _p(deg))
        if ncl < 0:
            raise ValueError(f"rejected (code {-ncl})")
        return labels, ncl, core, deg

    def fit_sngoptics_blocks(self, X, eps, minPts, *, dist="Cosine", samplingProb=0.01, seed=42, block_rows=32,
                             threads=-1):
        """sngOptics under the block-sampled rule.  Returns (ordering,
        reachability, core, core_dist, degree)."""
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        ordering = np.zeros(n, np.int32)
        reach = np.zeros(n, np.float32)
        core = np.zeros(n, np.uint8)
        cd = np.zeros(n, np.float32)
        deg = np.zeros(n, np.int32)
        r = self.L.orc_fit_sngoptics_blocks(_p(X), _i(n), _i(d), _i(DIST_CODES[dist]), _f(samplingProb),
                                            ctypes.c_uint32(seed & 0xFFFFFFFF), _i(block_rows), _f(eps), _i(minPts),
                                            _i(threads), _p(ordering), _p(reach), _p(core), _p(cd), _p(deg))
        if r < 0:
            raise ValueError(f"rejected (code {-r})")
        return ordering, reach, core, cd, deg

    def fit_sdbscan_sweep(self, X, eps_list, minPts, *, dist="Cosine", n_proj=1024, topK=10, topM=50, ker=1024,
                          sigma=1.0, L=0.4, seed=42, threads=-1):
        """The reference's index-once sweep restated (test_sDbscan, src/sDbscan.cpp:980-1039)."""
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        ker = d if dist == "Cosine" else ker
        fd = fht_dim(n_proj, ker)
        bits = self.hd3_bits(3 * fd, seed)
        R = self._R(dist, ker, d, sigma, seed)
        eps = np.ascontiguousarray(eps_list, np.float32)
        labels = np.zeros((len(eps), n), np.int32)
        ncl = np.zeros(len(eps), np.int32)
        times = np.zeros(5, np.float64)
        r = self.L.orc_fit_sdbscan_sweep(_p(X), _i(n), _i(d), _i(DIST_CODES[dist]), _i(n_proj), _i(topK), _i(topM),
                                         _i(ker), _f(L), _p(R), _p(bits), _i(fd), _p(eps), _i(len(eps)),
                                         _i(minPts), _i(threads), _p(labels), _p(ncl), _p(times))
        if r < 0:
            raise ValueError(_fit_error(-r))
        return labels, ncl, times

    def label_noise(self, P, topK, core, labels, samplingProb, seed):
        """labelNoise (clusterNoise = 1, src/sDbscan.cpp:648-807) on given projections,
        top-k rows, core flags and labels (returns the new labels)."""
        P = np.ascontiguousarray(P, np.float32)
        n, nproj = P.shape
        out = np.ascontiguousarray(labels, np.int32).copy()
        self.L.orc_label_noise(_p(P), _i(n), _i(nproj), _p(np.ascontiguousarray(topK, np.int32)),
                               _i(topK.shape[1] // 2), _p(np.ascontiguousarray(core, np.uint8)), _f(samplingProb),
                               ctypes.c_uint32(seed & 0xFFFFFFFF), _p(out))
        return out

    def fit_soptics(self, X, eps, minPts, *, dist="Cosine", n_proj=1024, topK=10, topM=50, ker=1024,
                    sigma=1.0, L=0.4, seed=42, threads=-1, tie_mode=1):
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        ker = d if dist == "Cosine" else ker
        fd = fht_dim(n_proj, ker)
        bits = self.hd3_bits(3 * fd, seed)
        R = self._R(dist, ker, d, sigma, seed)
        order = np.zeros(n, np.int32)
        reach = np.zeros(n, np.float32)
        core = np.zeros(n, np.uint8)
        cd = np.zeros(n, np.float32)
        times = np.zeros(5, np.float64)
        rc = self.L.orc_fit_soptics(_p(X), _i(n), _i(d), _i(DIST_CODES[dist]), _i(n_proj), _i(topK), _i(topM),
                                    _i(ker), _f(L), _p(R), _p(bits), _i(fd), _f(eps), _i(minPts), _i(threads),
                                    _i(tie_mode), _p(order), _p(reach), _p(core), _p(cd), _p(times))
        if rc < 0:
            raise ValueError(_fit_error(-rc))
        return order, reach, core, cd, times

    def _R(self, dist, ker, d, sigma, seed):
        if dist == "L2":
            return self.gauss(ker // 2, d, 0.0, 1.0 / sigma, seed)
        if dist == "L1":
            return self.cauchy(ker // 2, d, 0.0, 1.0 / sigma, seed)
        return None


def ref_load_txt(path, n: int, d: int, so: str = REF_SO) -> np.ndarray:
    """The reference's own text loader (loadtxtData) on a file of n lines of d
    numbers; (n, d) float32."""
    out = np.zeros((n, d), np.float32)
    ctypes.CDLL(so).ref_load_txt(str(path).encode(), _i(n), _i(d), _p(out))
    return out


class Ref:
    """The reference class itself (oracle/_ref), via oracle/ref_harness.cpp."""

    def __init__(self, n: int, d: int, path: str = REF_SO):
        L = ctypes.CDLL(path)
        L.ref_new.restype = _vp
        for f in ("ref_n_clusters", "ref_bits_size", "ref_R_rows", "ref_R_cols"):
            getattr(L, f).restype = _i
        L.ref_ordering_size.restype = _i64
        self.L = L
        self.n, self.d = n, d
        self.h = _vp(L.ref_new(_i(n), _i(d)))
        self.k = self.m = self.nproj = None

    def __del__(self):
        try:
            self.L.ref_free(self.h)
        except Exception:
            pass

    def set_params(self, n_proj=1024, topK=10, topM=50, distance="Cosine", ker_n_features=1024, ker_sigma=1.0,
                   ker_intervalSampling=0.4, clusterNoise=0, samplingProb=0.01, verbose=False, n_threads=1,
                   random_seed=42):
        self.k, self.m, self.nproj = topK, topM, n_proj
        self.L.ref_set_params(self.h, _i(n_proj), _i(topK), _i(topM), distance.encode(), _i(ker_n_features),
                              _f(ker_sigma), _f(ker_intervalSampling), _i(clusterNoise), _f(samplingProb),
                              _i(1 if verbose else 0), _i(n_threads), _i(random_seed))

    def fit_sDbscan(self, X, eps, minPts):
        X = np.ascontiguousarray(X, np.float32)
        self.L.ref_fit_sdbscan(self.h, _p(X), _i(self.n), _i(self.d), _f(eps), _i(minPts))

    def fit_sOptics(self, X, eps, minPts):
        X = np.ascontiguousarray(X, np.float32)
        self.L.ref_fit_soptics(self.h, _p(X), _i(self.n), _i(self.d), _f(eps), _i(minPts))

    def test_sDbscan(self, X, eps, rangeEps, n_tests, minPts, prefix):
        """The reference's index-once sweep; writes one labels file per eps."""
        X = np.ascontiguousarray(X, np.float32)
        self.L.ref_test_sdbscan(self.h, _p(X), _i(self.n), _i(self.d), _f(eps), _f(rangeEps), _i(n_tests),
                                _i(minPts), str(prefix).encode())

    def set_sngParams(self, distance="Cosine", samplingProb=0.01, clusterNoise=0, verbose=False, n_threads=1,
                      random_seed=42):
        self.L.ref_set_sng_params(self.h, distance.encode(), _f(samplingProb), _i(clusterNoise),
                                  _i(1 if verbose else 0), _i(n_threads), _i(random_seed))

    def fit_sngDbscan(self, X, eps, minPts):
        X = np.ascontiguousarray(X, np.float32)
        self.L.ref_fit_sngdbscan(self.h, _p(X), _i(self.n), _i(self.d), _f(eps), _i(minPts))

    def fit_sngOptics(self, X, eps, minPts):
        X = np.ascontiguousarray(X, np.float32)
        self.L.ref_fit_sngoptics(self.h, _p(X), _i(self.n), _i(self.d), _f(eps), _i(minPts))

    @property
    def labels_(self):
        out = np.zeros(self.n, np.int32)
        self.L.ref_labels(self.h, _p(out))
        return out

    @property
    def n_clusters_(self):
        return self.L.ref_n_clusters(self.h)

    @property
    def ordering_(self):
        out = np.zeros(self.L.ref_ordering_size(self.h), np.int32)
        self.L.ref_ordering(self.h, _p(out))
        return out

    @property
    def reachability_(self):
        out = np.zeros(self.n, np.float32)
        self.L.ref_reachability(self.h, _p(out))
        return out

    def topK(self):
        out = np.zeros((self.n, 2 * self.k), np.int32)
        self.L.ref_topk(self.h, _p(out))
        return out

    def topM(self):
        out = np.zeros((self.nproj, 2 * self.m), np.int32)
        self.L.ref_topm(self.h, _p(out))
        return out

    def core(self):
        out = np.zeros(self.n, np.uint8)
        self.L.ref_core(self.h, _p(out))
        return out

    def core_dist(self):
        out = np.zeros(self.n, np.float32)
        self.L.ref_core_dist(self.h, _p(out))
        return out

    def bits(self):
        out = np.zeros(self.L.ref_bits_size(self.h), np.uint8)
        self.L.ref_bits(self.h, _p(out))
        return out

    def R(self):
        r, c = self.L.ref_R_rows(self.h), self.L.ref_R_cols(self.h)
        out = np.zeros(r * c, np.float32)
        if r * c:
            self.L.ref_R(self.h, _p(out))
        return out

    def X(self):
        out = np.zeros((self.n, self.d), np.float32)
        self.L.ref_matrix_X(self.h, _p(out))
        return out

    def projections(self):
        out = np.zeros((self.n, self.nproj), np.float32)
        self.L.ref_project(self.h, _p(out))
        return out

    def neighbors(self):
        sizes = np.zeros(self.n, np.int64)
        self.L.ref_neighbor_sizes(self.h, _p(sizes))
        flat = np.zeros(int(sizes.sum()), np.int32)
        self.L.ref_neighbors(self.h, _p(flat))
        off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        return off, flat

    def neighbor_dist(self):
        sizes = np.zeros(self.n, np.int64)
        self.L.ref_neighbor_dist_sizes(self.h, _p(sizes))
        idx = np.zeros(int(sizes.sum()), np.int32)
        dd = np.zeros(int(sizes.sum()), np.float32)
        self.L.ref_neighbor_dist(self.h, _p(idx), _p(dd))
        off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        return off, idx, dd
