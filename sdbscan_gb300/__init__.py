"""sdbscan_gb300 — GB300-native (sm_103a) sDbscan / sOPTICS engine.

A drop-in for the fit path of NinhPham/sDbscan: the `sDbscan` class's
set_params / fit_sDbscan / fit_sOptics with labels_, n_clusters_, ordering_
and reachability_.  Compute runs in hand-written CUDA kernels behind the C ABI
of include/sdbscan_gb300.h.

    from sdbscan_gb300 import sDbscan          # pybind11 module, reference names
    dbs = sDbscan.sDbscan(n, d)
    dbs.set_params(n_proj=1024, topK=10, topM=50, distance="Cosine", random_seed=42)
    dbs.fit_sDbscan(X_dxn, eps, minPts)        # X: (d, n) float32
    dbs.labels_, dbs.n_clusters_

`sdbscan_gb300.capi.Engine` drives the same C ABI through ctypes.
"""
import importlib
import os

__all__ = ["capi", "datasets"]


def __getattr__(name):
    if name == "sDbscan":
        mod = importlib.import_module(".sDbscan", __name__)
        globals()["sDbscan"] = mod
        return mod
    if name in ("capi", "datasets"):
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)


def lib_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "libsdbscan_gb300.so")
