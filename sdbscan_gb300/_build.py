"""Builds the engine in-tree: every CUDA translation unit of csrc/ compiled in
parallel for sm_103a, linked into ``sdbscan_gb300/libsdbscan_gb300.so``; the
pybind11 drop-in module ``sDbscan`` (when pybind11 headers are available, e.g.
the copy bundled with PyTorch) links against it."""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsdbscan_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_lib(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    objs, jobs = [], []
    for src in sources:
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


def _pybind_include() -> str | None:
    try:
        import pybind11  # noqa: F401
        return pybind11.get_include()
    except Exception:
        pass
    try:
        import torch  # noqa: F401
        inc = os.path.join(os.path.dirname(torch.__file__), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    except Exception:
        pass
    return None


def build_pymodule() -> str | None:
    """The drop-in Python module `sDbscan` (same names as the reference's
    python/python_wrapper.cpp), linked against the engine library."""
    inc = _pybind_include()
    if inc is None:
        return None
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    target = os.path.join(PKG, "sDbscan" + suffix)
    srcs = [os.path.join(CSRC, "host", "sDbscan.cpp"), os.path.join(CSRC, "host", "python_module.cpp")]
    hdrs = [os.path.join(CSRC, "host", "sDbscan.h"), os.path.join(ROOT, "include", "sdbscan_gb300.h")]
    if not _stale(target, srcs + hdrs + [LIB]):
        return target
    cxx = os.environ.get("CXX", "g++")
    py_inc = sysconfig.get_paths()["include"]
    _run([cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden", f"-I{inc}", f"-I{py_inc}",
          f"-I{os.path.join(ROOT, 'include')}", *srcs, "-o", target, f"-L{PKG}", "-lsdbscan_gb300",
          "-Wl,-rpath,$ORIGIN"])
    return target


def build(verbose: bool = False) -> None:
    build_lib(verbose)
    build_pymodule()


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
