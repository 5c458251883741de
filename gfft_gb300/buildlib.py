"""Build the in-tree shared library ``gfft_gb300/libgfft_gb300.so`` for sm_103a.

Translation units are compiled in parallel with nvcc (CUDA sources) and g++
(host planner), then linked with the static CUDA runtime.  Objects go to
``gfft_gb300/_build/``; the library is written next to this file so the
package loads it from the tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgfft_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + CSRC, "-I" + INCLUDE] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-I" + CSRC, "-I" + INCLUDE]

CUDA_SOURCES = ["fft_engine.cu", "fft_fast.cu", "fft_spec.cu", "fft_lane.cu", "fft_tc.cu", "fft_mixed.cu", "fft_col.cu", "fft_col_real.cu", "fft_colmix.cu", "gfft_capi.cu", "gfft_dct.cu", "gfft_nd.cu", "gfft_noalloc.cu", "gfft_ragged.cu", "gfft_tune.cu", "gfft_peak.cu"]
CXX_SOURCES = ["planner.cpp", "colshape.cpp", "capi_host.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout[-4000:], r.stderr[-8000:]))
    return r.stdout + r.stderr


def lib_path(debug: bool = False) -> str:
    """The release library, or the debug build (-DGFFT_DEBUG: device-side
    bounds checks that record GFFT_E_BOUNDS instead of accessing memory)."""
    return os.path.join(HERE, "libgfft_gb300_debug.so") if debug else LIB


def _sources():
    out = []
    for f in os.listdir(CSRC):
        if f.endswith((".cu", ".cuh", ".h", ".cpp")):
            out.append(os.path.join(CSRC, f))
    out.append(os.path.join(INCLUDE, "gfft_gb300.h"))
    out.append(__file__)
    return out


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> str:
    lib = lib_path(debug)
    if not force and not _stale(lib):
        return lib
    bdir = BUILD + ("_debug" if debug else "")
    os.makedirs(bdir, exist_ok=True)
    nv = nvcc()
    dflag = ["-DGFFT_DEBUG"] if debug else []
    jobs, objs = [], []
    for s in CUDA_SOURCES:
        o = os.path.join(bdir, s + ".o")
        objs.append(o)
        extra = ["-Xptxas", "-v"] if verbose else []
        jobs.append([nv, *NVCC_FLAGS, *dflag, *extra, "-c", os.path.join(CSRC, s), "-o", o])
    for s in CXX_SOURCES:
        o = os.path.join(bdir, s + ".o")
        objs.append(o)
        jobs.append(["g++", *CXX_FLAGS, *dflag, "-c", os.path.join(CSRC, s), "-o", o])
    with ThreadPoolExecutor(len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            sys.stdout.write(lg)
    tmp = lib + ".tmp"
    _run([nv, *ARCH, "-shared", "-cudart", "static", *objs, "-o", tmp])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, debug="--debug" in sys.argv))
