"""Build recipes for the oracle (test infrastructure only).

- ``build_oracle()`` compiles the CPU restatement (gfft_restate.cpp) and the
  exact references (oracle_exact.c) into ``oracle/liboracle.so``.
- ``build_ref()`` compiles scpp/gfft's own headers, from where they lie in the
  reference tree, together with the two stand-in headers under
  ``oracle/refshim/`` (the reference's ``metafactor`` submodule is an empty
  directory), into ``oracle/_ref/libgfftref.so``.  It does nothing when the
  reference tree is absent.

Both use -ffp-contract=off so that no multiply-add is fused: the restatement
and the compiled reference then round identically on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: $GFFT_REFERENCE_ROOT, else a directory named
# `reference` beside this repository's checkout; absent on machines that only
# run the prebuilt fixtures.
REF_ROOT = os.environ.get("GFFT_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgfftref.so")
# a copy of the reference's headers (src/*.h, loki/*.h), made where the
# checkout exists, for machines that have only this working tree
# (git-ignored, never committed)
REF_STAGE = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "gfft")
REF_BENCH = os.path.join(HERE, "_ref", "ref_bench")

_CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fopenmp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr[-4000:]))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "oracle_exact.c"), os.path.join(HERE, "gfft_restate.cpp")]
    if not force and not _stale(ORACLE_SO, srcs + [__file__]):
        return ORACLE_SO
    bdir = os.path.join(HERE, "_build")
    os.makedirs(bdir, exist_ok=True)
    o1 = os.path.join(bdir, "oracle_exact.o")
    o2 = os.path.join(bdir, "gfft_restate.o")
    jobs = [
        ["gcc", "-std=gnu11", *_CFLAGS, "-c", srcs[0], "-o", o1],
        ["g++", "-std=c++14", *_CFLAGS, "-c", srcs[1], "-o", o2],
    ]
    with ThreadPoolExecutor(2) as ex:
        list(ex.map(_run, jobs))
    tmp = ORACLE_SO + ".tmp"
    _run(["g++", "-shared", "-fopenmp", o1, o2, "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force: bool = False) -> str | None:
    src_dir = os.path.join(REF_ROOT, "src")
    if not os.path.isdir(src_dir):
        return None
    drv = os.path.join(HERE, "ref_driver.cpp")
    shims = [os.path.join(HERE, "refshim", f) for f in ("sint.h", "metafactor.h")]
    if not force and not _stale(REF_SO, [drv, __file__] + shims):
        return REF_SO
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "refshim"), "-I", src_dir, "-I", os.path.join(REF_ROOT, "loki")]
    objs, jobs = [], []
    for vt in ("DOUBLE", "FLOAT", "COMPLEX_DOUBLE", "COMPLEX_FLOAT"):
        o = os.path.join(out_dir, "ref_%s.o" % vt.lower())
        objs.append(o)
        jobs.append(["g++", "-std=c++14", "-O2", "-fPIC", "-ffp-contract=off", "-w",
                     "-ftemplate-depth=100000", "-DREF_VTYPE=" + vt,
                     "-DREF_ROOTS=%d" % (vt in ("DOUBLE", "FLOAT")), *inc, "-c", drv, "-o", o])
    with ThreadPoolExecutor(4) as ex:
        list(ex.map(_run, jobs))
    tmp = REF_SO + ".tmp"
    _run(["g++", "-shared", *objs, "-o", tmp])
    os.replace(tmp, REF_SO)
    return REF_SO


def stage_ref() -> str | None:
    """Copy the reference's headers next to this tree (baseline/_ref/gfft),
    so that the benchmark's CPU arm can compile the reference where the
    checkout is absent.  Does nothing without the checkout."""
    if not os.path.isdir(os.path.join(REF_ROOT, "src")):
        return None
    for sub in ("src", "loki"):
        src = os.path.join(REF_ROOT, sub)
        dst = os.path.join(REF_STAGE, sub)
        os.makedirs(dst, exist_ok=True)
        for f in os.listdir(src):
            if f.endswith(".h"):
                shutil.copy2(os.path.join(src, f), os.path.join(dst, f))
    return REF_STAGE


def ref_include() -> list | None:
    """Include flags of the reference: the checkout if present, else the
    staged copy; None when neither exists."""
    for root in (REF_ROOT, REF_STAGE):
        if os.path.isdir(os.path.join(root, "src")) and os.path.isdir(os.path.join(root, "loki")):
            return ["-I", os.path.join(HERE, "refshim"), "-I", os.path.join(root, "src"), "-I",
                    os.path.join(root, "loki")]
    return None


def build_ref_bench(force: bool = False) -> str | None:
    """Compile ref_bench.cpp (the reference's serial objects, OpenMP over the
    batch) with -O3 -march=native -fopenmp into oracle/_ref/ref_bench; plain
    -O3 where the compiler rejects -march=native.  None without the
    reference's headers."""
    inc = ref_include()
    if inc is None:
        return None
    drv = os.path.join(HERE, "ref_bench.cpp")
    if not force and not _stale(REF_BENCH, [drv, __file__]):
        return REF_BENCH
    os.makedirs(os.path.dirname(REF_BENCH), exist_ok=True)
    base = ["g++", "-std=c++14", "-O3", "-fopenmp", "-w", "-ftemplate-depth=100000", *inc, drv, "-o",
            REF_BENCH + ".tmp"]
    try:
        _run(base[:3] + ["-march=native"] + base[3:])
    except RuntimeError:
        _run(base)
    os.replace(REF_BENCH + ".tmp", REF_BENCH)
    return REF_BENCH


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
