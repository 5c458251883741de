"""Compile tests/cpp/facade_test.cpp against include/gfft.h and the in-tree
library (test helper)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def build():
    from gfft_gb300 import buildlib
    lib = buildlib.build()
    out = os.path.join(ROOT, "gfft_gb300", "_build", "facade_test")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    src = os.path.join(HERE, "facade_test.cpp")
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(src), os.path.getmtime(lib),
                                                               os.path.getmtime(os.path.join(ROOT, "include",
                                                                                             "gfft.h"))):
        subprocess.run(["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", out,
                        "-L", os.path.dirname(lib), "-lgfft_gb300", "-Wl,-rpath," + os.path.dirname(lib)],
                       check=True, capture_output=True, text=True)
    return out
