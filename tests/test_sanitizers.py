"""CPU: the host code built with AddressSanitizer and UndefinedBehaviorSanitizer
(the planner, the host side of the C ABI and the oracle), run over a sweep
of plans and small oracle transforms (tests/cpp/sanitize_host.cpp).  Any
out-of-bounds access, leak, overflow of a signed integer or other undefined
behaviour aborts the program."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "gfft_gb300", "csrc")
SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g", "-O1"]


def _have(tool):
    return shutil.which(tool) is not None


@pytest.mark.skipif(not (_have("g++") and _have("gcc")), reason="needs gcc / g++")
def test_host_code_under_sanitizers():
    with tempfile.TemporaryDirectory() as d:
        objs = []
        for src, cc, std in ((os.path.join(ROOT, "oracle", "oracle_exact.c"), "gcc", "-std=gnu11"),):
            o = os.path.join(d, os.path.basename(src) + ".o")
            subprocess.run([cc, std, *SAN, "-ffp-contract=off", "-c", src, "-o", o], check=True)
            objs.append(o)
        cxx = [os.path.join(CSRC, "planner.cpp"), os.path.join(CSRC, "colshape.cpp"),
               os.path.join(CSRC, "capi_host.cpp"), os.path.join(ROOT, "oracle", "gfft_restate.cpp"),
               os.path.join(ROOT, "tests", "cpp", "sanitize_host.cpp")]
        for src in cxx:
            o = os.path.join(d, os.path.basename(src) + ".o")
            std = "-std=c++14" if src.endswith("gfft_restate.cpp") else "-std=c++17"
            subprocess.run(["g++", std, *SAN, "-ffp-contract=off", "-fopenmp", "-I" + CSRC,
                            "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", o], check=True)
            objs.append(o)
        exe = os.path.join(d, "sanitize_host")
        subprocess.run(["g++", *SAN, "-fopenmp", *objs, "-o", exe, "-lm"], check=True)
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1",
                   UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1", OMP_NUM_THREADS="2")
        r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-6000:])
        assert "0 failures" in r.stdout
