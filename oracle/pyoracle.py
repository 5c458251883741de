"""ctypes front end of the oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module; the product (``gfft_gb300``) never does.

Wraps ``oracle/liboracle.so`` (built by ``oracle/build.py``):
- ``gfft(n, vtype, trans, place, x, roots=None)``: the CPU restatement of the
  reference's algorithm (bit-exact with the compiled reference when its level
  roots are given);
- ``gfft_batch``: the same over a batch with OpenMP (the timed CPU baseline);
- ``dft_q``: binary128 direct DFT (double-double result);
- ``fft_ld``: long-double mixed-radix FFT with exact twiddles;
- ``rdft_q``: binary128 direct real DFT in the reference's packed layout;
- ``gen_uniform``: seeded splitmix64 uniform[-1,1) generator.
"""
from __future__ import annotations

import ctypes
import hashlib
import os

import numpy as np

from . import build as _build

_lib = None

VT_DOUBLE, VT_FLOAT, VT_COMPLEX_DOUBLE, VT_COMPLEX_FLOAT = 0, 1, 2, 3
DFT, IDFT, RDFT, IRDFT = 0, 1, 2, 3
IN_PLACE, OUT_OF_PLACE = 0, 1


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        i64, ci, vp, dp = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p
        L.orc_gfft_exec.argtypes = [i64, ci, ci, ci, vp, vp]
        L.orc_gfft_exec_roots.argtypes = [i64, ci, ci, ci, vp, vp, ci, dp, dp]
        L.orc_gfft_exec_batch.argtypes = [i64, i64, ci, ci, ci, vp, vp, ci]
        L.orc_dft_q.argtypes = [i64, dp, dp, dp, ci]
        L.orc_dft_bins_q.argtypes = [i64, dp, i64, vp, dp, ci]
        L.orc_fft_ld.argtypes = [i64, i64, dp, dp, ci]
        L.orc_rdft_q.argtypes = [i64, dp, dp]
        L.orc_dct_q.argtypes = [i64, ci, dp, dp]
        L.orc_gen_uniform.argtypes = [ctypes.c_uint64, i64, dp]
        L.orc_num_threads.restype = ci
        _lib = L
    return _lib


def _scalar(vtype):
    return np.float64 if vtype in (VT_DOUBLE, VT_COMPLEX_DOUBLE) else np.float32


def gfft(n, vtype, trans, place, x, roots=None):
    """One reference transform object applied to interleaved ``x`` (2n scalars)."""
    dt = _scalar(vtype)
    x = np.ascontiguousarray(x, dtype=dt)
    y = np.zeros_like(x)
    vt = 0 if dt == np.float64 else 1
    if roots is None:
        st = lib().orc_gfft_exec(n, vt, trans, place, x.ctypes.data, y.ctypes.data)
    else:
        re = np.ascontiguousarray(roots[0], dtype=np.float64)
        im = np.ascontiguousarray(roots[1], dtype=np.float64)
        st = lib().orc_gfft_exec_roots(n, vt, trans, place, x.ctypes.data, y.ctypes.data, len(re),
                                       re.ctypes.data, im.ctypes.data)
    if st != 0:
        raise ValueError("oracle rejected n=%d trans=%d place=%d (status %d)" % (n, trans, place, st))
    return y


def gfft_batch(n, batch, vtype, trans, place, x, y=None, nthreads=0):
    dt = _scalar(vtype)
    x = np.ascontiguousarray(x, dtype=dt)
    if y is None:
        y = np.zeros_like(x)
    vt = 0 if dt == np.float64 else 1
    st = lib().orc_gfft_exec_batch(n, batch, vt, trans, place, x.ctypes.data, y.ctypes.data, nthreads)
    if st != 0:
        raise ValueError("oracle rejected n=%d (status %d)" % (n, st))
    return y


def num_threads():
    return lib().orc_num_threads()


def dft_q(x, sign=1, lo=False):
    """binary128 direct DFT of interleaved complex double ``x``."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.size // 2
    hi = np.zeros_like(x)
    lw = np.zeros_like(x) if lo else None
    lib().orc_dft_q(n, x.ctypes.data, hi.ctypes.data, lw.ctypes.data if lo else None, sign)
    return (hi, lw) if lo else hi


def dft_bins_q(x, bins, sign=1):
    x = np.ascontiguousarray(x, dtype=np.float64)
    b = np.ascontiguousarray(bins, dtype=np.int64)
    out = np.zeros(2 * b.size)
    lib().orc_dft_bins_q(x.size // 2, x.ctypes.data, b.size, b.ctypes.data, out.ctypes.data, sign)
    return out


def fft_ld(x, n, batch=1, sign=1):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(2 * n * batch)
    lib().orc_fft_ld(n, batch, x.ctypes.data, y.ctypes.data, sign)
    return y


def rdft_q(x):
    """Direct DFT of 2n reals, packed X_0, X_n, X_1 .. X_{n-1}."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().orc_rdft_q(x.size // 2, x.ctypes.data, y.ctypes.data)
    return y


def dct_q(x, dct_type):
    """Direct cosine transform of the reference's direct.h (type 1 or 2) of
    the n reals ``x``, binary128 accumulation."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().orc_dct_q(x.size, int(dct_type), x.ctypes.data, y.ctypes.data)
    return y


def gen_uniform(seed, count):
    y = np.zeros(count)
    lib().orc_gen_uniform(seed, count, y.ctypes.data)
    return y


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_lib():
    """The compiled reference (oracle/_ref), or None where it was not built."""
    path = _build.REF_SO
    if not os.path.exists(path):
        return None
    L = ctypes.CDLL(path)
    for nm in ("DOUBLE", "FLOAT", "COMPLEX_DOUBLE", "COMPLEX_FLOAT"):
        f = getattr(L, "ref_exec_" + nm)
        f.argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    for nm in ("DOUBLE", "FLOAT"):
        f = getattr(L, "ref_roots_" + nm)
        f.argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return L
