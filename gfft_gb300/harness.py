"""The reference's accuracy and performance harnesses, run against this
library, so that a user of the reference can compare like with like.

- ``accuracy`` follows ``test/gfft_accuracy.cpp`` with ``GFFTcheck``
  (``test/gfft_accuracy.h:150-270``): for N = base^p, p in [pmin, pmax], one
  forward DFT of 2N inputs uniform in [-0.5, 0.5) (the reference draws them
  with ``rand()`` from seed 17, ``src/direct.h:43-51``; here a seeded
  splitmix64 stream), compared with a direct DFT in extended precision (the
  reference uses double-double, here long double with the angle reduced
  exactly); per N the 2-norm and the max-norm of the difference and the
  max-norm relative to the max-norm of the result; the summary line is the
  largest relative error, ``PLACE, TYPE, base^[pmin,pmax]: err``.
- ``matrix`` is ``test_accuracy.sh``: every value type x both places x
  {2^[2,11], 3^[2,7], 5^[2,4], 7^[2,3]}.
- ``performance`` follows ``test/gfft_performance.cpp`` with ``GFFTbench``
  (``test/gfft_performance.h:60-140``): N = 2^6 .. 2^9, DOUBLE and
  COMPLEX_DOUBLE, forward, out of place; ``it = 10^6 / N + 1`` transforms per
  timing, best of three, time per transform in ns and 5 N log2 N / t.  The
  reference times ``it`` consecutive calls with ``clock()``; here the ``it``
  transforms are one batched launch on device-resident data, timed with CUDA
  events.

Usage: ``python -m gfft_gb300.harness accuracy --type DOUBLE --place IN_PLACE
--base 2 --pmin 2 --pmax 11 [--full]``, ``... matrix``, ``... performance``.
"""
from __future__ import annotations

import argparse
import math
import sys

import numpy as np

from . import gfft as G
from . import inputs

TYPES = {"DOUBLE": G.DOUBLE, "FLOAT": G.FLOAT, "COMPLEX_DOUBLE": G.COMPLEX_DOUBLE, "COMPLEX_FLOAT": G.COMPLEX_FLOAT}
PLACES = {"IN_PLACE": G.IN_PLACE, "OUT_OF_PLACE": G.OUT_OF_PLACE}
SWEEP = [(2, 2, 11), (3, 2, 7), (5, 2, 4), (7, 2, 3)]  # test_accuracy.sh: base, pmin, pmax


def direct_dft(x: np.ndarray) -> np.ndarray:
    """Forward DFT of interleaved complex ``x`` (float64), summed in long
    double with the angle index k n reduced modulo N in integers."""
    n = x.size // 2
    xr = x[0::2].astype(np.longdouble)
    xi = x[1::2].astype(np.longdouble)
    out = np.empty(2 * n)
    j = np.arange(n, dtype=np.int64)
    two_pi = np.longdouble(2) * np.arccos(np.longdouble(-1))
    chunk = max(1, (1 << 22) // max(n, 1))
    for k0 in range(0, n, chunk):
        k = np.arange(k0, min(n, k0 + chunk), dtype=np.int64)
        m = (k[:, None] * j[None, :]) % n
        ang = two_pi * m.astype(np.longdouble) / np.longdouble(n)
        c, s = np.cos(ang), np.sin(ang)
        re = (c * xr + s * xi).sum(axis=1)
        im = (c * xi - s * xr).sum(axis=1)
        out[2 * k] = re.astype(np.float64)
        out[2 * k + 1] = im.astype(np.float64)
    return out


_REF = {}


def check_one(n: int, vtype, place, seed: int = 17):
    """One GFFTcheck step: (N, norm2, norm_inf, relative norm_inf)."""
    dt = np.float64 if vtype in (G.DOUBLE, G.COMPLEX_DOUBLE) else np.float32
    x = (inputs.uniform(seed + n, 2 * n) * 0.5).astype(dt)
    key = (n, seed, dt)
    if key not in _REF:  # the same inputs serve both places and both layouts of a precision
        _REF[key] = direct_dft(x.astype(np.float64))
    ref = _REF[key]
    obj = G.TransformObject(n, vtype, G.DFT, 1, G.Serial, place, 1)
    if place is G.IN_PLACE:
        y = x.copy()
        obj.fft(y)
    else:
        y = np.zeros_like(x)
        obj.fft(x, y)
    obj.close()
    y = y.astype(np.float64)
    d = float(np.max(np.abs(y)))
    diff = y - ref
    nr2 = float(np.sqrt(np.sum(diff * diff)))
    nrinf = float(np.max(np.abs(diff)))
    return n, nr2, nrinf, nrinf / d


def accuracy(tname: str, pname: str, base: int, pmin: int, pmax: int, full: bool = False, out=sys.stdout):
    vtype, place = TYPES[tname], PLACES[pname]
    worst = 0.0
    if full:
        print("-" * 61, file=out)
        print(" N         Norm2           NormInf       Relative NormInf    ", file=out)
        print("-" * 61, file=out)
    for p in range(pmin, pmax + 1):
        n, nr2, nrinf, rel = check_one(base ** p, vtype, place)
        if full:
            print("%d\t%.4g\t%.4g\t%.4g" % (n, nr2, nrinf, rel), file=out)
        worst = max(worst, rel)
    print("%s, %s, %d^[%d,%d]: %.4g" % (pname, tname, base, pmin, pmax, worst), file=out)
    return worst


def matrix(full: bool = False, out=sys.stdout):
    """The sweep of test_accuracy.sh; returns {(type, place, base): max rel}."""
    res = {}
    for t in TYPES:
        print(">>>>> Value type: %s" % t, file=out)
        for p in PLACES:
            print(">>>>> Transform mode: %s" % p, file=out)
            for base, lo, hi in SWEEP:
                res[(t, p, base)] = accuracy(t, p, base, lo, hi, full, out)
    return res


def performance(pmin: int = 6, pmax: int = 9, types=("DOUBLE", "COMPLEX_DOUBLE"), out=sys.stdout):
    """GFFTbench: rows (direction, value type, place, threads, N, ns, GFLOP/s)."""
    import torch
    names_t = {G.DFT: " forward", G.IDFT: "backward"}
    names_v = {"DOUBLE": "    double    ", "FLOAT": "     float    ", "COMPLEX_DOUBLE": "complex double",
               "COMPLEX_FLOAT": " complex float"}
    print("-" * 91, file=out)
    print(" Direction        Value type          Place       N-threads    Length   Time [ns]    GFLOPS", file=out)
    print("-" * 91, file=out)
    rows = []
    for t in types:
        vtype = TYPES[t]
        dt = torch.float64 if vtype in (G.DOUBLE, G.COMPLEX_DOUBLE) else torch.float32
        for p in range(pmin, pmax + 1):
            n = 1 << p
            it = int(1000000.0 / n) + 1
            x = torch.rand(2 * n * it, device="cuda", dtype=dt).sub_(0.5)
            y = torch.empty_like(x)
            obj = G.TransformObject(n, vtype, G.DFT, 1, G.Serial, G.OUT_OF_PLACE, it)
            obj.fft(x, y)
            best = math.inf
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            for _ in range(3):
                torch.cuda.synchronize()
                e0.record()
                obj.fft(x, y)
                e1.record()
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            obj.close()
            ns = best * 1e6 / it
            gf = 5.0 * n * math.log2(n) / ns
            rows.append(("forward", t, "out-of-place", 1, n, ns, gf))
            print("%s\t%s\t%s\t%d\t%d\t%.5g \t%.5g" % (names_t[G.DFT], names_v[t], "  out-of-place  ", 1, n, ns, gf),
                  file=out)
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m gfft_gb300.harness")
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("accuracy")
    a.add_argument("--type", default="DOUBLE", choices=list(TYPES))
    a.add_argument("--place", default="OUT_OF_PLACE", choices=list(PLACES))
    a.add_argument("--base", type=int, default=2)
    a.add_argument("--pmin", type=int, default=2)
    a.add_argument("--pmax", type=int, default=11)
    a.add_argument("--full", action="store_true", help="per-N rows (the reference's FOUT build)")
    m = sub.add_parser("matrix")
    m.add_argument("--full", action="store_true")
    pf = sub.add_parser("performance")
    pf.add_argument("--pmin", type=int, default=6)
    pf.add_argument("--pmax", type=int, default=9)
    args = ap.parse_args(argv)
    if args.cmd == "accuracy":
        accuracy(args.type, args.place, args.base, args.pmin, args.pmax, args.full)
    elif args.cmd == "matrix":
        matrix(args.full)
    else:
        performance(args.pmin, args.pmax)


if __name__ == "__main__":
    main()
