"""Generate the golden fixtures from the compiled reference (scpp/gfft).

Run in a container that holds the reference tree (it builds oracle/_ref from
the reference's own headers first):

    python tests/golden/make_golden.py

Writes ``tests/golden/reference_outputs.json``: for every (value type,
transform, place, N) the reference instantiates (oracle/ref_driver.cpp), the
SHA-256 of the reference's output bytes on the seeded input, the reference's
per-level root constants (so that the CPU restatement can be checked bit for
bit), and a few summary numbers.  ``reference_arrays.npz`` holds full output
arrays for a handful of small cases.

Inputs: uniform[-1,1) from gfft_gb300.inputs.uniform with seed 0x5EED0000 + N,
2N scalars, rounded to float32 for the single-precision types.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gfft_gb300 import inputs  # noqa: E402
from oracle import build as obuild  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

SIZES = [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 3, 9, 27, 81, 243, 729, 2187, 5, 25,
         125, 625, 3125, 7, 49, 343, 2401, 11, 13, 121, 6, 10, 12, 15, 18, 20, 24, 30, 36, 45, 48, 60,
         72, 96, 100, 120, 144, 192, 210, 240, 360, 384, 480, 500, 768, 1000, 1536, 2000, 3000, 3072,
         524288, 786432, 390625, 248832]
VTYPES = ["DOUBLE", "FLOAT", "COMPLEX_DOUBLE", "COMPLEX_FLOAT"]
ARRAY_CASES = [("DOUBLE", 0, 1, 16), ("DOUBLE", 0, 1, 60), ("DOUBLE", 1, 0, 243), ("FLOAT", 0, 1, 120),
               ("DOUBLE", 2, 0, 64), ("DOUBLE", 3, 0, 64), ("FLOAT", 2, 0, 128), ("COMPLEX_DOUBLE", 0, 1, 48),
               ("COMPLEX_FLOAT", 1, 1, 100), ("DOUBLE", 0, 1, 1024)]


def seed_for(n):
    return 0x5EED0000 + n


def main():
    if obuild.build_ref() is None:
        raise SystemExit("reference tree not found: fixtures cannot be regenerated here")
    ref = po.ref_lib()
    entries = []
    arrays = {}
    for vt in VTYPES:
        dt = np.float64 if vt in ("DOUBLE", "COMPLEX_DOUBLE") else np.float32
        fn = getattr(ref, "ref_exec_" + vt)
        for n in SIZES:
            x = inputs.uniform(seed_for(n), 2 * n).astype(dt)
            for trans in range(4):
                for place in (0, 1):
                    y = np.zeros_like(x)
                    if fn(n, trans, place, x.ctypes.data, y.ctypes.data) < 0:
                        continue
                    e = {"vtype": vt, "trans": trans, "place": place, "n": n, "seed": seed_for(n),
                         "sha256": po.digest(y), "absmax": float(np.max(np.abs(y))),
                         "sumsq": float(np.sum(y.astype(np.float64) ** 2))}
                    if vt in ("DOUBLE", "FLOAT"):
                        S = 1 if trans in (0, 2) else -1
                        re = np.zeros(64)
                        im = np.zeros(64)
                        nl = getattr(ref, "ref_roots_" + vt)(n, S, re.ctypes.data, im.ctypes.data)
                        e["roots_re"] = [float.hex(float(v)) for v in re[:nl]]
                        e["roots_im"] = [float.hex(float(v)) for v in im[:nl]]
                    entries.append(e)
                    if (vt, trans, place, n) in ARRAY_CASES:
                        arrays["%s_%d_%d_%d" % (vt, trans, place, n)] = y
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_outputs.json")
    with open(out, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "reference": "scpp/gfft v0.32 (Serial objects)",
                   "flags": "g++ -std=c++14 -O2 -ffp-contract=off (x86-64)", "entries": entries}, f, indent=0)
    np.savez_compressed(os.path.join(os.path.dirname(out), "reference_arrays.npz"), **arrays)
    print("wrote %d entries, %d arrays" % (len(entries), len(arrays)))


if __name__ == "__main__":
    main()
