"""GPU: the debug build (libgfft_gb300_debug.so, -DGFFT_DEBUG), in which the
column-tile and engine kernels test every checked shared- and global-memory
index before the access and record GFFT_E_BOUNDS (16) instead of touching
memory.  Small transforms of every kernel family run through it in a child
process; their results must match the exact oracle and leave no failed check
behind.  The check itself is exercised by one failing check with no access
behind it (gfft_selftest_bounds_check)."""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import ctypes, sys
    import numpy as np, torch
    sys.path.insert(0, %r)
    from gfft_gb300 import _lib, gfft as G, inputs
    from oracle import pyoracle
    L = _lib.lib()
    assert L.gfft_debug_build() == 1
    st, line = ctypes.c_int(), ctypes.c_int()
    _lib.check(L.gfft_selftest_bounds_check(ctypes.byref(st), ctypes.byref(line)))
    assert st.value == 16 and line.value > 0, (st.value, line.value)
    cases = [(4096, 1, 0, 3, None), (1 << 16, 1, 0, 2, None), (1 << 20, 1, 0, 1, None), (1 << 13, 0, 0, 2, None),
             (1 << 19, 0, 2, 1, None), (1 << 19, 0, 3, 1, None), (1 << 14, 1, 2, 2, None), (3 * 2 ** 14, 1, 0, 2, None),
             (1000, 0, 0, 3, {"kernel_variant": 1}), (5 ** 6, 1, 0, 2, None), (1 << 16, 1, 0, 2, {"decimation": 1}),
             (12288, 0, 1, 2, {"kernel_variant": 4}), (3 * 2 ** 18, 1, 0, 1, None), (5 ** 8, 1, 1, 1, None),
             (360 * 360, 1, 0, 1, None), (1 << 18, 1, 1, 2, {"blocks_per_sm": 2}), (8192, 1, 0, 3, None)]
    for n, vt, tr, b, opts in cases:
        dt = np.float64 if vt == 0 else np.float32
        x = inputs.gaussian(n + tr, 2 * n * b).astype(dt)
        obj = G.TransformObject(n, G.VALUE_TYPES[vt], G.TRANSFORM_TYPES[tr], 1, G.Serial, G.OUT_OF_PLACE, b, opts)
        xt = torch.from_numpy(x).cuda()
        y = torch.empty_like(xt)
        obj.fft(xt, y)
        torch.cuda.synchronize()
        s = ctypes.c_int(-1)
        _lib.check(L.gfft_get_device_status(obj._h, ctypes.byref(s)))
        assert s.value == 0, (n, vt, tr, opts, s.value)
        got = y.cpu().numpy().astype(np.float64)
        if tr in (0, 1):
            ex = pyoracle.fft_ld(x.astype(np.float64), n, b, 1 if tr == 0 else -1)
            err = np.linalg.norm(got - ex) / np.linalg.norm(ex)
            assert err <= (2e-15 if vt == 0 else 6e-7) * np.log2(n), (n, tr, err)
        obj.close()
    print("debug build ok")
""") % ROOT


def test_debug_build_bounds_checks(cuda):
    from gfft_gb300 import buildlib
    buildlib.build(debug=True)
    env = dict(os.environ, GFFT_GB300_DEBUG="1")
    r = subprocess.run([sys.executable, "-c", CHILD], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "debug build ok" in r.stdout
