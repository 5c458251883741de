"""GPU: the allocation-free entry point (gfft_exec_noalloc) against the
regular one (gfft_exec), through the C ABI.

gfft_exec_noalloc serves callers that may not allocate device memory when
they transform (fixed-memory real-time code, plugins inside applications
that own all allocations): its workspace and twiddle tables live in one
fixed device array.  Each case runs two calls in a row, with different
inputs, and checks both against gfft_exec on the same input; the array's
leftovers from the first call must not leak into the second.
"""
import ctypes

import numpy as np
import pytest

from gfft_gb300 import inputs

pytestmark = pytest.mark.gpu


def tol(n, dbl):
    return (2e-15 if dbl else 6e-7) * max(1.0, np.log2(max(n, 2)))


def rel(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b.astype(np.float64)) /
                 max(np.linalg.norm(b.astype(np.float64)), 1e-300))


# (n, double?, batch, in place?)
CASES = [(65536, 0, 4, False), (1 << 20, 0, 1, False), (12288, 1, 3, False), (1 << 21, 0, 1, True),
         (390625, 1, 2, False), (8192, 1, 2, True), (4096, 0, 16, False), (3 * 2 ** 14, 1, 1, True)]


def _regular(torch, n, dbl, tr, batch, x):
    from gfft_gb300 import gfft as G
    obj = G.TransformObject(n, G.DOUBLE if dbl else G.FLOAT, G.DFT if tr == 0 else G.IDFT, batch=batch)
    out = torch.empty_like(x)
    obj.fft(x, out)
    torch.cuda.synchronize()
    obj.close()
    return out.cpu().numpy()


def _noalloc(lib, torch, n, dbl, tr, batch, x, inplace):
    y = x.clone() if inplace else torch.empty_like(x)
    src = y if inplace else x
    st = lib.gfft_exec_noalloc(n, 0 if dbl else 1, tr, batch, ctypes.c_void_p(src.data_ptr()),
                               ctypes.c_void_p(y.data_ptr()), None)
    torch.cuda.synchronize()
    return st, y.cpu().numpy()


@pytest.mark.parametrize("case", CASES, ids=lambda c: "n%d-%s-b%d-%s" % (c[0], "f64" if c[1] else "f32", c[2],
                                                                           "inplace" if c[3] else "oop"))
def test_noalloc_matches_regular_entry_point(cuda, case):
    from gfft_gb300 import _lib
    torch = cuda
    lib = _lib.lib()
    n, dbl, batch, inplace = case
    dt = torch.float64 if dbl else torch.float32
    for tr in (0, 1):
        for call, seed in enumerate((11, 12)):  # two calls in a row, different data
            x = torch.from_numpy(inputs.uniform(seed * 1000 + n, 2 * n * batch)).to(dt).cuda()
            want = _regular(torch, n, dbl, tr, batch, x)
            st, got = _noalloc(lib, torch, n, dbl, tr, batch, x, inplace)
            assert st == 0, (case, tr, call, _lib.strerror(st))
            assert rel(got, want) <= tol(n, dbl), (case, tr, call, rel(got, want))


def test_noalloc_leaves_device_memory_alone(cuda):
    """After the first call (which looks up the array), calls change no
    device allocation."""
    from gfft_gb300 import _lib
    torch = cuda
    lib = _lib.lib()
    n, batch = 1 << 18, 2
    x = torch.from_numpy(inputs.uniform(5, 2 * n * batch)).float().cuda()
    y = torch.empty_like(x)
    assert lib.gfft_exec_noalloc(n, 1, 0, batch, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                 None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert lib.gfft_exec_noalloc(n, 1, 0, batch, ctypes.c_void_p(x.data_ptr()),
                                     ctypes.c_void_p(y.data_ptr()), None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_beyond_capacity(cuda):
    from gfft_gb300 import _lib
    torch = cuda
    lib = _lib.lib()
    x = torch.zeros(16, device="cuda", dtype=torch.float32)
    p = ctypes.c_void_p(x.data_ptr())
    # 2^23 complex FP32 = 64 MiB fits; one transform more does not
    assert lib.gfft_exec_noalloc(1 << 23, 1, 0, 2, p, p, None) == 15
    assert lib.gfft_exec_noalloc(1 << 24, 0, 0, 1, p, p, None) == 15
    assert lib.gfft_exec_noalloc(1024, 1, 2, 1, p, p, None) == 3  # real transforms are not offered
    assert lib.gfft_exec_noalloc(0, 1, 0, 1, p, p, None) == 1
    assert lib.gfft_exec_noalloc(64, 1, 0, 1, None, p, None) == 7
