"""GPU: multi-dimensional complex transforms (gfft_create_nd, and gfft_create
with dim = 2 / 3) against the long-double oracle applied along every axis.

Tolerance: the 1-D bound of the total length (FP64 2e-15 log2 N, FP32
6e-7 log2 N, N = product of the dims)."""
import numpy as np
import pytest

from gfft_gb300 import inputs

pytestmark = pytest.mark.gpu


def tol(n, dbl):
    return (2e-15 if dbl else 6e-7) * max(1.0, np.log2(max(n, 2)))


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def exact_nd(oracle, x, dims, batch, sign):
    """Interleaved float64 -> interleaved: the oracle's 1-D FFT along each axis."""
    c = (x[0::2] + 1j * x[1::2]).reshape((batch,) + tuple(dims))
    for ax in range(1, len(dims) + 1):
        m = np.moveaxis(c, ax, -1)
        shp = m.shape
        flat = np.ascontiguousarray(m).reshape(-1, shp[-1])
        inter = np.empty(2 * flat.size)
        inter[0::2], inter[1::2] = flat.real.ravel(), flat.imag.ravel()
        y = oracle.fft_ld(inter, shp[-1], flat.shape[0], sign)
        m = (y[0::2] + 1j * y[1::2]).reshape(shp)
        c = np.moveaxis(m, -1, ax)
    out = np.empty(2 * c.size)
    out[0::2], out[1::2] = c.real.ravel(), c.imag.ravel()
    return out


def run_nd(torch, dims, dbl, trans, place, x, batch):
    from gfft_gb300 import gfft as G
    obj = G.TransformND(dims, G.DOUBLE if dbl else G.FLOAT, G.TRANSFORM_TYPES[trans], G.PLACES[place], batch)
    src = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if place == 0:
        obj.fft(src)
        out = src
    else:
        out = torch.empty_like(src)
        obj.fft(src, out)
    torch.cuda.synchronize()
    r = out.cpu().numpy()
    obj.close()
    return r


SHAPES = [(8, 8), (64, 48), (5, 7, 9), (256, 256), (3, 1000), (1000, 3), (16, 32, 64), (1, 64), (12, 1, 10),
          (1024, 1024), (3, 5, 4096)]


@pytest.mark.parametrize("dbl", [1, 0])
@pytest.mark.parametrize("dims", SHAPES)
def test_nd_vs_oracle(cuda, oracle, dims, dbl):
    batch = 2
    total = int(np.prod(dims))
    dt = np.float64 if dbl else np.float32
    x = inputs.uniform(9000 + total, 2 * total * batch).astype(dt)
    for trans, sign in ((0, 1), (1, -1)):
        ex = exact_nd(oracle, x.astype(np.float64), dims, batch, sign)
        for place in (1, 0):
            y = run_nd(cuda, dims, dbl, trans, place, x, batch)
            assert rel(y, ex) <= tol(total, dbl), (dims, trans, place, rel(y, ex))


def test_nd_long_outer_axes(cuda, oracle):
    """Outer axes of a full tile (4096 FP32, 2048 FP64) and a rejected longer one."""
    from gfft_gb300 import _lib
    from gfft_gb300 import gfft as G
    for dims, dbl in (((4096, 6), 0), ((2048, 6), 1)):
        total = int(np.prod(dims))
        x = inputs.uniform(31 + total, 2 * total).astype(np.float64 if dbl else np.float32)
        ex = exact_nd(oracle, x.astype(np.float64), dims, 1, 1)
        y = run_nd(cuda, dims, dbl, 0, 1, x, 1)
        assert rel(y, ex) <= tol(total, dbl)
    with pytest.raises(_lib.GfftError):
        G.TransformND((8192, 4), G.FLOAT)


def test_create_with_dim(cuda, oracle):
    """gfft_create(n, ..., dim = 2) is the n x n transform."""
    import ctypes

    from gfft_gb300 import _lib
    n = 48
    x = inputs.uniform(5, 2 * n * n)
    h = ctypes.c_void_p()
    _lib.check(_lib.lib().gfft_create(ctypes.byref(h), n, 0, 0, 2, 0, 1, 1))
    src = cuda.from_numpy(x).cuda()
    dst = cuda.empty_like(src)
    _lib.check(_lib.lib().gfft_exec(h, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()), None))
    cuda.cuda.synchronize()
    _lib.lib().gfft_destroy(h)
    ex = exact_nd(oracle, x, (n, n), 1, 1)
    assert rel(dst.cpu().numpy(), ex) <= tol(n * n, 1)
