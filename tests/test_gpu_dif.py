"""Frequency decimation (plan option decimation = 1) through the C ABI: the
transposed Stockham passes, last to first, twiddles after the butterflies
(the reference's InFreq / T_DFTk_x_Im, src/gfftalgfreq.h:106-432, unused by
its own factory).  Against the exact oracle within the benchmark spec's bounds
(relative L2: FP64 <= 2e-15 log2 N, FP32 <= 6e-7 log2 N) and against the
time-decimation plan on the same input."""
import numpy as np
import pytest

from gfft_gb300 import inputs

pytestmark = pytest.mark.gpu
DIF = {"decimation": 1}


def tol(n, dbl):
    return (2e-15 if dbl else 6e-7) * max(1.0, np.log2(max(n, 2)))


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run(torch, n, vt, tr, pl, x, batch=1, opts=None):
    from gfft_gb300 import gfft as G
    obj = G.TransformObject(n, G.VALUE_TYPES[vt], G.TRANSFORM_TYPES[tr], 1, G.Serial, G.PLACES[pl], batch, opts)
    src = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if pl == 0:
        obj.fft(src)
        out = src
    else:
        out = torch.empty_like(src)
        obj.fft(src, out)
    torch.cuda.synchronize()
    r = out.cpu().numpy()
    obj.close()
    return r


SIZES = [2, 8, 16, 60, 64, 97, 1000, 1009, 4096, 8192, 3 * 2 ** 14, 5 ** 6, 1 << 20]


@pytest.mark.parametrize("dbl", [1, 0])
@pytest.mark.parametrize("n", SIZES)
def test_dif_vs_exact_and_dit(cuda, oracle, n, dbl):
    from gfft_gb300 import _lib
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    B = 3 if n <= 4096 else 1
    info = _lib.plan_query(n, vt, 0, 1, B, DIF)
    assert set(info["kernel_variant"]) == {1}, info
    x = inputs.gaussian(41 + n, 2 * n * B).astype(dt)
    for tr in (0, 1):
        y = run(cuda, n, vt, tr, 1, x, batch=B, opts=DIF)
        ex = oracle.fft_ld(x.astype(np.float64), n, B, 1 if tr == 0 else -1)
        assert rel(y, ex) <= tol(n, dbl), (n, tr, rel(y, ex))
        dit = run(cuda, n, vt, tr, 1, x, batch=B)
        assert rel(y, dit) <= 2 * tol(n, dbl)
        inp = run(cuda, n, vt, tr, 0, x, batch=B, opts=DIF)
        assert np.array_equal(y, inp), (n, tr)


@pytest.mark.parametrize("n,dbl", [(1 << 22, 0), (1 << 12, 1), (1 << 19, 1)])
def test_dif_multipass_and_real(cuda, n, dbl):
    """Three-pass FP32 and real transforms (packed spectrum against numpy's
    FP64 real DFT, inverse round trip) with frequency decimation."""
    from gfft_gb300 import _lib
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    x = inputs.uniform(7 + n, 2 * n).astype(dt)
    if n == 1 << 22:
        assert _lib.plan_query(n, vt, 0, 1, 1, DIF)["n_global_passes"] == 3
        y = run(cuda, n, vt, 0, 1, x, opts=DIF)
        dit = run(cuda, n, vt, 0, 1, x)
        assert rel(y, dit) <= 2 * tol(n, dbl)
        back = run(cuda, n, vt, 1, 1, y, opts=DIF)
        assert rel(back, x) <= 2 * tol(n, dbl)
        return
    y = run(cuda, n, vt, 2, 1, x, opts=DIF)
    f = np.fft.rfft(x.astype(np.float64))
    want = np.empty(2 * n)
    want[0], want[1] = f[0].real, f[n].real
    want[2::2], want[3::2] = f[1:n].real, f[1:n].imag
    assert rel(y, want) <= tol(2 * n, dbl)
    z = run(cuda, n, vt, 3, 1, y, opts=DIF)
    assert rel(z, x) <= 2 * tol(2 * n, dbl)
