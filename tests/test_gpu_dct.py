"""GPU: cosine transforms (transform IDs 4-7) against the binary128 direct
sums of the reference's direct.h (oracle.dct_q).

Tolerance: relative L2 <= 2x the real-transform bound of length 2n (FP64
2e-15 log2(2n), FP32 6e-7 log2(2n)): a cosine transform is one real
transform of 2n (type 2) or 2(n-1) (type 1) reals plus O(1) work per output.
"""
import numpy as np
import pytest

from gfft_gb300 import inputs

pytestmark = pytest.mark.gpu


def tol(n, dbl):
    return 2 * (2e-15 if dbl else 6e-7) * max(1.0, np.log2(2 * max(n, 2)))


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)


def run(torch, n, vt, tr, pl, x, batch):
    from gfft_gb300 import gfft as G
    obj = G.TransformObject(n, G.VALUE_TYPES[vt], G.TRANSFORM_TYPES[tr], 1, G.Serial, G.PLACES[pl], batch)
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


@pytest.mark.parametrize("dbl", [1, 0])
@pytest.mark.parametrize("tr", [4, 5, 6, 7])
@pytest.mark.parametrize("n", [2, 3, 5, 8, 17, 64, 100, 257, 1000, 1024, 1025, 4097])
def test_dct_vs_direct_sum(cuda, oracle, n, tr, dbl):
    if tr in (4, 5) and n < 2:
        pytest.skip("type 1 needs two points")
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    B = 3
    x = inputs.uniform(6000 + n + tr, n * B).astype(dt)
    kind = 1 if tr in (4, 5) else 2
    ex = np.concatenate([oracle.dct_q(x[b * n:(b + 1) * n].astype(np.float64), kind) for b in range(B)])
    if tr in (5, 7):
        ex = ex / n
    for pl in (1, 0):
        y = run(cuda, n, vt, tr, pl, x, B)
        assert rel(y, ex) <= tol(n, dbl), (n, tr, pl, rel(y, ex))


def test_dct_large_and_host_path(cuda, oracle):
    """A 2^20-point DCT2 in FP32 (sampled outputs against direct sums of the
    oracle on a reduced problem would not be exact, so: DCT2 of a cosine
    is a pair of spikes) and the host-pointer entry point on a small case."""
    from gfft_gb300 import gfft as G
    n = 1 << 20
    k0 = 12345
    l = np.arange(n)
    # x_l = cos(pi k0 l / n): X_k = sum_l cos(pi k0 l/n) cos(pi k l/n), largest at k = k0
    x = np.cos(np.pi * ((k0 * l) % (2 * n)) / n).astype(np.float32)
    y = run(cuda, n, 1, 6, 1, x, 1)
    assert int(np.argmax(np.abs(y))) == k0
    assert abs(y[k0] - n / 2) <= 1e-3 * n
    # host arrays through gfft_exec_host
    m, B = 300, 2
    xh = inputs.uniform(77, m * B)
    obj = G.TransformObject(m, G.DOUBLE, G.DCT1, 1, G.Serial, G.OUT_OF_PLACE, B)
    yh = np.empty_like(xh)
    obj.fft(xh, yh)
    obj.close()
    ex = np.concatenate([oracle.dct_q(xh[b * m:(b + 1) * m], 1) for b in range(B)])
    assert rel(yh, ex) <= tol(m, 1)
