"""Tensor-copy column tiles (plan option kernel_variant = 9), the default for
multi-pass power-of-two lengths, through the C ABI.

Against the exact oracle (long-double FFT with exact twiddles) within the
spec bounds FP64 <= 2e-15 log2 N and FP32 <= 6e-7 log2 N (relative L2),
and against the generic engine (variant 1) and the specialised column tiles
(variant 5) on the same inputs; in place must equal out of place bit for bit.
"""
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


def run(torch, n, vt, tr, pl, x, batch=1, opts=None, offset=0):
    """One transform object; `offset` shifts the device buffers by that many
    scalars (8 bytes for FP32 complex: aligned to the element, not to 16)."""
    from gfft_gb300 import gfft as G
    obj = G.TransformObject(n, G.VALUE_TYPES[vt], G.TRANSFORM_TYPES[tr], 1, G.Serial, G.PLACES[pl], batch, opts)
    m = x.size
    src_all = torch.zeros(m + 8, dtype=torch.float64 if x.dtype == np.float64 else torch.float32, device="cuda")
    src = src_all[offset:offset + m]
    src.copy_(torch.from_numpy(np.ascontiguousarray(x)))
    if pl == 0:
        obj.fft(src)
        out = src
    else:
        out_all = torch.zeros_like(src_all)
        out = out_all[offset:offset + m]
        obj.fft(src, out)
    torch.cuda.synchronize()
    r = out.cpu().numpy()
    obj.close()
    return r


CASES = [(1 << 13, 1, 2), (1 << 14, 1, 5), (1 << 15, 0, 3), (1 << 16, 0, 2), (1 << 17, 0, 2),
         (1 << 18, 0, 2), (1 << 19, 0, 1), (1 << 20, 0, 2), (1 << 21, 0, 1), (1 << 22, 0, 1), (1 << 16, 1, 3),
         (1 << 19, 1, 1), (1 << 20, 1, 1), (1 << 22, 1, 1)]


@pytest.mark.parametrize("n,dbl,B", CASES)
def test_col_vs_exact_and_engine(cuda, oracle, n, dbl, B):
    from gfft_gb300 import _lib
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    info = _lib.plan_query(n, vt, 0, 1, B)
    P = info["n_global_passes"]
    assert P >= 2 and info["kernel_variant"][:P] == [9] * P, info
    x = inputs.gaussian(3 + n + B, 2 * n * B).astype(dt)
    for tr in (0, 1):
        y = run(cuda, n, vt, tr, 1, x, batch=B)
        gen = run(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 1})
        assert rel(y, gen) <= tol(n, dbl), (n, tr, rel(y, gen))
        inp = run(cuda, n, vt, tr, 0, x, batch=B)
        assert np.array_equal(y, inp), (n, tr)
        if n <= 1 << 20:
            k = min(B, 2)
            ex = oracle.fft_ld(x[:2 * n * k].astype(np.float64), n, k, 1 if tr == 0 else -1)
            assert rel(y[:2 * n * k], ex) <= tol(n, dbl), (n, tr, rel(y[:2 * n * k], ex))


@pytest.mark.parametrize("n,opts", [(1 << 24, None), (1 << 24, {"max_pass_len": 4096}), (1 << 23, None),
                                    (1 << 23, {"max_pass_len": 4096}), (1 << 13, {"max_pass_len": 4096})])
def test_col_large_fp32(cuda, oracle, n, opts):
    """2^23 / 2^24 in three passes (default) or two with a 4096-point pass,
    and 2^13 as two passes: against the specialised column tiles and, on
    sampled bins, the binary128 direct sum."""
    from gfft_gb300 import _lib
    info = _lib.plan_query(n, 1, 0, 1, 1, opts)
    P = info["n_global_passes"]
    assert info["kernel_variant"][:P] == [9] * P, info
    if opts:
        assert max(info["pass_len"][:P]) == min(4096, n // 64) or n == 1 << 13, info
    x = (inputs.gaussian(11 + n, 2 * n) + inputs.tone_mix(11 + n, n, 1)).astype(np.float32)
    y = run(cuda, n, 1, 0, 1, x, opts=opts)
    ref = run(cuda, n, 1, 0, 1, x, opts={"kernel_variant": 5})
    assert rel(y, ref) <= tol(n, 0), rel(y, ref)
    if n <= 1 << 20:
        ex = oracle.fft_ld(x.astype(np.float64), n, 1, 1)
        assert rel(y, ex) <= tol(n, 0)
    else:
        c = x.astype(np.float64)[0::2] + 1j * x.astype(np.float64)[1::2]
        rng = np.random.default_rng(n)
        ks = rng.integers(0, n, 6)
        nn = np.arange(n, dtype=np.int64)
        scale = np.sqrt(n)
        for k in ks:
            ph = np.exp(-2j * np.pi * ((int(k) * nn) % n) / n)
            want = np.sum(c * ph)
            got = complex(y[2 * k], y[2 * k + 1])
            assert abs(got - want) <= 6e-7 * np.log2(n) * scale * 8, (k, got, want)
    back = run(cuda, n, 1, 1, 1, y, opts=opts)
    assert rel(back, x) <= 2 * tol(n, 0)


@pytest.mark.parametrize("n", [1 << 16, 1 << 22, 3 * 2 ** 18, 5 ** 8])
def test_col_unaligned_buffers(cuda, n):
    """FP32 buffers aligned to one complex element (8 bytes) but not to 16:
    plans with tensor copies run through the handle's second plan (column
    tiles of variant 5 / the engine), gathered mixed-radix tiles (5^8) run
    as they are; the same result within tolerance, repeatably."""
    x = inputs.gaussian(29 + n, 2 * n).astype(np.float32)
    a = run(cuda, n, 1, 0, 1, x)
    b = run(cuda, n, 1, 0, 1, x, offset=2)
    assert rel(a, b) <= tol(n, 0)
    b2 = run(cuda, n, 1, 0, 1, x, offset=2)
    assert np.array_equal(b, b2)


@pytest.mark.parametrize("n,B", [(1 << 15, 3), (1 << 16, 2), (1 << 17, 2), (1 << 18, 2), (1 << 19, 1),
                                 (1 << 23, 1)])
def test_col_half_tiles(cuda, oracle, n, B):
    """FP32 passes of 128 .. 512 run 32 KB tiles by default (half the units
    of the 64 KB tiles that blocks_per_sm = 1 keeps): against the exact
    oracle (up to 2^19) and the 64 KB plan, forward and inverse, in and out
    of place."""
    from gfft_gb300 import _lib
    one = {"blocks_per_sm": 1}
    d1 = _lib.plan_query(n, 1, 0, 1, B, one)
    d = _lib.plan_query(n, 1, 0, 1, B)
    P = d["n_global_passes"]
    assert d["kernel_variant"][:P] == [9] * P, d
    for g in range(P):
        if 128 <= d["pass_len"][g] <= 512:
            assert 2 * d["units"][g] == d1["units"][g] and d["threads"][g] == 256, (d, d1)
    x = inputs.gaussian(41 + n + B, 2 * n * B).astype(np.float32)
    for tr in (0, 1):
        y = run(cuda, n, 1, tr, 1, x, batch=B)
        ref = run(cuda, n, 1, tr, 1, x, batch=B, opts=one)
        assert rel(y, ref) <= tol(n, 0), (n, tr, rel(y, ref))
        inp = run(cuda, n, 1, tr, 0, x, batch=B)
        assert np.array_equal(y, inp), (n, tr)
        if n > 1 << 19:
            continue
        ex = oracle.fft_ld(x.astype(np.float64), n, B, 1 if tr == 0 else -1)
        assert rel(y, ex) <= tol(n, 0), (n, tr, rel(y, ex))


@pytest.mark.parametrize("n,B", [(1 << 19, 2), (1 << 20, 1), (1 << 21, 1)])
def test_col_half_tiles_1024(cuda, oracle, n, B):
    """blocks_per_sm = 2 extends the 32 KB tiles to FP32 passes of 1024 (4
    units, 32-byte rows): against the default plan and, up to 2^20, the
    exact oracle, forward and inverse."""
    from gfft_gb300 import _lib
    two = {"blocks_per_sm": 2}
    d = _lib.plan_query(n, 1, 0, 1, B, two)
    P = d["n_global_passes"]
    assert 1024 in d["pass_len"][:P], d
    for g in range(P):
        if d["pass_len"][g] == 1024:
            assert d["units"][g] == 4 and d["threads"][g] == 256, d
    x = inputs.gaussian(43 + n + B, 2 * n * B).astype(np.float32)
    for tr in (0, 1):
        y = run(cuda, n, 1, tr, 1, x, batch=B, opts=two)
        ref = run(cuda, n, 1, tr, 1, x, batch=B)
        assert rel(y, ref) <= tol(n, 0), (n, tr, rel(y, ref))
        if n <= 1 << 20:
            ex = oracle.fft_ld(x.astype(np.float64), n, B, 1 if tr == 0 else -1)
            assert rel(y, ex) <= tol(n, 0), (n, tr, rel(y, ex))


REAL = [(1 << 19, 1, 2, 0), (1 << 19, 1, 3, 1), (1 << 13, 1, 3, 1), (1 << 14, 0, 2, 1), (1 << 16, 0, 2, 0),
        (1 << 17, 1, 1, 1), (1 << 20, 0, 1, 1), (1 << 21, 0, 1, 1), (1 << 23, 0, 1, 1)]


@pytest.mark.parametrize("n,dbl,B,pl", REAL)
def test_col_real_transforms(cuda, n, dbl, B, pl):
    """Real transforms of 2n reals whose complex half-length n runs through
    variant 9, with the real post pass fused into the last pass (RDFT) and
    the pre pass into the first (IRDFT) where the tiles fit: forward against
    numpy's FP64 real DFT in the packed layout (X_0, X_n, X_1 .. X_{n-1}),
    against the unfused plan (column tiles of variant 5 and the separate real
    pass), and the inverse round trip; in and out of place."""
    from gfft_gb300 import _lib
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    for tr in (2, 3):
        d = _lib.plan_query(n, vt, tr, pl, B)
        if (n, dbl, tr) != (1 << 21, 0, 3):  # an FP32 first pass of 2048 keeps the separate pre pass
            assert d["real_fused"] == 1 and d["kernels_per_exec"] == d["n_global_passes"], d
    x = inputs.uniform(5 + n + B, 2 * n * B).astype(dt)
    y = run(cuda, n, vt, 2, pl, x, batch=B)
    for t in range(B):
        f = np.fft.rfft(x[2 * n * t:2 * n * (t + 1)].astype(np.float64))
        want = np.empty(2 * n)
        want[0], want[1] = f[0].real, f[n].real
        want[2::2], want[3::2] = f[1:n].real, f[1:n].imag
        got = y[2 * n * t:2 * n * (t + 1)]
        assert rel(got, want) <= tol(2 * n, dbl), (t, rel(got, want))
    unf = run(cuda, n, vt, 2, pl, x, batch=B, opts={"kernel_variant": 5})
    assert rel(y, unf) <= tol(2 * n, dbl)
    z = run(cuda, n, vt, 3, pl, y, batch=B)
    assert rel(z, x) <= 2 * tol(2 * n, dbl)
    zu = run(cuda, n, vt, 3, pl, y, batch=B, opts={"kernel_variant": 5})
    assert rel(z, zu) <= 2 * tol(2 * n, dbl)
