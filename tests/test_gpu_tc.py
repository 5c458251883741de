"""The split-precision tensor-core form (plan option kernel_variant = 6)
against the exact oracle.

Bar: relative L2 error <= 1e-6 against the FP64/long-double oracle (the
precision target of the split form), with the plain FP32 path's error
measured beside it on the same input.  Inputs: seeded Gaussian N(0,1) plus a
1e-4-amplitude mix of 8 tones (the dynamic-range probe).
"""
import numpy as np
import pytest

from gfft_gb300 import inputs

pytestmark = pytest.mark.gpu

TC = {"kernel_variant": 6}
TOL_TC = 1e-6


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run(torch, n, tr, pl, x, batch=1, opts=None):
    from gfft_gb300 import gfft as G
    obj = G.TransformObject(n, G.FLOAT, G.TRANSFORM_TYPES[tr], 1, G.Serial, G.PLACES[pl], batch, opts)
    src = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda()
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


def probe_input(n, batch, seed):
    x = inputs.gaussian(seed, 2 * n * batch) + inputs.tone_mix(seed, n, batch)
    return x.astype(np.float32)


@pytest.mark.parametrize("n,batch", [(64, 7), (256, 100), (1024, 9), (4096, 33), (1 << 16, 2), (1 << 20, 1),
                                     (12288, 3), (1 << 24, 1)])
def test_tc_split_vs_oracle(cuda, oracle, n, batch):
    from gfft_gb300 import _lib
    info = _lib.plan_query(n, 1, 0, 1, batch, TC)
    assert 6 in info["kernel_variant"], info
    x = probe_input(n, batch, 0x5EED0003 + n)
    k = batch if n * batch <= 1 << 20 else 1
    ex = oracle.fft_ld(x[:2 * n * k].astype(np.float64), n, k, 1)
    y = run(cuda, n, 0, 1, x, batch, TC)
    e_tc = rel(y[:2 * n * k], ex)
    e_plain = rel(run(cuda, n, 0, 1, x[:2 * n * k], k), ex)
    print("tc-split n=%d batch=%d rel_l2 tc %.3e plain %.3e max_abs tc %.3e" %
          (n, batch, e_tc, e_plain, np.max(np.abs(y[:2 * n * k] - ex))))
    assert e_tc <= TOL_TC, (n, e_tc, e_plain)
    # inverse (with its 1/N) and in place
    exi = oracle.fft_ld(x[:2 * n * k].astype(np.float64), n, k, -1)
    yi = run(cuda, n, 1, 0, x, batch, TC)
    assert rel(yi[:2 * n * k], exi) <= TOL_TC, (n, rel(yi[:2 * n * k], exi))
    # the whole batch: every transform, forward then inverse, returns the input
    back = run(cuda, n, 1, 1, y, batch, TC)
    assert rel(back, x) <= 2 * TOL_TC


def test_tc_split_ragged_tiles(cuda, oracle):
    """256-point transforms, 16 per tile: a batch of 37 leaves a last tile of
    5; every transform matches the oracle."""
    n, batch = 256, 37
    x = probe_input(n, batch, 11)
    y = run(cuda, n, 0, 1, x, batch, TC)
    ex = oracle.fft_ld(x.astype(np.float64), n, batch, 1)
    for b in range(batch):
        s = slice(2 * n * b, 2 * n * (b + 1))
        assert rel(y[s], ex[s]) <= TOL_TC, b


def test_tc_split_is_deterministic_and_distinct(cuda):
    """Two runs agree bit for bit; the split form's rounding differs from the
    plain FP32 path's (the tensor-core path really ran)."""
    n, batch = 4096, 8
    x = probe_input(n, batch, 5)
    a = run(cuda, n, 0, 1, x, batch, TC)
    b = run(cuda, n, 0, 1, x, batch, TC)
    p = run(cuda, n, 0, 1, x, batch)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, p)


def test_tc_split_full_c3_config(cuda, oracle):
    """The precision configuration at full size: 65536 FP32 transforms of
    4096 points (2 GiB), Gaussian plus the 1e-4 tone mix, through the split
    form.  Sampled transforms against the long-double oracle at the 1e-6 bar,
    the plain FP32 path's error beside them on the same transforms, and the
    whole batch's Parseval ratio (sum |X|^2 / (N sum |x|^2) = 1)."""
    import torch
    from gfft_gb300 import gfft as G
    n, batch = 4096, 65536
    xt = torch.from_numpy(inputs.gaussian(0x5EED0003, 2 * n * batch, dtype=np.float32)).cuda()
    tone = torch.from_numpy(inputs.tone_mix(0x5EED0003, n, 1)).cuda()  # the same tones in every transform
    xt.view(batch, 2 * n).add_(tone.float())
    y = torch.empty_like(xt)
    G.TransformObject(n, G.FLOAT, G.DFT, 1, G.Serial, G.OUT_OF_PLACE, batch, TC).fft(xt, y)
    yp = torch.empty_like(xt)
    G.TransformObject(n, G.FLOAT, G.DFT, 1, G.Serial, G.OUT_OF_PLACE, batch).fft(xt, yp)
    torch.cuda.synchronize()
    for t in (0, 1, 4097, 33333, batch - 1):
        s = slice(2 * n * t, 2 * n * (t + 1))
        xs = xt[s].double().cpu().numpy()
        ex = oracle.fft_ld(xs, n, 1, 1)
        e_tc = rel(y[s].cpu().numpy(), ex)
        e_pl = rel(yp[s].cpu().numpy(), ex)
        assert e_tc <= TOL_TC, (t, e_tc, e_pl)
    ex2 = float(torch.sum(xt.double() ** 2))
    ey2 = float(torch.sum(y.double() ** 2))
    assert abs(ey2 / (n * ex2) - 1) <= 1e-5
