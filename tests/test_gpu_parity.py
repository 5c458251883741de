"""GPU parity: the CUDA path (through the C ABI) against the oracle.

Tolerances (relative L2 error against the exact oracle, binary128 DFT or
long-double FFT): FP64 <= 2e-15*log2(N), FP32 <= 6e-7*log2(N).  Against the
CPU restatement of the reference's algorithm the bound is that tolerance
plus the restatement's own measured error (the reference's twiddle
recurrences lose accuracy with N, to ~1e-11 in FP64 at 3*2^18).
"""
import json
import os
import platform

import numpy as np
import pytest

from gfft_gb300 import inputs

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def tol(n, dbl):
    return (2e-15 if dbl else 6e-7) * max(1.0, np.log2(max(n, 2)))


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)


def run_gpu(torch, n, vt, tr, pl, x, batch=1, opts=None):
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


def packed_rfft(x):
    """FP64 real DFT of 2n reals in the reference's packed layout."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size // 2
    f = np.fft.rfft(x)
    out = np.empty(2 * n)
    out[0], out[1] = f[0].real, f[n].real
    out[2::2], out[3::2] = f[1:n].real, f[1:n].imag
    return out


def exact(oracle, x, n, tr, batch=1):
    x = np.asarray(x, dtype=np.float64)
    if tr in (0, 1):
        s = 1 if tr == 0 else -1
        if n <= 512 and batch == 1:
            return oracle.dft_q(x, s)
        return oracle.fft_ld(x, n, batch, s)
    raise ValueError


SMALL = list(range(1, 65)) + [81, 96, 100, 121, 125, 128, 243, 256, 343, 360, 500, 512, 625, 729, 1000, 1024,
                                1536, 2048, 2187, 2401, 3000, 3072, 3125, 4096]
PRIMES = [11, 13, 17, 19, 23, 29, 31, 37, 41, 97, 127, 257, 1009]
MULTI = [8192, 12288, 15625, 16384, 65536, 3 * 2 ** 14, 2 ** 20, 5 ** 8]


@pytest.mark.parametrize("dbl", [1, 0])
@pytest.mark.parametrize("n", SMALL + PRIMES)
def test_c2c_vs_exact(cuda, oracle, n, dbl):
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    x = inputs.uniform(1000 + n, 2 * n).astype(dt)
    for tr in (0, 1):
        y = run_gpu(cuda, n, vt, tr, 1, x)
        ex = exact(oracle, x, n, tr)
        assert rel(y, ex) <= tol(n, dbl), (n, tr, rel(y, ex))


@pytest.mark.parametrize("dbl", [1, 0])
@pytest.mark.parametrize("n", MULTI)
def test_multipass_vs_exact(cuda, oracle, n, dbl):
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    x = inputs.gaussian(2000 + n, 2 * n).astype(dt)
    for tr in (0, 1):
        for pl in (1, 0):
            y = run_gpu(cuda, n, vt, tr, pl, x)
            ex = exact(oracle, x, n, tr)
            assert rel(y, ex) <= tol(n, dbl), (n, tr, pl, rel(y, ex))


@pytest.mark.parametrize("dbl", [1, 0])
@pytest.mark.parametrize("n", [16, 60, 243, 1024, 3000, 4096, 8192, 786432])
def test_vs_restatement(cuda, oracle, n, dbl):
    """Against the reference's own algorithm restated on the CPU."""
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    x = inputs.uniform(0x5EED0000 + n, 2 * n).astype(dt)
    ex = exact(oracle, x, n, 0)
    ref = oracle.gfft(n, vt, 0, 1, x)
    ref_err = rel(ref, ex)
    y = run_gpu(cuda, n, vt, 0, 1, x)
    assert rel(y, ref) <= tol(n, dbl) + 2 * ref_err, (n, rel(y, ref), ref_err)
    assert rel(y, ex) <= tol(n, dbl)


def test_golden_reference_arrays(cuda, oracle):
    """The compiled reference's stored outputs (DOUBLE/FLOAT objects)."""
    arr = np.load(os.path.join(GOLD, "reference_arrays.npz"))
    checked = 0
    for key in arr.files:
        vt_name, tr, pl, n = key.rsplit("_", 3)
        tr, pl, n = int(tr), int(pl), int(n)
        dbl = "DOUBLE" in vt_name
        dt = np.float64 if dbl else np.float32
        x = inputs.uniform(0x5EED0000 + n, 2 * n).astype(dt)
        vt = {"DOUBLE": 0, "FLOAT": 1, "COMPLEX_DOUBLE": 2, "COMPLEX_FLOAT": 3}[vt_name]
        y = run_gpu(cuda, n, vt, tr, pl, x)
        ref = arr[key]
        if vt >= 2 and tr < 2 and pl == 1 and n % 10 == 0:
            continue  # the reference's std::complex path is defective here (test_oracle.py)
        assert rel(y, ref) <= tol(n, dbl) * 4, (key, rel(y, ref))
        checked += 1
    assert checked >= 8


def test_golden_digests_match_within_tolerance(cuda, oracle):
    """For the fixture sizes the GPU result is within tolerance of the
    reference output (recomputed by the pinned restatement)."""
    with open(os.path.join(GOLD, "reference_outputs.json")) as f:
        entries = [e for e in json.load(f)["entries"] if e["vtype"] in ("DOUBLE", "FLOAT") and e["n"] <= 4096]
    for e in entries[::7]:
        dbl = e["vtype"] == "DOUBLE"
        dt = np.float64 if dbl else np.float32
        x = inputs.uniform(e["seed"], 2 * e["n"]).astype(dt)
        roots = ([float.fromhex(v) for v in e["roots_re"]], [float.fromhex(v) for v in e["roots_im"]])
        ref = oracle.gfft(e["n"], 0 if dbl else 1, e["trans"], e["place"], x, roots=roots)
        if platform.machine() == "x86_64":
            # fixtures were made on x86-64, where the reference's long double
            # TempType is 80-bit; on aarch64 it is binary128 and rounds differently
            assert oracle.digest(ref) == e["sha256"]
        y = run_gpu(cuda, e["n"], 0 if dbl else 1, e["trans"], e["place"], x)
        t = tol(e["n"], dbl) * 8
        assert rel(y, ref) <= t, (e["n"], e["trans"], e["place"], rel(y, ref))


@pytest.mark.parametrize("dbl", [1, 0])
@pytest.mark.parametrize("n", [1, 2, 4, 8, 16, 64, 256, 1024, 4096, 8192, 1 << 15, 1 << 19])
def test_real_forward_inverse(cuda, oracle, n, dbl):
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    x = inputs.uniform(3000 + n, 2 * n).astype(dt)
    y = run_gpu(cuda, n, vt, 2, 0, x)
    ex = oracle.rdft_q(x.astype(np.float64)) if n <= 256 else packed_rfft(x)
    assert rel(y, ex) <= tol(2 * n, dbl), (n, rel(y, ex))
    back = run_gpu(cuda, n, vt, 3, 0, y)
    assert rel(back, x) <= 2 * tol(2 * n, dbl), (n, rel(back, x))
    # against the restatement of the reference's IRDFT on the same spectrum
    ri = oracle.gfft(n, vt, 3, 0, y)
    assert rel(back, ri) <= 2 * tol(2 * n, dbl) + 2 * rel(ri, x)


@pytest.mark.parametrize("n", [6, 12, 48, 100, 1000, 3 * 1024, 12288])
def test_real_beyond_reference(cuda, oracle, n):
    """Non-power-of-two and out-of-place real transforms (the reference
    rejects both: src/gfftswap.h:282-286)."""
    x = inputs.uniform(4000 + n, 2 * n)
    ex = packed_rfft(x)
    for pl in (0, 1):
        y = run_gpu(cuda, n, 0, 2, pl, x)
        assert rel(y, ex) <= 4 * tol(2 * n, 1), (n, pl, rel(y, ex))
        back = run_gpu(cuda, n, 0, 3, pl, y)
        assert rel(back, x) <= 4 * tol(2 * n, 1)


def test_batch_equals_single(cuda, oracle):
    for n, dbl in ((1024, 1), (4096, 0), (60, 0), (12288, 1)):
        dt = np.float64 if dbl else np.float32
        vt = 0 if dbl else 1
        B = 5
        x = inputs.uniform(77 + n, 2 * n * B).astype(dt)
        yb = run_gpu(cuda, n, vt, 0, 1, x, batch=B)
        for b in range(B):
            ys = run_gpu(cuda, n, vt, 0, 1, x[2 * n * b:2 * n * (b + 1)])
            assert np.array_equal(ys, yb[2 * n * b:2 * n * (b + 1)]), (n, b)


def test_inplace_equals_outofplace(cuda):
    for n in (1024, 3000, 65536, 1 << 20):
        x = inputs.uniform(5 + n, 2 * n)
        a = run_gpu(cuda, n, 0, 0, 0, x)
        b = run_gpu(cuda, n, 0, 0, 1, x)
        assert np.array_equal(a, b)


def test_complex_dtypes_same_bytes(cuda):
    import torch
    from gfft_gb300 import gfft as G
    n = 1000
    x = inputs.uniform(9, 2 * n)
    a = run_gpu(cuda, n, 0, 0, 1, x)
    obj = G.TransformObject(n, G.COMPLEX_DOUBLE, G.DFT)
    src = torch.from_numpy(x).cuda().view(torch.complex128)
    dst = torch.empty_like(src)
    obj.fft(src, dst)
    b = dst.view(torch.float64).cpu().numpy()
    assert np.array_equal(a, b)


def test_plan_options_agree(cuda, oracle):
    """Every autotuner knob gives the same transform within tolerance."""
    n = 4096
    x = inputs.uniform(31, 2 * n * 3).astype(np.float32)
    ex = oracle.fft_ld(x, n, 3, 1)
    for opts in ({"max_radix": 8}, {"max_radix": 4}, {"max_radix": 2}, {"radix_order": 1},
                 {"threads_per_block": 128}, {"units_per_block": 2}, {"max_pass_len": 64}):
        y = run_gpu(cuda, n, 1, 0, 1, x, batch=3, opts=opts)
        assert rel(y, ex) <= tol(n, 0), (opts, rel(y, ex))


def test_host_entry_point(cuda, oracle):
    from gfft_gb300 import gfft as G
    n = 2048
    x = inputs.uniform(41, 2 * n)
    obj = G.TransformObject(n, G.DOUBLE, G.DFT)
    y = np.zeros_like(x)
    obj.fft(x, y)
    assert rel(y, oracle.fft_ld(x, n, 1, 1)) <= tol(n, 1)
    inp = G.TransformObject(n, G.DOUBLE, G.DFT, place=G.IN_PLACE)
    z = x.copy()
    inp.fft(z)
    assert np.array_equal(z, y)


def test_host_entry_point_chunked(cuda, oracle):
    """Host arrays of >= 64 MiB run the pipelined path (slices uploaded,
    transformed and downloaded on three streams); same result as the device
    path, in and out of place, with a ragged last slice."""
    import torch
    from gfft_gb300 import gfft as G
    for n, B, vt, tt, place in ((4096, 4099, G.FLOAT, G.DFT, G.OUT_OF_PLACE),
                                (1 << 19, 16, G.DOUBLE, G.RDFT, G.IN_PLACE),
                                (3 * 2 ** 18, 8, G.DOUBLE, G.IDFT, G.OUT_OF_PLACE)):
        dt = np.float64 if vt is G.DOUBLE else np.float32
        x = inputs.uniform(61 + n, 2 * n * B).astype(dt)
        obj = G.TransformObject(n, vt, tt, place=place, batch=B)
        dev = torch.from_numpy(x).cuda()
        if place is G.IN_PLACE:
            obj.fft(dev)
            want = dev.cpu().numpy()
            host = torch.from_numpy(x.copy()).pin_memory()
            obj.fft(host)
            got = host.numpy()
        else:
            out = torch.empty_like(dev)
            obj.fft(dev, out)
            want = out.cpu().numpy()
            hx = torch.from_numpy(x).pin_memory()
            hy = torch.empty_like(hx).pin_memory()
            obj.fft(hx, hy)
            got = hy.numpy()
        assert np.array_equal(got, want), (n, B)


def test_error_codes(cuda):
    import ctypes
    from gfft_gb300 import _lib
    from gfft_gb300 import gfft as G
    L = _lib.lib()
    obj = G.TransformObject(64, G.DOUBLE, G.DFT, place=G.IN_PLACE)
    t = cuda.zeros(256, dtype=cuda.float64, device="cuda")
    p = t.data_ptr()
    assert L.gfft_exec(obj._h, None, ctypes.c_void_p(p), None) == 7
    assert L.gfft_exec(obj._h, ctypes.c_void_p(p + 8), ctypes.c_void_p(p + 8), None) == 8
    assert L.gfft_exec(obj._h, ctypes.c_void_p(p), ctypes.c_void_p(p + 1024), None) == 4
    assert L.gfft_exec(None, ctypes.c_void_p(p), ctypes.c_void_p(p), None) == 11
    assert L.gfft_exec(obj._h, ctypes.c_void_p(p), ctypes.c_void_p(p), None) == 0
    h = ctypes.c_void_p()
    assert L.gfft_create(ctypes.byref(h), 2 * 4099, 1, 0, 1, 0, 1, 1) == 1
    assert L.gfft_create(ctypes.byref(h), 64, 0, 0, 4, 0, 1, 1) == 5  # four dimensions
    assert L.gfft_create(ctypes.byref(h), 64, 0, 0, 2, 0, 1, 1) == 0  # 64 x 64
    assert L.gfft_destroy(h) == 0
    cuda.cuda.synchronize()
    # the context is still usable
    y = run_gpu(cuda, 16, 0, 0, 1, inputs.uniform(1, 32))
    assert np.isfinite(y).all()


# ---- full-size configurations, size-independent properties --------------
def test_c1_fp64_1024_batch4096_inplace_roundtrip(cuda, oracle):
    import torch
    from gfft_gb300 import gfft as G
    n, B = 1024, 4096
    x = inputs.uniform(0x5EED0001, 2 * n * B)
    t = torch.from_numpy(x).cuda()
    f = G.TransformObject(n, G.DOUBLE, G.DFT, place=G.IN_PLACE, batch=B)
    f.fft(t)
    torch.cuda.synchronize()
    y = t.cpu().numpy()
    for b in (0, 1, 2047, 4095):  # spot transforms against the exact oracle
        seg = slice(2 * n * b, 2 * n * (b + 1))
        assert rel(y[seg], oracle.fft_ld(x[seg], n, 1, 1)) <= tol(n, 1)
    f.ifft(t)
    torch.cuda.synchronize()
    assert rel(t.cpu().numpy(), x) <= 2 * tol(n, 1)


@pytest.mark.parametrize("n", [3 * 2 ** 18, 5 ** 8, 2 ** 10 * 3 ** 5])
@pytest.mark.parametrize("dbl", [1, 0])
def test_c2_mixed_radix_batch8(cuda, oracle, n, dbl):
    dt = np.float64 if dbl else np.float32
    B = 8
    x = inputs.gaussian(0x5EED0002 + n, 2 * n * B).astype(dt)
    y = run_gpu(cuda, n, 0 if dbl else 1, 0, 1, x, batch=B)
    seg = slice(2 * n * 5, 2 * n * 6)
    assert rel(y[seg], oracle.fft_ld(x[seg], n, 1, 1)) <= tol(n, dbl)
    # Parseval over the batch
    e_in = np.sum(x.astype(np.float64) ** 2) * n
    e_out = np.sum(y.astype(np.float64) ** 2)
    assert abs(e_out / e_in - 1) <= 10 * tol(n, dbl)
    back = run_gpu(cuda, n, 0 if dbl else 1, 1, 1, y, batch=B)
    assert rel(back, x) <= 2 * tol(n, dbl)


def test_c2b_real_2pow20_batch16(cuda, oracle):
    n, B = 1 << 19, 16
    x = inputs.uniform(0x5EED0003, 2 * n * B)
    y = run_gpu(cuda, n, 0, 2, 0, x, batch=B)
    seg = slice(2 * n * 3, 2 * n * 4)
    ref = oracle.gfft(n, 0, 2, 0, x[seg])
    exact_packed = packed_rfft(x[seg])
    assert rel(y[seg], exact_packed) <= tol(2 * n, 1) * 2
    assert rel(y[seg], ref) <= tol(2 * n, 1) * 2 + 2 * rel(ref, exact_packed)
    back = run_gpu(cuda, n, 0, 3, 0, y, batch=B)
    assert rel(back, x) <= 2 * tol(2 * n, 1)


def test_c3_fp32_4096_batch65536(cuda, oracle):
    import torch
    from gfft_gb300 import gfft as G
    n, B = 4096, 65536
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    x = torch.randn(2 * n * B, device="cuda", dtype=torch.float32, generator=g)
    y = torch.empty_like(x)
    G.TransformObject(n, G.FLOAT, G.DFT, batch=B).fft(x, y)
    torch.cuda.synchronize()
    for b in (0, 12345, 65535):
        seg = slice(2 * n * b, 2 * n * (b + 1))
        xs = x[seg].cpu().numpy().astype(np.float64)
        assert rel(y[seg].cpu().numpy(), oracle.fft_ld(xs, n, 1, 1)) <= tol(n, 0)
    z = torch.empty_like(x)
    G.TransformObject(n, G.FLOAT, G.IDFT, batch=B).fft(y, z)
    torch.cuda.synchronize()
    assert (torch.linalg.vector_norm(z - x) / torch.linalg.vector_norm(x)).item() <= 2 * tol(n, 0)


def test_c3_fp32_2pow24(cuda, oracle):
    import torch
    from gfft_gb300 import gfft as G
    n = 1 << 24
    x = inputs.gaussian(0x5EED0004, 2 * n).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    y = torch.empty_like(xt)
    G.TransformObject(n, G.FLOAT, G.DFT).fft(xt, y)
    torch.cuda.synchronize()
    yn = y.cpu().numpy()
    bins = np.array([0, 1, 2, 777, n // 2, n - 1, 123456, 9999999])
    exb = oracle.dft_bins_q(x.astype(np.float64), bins, 1)
    got = np.empty(2 * len(bins))
    got[0::2], got[1::2] = yn[2 * bins], yn[2 * bins + 1]
    scale = np.sqrt(np.sum(x.astype(np.float64) ** 2))  # ~|X_k| for noise input
    assert np.max(np.abs(got - exb)) / scale <= 10 * tol(n, 0)
    e_in = np.sum(x.astype(np.float64) ** 2) * n
    assert abs(np.sum(yn.astype(np.float64) ** 2) / e_in - 1) <= 10 * tol(n, 0)


@pytest.mark.parametrize("n,B", [(4096, 9), (8192, 5), (16384, 3)])
def test_direct_single_pass(cuda, oracle, n, B):
    """One transform per block with no stage (FP32 4096 / 8192 / 16384, the
    defaults): against the exact oracle and the staged single pass (or the
    two-pass plan at 16384), forward and inverse, in and out of place."""
    from gfft_gb300 import _lib
    opts = None
    d = _lib.plan_query(n, 1, 0, 1, B, opts)
    assert d["kernel_variant"] == [3] and d["threads"] == [n // 16], d
    x = inputs.gaussian(61 + n, 2 * n * B).astype(np.float32)
    for tr in (0, 1):
        y = run_gpu(cuda, n, 1, tr, 1, x, batch=B, opts=opts)
        ex = oracle.fft_ld(x.astype(np.float64), n, B, 1 if tr == 0 else -1)
        assert rel(y, ex) <= tol(n, 0), (n, tr, rel(y, ex))
        ref = run_gpu(cuda, n, 1, tr, 1, x, batch=B, opts={"stages": 1})
        assert rel(y, ref) <= tol(n, 0), (n, tr, rel(y, ref))
        yi = run_gpu(cuda, n, 1, tr, 0, x, batch=B, opts=opts)
        assert np.array_equal(y, yi), (n, tr)


def test_fast_path_matches_generic_engine(cuda, oracle):
    """The pipelined register-resident kernel (variant 2) against the generic
    engine (variant 1) and the exact oracle, single and partial tiles."""
    for n, dbl, B in ((4096, 0, 7), (1024, 1, 9), (16, 0, 1000), (64, 0, 300), (8192, 0, 3), (2048, 1, 5),
                      (256, 1, 33), (16384, 0, 5)):
        dt = np.float64 if dbl else np.float32
        vt = 0 if dbl else 1
        x = inputs.uniform(55 + n, 2 * n * B).astype(dt)
        ex = oracle.fft_ld(x.astype(np.float64), n, B, 1)
        for tr in (0, 1):
            spec = run_gpu(cuda, n, vt, tr, 1, x, batch=B)
            fast = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 2})
            gen = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 1})
            if tr == 0:
                assert rel(spec, ex) <= tol(n, dbl), (n, rel(spec, ex))
                assert rel(fast, ex) <= tol(n, dbl), (n, rel(fast, ex))
            assert rel(fast, gen) <= tol(n, dbl), (n, tr, rel(fast, gen))
            assert rel(spec, gen) <= tol(n, dbl), (n, tr, rel(spec, gen))
        for stages in (1, 2, 3, 4):
            y = run_gpu(cuda, n, vt, 0, 1, x, batch=B, opts={"stages": stages})
            assert rel(y, ex) <= tol(n, dbl), (n, stages)


def test_bounded_wait_selftest(cuda):
    """A wait that nothing completes runs out, reports GFFT_E_TIMEOUT, and the
    context stays usable."""
    import ctypes
    from gfft_gb300 import _lib
    L = _lib.lib()
    st = ctypes.c_int(-1)
    assert L.gfft_selftest_bounded_wait(1 << 12, ctypes.byref(st)) == 0
    assert st.value == 13
    y = run_gpu(cuda, 4096, 1, 0, 1, inputs.uniform(2, 2 * 4096 * 4).astype(np.float32), batch=4)
    assert np.isfinite(y).all()


def test_device_status_clean_after_runs(cuda):
    import ctypes
    from gfft_gb300 import _lib
    from gfft_gb300 import gfft as G
    obj = G.TransformObject(4096, G.FLOAT, G.DFT, batch=256)
    x = cuda.zeros(2 * 4096 * 256, device="cuda", dtype=cuda.float32)
    y = cuda.empty_like(x)
    for _ in range(3):
        obj.fft(x, y)
    st = ctypes.c_int(-1)
    assert _lib.lib().gfft_get_device_status(obj._h, ctypes.byref(st)) == 0
    assert st.value == 0


def test_cpp_facade_on_gpu(cuda):
    import subprocess
    from tests.cpp import build_facade
    exe = build_facade.build()
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade ok (gpu)" in r.stdout


@pytest.mark.parametrize("dbl", [0, 1])
@pytest.mark.parametrize("n,B", [(768, 7), (625, 5), (576, 3), (432, 9), (1000, 3), (729, 2), (480, 5), (360, 11),
                                 (3 * 2 ** 18, 2), (5 ** 8, 2), (2 ** 10 * 3 ** 5, 3), (1000 * 1000, 1)])
def test_mixed_columns(cuda, oracle, n, B, dbl):
    """The compile-time mixed-radix column tiles (variant 7): single-pass
    lengths (batches whose last tile is partial) and the passes of multi-pass
    lengths, forward and inverse, out of place and in place, against the
    generic engine and the exact oracle."""
    from gfft_gb300 import _lib
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    v7 = {"kernel_variant": 7}
    assert 7 in _lib.plan_query(n, vt, 0, 1, B, v7)["kernel_variant"]
    x = inputs.gaussian(23 + n, 2 * n * B).astype(dt)
    for tr in (0, 1):
        y = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts=v7)
        gen = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 1})
        assert rel(y, gen) <= tol(n, dbl), (n, tr, rel(y, gen))
        yi = run_gpu(cuda, n, vt, tr, 0, x, batch=B, opts=v7)
        assert np.array_equal(y, yi), (n, tr)
    k = min(B, max(1, (1 << 20) // n))
    ex = oracle.fft_ld(x[:2 * n * k].astype(np.float64), n, k, 1)
    y = run_gpu(cuda, n, vt, 0, 1, x[:2 * n * k], batch=k, opts=v7)
    assert rel(y, ex) <= tol(n, dbl), (n, rel(y, ex))


@pytest.mark.parametrize("dbl", [0, 1])
@pytest.mark.parametrize("n,B", [(3 * 2 ** 18, 3), (2 ** 10 * 3 ** 5, 3), (1000 * 1000, 1), (480 * 1024, 2),
                                 (768 * 768, 1), (432 * 432, 2), (576 * 576, 1), (480 * 480, 2), (360 * 360, 2),
                                 (5 ** 8, 3), (3 ** 12, 1)])
def test_mixed_tensor_copy_columns(cuda, oracle, n, B, dbl):
    """Mixed-radix passes of variant 9 (a pass length that is not a power of
    two): moved by 2-D tensor copies where W divides N / L and Ns and the
    rows fit a tensor map, else gathered by cp.async (FP32 360 x 360: 16
    units do not divide 360; 5^8 and 3^12: odd rows, tiles spanning
    transforms, a partial last tile); against the copy-free mixed tiles
    (variant 7), the generic engine and, up to 2^20 points, the exact
    oracle; forward and inverse, in and out of place."""
    from gfft_gb300 import _lib
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    d = _lib.plan_query(n, vt, 0, 1, B)
    P = d["n_global_passes"]
    mixed9 = [g for g in range(P) if d["kernel_variant"][g] == 9 and d["pass_len"][g] & (d["pass_len"][g] - 1)]
    if not (dbl and n in (5 ** 8, 3 ** 12)):  # FP64 tiles that need gathers stay on variant 7
        assert mixed9, d
    x = inputs.gaussian(31 + n + B, 2 * n * B).astype(dt)
    for tr in (0, 1):
        y = run_gpu(cuda, n, vt, tr, 1, x, batch=B)
        v7 = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 7})
        gen = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 1})
        assert rel(y, v7) <= tol(n, dbl), (n, tr, rel(y, v7))
        assert rel(y, gen) <= tol(n, dbl), (n, tr, rel(y, gen))
        yi = run_gpu(cuda, n, vt, tr, 0, x, batch=B)
        assert np.array_equal(y, yi), (n, tr)
        if n * B <= 1 << 20:
            ex = oracle.fft_ld(x.astype(np.float64), n, B, 1 if tr == 0 else -1)
            assert rel(y, ex) <= tol(n, dbl), (n, tr, rel(y, ex))


@pytest.mark.parametrize("n,dbl,B,cap", [(1 << 13, 0, 3, 1024), (1 << 16, 0, 2, 0), (1 << 20, 0, 1, 0),
                                         (1 << 24, 0, 1, 0), (1 << 18, 0, 2, 64), (1 << 12, 1, 5, 64),
                                         (1 << 18, 1, 2, 0), (1 << 22, 1, 1, 0), (1 << 15, 0, 3, 256)])
def test_multipass_spec_columns(cuda, oracle, n, dbl, B, cap):
    """The length-specialised column-tile kernel (variant 5, for power-of-two
    passes of 64..1024) against the generic engine and the prefetching
    column-tile kernel, forward and inverse, out of place and in place, and
    against the exact oracle."""
    from gfft_gb300 import _lib
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    base = {"max_pass_len": cap, "kernel_variant": 5} if cap else {"kernel_variant": 5}
    info = _lib.plan_query(n, vt, 0, 1, B, base or None)
    assert info["n_global_passes"] >= 2 and all(v == 5 for v in info["kernel_variant"]), info
    x = inputs.gaussian(17 + n, 2 * n * B).astype(dt)
    for tr in (0, 1):
        spec = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts=base or None)
        gen = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts=dict(base, kernel_variant=1))
        lane = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts=dict(base, kernel_variant=4))
        inp = run_gpu(cuda, n, vt, tr, 0, x, batch=B, opts=base or None)
        assert rel(spec, gen) <= tol(n, dbl), (n, tr, rel(spec, gen))
        assert rel(spec, lane) <= tol(n, dbl), (n, tr, rel(spec, lane))
        assert np.array_equal(spec, inp), (n, tr)
    if n <= 1 << 20:
        for tr in (0, 1):
            k = min(B, 2)
            ex = oracle.fft_ld(x[:2 * n * k].astype(np.float64), n, k, 1 if tr == 0 else -1)
            y = run_gpu(cuda, n, vt, tr, 1, x[:2 * n * k], batch=k, opts=base or None)
            assert rel(y, ex) <= tol(n, dbl), (n, tr, rel(y, ex))


@pytest.mark.parametrize("n,dbl", [(1 << 14, 0), (1 << 21, 0), (1 << 16, 1)])
def test_multipass_spec_columns_real(cuda, n, dbl):
    """Real transforms whose complex half-length runs through variant 5:
    forward against numpy's FP64 real DFT in the packed layout, and the
    inverse round trip."""
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    x = inputs.gaussian(5 + n, 2 * n).astype(dt)
    y = run_gpu(cuda, n, vt, 2, 1, x)
    assert rel(y, packed_rfft(x)) <= tol(2 * n, dbl)
    z = run_gpu(cuda, n, vt, 3, 1, y)
    assert rel(z, x) <= 2 * tol(2 * n, dbl)


@pytest.mark.parametrize("n,dbl,B", [(786432, 0, 3), (390625, 1, 2), (248832, 0, 5), (1 << 20, 1, 1),
                                     (12288, 0, 7), (1 << 24, 0, 1), (3 * 5 * 7 * 11 * 13 * 16, 0, 1)])
def test_multipass_pipelined_matches_engine(cuda, oracle, n, dbl, B):
    """The prefetching column-tile kernel (variant 4) against the one-tile-per-
    block engine (variant 1), forward and inverse, with a ragged last tile."""
    vt = 0 if dbl else 1
    dt = np.float64 if dbl else np.float32
    x = inputs.gaussian(91 + n, 2 * n * B).astype(dt)
    for tr in (0, 1):
        fast = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 4})
        gen = run_gpu(cuda, n, vt, tr, 1, x, batch=B, opts={"kernel_variant": 1})
        assert rel(fast, gen) <= tol(n, dbl), (n, tr, rel(fast, gen))
    if n <= 1 << 20:
        ex = oracle.fft_ld(x[:2 * n].astype(np.float64), n, 1, 1)
        for opts in (None, {"kernel_variant": 4}):  # the default plan and the prefetching column tiles
            y = run_gpu(cuda, n, vt, 0, 1, x[:2 * n], opts=opts)
            assert rel(y, ex) <= tol(n, dbl)
