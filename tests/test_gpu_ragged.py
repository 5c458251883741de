"""GPU: ragged batches (many lengths, one persistent launch from a CUDA
graph) against numpy's FP64 FFT per transform and against the per-length
transform objects."""
import numpy as np
import pytest

from gfft_gb300 import inputs

pytestmark = pytest.mark.gpu


def tol(n, dbl):
    return (2e-15 if dbl else 6e-7) * max(1.0, np.log2(max(n, 2)))


def _check(y, x, sizes, sign, dbl, scale=1.0):
    off = 0
    worst = 0.0
    for n in sizes:
        n = int(n)
        xs = x[2 * off:2 * (off + n)].astype(np.float64)
        c = xs[0::2] + 1j * xs[1::2]
        f = np.fft.fft(c) if sign > 0 else np.fft.ifft(c)
        ref = np.empty(2 * n)
        ref[0::2], ref[1::2] = f.real, f.imag
        got = y[2 * off:2 * (off + n)].astype(np.float64)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)
        assert err <= tol(n, dbl), (n, err)
        worst = max(worst, err)
        off += n
    return worst


@pytest.mark.parametrize("dbl", [0, 1])
def test_ragged_matches_exact(cuda, dbl):
    import torch
    from gfft_gb300 import gfft as G
    sizes = np.concatenate([inputs.ragged_sizes(71, 240, 6, 13), inputs.ragged_sizes(72, 12, 13, 18),
                            [1, 2, 3, 64, 4096, 4097 - 1, 2 ** 18]])
    vt = G.DOUBLE if dbl else G.FLOAT
    dt = torch.float64 if dbl else torch.float32
    total = int(sizes.sum())
    x = inputs.uniform(5, 2 * total)
    xt = torch.from_numpy(x).to(dt).cuda()
    fwd = G.RaggedBatch(sizes, vt, G.DFT)
    inv = G.RaggedBatch(sizes, vt, G.IDFT)
    info = fwd.info()
    assert info["total_points"] == total and info["max_passes"] >= 2
    y = torch.empty_like(xt)
    fwd.fft(xt, y)
    torch.cuda.synchronize()
    _check(y.cpu().numpy(), xt.cpu().numpy(), sizes, 1, dbl)
    z = torch.empty_like(xt)
    inv.fft(y, z)
    torch.cuda.synchronize()
    _check(z.cpu().numpy(), y.cpu().numpy(), sizes, -1, dbl)
    assert fwd.status() == 0 and inv.status() == 0


def test_ragged_graph_replay_and_new_pointers(cuda):
    import torch
    from gfft_gb300 import gfft as G
    sizes = inputs.ragged_sizes(81, 64, 6, 16)
    total = int(sizes.sum())
    rb = G.RaggedBatch(sizes, G.FLOAT, G.DFT)
    a = torch.from_numpy(inputs.uniform(1, 2 * total)).float().cuda()
    out = torch.empty_like(a)
    rb.fft(a, out)                      # captures the graph
    b = torch.from_numpy(inputs.uniform(2, 2 * total)).float().cuda()
    a.copy_(b)
    rb.fft(a, out)                      # replays it on new data
    torch.cuda.synchronize()
    _check(out.cpu().numpy(), b.cpu().numpy(), sizes, 1, 0)
    out2 = torch.empty_like(a)
    rb.fft(b, out2)                     # new pointers: captured again
    torch.cuda.synchronize()
    assert torch.equal(out, out2)
    assert rb.status() == 0


def test_ragged_equals_per_length_objects(cuda):
    import torch
    from gfft_gb300 import gfft as G
    sizes = np.array([4096, 1000, 8192, 786432 // 3, 60, 4096])
    total = int(sizes.sum())
    x = torch.from_numpy(inputs.uniform(3, 2 * total)).float().cuda()
    y = torch.empty_like(x)
    G.RaggedBatch(sizes, G.FLOAT, G.DFT).fft(x, y)
    off = 0
    for n in sizes:
        n = int(n)
        seg = slice(2 * off, 2 * (off + n))
        want = torch.empty(2 * n, device="cuda")
        G.TransformObject(n, G.FLOAT, G.DFT).fft(x[seg].contiguous(), want)
        torch.cuda.synchronize()
        r = (torch.linalg.vector_norm(y[seg] - want) / torch.linalg.vector_norm(want)).item()
        assert r <= tol(n, 0), (n, r)
        off += n


def test_ragged_shape_functions_cover_and_match(cuda, oracle):
    """Lengths whose passes run the compile-time pass functions (360 x 400,
    300 x 450, 480 x 324, ...) and lengths that do not, in one launch,
    against the exact oracle."""
    from gfft_gb300 import _lib
    from gfft_gb300 import gfft as G
    sizes = np.array([360 * 400, 300 * 450, 480 * 324, 375 * 500, 240, 225, 1000, 7 * 11 * 13, 360, 432 * 576])
    shaped = 0
    for n in sizes:
        d = _lib.plan_query(int(n), 1, 0, 1, 1, {"units_per_block": 4, "max_pass_len": 4096, "kernel_variant": 1})
        shaped += sum(1 for rs in d["radices"] if tuple(rs) in SHAPES)
    assert shaped >= 8
    total = int(sizes.sum())
    x = inputs.uniform(99, 2 * total).astype(np.float32)
    rb = G.RaggedBatch(sizes, G.FLOAT, G.DFT)
    import torch
    xs = torch.from_numpy(x).cuda()
    ys = torch.empty_like(xs)
    rb.fft(xs, ys)
    torch.cuda.synchronize()
    assert rb.status() == 0
    y = ys.cpu().numpy()
    off = 0
    for n in sizes:
        n = int(n)
        seg = slice(2 * off, 2 * (off + n))
        ex = oracle.fft_ld(x[seg].astype(np.float64), n, 1, 1)
        err = np.linalg.norm(y[seg] - ex) / np.linalg.norm(ex)
        assert err <= 6e-7 * np.log2(n), (n, err)
        off += n


SHAPES = {(15, 12, 2), (15, 10, 2), (15, 15, 2), (16, 5, 5), (16, 15, 2), (12, 9, 3), (15, 5, 5), (10, 10, 5),
          (16, 10, 2), (16, 12, 2), (16, 9, 2), (16, 15), (10, 5, 5), (15, 9, 2), (16, 9, 3), (15, 15), (15, 9, 3),
          (15, 10, 4), (9, 9, 6), (16, 12, 3), (9, 9, 3), (10, 10, 2), (15, 12, 3), (16, 10, 4), (15, 12), (15, 10),
          (9, 9, 2), (16, 10), (12, 9, 2), (16, 9)}


def test_ragged_schedule_from_tuner(cuda):
    """The autotuner's ragged schedule (tuner.ragged_schedule: every candidate
    timed inside the ragged kernel on that length's transforms) is what the
    handle runs: for every scheduled length, the plan the handle reports
    reflects the chosen options; explicit schedules give the same kind of
    change; results stay within the oracle bound."""
    import torch
    from gfft_gb300 import gfft as G
    from gfft_gb300 import tuner
    sizes = np.concatenate([inputs.ragged_sizes(91, 60, 8, 12), [3 * 2 ** 14] * 6, [5 ** 7] * 4, [2 ** 16] * 5])
    sched = tuner.ragged_schedule(sizes, 1, 0, coverage=0.8, max_members=8, reps=3)
    rb = G.RaggedBatch(sizes, G.FLOAT, G.DFT, schedule=sched)
    assert rb.schedule == sched
    for n, opts in sched.items():
        p = rb.plan(n)
        alone = G.RaggedBatch([n], G.FLOAT, G.DFT, schedule={n: opts})
        assert alone.plan(n) == p, (n, opts, p)  # the tuned schedule, as measured
        if "max_pass_len" in opts:
            assert max(p["pass_len"]) <= opts["max_pass_len"], (n, p)
        if "units_per_block" in opts:
            assert all(u <= opts["units_per_block"] for u in p["units"]), (n, p)
    # explicit schedules change what the handle reports
    big = 3 * 2 ** 14
    r2 = G.RaggedBatch(sizes, G.FLOAT, G.DFT, schedule={big: {"max_pass_len": 128, "units_per_block": 2}})
    p2 = r2.plan(big)
    assert max(p2["pass_len"]) <= 128 and p2["n_global_passes"] >= 3 and max(p2["units"]) <= 2, p2
    total = int(sizes.sum())
    x = torch.from_numpy(inputs.uniform(9, 2 * total)).float().cuda()
    for h in (rb, r2):
        y = torch.empty_like(x)
        h.fft(x, y)
        torch.cuda.synchronize()
        _check(y.cpu().numpy(), x.cpu().numpy(), sizes, 1, 0)
        assert h.status() == 0
