"""CPU: tuner candidate enumeration and plan features (no GPU), and the FP64
reference of the cost model pinned by finite differences."""
import numpy as np
import pytest

from gfft_gb300 import _lib
from gfft_gb300 import tuner


def test_candidates_distinct_and_plannable():
    for n in (4096, 786432, 1000, 1 << 20):
        c = tuner.candidates(n, 1, 0, 1, 4)
        assert 3 <= len(c) <= 64
        assert {} in c  # the planner's default is always a candidate
        shapes = set()
        for o in c:
            d = _lib.plan_query(n, 1, 0, 1, 4, o or None)
            key = (tuple(d["pass_len"]), tuple(map(tuple, d["radices"])), tuple(d["kernel_variant"]),
                   tuple(d["units"]), o.get("stages", 0))
            assert key not in shapes
            shapes.add(key)


def test_features():
    f = tuner.features(2 ** 10 * 3 ** 5, 1, 0, 1, 8, {})
    assert f.shape == (_lib.NFEAT,)
    assert abs(f[0] - np.log2(2 ** 10 * 3 ** 5)) < 1e-5
    assert list(f[1:5]) == [10, 5, 0, 0]
    assert f[5] == 3 and f[6] == 0 and f[7] == 2
    assert f[8:15].sum() >= 4  # radices counted
    assert f[18:22].sum() + f[24] == 2  # one kernel class per global pass
    assert abs(f[16] - np.log2(576)) < 1e-5 and abs(f[17] - np.log2(432)) < 1e-5
    g = tuner.features(4096, 0, 0, 1, 1, {"max_radix": 4})
    assert g[6] == 1 and g[10] == 6  # six radix-4 passes, FP64
    assert g[23] == 4 / 16
    # candidates that differ only in their pipeline depth or lane width differ in features
    h1 = tuner.features(4096, 1, 0, 1, 64, {"stages": 3})
    h0 = tuner.features(4096, 1, 0, 1, 64, {})
    assert h1[22] == 3 and h0[22] == 0
    w0 = tuner.features(1 << 20, 1, 0, 1, 1, {"kernel_variant": 4})
    w1 = tuner.features(1 << 20, 1, 0, 1, 1, {"units_per_block": 16})
    assert w1[15] > w0[15]


def test_mlp_reference_gradients_finite_difference():
    from oracle import mlp_ref
    rng = np.random.default_rng(0)
    nin, width, depth = 5, 7, 3
    npar = sum((nin if l == 0 else width) * (1 if l == depth else width) + (1 if l == depth else width)
               for l in range(depth + 1))
    p = rng.normal(size=npar) * 0.5
    X = rng.normal(size=(13, nin))
    y = rng.normal(size=13)
    g = mlp_ref.gradients(p, X, y, nin, width, depth)

    def loss(q):
        return np.mean((mlp_ref.forward(q, X, nin, width, depth) - y) ** 2)

    for i in rng.choice(npar, 40, replace=False):
        e = np.zeros(npar)
        e[i] = 1e-6
        fd = (loss(p + e) - loss(p - e)) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_mlp_rejects_rows_of_the_wrong_width():
    """The library reads len(X) * nin features: a matrix of another width is
    refused on the host before any copy."""
    m = tuner.MLP.__new__(tuner.MLP)  # no device state: only the host-side check
    m.nin = 25
    with pytest.raises(ValueError):
        m._rows(np.zeros((3, 24), dtype=np.float32))
    with pytest.raises(ValueError):
        m._rows(np.zeros((3, 25), dtype=np.float32), np.zeros(4, dtype=np.float32))
    X, y = m._rows(np.zeros((3, 25)), np.zeros(3))
    assert X.dtype == np.float32 and X.flags.c_contiguous and y.shape == (3,)
