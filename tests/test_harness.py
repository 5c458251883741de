"""The reference-style accuracy / performance harness (gfft_gb300.harness)."""
import io

import numpy as np
import pytest

from gfft_gb300 import harness


def test_direct_dft_matches_numpy():
    rng = np.random.default_rng(0)
    for n in (1, 2, 3, 8, 49, 125):
        x = rng.uniform(-0.5, 0.5, 2 * n)
        c = np.fft.fft(x[0::2] + 1j * x[1::2])
        y = harness.direct_dft(x)
        assert np.max(np.abs(y[0::2] - c.real)) < 1e-13 and np.max(np.abs(y[1::2] - c.imag)) < 1e-13


@pytest.mark.gpu
def test_accuracy_matrix_small(cuda):
    """The test_accuracy.sh sweep (every value type and place, bases 2, 3, 5,
    7) over shortened power ranges; the summary lines and their bounds."""
    out = io.StringIO()
    worst = {}
    for t in harness.TYPES:
        for p in harness.PLACES:
            for base, lo, hi in ((2, 2, 9), (3, 2, 5), (5, 2, 3), (7, 2, 3)):
                worst[(t, p, base)] = harness.accuracy(t, p, base, lo, hi, full=True, out=out)
    text = out.getvalue()
    assert "IN_PLACE, DOUBLE, 2^[2,9]:" in text and "Relative NormInf" in text
    for (t, p, base), e in worst.items():
        bound = 1e-14 if "DOUBLE" in t else 5e-6
        assert e <= bound, (t, p, base, e)


@pytest.mark.gpu
def test_performance_table(cuda):
    out = io.StringIO()
    rows = harness.performance(6, 7, out=out)
    assert len(rows) == 4 and all(r[5] > 0 and r[6] > 0 for r in rows)
    assert "Time [ns]" in out.getvalue()
