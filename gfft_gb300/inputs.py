"""Seeded synthetic inputs (host side, numpy).

The same splitmix64 stream everywhere: element i of a stream with seed s is
splitmix64 state s + (i+1)*0x9E3779B97F4A7C15, finalised; doubles in [-1, 1)
come from its top 53 bits.  Gaussian values use Box-Muller on consecutive
pairs of the stream; float32 inputs are generated in float64 and rounded.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(seed: int, start: int, count: int) -> np.ndarray:
    i = np.arange(start + 1, start + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, count: int, dtype=np.float64, chunk: int = 1 << 24) -> np.ndarray:
    """``count`` values uniform in [-1, 1)."""
    out = np.empty(count, dtype=dtype)
    for s in range(0, count, chunk):
        c = min(chunk, count - s)
        r = (_mix(seed, s, c) >> np.uint64(11)).astype(np.float64)
        out[s:s + c] = r * (1.0 / 4503599627370496.0) - 1.0
    return out


def gaussian(seed: int, count: int, dtype=np.float64, chunk: int = 1 << 24) -> np.ndarray:
    """``count`` N(0,1) values (Box-Muller on pairs of the uniform stream)."""
    out = np.empty(count, dtype=dtype)
    npair = (count + 1) // 2
    for s in range(0, npair, chunk):
        c = min(chunk, npair - s)
        z = _mix(seed, 2 * s, 2 * c)
        u = ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
        u1, u2 = u[0::2], u[1::2]
        r = np.sqrt(-2.0 * np.log(u1))
        g = np.empty(2 * c)
        g[0::2] = r * np.cos(2 * np.pi * u2)
        g[1::2] = r * np.sin(2 * np.pi * u2)
        lo = 2 * s
        hi = min(count, lo + 2 * c)
        out[lo:hi] = g[: hi - lo]
    return out


def tone_mix(seed: int, n: int, batch: int, amp: float = 1e-4, tones: int = 8) -> np.ndarray:
    """``tones`` complex exponentials of amplitude ``amp`` at bins drawn from
    the stream, random phase; the phase argument uses the exact integer
    reduction (k*t mod n).  Returns interleaved float64 of length 2*n*batch."""
    z = _mix(seed ^ 0x70AE, 0, 2 * tones)
    bins = (z[:tones] % np.uint64(n)).astype(np.int64)
    phase = (z[tones:] >> np.uint64(11)).astype(np.float64) * (2 * np.pi / 9007199254740992.0)
    t = np.arange(n, dtype=np.int64)
    sig = np.zeros(n, dtype=np.complex128)
    for k, ph in zip(bins, phase):
        m = (k * t) % n
        sig += amp * np.exp(1j * (2 * np.pi * m / n + ph))
    out = np.empty(2 * n * batch)
    inter = np.empty(2 * n)
    inter[0::2] = sig.real
    inter[1::2] = sig.imag
    out.reshape(batch, 2 * n)[:] = inter
    return out


def smooth235(limit: int) -> np.ndarray:
    """All 2^a 3^b 5^c <= limit, ascending."""
    out = []
    p2 = 1
    while p2 <= limit:
        p3 = p2
        while p3 <= limit:
            p5 = p3
            while p5 <= limit:
                out.append(p5)
                p5 *= 5
            p3 *= 3
        p2 *= 2
    return np.array(sorted(out), dtype=np.int64)


def ragged_sizes(seed: int, count: int, lo: int = 6, hi: int = 18) -> np.ndarray:
    """``count`` lengths log-uniform in [2^lo, 2^hi], each snapped to the
    nearest 5-smooth value inside that range (ties go down)."""
    z = _mix(seed, 0, count)
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    target = 2.0 ** (lo + u * (hi - lo))
    cand = smooth235(2 ** hi)
    cand = cand[cand >= 2 ** lo]
    idx = np.searchsorted(cand, target)
    idx = np.clip(idx, 1, len(cand) - 1)
    below, above = cand[idx - 1], cand[idx]
    pick = np.where(target - below <= above - target, below, above)
    return pick.astype(np.int64)
