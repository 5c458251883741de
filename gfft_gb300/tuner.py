"""Autotuner and learned planner over the C ABI.

- ``candidates``: the distinct plans reachable through the plan options;
- ``measure``: exhaustive measured search (every candidate timed with CUDA
  events in the library);
- ``CostModel``: a 3 x 64 FP32 MLP on ``gfft_plan_features``, trained and
  evaluated on the GPU by the library's own kernels (``gfft_mlp_*``), with the
  feature normalisation kept beside the weights; ``save`` / ``load`` persist
  both (the tuner's only state, with the timing table);
- ``choose``: the plan the model ranks first, or the best measured among its
  top ``k`` (a pruned search; ``k=None`` falls back to the exhaustive one);
- ``ragged_schedule``: the tile / radix schedule of a ragged batch, measured
  per length inside the ragged kernel itself.
"""
from __future__ import annotations

import ctypes
import json
import math
import os

import numpy as np

from . import _lib

OPT_FIELDS = ["radix_order", "max_radix", "threads_per_block", "units_per_block", "max_pass_len", "kernel_variant",
              "stages", "blocks_per_sm"]


def _opts_to_dict(o: _lib.PlanOpts) -> dict:
    return {k: int(getattr(o, k)) for k in OPT_FIELDS if int(getattr(o, k))}


def candidates(n, vtype=1, trans=0, place=1, batch=1, max_cands=64):
    arr = (_lib.PlanOpts * max_cands)()
    cnt = ctypes.c_int()
    _lib.check(_lib.lib().gfft_tune_candidates(n, vtype, trans, place, batch, arr, max_cands, ctypes.byref(cnt)),
               "gfft_tune_candidates")
    return [_opts_to_dict(arr[i]) for i in range(cnt.value)]


def features(n, vtype, trans, place, batch, opts: dict) -> np.ndarray:
    f = np.zeros(_lib.NFEAT, dtype=np.float32)
    o = _lib.make_opts(opts) if opts else None
    _lib.check(_lib.lib().gfft_plan_features(n, vtype, trans, place, batch, ctypes.byref(o) if o else None,
                                             f.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "gfft_plan_features")
    return f


def measure(n, vtype, trans, place, batch, cands, reps=5, src=None, dst=None):
    """Time every candidate (ms per launch) on device buffers (allocated here
    with torch when not given)."""
    import torch
    if src is None:
        dt = torch.float64 if vtype in (0, 2) else torch.float32
        src = torch.rand(2 * n * batch, device="cuda", dtype=dt)
        dst = torch.empty_like(src)
    arr = (_lib.PlanOpts * len(cands))()
    for i, c in enumerate(cands):
        for k, v in c.items():
            setattr(arr[i], k, int(v))
    ms = np.zeros(len(cands), dtype=np.float32)
    _lib.check(_lib.lib().gfft_tune_measure(n, vtype, trans, place, batch, arr, len(cands),
                                            ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()), reps,
                                            ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "gfft_tune_measure")
    return ms


class MLP:
    """The library's GPU-trained perceptron (gfft_mlp_*)."""

    def __init__(self, nin=_lib.NFEAT, width=64, depth=3, seed=1):
        self.nin, self.width, self.depth = nin, width, depth
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().gfft_mlp_create(ctypes.byref(h), nin, width, depth, seed), "gfft_mlp_create")
        self._h = h
        self.nparams = _lib.lib().gfft_mlp_num_params(h)

    @staticmethod
    def _fp(a):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def _rows(self, X, y=None):
        """X as C-contiguous FP32 rows of exactly `nin` features (the library
        reads len(X) * nin values), y one target per row."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        if X.ndim != 2 or X.shape[1] != self.nin:
            raise ValueError("features must have shape (rows, %d), got %s" % (self.nin, X.shape))
        if y is None:
            return X
        y = np.ascontiguousarray(y, dtype=np.float32)
        if y.shape != (len(X),):
            raise ValueError("targets must have shape (%d,), got %s" % (len(X), y.shape))
        return X, y

    def params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        _lib.check(_lib.lib().gfft_mlp_get_params(self._h, self._fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _lib.check(_lib.lib().gfft_mlp_set_params(self._h, self._fp(p)))

    def train(self, X, y, epochs=2000, lr=3e-3):
        X, y = self._rows(X, y)
        loss = ctypes.c_float()
        _lib.check(_lib.lib().gfft_mlp_train(self._h, self._fp(X), self._fp(y), len(y), epochs, lr,
                                             ctypes.byref(loss)), "gfft_mlp_train")
        return loss.value

    def predict(self, X):
        X = self._rows(X)
        out = np.zeros(len(X), dtype=np.float32)
        _lib.check(_lib.lib().gfft_mlp_predict(self._h, self._fp(X), len(X), self._fp(out)), "gfft_mlp_predict")
        return out

    def gradients(self, X, y):
        X, y = self._rows(X, y)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = ctypes.c_float()
        _lib.check(_lib.lib().gfft_mlp_gradients(self._h, self._fp(X), self._fp(y), len(y), self._fp(g),
                                                 ctypes.byref(loss)), "gfft_mlp_gradients")
        return g, loss.value

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gfft_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CostModel:
    """log(ms) of a plan from its features; inputs standardised with the
    training set's mean and spread.

    With ``groups`` (one key per row, e.g. the transform length) the target is
    the log-time relative to the mean over the rows of the same group: plans
    are only ever compared within one (length, batch), so the network spends
    its capacity on the differences between plans rather than on the overall
    scale, and predictions rank the candidates of a length directly."""

    def __init__(self, seed=1, members=1):
        # an ensemble of `members` networks of different initial weights; the
        # prediction is the mean of their log-times
        self.nets = [MLP(seed=seed + 1000 * k) for k in range(max(1, members))]
        self.mu = np.zeros(_lib.NFEAT, dtype=np.float32)
        self.sd = np.ones(_lib.NFEAT, dtype=np.float32)

    @property
    def net(self):
        return self.nets[0]

    @staticmethod
    def relative_log(ms, groups):
        y = np.log(np.asarray(ms, dtype=np.float64))
        g = np.asarray(groups)
        out = np.empty_like(y)
        for key in np.unique(g):
            sel = g == key
            out[sel] = y[sel] - y[sel].mean()
        return out.astype(np.float32)

    def fit(self, X, ms, epochs=3000, lr=3e-3, groups=None):
        X = np.asarray(X, dtype=np.float32)
        self.mu = X.mean(0)
        self.sd = np.where(X.std(0) > 1e-6, X.std(0), 1.0).astype(np.float32)
        y = self.relative_log(ms, groups) if groups is not None else np.log(np.asarray(ms, dtype=np.float32))
        Xs = (X - self.mu) / self.sd
        return float(np.mean([net.train(Xs, y, epochs, lr) for net in self.nets]))

    def predict_ms(self, X):
        X = (np.asarray(X, dtype=np.float32) - self.mu) / self.sd
        return np.exp(np.mean([net.predict(X) for net in self.nets], axis=0))

    def save(self, path):
        np.savez(path, params=np.stack([net.params() for net in self.nets]), mu=self.mu, sd=self.sd)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        p = d["params"]
        p = p[None, :] if p.ndim == 1 else p
        m = cls(members=len(p))
        for net, q in zip(m.nets, p):
            net.set_params(q)
        m.mu, m.sd = d["mu"], d["sd"]
        return m


MODEL_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "cost_model_gb300.npz")


def default_model():
    """The cost model trained on a GB300 by ``bench.py --planner`` (FP32
    plans, lengths 256 .. 2^27), shipped with the package; None if absent."""
    return CostModel.load(MODEL_FILE) if os.path.exists(MODEL_FILE) else None


def choose(model, n, vtype=1, trans=0, place=1, batch=1, k=1, reps=5):
    """Plan options for (n, ...): the model's first choice (k=1), the best
    measured of its top k and the planner's default plan (so the measured
    choice is never slower than the default), or the exhaustive measured best
    (model=None)."""
    cands = candidates(n, vtype, trans, place, batch)
    if model is None:
        ms = measure(n, vtype, trans, place, batch, cands, reps)
        ok = np.where(ms > 0, ms, np.inf)
        return cands[int(np.argmin(ok))], float(np.min(ok))
    X = np.stack([features(n, vtype, trans, place, batch, c) for c in cands])
    pred = model.predict_ms(X)
    order = np.argsort(pred)[:max(1, k)]
    if len(order) == 1:
        return cands[int(order[0])], float(pred[order[0]])
    sub = [cands[int(i)] for i in order]
    if {} in cands and {} not in sub:
        sub.append({})
    ms = measure(n, vtype, trans, place, batch, sub, reps)
    ok = np.where(ms > 0, ms, np.inf)
    return sub[int(np.argmin(ok))], float(np.min(ok))


def timing_table(sizes, vtype=1, batch_points=1 << 20, reps=5, log=None):
    """Measured timings of every candidate of every size: rows of
    (n, batch, opts, features, ms).  batch = max(1, batch_points // n)."""
    rows = []
    for n in sizes:
        n = int(n)
        batch = max(1, batch_points // n)
        cands = candidates(n, vtype, 0, 1, batch)
        ms = measure(n, vtype, 0, 1, batch, cands, reps)
        for c, t in zip(cands, ms):
            if t > 0:
                rows.append({"n": n, "batch": batch, "opts": c, "ms": float(t),
                             "features": features(n, vtype, 0, 1, batch, c).tolist()})
        if log:
            log(n, len(cands))
    return rows


def save_table(rows, path):
    with open(path, "w") as f:
        json.dump(rows, f)


def load_table(path):
    with open(path) as f:
        return json.load(f)


def default_plan_ms(row_group):
    """Time of the planner's default plan (no options) within a size's rows."""
    for r in row_group:
        if not r["opts"]:
            return r["ms"]
    return None


def gflops(n, batch, ms):
    return 5.0 * n * math.log2(max(n, 2)) * batch / ms / 1e6


# schedules a ragged batch may give one length (gfft_ragged_create_opts):
# radix order, units per work item, pass split
RAGGED_CANDIDATES = [{}, {"radix_order": 1}, {"radix_order": 2}, {"units_per_block": 2}, {"units_per_block": 8},
                     {"max_pass_len": 256}, {"max_pass_len": 512}]


def time_ragged(n, members, vtype=1, trans=0, opts=None, reps=5):
    """ms of one ragged launch over `members` transforms of length n with the
    schedule `opts` for n (None when the schedule cannot be built)."""
    import torch

    from . import gfft as G
    try:
        rb = G.RaggedBatch([n] * members, G.VALUE_TYPES[vtype], G.TRANSFORM_TYPES[trans],
                           schedule={n: opts} if opts else None)
    except _lib.GfftError:
        return None
    dt = torch.float64 if vtype in (0, 2) else torch.float32
    x = torch.rand(2 * n * members, device="cuda", dtype=dt)
    y = torch.empty_like(x)
    for _ in range(2):
        rb.fft(x, y)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        rb.fft(x, y)
    e1.record()
    torch.cuda.synchronize()
    rb.close()
    return e0.elapsed_time(e1) / reps


def ragged_schedule(sizes, vtype=1, trans=0, cands=None, coverage=0.9, max_members=512, min_points=1 << 21, reps=5,
                    margin=0.03, log=None):
    """The measured schedule of a ragged batch: for the distinct lengths that
    carry `coverage` of the points (largest share first), every candidate in
    `cands` (default RAGGED_CANDIDATES) is timed inside the ragged kernel on
    transforms of that length -- as many as the batch holds, raised to at
    least `min_points` points so that a launch fills the GPU as the whole
    batch does, at most `max_members`; returns {length: opts} for the
    lengths whose fastest schedule beats the default by more than `margin`."""
    cands = RAGGED_CANDIDATES if cands is None else cands
    sizes = np.asarray(sizes, dtype=np.int64)
    lengths, counts = np.unique(sizes, return_counts=True)
    pts = lengths * counts
    total = float(pts.sum())
    chosen, acc = {}, 0.0
    for idx in np.argsort(-pts, kind="stable"):
        if acc >= coverage * total:
            break
        acc += float(pts[idx])
        n = int(lengths[idx])
        m = int(min(max(counts[idx], -(-min_points // n)), max_members))
        best, t_default = None, None
        for c in cands:
            t = time_ragged(n, m, vtype, trans, c, reps)
            if t is None:
                continue
            if not c:
                t_default = t
            if best is None or t < best[0]:
                best = (t, c)
        if log:
            log(n, m, best, t_default)
        if best and best[1] and (t_default is None or best[0] < (1.0 - margin) * t_default):
            chosen[n] = dict(best[1])
    return chosen
