"""ctypes binding of the in-tree C ABI library (include/gfft_gb300.h).

There is no CPU fallback: when ``libgfft_gb300.so`` is missing the import of
a compute entry point raises.  ``build()`` compiles it in place.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# GFFT_GB300_DEBUG=1 loads the debug build (device-side bounds checks)
DEBUG = os.environ.get("GFFT_GB300_DEBUG") == "1"
LIB_PATH = os.path.join(HERE, "libgfft_gb300_debug.so" if DEBUG else "libgfft_gb300.so")

# status codes (include/gfft_gb300.h)
GFFT_OK = 0
STATUS_NAMES = {
    0: "GFFT_OK", 1: "GFFT_E_INVALID_SIZE", 2: "GFFT_E_INVALID_TYPE", 3: "GFFT_E_INVALID_TRANSFORM",
    4: "GFFT_E_INVALID_PLACE", 5: "GFFT_E_INVALID_DIM", 6: "GFFT_E_INVALID_PARALL", 7: "GFFT_E_NULL_POINTER",
    8: "GFFT_E_MISALIGNED", 9: "GFFT_E_ALLOC", 10: "GFFT_E_CUDA", 11: "GFFT_E_INVALID_HANDLE",
    12: "GFFT_E_NOT_IN_LIST", 13: "GFFT_E_TIMEOUT", 14: "GFFT_E_INVALID_PLAN", 15: "GFFT_E_TOO_LARGE",
    16: "GFFT_E_BOUNDS",
}

# every symbol the header declares, checked by the CPU tests
EXPORTED = ["gfft_create", "gfft_create_opts", "gfft_create_nd", "gfft_exec", "gfft_exec_host", "gfft_destroy", "gfft_strerror",
            "gfft_get_info", "gfft_plan_query", "gfft_get_device_status", "gfft_selftest_bounded_wait",
            "gfft_exec_noalloc", "gfft_ragged_create", "gfft_ragged_create_opts", "gfft_ragged_get_plan", "gfft_ragged_exec", "gfft_ragged_get_info",
            "gfft_ragged_get_status", "gfft_ragged_destroy", "gfft_tune_candidates", "gfft_tune_measure",
            "gfft_plan_features", "gfft_mlp_create", "gfft_mlp_num_params", "gfft_mlp_get_params", "gfft_mlp_set_params",
            "gfft_mlp_train", "gfft_mlp_predict", "gfft_mlp_gradients", "gfft_mlp_destroy", "gfft_version",
            "gfft_measure_fma_peak", "gfft_debug_build", "gfft_selftest_bounds_check"]
NFEAT = 25


class PlanOpts(ctypes.Structure):
    _fields_ = [("radix_order", ctypes.c_int), ("max_radix", ctypes.c_int), ("threads_per_block", ctypes.c_int),
                ("units_per_block", ctypes.c_int), ("max_pass_len", ctypes.c_int),
                ("kernel_variant", ctypes.c_int), ("stages", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("decimation", ctypes.c_int), ("reserved", ctypes.c_int * 3)]


class PlanInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("batch", ctypes.c_uint64), ("vtype_id", ctypes.c_int),
                ("trans_id", ctypes.c_int), ("place_id", ctypes.c_int), ("n_global_passes", ctypes.c_int),
                ("pass_len", ctypes.c_int * 4), ("radices", (ctypes.c_int * 16) * 4), ("threads", ctypes.c_int * 4),
                ("units", ctypes.c_int * 4), ("kernel_variant", ctypes.c_int * 4),
                ("workspace_bytes", ctypes.c_uint64), ("table_bytes", ctypes.c_uint64),
                ("real_fused", ctypes.c_int), ("kernels_per_exec", ctypes.c_int)]


class GfftError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = "%s (%d): %s" % (STATUS_NAMES.get(status, "?"), status, strerror(status) if _lib else "")
        if what:
            msg = what + ": " + msg
        super().__init__(msg)


_lib = None


def build(force=False):
    from . import buildlib
    return buildlib.build(force=force, debug=DEBUG)


def lib():
    """The loaded library; raises if the CUDA extension has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("gfft_gb300 CUDA extension not built (%s missing); run "
                               "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        vp, ci, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64
        L.gfft_create.argtypes = [ctypes.POINTER(vp), u64, ci, ci, ci, ci, ci, u64]
        L.gfft_create_opts.argtypes = [ctypes.POINTER(vp), u64, ci, ci, ci, ci, ci, u64, ctypes.POINTER(PlanOpts)]
        L.gfft_create_nd.argtypes = [ctypes.POINTER(vp), ci, ctypes.POINTER(u64), ci, ci, ci, u64]
        L.gfft_exec.argtypes = [vp, vp, vp, vp]
        L.gfft_exec_host.argtypes = [vp, vp, vp, vp]
        L.gfft_destroy.argtypes = [vp]
        L.gfft_strerror.argtypes = [ci]
        L.gfft_strerror.restype = ctypes.c_char_p
        L.gfft_get_info.argtypes = [vp, ctypes.POINTER(PlanInfo)]
        L.gfft_plan_query.argtypes = [u64, ci, ci, ci, u64, ctypes.POINTER(PlanOpts), ctypes.POINTER(PlanInfo)]
        L.gfft_version.restype = ctypes.c_char_p
        L.gfft_get_device_status.argtypes = [vp, ctypes.POINTER(ci)]
        L.gfft_selftest_bounded_wait.argtypes = [ctypes.c_longlong, ctypes.POINTER(ci)]
        L.gfft_exec_noalloc.argtypes = [u64, ci, ci, u64, vp, vp, vp]
        L.gfft_ragged_create.argtypes = [ctypes.POINTER(vp), u64, ctypes.POINTER(u64), ci, ci]
        L.gfft_ragged_create_opts.argtypes = [ctypes.POINTER(vp), u64, ctypes.POINTER(u64), ci, ci, u64,
                                              ctypes.POINTER(u64), ctypes.POINTER(PlanOpts)]
        L.gfft_ragged_get_plan.argtypes = [vp, u64, ctypes.POINTER(PlanInfo)]
        L.gfft_ragged_exec.argtypes = [vp, vp, vp, vp]
        L.gfft_ragged_get_info.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(ci),
                                           ctypes.POINTER(ci), ctypes.POINTER(ctypes.c_uint)]
        L.gfft_ragged_get_status.argtypes = [vp, ctypes.POINTER(ci)]
        L.gfft_ragged_destroy.argtypes = [vp]
        fp = ctypes.POINTER(ctypes.c_float)
        L.gfft_tune_candidates.argtypes = [u64, ci, ci, ci, u64, ctypes.POINTER(PlanOpts), ci, ctypes.POINTER(ci)]
        L.gfft_tune_measure.argtypes = [u64, ci, ci, ci, u64, ctypes.POINTER(PlanOpts), ci, vp, vp, ci, fp]
        L.gfft_plan_features.argtypes = [u64, ci, ci, ci, u64, ctypes.POINTER(PlanOpts), fp]
        L.gfft_mlp_create.argtypes = [ctypes.POINTER(vp), ci, ci, ci, u64]
        L.gfft_mlp_num_params.argtypes = [vp]
        L.gfft_mlp_get_params.argtypes = [vp, fp]
        L.gfft_mlp_set_params.argtypes = [vp, fp]
        L.gfft_mlp_train.argtypes = [vp, fp, fp, ci, ci, ctypes.c_float, fp]
        L.gfft_mlp_predict.argtypes = [vp, fp, ci, fp]
        L.gfft_mlp_gradients.argtypes = [vp, fp, fp, ci, fp, fp]
        L.gfft_mlp_destroy.argtypes = [vp]
        dp = ctypes.POINTER(ctypes.c_double)
        L.gfft_measure_fma_peak.argtypes = [ci, ci, dp, dp]
        L.gfft_debug_build.argtypes = []
        L.gfft_selftest_bounds_check.argtypes = [ctypes.POINTER(ci), ctypes.POINTER(ci)]
        for name in EXPORTED:
            getattr(L, name).restype = getattr(L, name).restype or ci
        L.gfft_strerror.restype = ctypes.c_char_p
        L.gfft_version.restype = ctypes.c_char_p
        _lib = L
    return _lib


def info_dict(inf: "PlanInfo") -> dict:
    d = {f: getattr(inf, f) for f, _ in PlanInfo._fields_}
    g = inf.n_global_passes
    d["pass_len"] = list(inf.pass_len)[:g]
    d["radices"] = [[r for r in inf.radices[i] if r] for i in range(g)]
    d["threads"] = list(inf.threads)[:g]
    d["units"] = list(inf.units)[:g]
    d["kernel_variant"] = list(inf.kernel_variant)[:g]
    return d


def make_opts(opts: dict | None):
    if not opts:
        return None
    o = PlanOpts()
    for k, v in opts.items():
        setattr(o, k, int(v))
    return o


def plan_query(n, vtype_id, trans_id, place_id, batch=1, opts=None) -> dict:
    """Plan without a GPU (gfft_plan_query)."""
    inf = PlanInfo()
    o = make_opts(opts)
    check(lib().gfft_plan_query(n, vtype_id, trans_id, place_id, batch, ctypes.byref(o) if o else None,
                                ctypes.byref(inf)), "gfft_plan_query")
    return info_dict(inf)


def strerror(status: int) -> str:
    return lib().gfft_strerror(status).decode()


def check(status: int, what: str = ""):
    if status != GFFT_OK:
        raise GfftError(status, what)


def measure_fma_peak(dbl: int, iters: int = 1 << 16) -> dict:
    """Multiply-add throughput of the CUDA cores (FP64 or FP32), best of five
    timed launches over every SM (gfft_measure_fma_peak)."""
    g, ms = ctypes.c_double(), ctypes.c_double()
    check(lib().gfft_measure_fma_peak(int(dbl), int(iters), ctypes.byref(g), ctypes.byref(ms)),
          "gfft_measure_fma_peak")
    return {"gflops": g.value, "ms": ms.value, "iters": iters}
