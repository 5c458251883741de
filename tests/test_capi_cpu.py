"""CPU: the C-ABI library builds, loads and exports every declared symbol;
host logic (planner, option validation, facade errors) without a GPU."""
import ctypes
import glob
import os
import re

import pytest

import gfft_gb300
from gfft_gb300 import _lib
from gfft_gb300 import gfft as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        if "extern \"C\"" not in text and "extern \"C\" {" not in text:
            continue
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(gfft_\w+)\s*\(", text, re.M):
            syms.add(m.group(1))
    return syms


def test_build_and_load():
    path = gfft_gb300.build()
    assert os.path.exists(path)
    L = _lib.lib()
    assert L.gfft_version().decode().startswith("gfft_gb300")


def test_exports_every_declared_symbol():
    L = _lib.lib()
    declared = _declared_symbols()
    assert {"gfft_create", "gfft_exec", "gfft_destroy", "gfft_strerror"} <= declared
    for s in declared:
        assert hasattr(L, s), s
    assert set(_lib.EXPORTED) <= declared


def test_strerror():
    assert _lib.strerror(0) == "success"
    assert _lib.strerror(12) == ("Requested transform is not compiled! Check your instantiation of "
                                 "GenerateTransform class!")
    assert _lib.strerror(999) == "unknown status"


@pytest.mark.parametrize("n,vt,passes", [(1, 0, 1), (2, 1, 1), (1024, 0, 1), (4096, 1, 1), (8192, 1, 1),
                                         (8192, 0, 2), (65536, 0, 2), (786432, 0, 2), (390625, 1, 2), (248832, 0, 2),
                                         (1 << 24, 1, 3), (1 << 27, 1, 3)])
def test_plan_shapes(n, vt, passes):
    d = _lib.plan_query(n, vt, 0, 1, 1)
    assert d["n_global_passes"] == passes
    prod = 1
    for L, rs in zip(d["pass_len"], d["radices"]):
        p = 1
        for r in rs:
            p *= r
        assert p == L
        prod *= L
    assert prod == n
    if passes > 1:
        assert d["workspace_bytes"] == n * (16 if vt in (0, 2) else 8)


def test_plan_power_of_two_uses_radix16():
    d = _lib.plan_query(4096, 1, 0, 1, 65536)
    assert d["radices"] == [[16, 16, 16]]
    # FP32 8192: the length-specialised single pass, one transform per
    # block, 512 threads; variant 2 on request
    d = _lib.plan_query(8192, 1, 0, 1, 100)
    assert d["kernel_variant"] == [3] and d["threads"] == [512] and d["units"] == [1], d
    assert d["radices"] == [[16, 16, 8, 4]]
    assert _lib.plan_query(8192, 1, 0, 1, 100, {"kernel_variant": 2})["kernel_variant"] == [2]
    # FP32 16384: one pass of 1024 threads, straight from global memory; two
    # column-tile passes with any tuning option
    d = _lib.plan_query(16384, 1, 0, 1, 100)
    assert d["kernel_variant"] == [3] and d["threads"] == [1024] and d["radices"] == [[16, 16, 16, 4]], d
    assert _lib.plan_query(16384, 1, 0, 1, 100, {"stages": 1})["kernel_variant"] == [9, 9]
    assert _lib.plan_query(16384, 0, 0, 1, 100)["kernel_variant"] == [9, 9]
    d = _lib.plan_query(4096, 1, 0, 1, 1, {"max_radix": 4})
    assert d["radices"] == [[4] * 6]


def test_plan_column_kernel_selection():
    """Multi-pass power-of-two lengths take the tensor-copy column tiles (9)
    with passes of 64..2048 (two passes up to 2^22); on request, power-of-two
    passes of 64..1024 take the length-specialised column tiles (5); other
    lengths, explicit options and short transforms keep the prefetching
    column tiles (4)."""
    for n, vt, passes in ((1 << 13, 0, 2), (1 << 16, 1, 2), (1 << 20, 1, 2), (1 << 22, 1, 2), (1 << 24, 1, 3),
                          (1 << 20, 0, 2), (1 << 22, 0, 2), (1 << 27, 1, 3)):
        d = _lib.plan_query(n, vt, 0, 1, 1)
        assert d["n_global_passes"] == passes and set(d["kernel_variant"]) == {9}, (n, vt, d)
        assert all(64 <= L <= 2048 for L in d["pass_len"][:passes])
        # tiles of about 64 KB: units = 64 KB / (L * element size), 2 .. 64;
        # FP32 passes of 128 .. 512: 32 KB tiles (64 KB with blocks_per_sm 1)
        esz = 16 if vt == 0 else 8
        d1 = _lib.plan_query(n, vt, 0, 1, 1, {"blocks_per_sm": 1})
        for L, W, W1 in zip(d["pass_len"][:passes], d["units"][:passes], d1["units"][:passes]):
            assert W1 == max(2, min(64, 65536 // esz // L)), (L, W1)
            half = esz == 8 and 128 <= L <= 512
            assert W == (W1 // 2 if half else W1), (L, W, W1)
    # two passes of 4096 x 4096 on request
    d = _lib.plan_query(1 << 24, 1, 0, 1, 1, {"max_pass_len": 4096})
    assert d["pass_len"][:2] == [4096, 4096] and d["kernel_variant"][:2] == [9, 9], d
    for n, vt in ((1 << 16, 1), (1 << 20, 1), (1 << 24, 1), (1 << 20, 0), (1 << 22, 0)):
        d = _lib.plan_query(n, vt, 0, 1, 1, {"kernel_variant": 5})
        assert d["n_global_passes"] >= 2 and set(d["kernel_variant"]) == {5}, (n, vt, d)
        assert all(64 <= L <= 1024 for L in d["pass_len"])
    # FP32 passes without a compiled shape: the generic engine, radices in reverse order
    d = _lib.plan_query(5 ** 8 * 3, 1, 0, 1, 1)
    assert set(d["kernel_variant"]) <= {1, 7}, d
    assert set(_lib.plan_query(5 ** 8 * 3, 0, 0, 1, 1)["kernel_variant"]) <= {4, 7}  # FP64 keeps variant 4
    assert set(_lib.plan_query(1 << 20, 1, 0, 1, 1, {"kernel_variant": 4})["kernel_variant"]) == {4}
    assert set(_lib.plan_query(1 << 20, 1, 0, 1, 1, {"max_radix": 8})["kernel_variant"]) == {4}
    # an 8192-point FP64 transform of two 64 x 128 passes: tile (2048) divides n
    d = _lib.plan_query(8192, 0, 0, 1, 1, {"max_pass_len": 128, "kernel_variant": 5})
    assert set(d["kernel_variant"]) == {5}, d
    # 1024 points in two passes: a 2048-value tile would span transforms
    d = _lib.plan_query(1024, 0, 0, 1, 4, {"max_pass_len": 64})
    assert 5 not in d["kernel_variant"], d


def test_plan_mixed_kernel_selection():
    """Mixed-radix pass shapes with a compile-time kernel take variant 7."""
    # the 768-point pass too: mixed shapes move by tensor copies where W divides N / L and Ns
    assert _lib.plan_query(3 * 2 ** 18, 1, 0, 1, 8)["kernel_variant"] == [9, 9]
    assert _lib.plan_query(2 ** 10 * 3 ** 5, 1, 0, 1, 8)["kernel_variant"] == [9, 9]
    assert _lib.plan_query(3 * 2 ** 18, 1, 0, 1, 8, {"kernel_variant": 7})["kernel_variant"][1] == 7
    # tiles that do not fit a tensor map (16 units do not divide 360; 625-element rows are not a
    # multiple of 16 bytes) are gathered by cp.async, still variant 9; variant 7 on request
    assert _lib.plan_query(360 * 360, 1, 0, 1, 8)["kernel_variant"] == [9, 9]
    assert _lib.plan_query(5 ** 8, 1, 0, 1, 8)["kernel_variant"] == [9, 9]
    assert _lib.plan_query(5 ** 8, 1, 0, 1, 8, {"kernel_variant": 7})["kernel_variant"] == [7, 7]
    assert _lib.plan_query(5 ** 8, 0, 0, 1, 8)["kernel_variant"] == [7, 7]  # FP64: no gathered tiles
    assert _lib.plan_query(768, 1, 0, 1, 100)["kernel_variant"] == [7]
    assert _lib.plan_query(768, 1, 0, 1, 100, {"kernel_variant": 1})["kernel_variant"] == [1]
    assert 7 not in _lib.plan_query(768, 1, 2, 1, 100)["kernel_variant"]  # real: fused pre/post in the engine


def test_plan_errors():
    with pytest.raises(_lib.GfftError) as e:
        _lib.plan_query(0, 0, 0, 1)
    assert e.value.status == 1
    with pytest.raises(_lib.GfftError) as e:
        _lib.plan_query(16, 7, 0, 1)
    assert e.value.status == 2
    with pytest.raises(_lib.GfftError) as e:
        _lib.plan_query(16, 0, 9, 1)
    assert e.value.status == 3
    with pytest.raises(_lib.GfftError) as e:
        _lib.plan_query(16, 0, 0, 3)
    assert e.value.status == 4
    with pytest.raises(_lib.GfftError) as e:
        _lib.plan_query(16, 0, 0, 1, 1, {"max_radix": 6})
    assert e.value.status == 14
    # a prime factor larger than one block holds cannot be planned
    with pytest.raises(_lib.GfftError) as e:
        _lib.plan_query(2 * 4099, 1, 0, 1)
    assert e.value.status == 1


def test_real_plans():
    """The real pre/post pass runs inside the transform's own launches: the
    single pass of a short length, the last (forward) / first (inverse) pass
    of a multi-pass power-of-two length on the tensor-copy column tiles
    (C2b: FP64 N_real = 2^20 in two launches).  A pass whose real-pair tiles
    do not fit the shared memory (FP32 passes of 2048) keeps the separate
    pass; so do plans on other kernels."""
    for tr in (2, 3):
        d = _lib.plan_query(1 << 19, 0, tr, 0, 16)
        assert d["real_fused"] == 1 and d["kernels_per_exec"] == d["n_global_passes"] == 2, d
        assert d["kernel_variant"] == [9, 9]
    d = _lib.plan_query(2048, 0, 2, 0, 16)
    assert d["real_fused"] == 1 and d["kernels_per_exec"] == 1
    d = _lib.plan_query(1 << 21, 1, 3, 1, 1)  # first pass 2048 FP32
    assert d["real_fused"] == 0 and d["kernels_per_exec"] == d["n_global_passes"] + 1, d
    d = _lib.plan_query(1 << 19, 0, 2, 0, 16, {"kernel_variant": 5})
    assert d["real_fused"] == 0 and d["kernels_per_exec"] == d["n_global_passes"] + 1, d


def test_tags_and_ids():
    assert (G.DOUBLE.ID, G.FLOAT.ID, G.COMPLEX_DOUBLE.ID, G.COMPLEX_FLOAT.ID) == (0, 1, 2, 3)
    assert (G.DFT.ID, G.IDFT.ID, G.RDFT.ID, G.IRDFT.ID) == (0, 1, 2, 3)
    assert (G.IN_PLACE.ID, G.OUT_OF_PLACE.ID) == (0, 1)
    assert G.Serial.ID == 0 and G.OpenMP(4).ID == 3 and G.OpenMP(1) is G.Serial
    assert G.DFT.Inverse is G.IDFT and G.RDFT.Inverse is G.IRDFT
    assert G.PlaceGroup.Default is G.OUT_OF_PLACE and G.TransformTypeGroup.Default is G.DFT


def test_factory_unknown_combination_raises():
    ts = G.GenerateTransform([16, 32], G.DOUBLE, [G.DFT, G.IDFT], 1, G.Serial, G.OUT_OF_PLACE)
    assert len(ts.Result) == 4
    for bad in [dict(n=64, vtype_id=0), dict(n=16, vtype_id=1), dict(n=16, vtype_id=0, trans_id=2),
                dict(n=16, vtype_id=0, parall_id=3), dict(n=16, vtype_id=0, place_id=0),
                dict(n=16, vtype_id=0, dim=2)]:
        with pytest.raises(G.TransformFactoryError.Exception) as e:
            ts.CreateTransformObject(**bad)
        assert e.value.what() == ("Requested transform is not compiled! Check your instantiation of "
                                  "GenerateTransform class!")


def test_plan_opts_layout():
    assert ctypes.sizeof(_lib.PlanOpts) == 12 * 4


def test_cpp_facade_factory_errors():
    """include/gfft.h compiles as the reference's user code does and throws
    TransformFactoryError for unknown combinations (no GPU needed)."""
    import subprocess
    from tests.cpp import build_facade
    exe = build_facade.build()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade ok (cpu)" in r.stdout


def test_empty_options_mean_default_plan():
    from gfft_gb300 import tuner
    assert tuner.features(4096, 1, 0, 1, 8, {}).tolist() == tuner.features(4096, 1, 0, 1, 8, None).tolist()


def test_cosine_transform_plans_and_errors():
    """Cosine transforms (IDs 4-7) plan as the inner real transform of n - 1
    (type 1) or n (type 2) complex points; complex value types and a type-1
    length below two are rejected."""
    d = _lib.plan_query(1000, 0, 4, 1, 3)
    assert d["trans_id"] == 4 and d["pass_len"] == [999] and d["kernels_per_exec"] == 3
    assert _lib.plan_query(1000, 1, 6, 0, 1)["pass_len"] == [1000]
    with pytest.raises(_lib.GfftError):
        _lib.plan_query(64, 2, 6, 1)
    with pytest.raises(_lib.GfftError):
        _lib.plan_query(1, 0, 4, 1)
    with pytest.raises(_lib.GfftError):
        _lib.plan_query(64, 0, 8, 1)


def test_create_nd_argument_errors():
    """gfft_create_nd checks its arguments before touching a device."""
    L = _lib.lib()
    h = ctypes.c_void_p()
    dims = (ctypes.c_uint64 * 3)(64, 64, 64)
    assert L.gfft_create_nd(ctypes.byref(h), 4, dims, 1, 0, 1, 1) == 5      # rank
    assert L.gfft_create_nd(ctypes.byref(h), 2, dims, 1, 2, 1, 1) == 3      # real: not multi-dimensional
    assert L.gfft_create_nd(ctypes.byref(h), 2, dims, 7, 0, 1, 1) == 2      # value type
    assert L.gfft_create_nd(ctypes.byref(h), 2, dims, 1, 0, 5, 1) == 4      # place
    assert L.gfft_create_nd(ctypes.byref(h), 2, None, 1, 0, 1, 1) == 7      # null dims
    big = (ctypes.c_uint64 * 2)(8192, 16)
    assert L.gfft_create_nd(ctypes.byref(h), 2, big, 1, 0, 1, 1) == 1      # outer axis above one tile


def _header_shapes():
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gfft_gb300", "csrc",
                            "mixed_shapes.h")).read()
    mixed = [tuple(int(v) for v in m.group(2).split(",") if int(v) > 1)
             for m in re.finditer(r"\{(\d+), \{([\d, ]+)\}\}", src)]
    ragged = [tuple(int(v) for v in m.group(1).split(",") if int(v) > 1)
              for m in re.finditer(r"X\(\d+, ([\d, ]+)\)", src)]
    return mixed, ragged


def test_compiled_shapes_are_planner_shapes():
    """Every compiled pass shape (mixed_shapes.h) is the planner's own radix
    sequence for its length, so none is unreachable; the mixed-radix column
    kernel is chosen for each of its single-pass lengths."""
    mixed, ragged = _header_shapes()
    assert len(mixed) >= 8 and len(ragged) >= 30
    for rs in mixed + ragged:
        L = 1
        for r in rs:
            L *= r
        d = _lib.plan_query(L, 1, 0, 1, 16)
        assert tuple(d["radices"][0]) == rs, (L, rs, d["radices"])
    for rs in mixed:
        L = 1
        for r in rs:
            L *= r
        assert _lib.plan_query(L, 1, 0, 1, 16)["kernel_variant"] == [7], rs


def test_decimation_option():
    """decimation = 1 (frequency decimation) plans every pass on the generic
    engine; other values, or another kernel variant with it, are rejected."""
    for n, vt in ((64, 0), (1000, 1), (1 << 20, 1), (3 * 2 ** 14, 0)):
        d = _lib.plan_query(n, vt, 0, 1, 1, {"decimation": 1})
        assert set(d["kernel_variant"]) == {1}, d
    for bad in ({"decimation": 2}, {"decimation": -1}, {"decimation": 1, "kernel_variant": 9}):
        with pytest.raises(_lib.GfftError) as e:
            _lib.plan_query(64, 0, 0, 1, 1, bad)
        assert e.value.status == 14


def test_mixed_column_tile_shapes():
    """Shape arithmetic of the mixed-radix column tiles (host only): units per
    tile (power of two, tile <= 64 KB), 512 threads, shared memory within one
    SM for one stage; tensor copies need boxes starting on 128-byte
    boundaries (729 = 9.9.9 and 625 = 5.5.5.5: odd row counts per box of
    64-byte rows do not), gathers take any shape of the compiled list, at
    most two stages."""
    import ctypes
    L = _lib.lib()
    f = L.gfft_colmix_shape
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t)]

    def shape(dbl, n, rs, stages, gather):
        arr = (ctypes.c_int * 4)(*(list(rs) + [1] * (4 - len(rs))))
        w, t, sm = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        st = f(dbl, n, arr, len(rs), stages, gather, ctypes.byref(w), ctypes.byref(t), ctypes.byref(sm))
        return st, w.value, t.value, sm.value

    for n, rs in ((768, (16, 16, 3)), (576, (16, 12, 3)), (432, (16, 9, 3)), (1000, (10, 10, 10)),
                  (480, (16, 15, 2)), (360, (15, 12, 2))):
        for dbl in (0, 1):
            esz = 16 if dbl else 8
            st, w, t, sm = shape(dbl, n, rs, 1, 0)
            assert st == 0 and t == 512, (n, dbl)
            assert w & (w - 1) == 0 and w * n * esz <= 65536 < 2 * w * n * esz, (n, dbl, w)
            assert sm <= 227 * 1024, (n, dbl, sm)
            assert shape(dbl, n, rs, 1, 1)[0] == 0
    assert shape(0, 729, (9, 9, 9), 1, 0)[0] == 1   # no tensor copies
    assert shape(0, 625, (5, 5, 5, 5), 1, 0)[0] == 1
    assert shape(0, 625, (5, 5, 5, 5), 2, 1)[0] == 0
    assert shape(0, 729, (9, 9, 9), 1, 1)[0] == 0   # gathers
    assert shape(0, 729, (9, 9, 9), 3, 1)[0] == 1   # gathers: one or two stages
    assert shape(0, 768, (16, 8, 6), 1, 0)[0] == 1  # not a compiled shape
    assert shape(0, 1024, (16, 16, 4), 1, 0)[0] == 1  # powers of two are col.cuh's
