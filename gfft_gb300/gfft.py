"""Python mirror of GFFT's factory / transform-object API over the C ABI.

Same names, IDs, argument meaning and error behaviour as the reference
(scpp/gfft):

- value types ``DOUBLE, FLOAT, COMPLEX_DOUBLE, COMPLEX_FLOAT`` (IDs 0..3),
  transform types ``DFT, IDFT, RDFT, IRDFT`` (IDs 0..3, with ``Sign`` and
  ``Inverse``), places ``IN_PLACE, OUT_OF_PLACE`` (0, 1), parallel policies
  ``Serial`` (0) and ``OpenMP(NT)`` (NT-1)  -- src/gfftpolicy.h:78-453;
- ``GenerateTransform(NList, VType, TransType, Dim, Parall, Place)`` builds the
  cartesian product of the parameter lists and
  ``CreateTransformObject(n, vtype_id, trans_id, dim, parall_id, place_id)``
  returns an object or raises ``TransformFactoryError.Exception`` whose
  ``what()`` is the reference's text  -- src/gfftgen.h:133-231;
- objects have ``fft(data)`` (in place) or ``fft(src, dst)`` (out of place)
  -- src/gfftpolicy.h:46-58; ``ifft`` is an added convenience that runs the
  inverse object (IDFT for DFT, IRDFT for RDFT and vice versa).

Arrays: ``torch`` CUDA tensors run on the device (current stream, async);
numpy arrays (or CPU tensors) go through the host entry point (copy in,
transform, copy out).  Real dtypes hold interleaved (re, im); complex dtypes
are the same bytes.  An optional ``batch`` (transforms back to back) is the
one extension of the signatures.
"""
from __future__ import annotations

import ctypes
import itertools
from typing import Iterable

import numpy as np

from . import _lib


# ---------------------------------------------------------------- tags ----
class _Tag:
    ID = -1

    @classmethod
    def name(cls):
        return cls.__name__


class DOUBLE(_Tag):
    ID = 0
    np_dtype = np.float64
    per_point = 2


class FLOAT(_Tag):
    ID = 1
    np_dtype = np.float32
    per_point = 2


class COMPLEX_DOUBLE(_Tag):
    ID = 2
    np_dtype = np.complex128
    per_point = 1


class COMPLEX_FLOAT(_Tag):
    ID = 3
    np_dtype = np.complex64
    per_point = 1


class DFT(_Tag):
    ID = 0
    Sign = 1


class IDFT(_Tag):
    ID = 1
    Sign = -1


class RDFT(_Tag):
    ID = 2
    Sign = 1


class IRDFT(_Tag):
    ID = 3
    Sign = -1


class DCT1(_Tag):
    """X_k = sum_l x_l cos(pi k l / (n-1)) (the reference's direct.h DCT1)."""
    ID = 4
    Sign = 1


class IDCT1(_Tag):
    """The DCT1 sum divided by n (the reference's Backward policy)."""
    ID = 5
    Sign = -1


class DCT2(_Tag):
    """X_k = sum_l x_l cos(pi k l / n) (the reference's direct.h DCT2)."""
    ID = 6
    Sign = 1


class IDCT2(_Tag):
    """The DCT2 sum divided by n."""
    ID = 7
    Sign = -1


DFT.Inverse, IDFT.Inverse, RDFT.Inverse, IRDFT.Inverse = IDFT, DFT, IRDFT, RDFT
DCT1.Inverse, IDCT1.Inverse, DCT2.Inverse, IDCT2.Inverse = IDCT1, DCT1, IDCT2, DCT2
COSINE_TYPES = (DCT1, IDCT1, DCT2, IDCT2)


class IN_PLACE(_Tag):
    ID = 0


class OUT_OF_PLACE(_Tag):
    ID = 1


class Serial(_Tag):
    ID = 0
    NParProc = 1


_OPENMP = {}


def OpenMP(NT: int):
    """``OpenMP<NT>`` tag (ID = NT-1; OpenMP<0>, OpenMP<1> are Serial)."""
    if NT <= 1:
        return Serial
    if NT not in _OPENMP:
        _OPENMP[NT] = type("OpenMP<%d>" % NT, (_Tag,), {"ID": NT - 1, "NParProc": NT})
    return _OPENMP[NT]


VALUE_TYPES = {0: DOUBLE, 1: FLOAT, 2: COMPLEX_DOUBLE, 3: COMPLEX_FLOAT}
TRANSFORM_TYPES = {0: DFT, 1: IDFT, 2: RDFT, 3: IRDFT, 4: DCT1, 5: IDCT1, 6: DCT2, 7: IDCT2}
PLACES = {0: IN_PLACE, 1: OUT_OF_PLACE}


class ValueTypeGroup:
    FullList = [DOUBLE, FLOAT, COMPLEX_DOUBLE, COMPLEX_FLOAT]
    Default = DOUBLE


class TransformTypeGroup:
    FullList = [DFT, IDFT, RDFT, IRDFT]
    Default = DFT


class ParallelizationGroup:
    FullList = [Serial, OpenMP(2), OpenMP(4), OpenMP(8)]
    Default = Serial


class PlaceGroup:
    FullList = [IN_PLACE, OUT_OF_PLACE]
    Default = OUT_OF_PLACE


class TransformFactoryError:
    """Raised for a combination that GenerateTransform did not generate."""

    class Exception(Exception):  # noqa: A001 - the reference's nested name
        def what(self):
            return "Requested transform is not compiled! Check your instantiation of GenerateTransform class!"

        def __str__(self):
            return self.what()


# ---------------------------------------------------------- objects ----
def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _as_list(x) -> list:
    if isinstance(x, (list, tuple)):
        return list(x)
    return [x]


def _learned_opts(n, vtype, trans, place, batch, plan):
    """Plan options from the learned planner (gfft_gb300.tuner)."""
    from . import tuner
    if plan not in ("learned", "measured"):
        raise ValueError("plan: None, 'learned' or 'measured'")
    model = tuner.default_model()
    if model is None:
        raise RuntimeError("no shipped cost model")
    opts, _ = tuner.choose(model, n, vtype, trans, place, batch, k=1 if plan == "learned" else 5)
    return opts


class TransformObject:
    """A transform object (the reference's ``Transform<...>::Instance``).

    Owns a C-ABI handle: device twiddle tables and workspace.  ``fft`` is
    asynchronous on the current torch stream for device tensors.
    """

    def __init__(self, n, vtype, trans, dim=1, parall=Serial, place=OUT_OF_PLACE, batch=1, opts=None, plan=None):
        """``plan``: None (the planner's rules, or ``opts``), "learned" (the
        shipped cost model's first choice among the tuner's candidates, no
        measurement) or "measured" (the best measured of the model's top 5:
        the pruned search)."""
        self.n = int(n)
        self.VType = vtype
        self.Type = trans
        self.Parall = parall
        self.Place = place
        self.batch = int(batch)
        self.dim = int(dim)
        if plan is not None and not opts:
            opts = _learned_opts(self.n, vtype.ID, trans.ID, place.ID, self.batch, plan)
        L = _lib.lib()
        h = ctypes.c_void_p()
        if not opts:  # None or {}: the default plan
            st = L.gfft_create(ctypes.byref(h), self.n, vtype.ID, trans.ID, self.dim, parall.ID, place.ID,
                               self.batch)
        else:
            o = _lib.make_opts(opts)
            st = L.gfft_create_opts(ctypes.byref(h), self.n, vtype.ID, trans.ID, self.dim, parall.ID, place.ID,
                                    self.batch, ctypes.byref(o))
        _lib.check(st, "gfft_create(n=%d, %s, %s, %s)" % (self.n, vtype.name(), trans.name(), place.name()))
        self._h = h
        self._inverse = None
        self._opts = opts

    # number of scalars (real dtype) of one batch
    @property
    def scalars(self):
        return (1 if self.Type in COSINE_TYPES else 2) * self.n * self.batch

    def info(self):
        inf = _lib.PlanInfo()
        _lib.check(_lib.lib().gfft_get_info(self._h, ctypes.byref(inf)))
        return _lib.info_dict(inf)

    def _check_array(self, x, name):
        if _is_torch(x):
            import torch
            ok = {DOUBLE: (torch.float64, torch.complex128), COMPLEX_DOUBLE: (torch.float64, torch.complex128),
                  FLOAT: (torch.float32, torch.complex64), COMPLEX_FLOAT: (torch.float32, torch.complex64)}
            if x.dtype not in ok[self.VType]:
                raise TypeError("%s: dtype %s does not match %s" % (name, x.dtype, self.VType.name()))
            if not x.is_contiguous():
                raise ValueError("%s must be contiguous" % name)
            nbytes = x.numel() * x.element_size()
        else:
            x = np.asarray(x)
            nbytes = x.nbytes
        want = self.scalars * (8 if self.VType in (DOUBLE, COMPLEX_DOUBLE) else 4)
        if nbytes != want:
            raise ValueError("%s holds %d bytes, the transform needs %d" % (name, nbytes, want))
        return x

    def fft(self, src, dst=None):
        """``fft(data)`` in place, ``fft(src, dst)`` out of place (reference
        semantics).  Returns the output array."""
        if self.Place is IN_PLACE:
            if dst is not None and dst is not src:
                raise _lib.GfftError(4, "in-place object called with two arrays")
            dst = src
        elif dst is None:
            raise TypeError("an OUT_OF_PLACE object needs fft(src, dst)")
        src = self._check_array(src, "src")
        dst = self._check_array(dst, "dst")
        L = _lib.lib()
        if _is_torch(src) and src.is_cuda:
            import torch
            if not (_is_torch(dst) and dst.is_cuda):
                raise TypeError("src is on the device, dst is not")
            stream = torch.cuda.current_stream(src.device).cuda_stream
            st = L.gfft_exec(self._h, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                             ctypes.c_void_p(stream))
            _lib.check(st, "gfft_exec")
            return dst
        # host arrays: the C ABI's host entry point stages through the device
        if _is_torch(src):
            s_ptr, d_ptr = src.data_ptr(), dst.data_ptr()
        else:
            if not (isinstance(dst, np.ndarray) and dst.flags.c_contiguous and dst.flags.writeable):
                raise ValueError("dst must be a writeable contiguous array")
            src = np.ascontiguousarray(src)
            s_ptr, d_ptr = src.ctypes.data, dst.ctypes.data
        st = L.gfft_exec_host(self._h, ctypes.c_void_p(s_ptr), ctypes.c_void_p(d_ptr), None)
        _lib.check(st, "gfft_exec_host")
        return dst

    def inverse_object(self):
        if self._inverse is None:
            self._inverse = TransformObject(self.n, self.VType, self.Type.Inverse, self.dim, self.Parall, self.Place,
                                            self.batch, self._opts)
        return self._inverse

    def ifft(self, src, dst=None):
        """Run the inverse transform type on the same length and layout."""
        return self.inverse_object().fft(src, dst)

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gfft_destroy(self._h)
            self._h = None
        if self._inverse is not None:
            self._inverse.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TransformND(TransformObject):
    """A multi-dimensional complex DFT / IDFT of ``batch`` row-major arrays of
    shape ``dims`` (1 to 3 axes, the last fastest) through
    ``gfft_create_nd``; ``fft`` as for ``TransformObject``.  No reference
    counterpart (the reference implements only ``Dim = 1``)."""

    def __init__(self, dims, vtype, trans=None, place=None, batch=1):
        self.dims = tuple(int(d) for d in dims)
        self.n = int(np.prod(self.dims))
        self.VType = vtype
        self.Type = trans or DFT
        self.Parall = Serial
        self.Place = place or OUT_OF_PLACE
        self.batch = int(batch)
        self.dim = len(self.dims)
        self._inverse = None
        self._opts = None
        L = _lib.lib()
        arr = (ctypes.c_uint64 * len(self.dims))(*self.dims)
        h = ctypes.c_void_p()
        _lib.check(L.gfft_create_nd(ctypes.byref(h), len(self.dims), arr, vtype.ID, self.Type.ID, self.Place.ID,
                                    self.batch), "gfft_create_nd(%s, %s, %s)" % (self.dims, vtype.name(),
                                                                                 self.Type.name()))
        self._h = h

    def inverse_object(self):
        if self._inverse is None:
            self._inverse = TransformND(self.dims, self.VType, self.Type.Inverse, self.Place, self.batch)
        return self._inverse


class RaggedBatch:
    """Transforms of many lengths (back to back, in the order of ``sizes``)
    in one persistent launch replayed from a CUDA graph (gfft_ragged_*).
    ``fft(src, dst)`` takes device tensors on the current stream.

    ``schedule``: None (the planner's defaults), ``{length: plan options}``
    (gfft_ragged_create_opts: pass split, radix order, units per work item)
    or ``"tuned"``: the autotuner's measured schedule
    (``tuner.ragged_schedule``)."""

    def __init__(self, sizes, VType=FLOAT, Type=DFT, schedule=None):
        import numpy as _np
        self.sizes = _np.ascontiguousarray(_np.asarray(sizes, dtype=_np.uint64))
        self.VType, self.Type = VType, Type
        if isinstance(schedule, str):
            if schedule != "tuned":
                raise ValueError("schedule: None, a dict or 'tuned'")
            from . import tuner
            schedule = tuner.ragged_schedule(self.sizes, VType.ID, Type.ID)
        self.schedule = dict(schedule or {})
        L = _lib.lib()
        h = ctypes.c_void_p()
        lens = _np.ascontiguousarray(_np.array(sorted(self.schedule), dtype=_np.uint64))
        opts = (_lib.PlanOpts * max(1, len(lens)))()
        for i, n in enumerate(lens):
            for k, v in self.schedule[int(n)].items():
                setattr(opts[i], k, int(v))
        st = L.gfft_ragged_create_opts(ctypes.byref(h), int(self.sizes.size),
                                       self.sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), VType.ID, Type.ID,
                                       int(lens.size), lens.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), opts)
        _lib.check(st, "gfft_ragged_create_opts")
        self._h = h
        self.total_points = int(self.sizes.sum())

    def plan(self, n):
        """The schedule used for length n (gfft_ragged_get_plan)."""
        inf = _lib.PlanInfo()
        _lib.check(_lib.lib().gfft_ragged_get_plan(self._h, int(n), ctypes.byref(inf)), "gfft_ragged_get_plan")
        return _lib.info_dict(inf)

    def info(self):
        tp, it = ctypes.c_uint64(), ctypes.c_uint64()
        nd, mp, gr = ctypes.c_int(), ctypes.c_int(), ctypes.c_uint()
        _lib.check(_lib.lib().gfft_ragged_get_info(self._h, ctypes.byref(tp), ctypes.byref(it), ctypes.byref(nd),
                                                   ctypes.byref(mp), ctypes.byref(gr)))
        return {"total_points": tp.value, "items": it.value, "distinct_lengths": nd.value, "max_passes": mp.value,
                "grid": gr.value}

    def status(self):
        st = ctypes.c_int(-1)
        _lib.check(_lib.lib().gfft_ragged_get_status(self._h, ctypes.byref(st)))
        return st.value

    def fft(self, src, dst):
        import torch
        stream = torch.cuda.current_stream(src.device).cuda_stream
        _lib.check(_lib.lib().gfft_ragged_exec(self._h, ctypes.c_void_p(src.data_ptr()),
                                               ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(stream)),
                   "gfft_ragged_exec")
        return dst

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gfft_ragged_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Transform:
    """``Transform<N, VType, Type, Dim, Parall, Place>`` (src/gfftgen.h:46-87):
    ``Transform(...).Instance()`` / ``Create()`` return a new object."""

    def __init__(self, N, VType=DOUBLE, Type=DFT, Dim=1, Parall=Serial, Place=OUT_OF_PLACE, batch=1):
        self.Len = int(N)
        self.args = (N, VType, Type, Dim, Parall, Place, batch)

    def Instance(self):
        N, VType, Type, Dim, Parall, Place, batch = self.args
        return TransformObject(N, VType, Type, Dim, Parall, Place, batch)

    Create = Instance


class GenerateTransform:
    """``GenerateTransform<NList, VType, TransType, Dim, Parall, Place>``.

    Every parameter but ``NList`` is a tag or a list of tags; ``NList`` is a
    list of lengths (or a single length).  Objects are created on demand
    (the reference compiles them all up front) and each call returns a new
    object owned by the caller."""

    def __init__(self, NList, VType=ValueTypeGroup.Default, TransType=TransformTypeGroup.Default, Dim=1,
                 Parall=ParallelizationGroup.Default, Place=PlaceGroup.Default, batch=1):
        self.NList = [int(n) for n in _as_list(NList)]
        self.VTypes = _as_list(VType)
        self.TransTypes = _as_list(TransType)
        self.Dims = [int(d) for d in _as_list(Dim)]
        self.Paralls = _as_list(Parall)
        self.Places = _as_list(Place)
        self.batch = batch
        self.Result = list(itertools.product(self.NList, self.VTypes, self.TransTypes, self.Dims, self.Paralls,
                                             self.Places))

    def CreateTransformObject(self, n, vtype_id, trans_id=TransformTypeGroup.Default.ID, dim=1,
                              parall_id=ParallelizationGroup.Default.ID, place_id=PlaceGroup.Default.ID, batch=None):
        def pick(tags: Iterable, tid):
            for t in tags:
                if t.ID == tid:
                    return t
            return None

        vt = pick(self.VTypes, vtype_id)
        tt = pick(self.TransTypes, trans_id)
        pa = pick(self.Paralls, parall_id)
        pl = pick(self.Places, place_id)
        if int(n) not in self.NList or vt is None or tt is None or pa is None or pl is None or dim not in self.Dims:
            raise TransformFactoryError.Exception()
        return TransformObject(n, vt, tt, dim, pa, pl, self.batch if batch is None else batch)
