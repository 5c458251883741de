"""gfft_gb300: GFFT's transform hot path on one GB300 (sm_103a).

Public API mirrors scpp/gfft's factory and transform objects (see gfft.py);
the compute runs in the in-tree CUDA library ``libgfft_gb300.so`` through its
C ABI (include/gfft_gb300.h).  There is no CPU fallback.
"""
from .gfft import (COMPLEX_DOUBLE, COMPLEX_FLOAT, DFT, DOUBLE, FLOAT, IDFT, IN_PLACE, IRDFT, OUT_OF_PLACE, RDFT,
                   GenerateTransform, OpenMP, ParallelizationGroup, PlaceGroup, RaggedBatch, Serial, Transform,
                   TransformFactoryError, TransformObject, TransformTypeGroup, ValueTypeGroup)
from ._lib import GfftError, build, lib

__all__ = ["COMPLEX_DOUBLE", "COMPLEX_FLOAT", "DFT", "DOUBLE", "FLOAT", "IDFT", "IN_PLACE", "IRDFT", "OUT_OF_PLACE",
           "RDFT", "RaggedBatch", "GenerateTransform", "OpenMP", "ParallelizationGroup", "PlaceGroup", "Serial", "Transform",
           "TransformFactoryError", "TransformObject", "TransformTypeGroup", "ValueTypeGroup", "GfftError", "build",
           "lib"]
