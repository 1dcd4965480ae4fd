"""GB300-native streaming DBSCAN: the per-slide clustering path of RTDBStream.

The numeric work runs in librtdbs.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/rtdbs.h).  This package holds the ctypes binding, the
nvcc build step and seeded workload generators.
"""
from .engine import (PREC_FP32, PREC_FP64, Engine, RtdbsError, load_library)  # noqa: F401

__all__ = ["Engine", "RtdbsError", "load_library", "PREC_FP32", "PREC_FP64"]
