"""GB300-native streaming DBSCAN: the per-slide clustering path of RTDBStream.

The numeric work runs in librtdbs.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/rtdbs.h).  This package holds the ctypes binding, the
nvcc build step, the launch-configuration autotuner and seeded workload
generators.
"""
from .engine import (PREC_FP32, PREC_FP64, Engine, Pool, RtdbsError, load_library,  # noqa: F401
                     make_params, stream_bytes)

__all__ = ["Engine", "Pool", "RtdbsError", "load_library", "make_params", "stream_bytes", "PREC_FP32",
           "PREC_FP64"]
