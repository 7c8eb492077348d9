"""GB300-native tTV-NESTA: OpenCLIPER's compressed-sensing hot path on sm_103a.

The compute path is libgbnesta.so (CUDA kernels behind the C ABI in
include/gbn.h).  This package holds its in-tree build recipe and a ctypes
binding; there is no CPU fallback.
"""
from ._abi import GbnError, NestaParams, NestaStats, lib  # noqa: F401
from .api import (PRECISION_FP32, PRECISION_MIXED, Batch, Context, DeviceArray, Problem,  # noqa: F401
                  nesta_params, nesta_run_host, registration, registration_info, registration_params,
                  supported_lengths)

__all__ = ["GbnError", "NestaParams", "NestaStats", "lib", "Context", "DeviceArray", "Problem", "Batch",
           "PRECISION_FP32", "PRECISION_MIXED", "nesta_params", "nesta_run_host", "supported_lengths",
           "registration", "registration_params", "registration_info"]
