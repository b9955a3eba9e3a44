"""GB300-native compressible RHS + SSP-RK path of amrsolver (sm_103a).

C-ABI: include/amrs_gb300.h (library built by amrsolver_gb300.build).
Python access: amrsolver_gb300.capi (ctypes; torch tensors hold device
memory).  Problem definitions and synthetic inputs: amrsolver_gb300.problems.
"""
from . import problems  # noqa: F401

__all__ = ["problems", "capi", "build"]
