"""nav24_gb300 - GB300-native bundle-adjustment back end for nav24.

The product is the native library libnavba.so (CUDA sm_103a kernels behind the C ABI of
include/nav_ba.h).  This package holds its build recipe, a ctypes binding (``Context``), the
seeded synthetic workloads and the reference-shaped Python interface (``GraphOptimGpu``).
"""
from . import abi
from ._lib import BAError, Context, NativeLibraryMissing, load

__all__ = ["abi", "Context", "BAError", "NativeLibraryMissing", "load"]
