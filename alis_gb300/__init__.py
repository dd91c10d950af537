"""GB300-native ALiS engine.

The product is a C library (alis_gb300/lib/libalis_gb300.so) exporting
the ALiS C API (include/alis_c.h) on top of hand-written sm_103a kernels
reached through the device C-ABI (include/alisgpu.h).  This package
builds it (alis_gb300.build) and loads it for Python callers.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libalis_gb300.so")
_lib = None


def library():
    """Load the engine library, building it first if needed."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build
            build.build_engine()
        _lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    return _lib
