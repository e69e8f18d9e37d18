"""GB300-native (sm_103a) acceleration structures for LuisaCompute's Mesh/Accel path.

The compute path is liblcx_accel.so (hand-written CUDA kernels behind the C ABI
of include/lcx_accel.h); this package builds it, binds it and mirrors the
reference's host API.  There is no CPU fallback: without the library the
calls raise.
"""
from . import scenes  # noqa: F401
from ._capi import LcxError, load  # noqa: F401

__version__ = "0.1.0"


def library():
    """The loaded liblcx_accel.so (ctypes.CDLL)."""
    return load()
