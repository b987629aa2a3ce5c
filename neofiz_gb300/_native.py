"""Loader for libneofiz_gpu.so, the CUDA implementation behind include/neofiz.h.

The library is built in-tree by ``neofiz_gb300.build.build()`` into ``neofiz_gb300/_build``.
There is no fallback: if the library is missing, or no CUDA device is visible, ``api()``
raises ``NativeUnavailable`` with the reason.
"""
from __future__ import annotations

import ctypes
import os

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY = os.path.join(_HERE, "_build", "libneofiz_gpu.so")


class NativeUnavailable(RuntimeError):
    pass


_api = None


def load_library() -> ctypes.CDLL:
    """Loads the shared object without touching the GPU (used to check its exports)."""
    if not os.path.exists(LIBRARY):
        raise NativeUnavailable(
            f"{LIBRARY} is missing; build it with neofiz_gb300.build.build()")
    return ctypes.CDLL(LIBRARY, mode=ctypes.RTLD_GLOBAL)


def api():
    global _api
    if _api is None:
        lib = load_library()
        _api = _abi.bind(lib, "nf_")
        lib.nf_device_count.restype = ctypes.c_int
        if lib.nf_device_count() < 1:
            raise NativeUnavailable("libneofiz_gpu.so loaded but no CUDA device is visible")
    return _api


def fp64_rate():
    """(FP64 DFMA warp instructions per second, FP64 FLOPs per second) of the current device,
    measured by nf_device_fp64_rate."""
    a = api()
    fn = a.lib.nf_device_fp64_rate
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    w, f = ctypes.c_double(), ctypes.c_double()
    st = fn(ctypes.byref(w), ctypes.byref(f))
    if st:
        raise RuntimeError(f"nf_device_fp64_rate failed: {a.last_error(None)}")
    return w.value, f.value
