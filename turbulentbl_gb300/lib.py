"""Loader for libtblgpu.so and the GPU runner.

The library is built in-tree (turbulentbl_gb300/_build) by build.py.  There is
no CPU fallback: if the library or a CUDA device is missing, this raises.
"""
import ctypes as C
import os

from . import abi
from .runner import AbiRunner

_lib = None


def lib_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libtblgpu.so")


def load(build_if_missing=False):
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libtblgpu.so not built ({path}); run turbulentbl_gb300/build.py")
        from .build import build
        build()
    _lib = C.CDLL(path)
    _lib.tbl_status_string.argtypes = [C.c_int]
    _lib.tbl_status_string.restype = C.c_char_p
    _lib.tbl_launch_count.argtypes = [C.c_void_p]
    _lib.tbl_launch_count.restype = C.c_int64
    return _lib


class TblGpu(AbiRunner):
    """The time-step library on the current CUDA device."""

    def __init__(self, mesh, rp):
        super().__init__(load(), "tbl_", mesh, rp)

    def launches(self):
        return int(self.lib.tbl_launch_count(self._h))
