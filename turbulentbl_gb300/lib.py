"""Loader for libtblgpu.so and the GPU runner.

The library is built in-tree (turbulentbl_gb300/_build) by build.py.  There is
no CPU fallback: if the library or a CUDA device is missing, this raises.
"""
import ctypes as C
import os

from . import abi
import numpy as np

from .runner import AbiRunner, TblError

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


def _declare_adjoint(lib):
    _dp = C.POINTER(C.c_double)
    lib.tbl_set_wall_control.argtypes = [C.c_void_p, _dp]
    lib.tbl_set_wall_control.restype = C.c_int
    lib.tbl_forward_window.argtypes = [C.c_void_p, C.c_int32, C.POINTER(abi.TblWindowConfig), _dp,
                                       C.POINTER(abi.TblStepStats)]
    lib.tbl_forward_window.restype = C.c_int
    lib.tbl_backward_window.argtypes = [C.c_void_p, C.c_double, C.POINTER(abi.TblFields), _dp,
                                        C.POINTER(abi.TblFields), C.POINTER(abi.TblAdjointStats)]
    lib.tbl_backward_window.restype = C.c_int


class TblGpu(AbiRunner):
    """The time-step library on the current CUDA device."""

    def __init__(self, mesh, rp):
        super().__init__(load(), "tbl_", mesh, rp)
        _declare_adjoint(self.lib)

    def launches(self):
        return int(self.lib.tbl_launch_count(self._h))

    # ------------------------------------------------ wall control / adjoint
    def set_wall_control(self, c):
        """c: (nx, ny-2) wall-normal wall velocity (None = the reference's w = 0)."""
        if c is None:
            st = self.lib.tbl_set_wall_control(self._h, None)
        else:
            c = np.asfortranarray(c, dtype=np.float64)
            assert c.shape == (self.mesh.nx, self.mesh.ny - 2)
            st = self.lib.tbl_set_wall_control(self._h, abi.dptr(c))
        if st != abi.TBL_OK:
            raise TblError(st, "tbl_set_wall_control")

    def forward_window(self, nsteps, x_lo, x_hi, ckpt_every, branch_mode=abi.TBL_BRANCH_FREE):
        """Run nsteps recorded steps; returns (objective, per-step stats dicts)."""
        wc = abi.TblWindowConfig(x_lo, x_hi, int(ckpt_every), int(branch_mode))
        J = C.c_double(0.0)
        stats = (abi.TblStepStats * nsteps)()
        st = self.lib.tbl_forward_window(self._h, int(nsteps), C.byref(wc), C.byref(J), stats)
        if st != abi.TBL_OK:
            raise TblError(st, "tbl_forward_window")
        return J.value, [s.as_dict() for s in stats]

    def backward_window(self, dL_dJ=1.0, dL_dfinal=None, want_initial=False):
        """Adjoint of the last window.  dL_dfinal: dict of (nx,ny,nz) arrays for
        some of u, v, w, p.  Returns (dL/dc (nx, ny-2), dL/dinitial dict or None,
        adjoint stats dict)."""
        nx, ny, nz = self.n3d
        keep = []
        fin = None
        if dL_dfinal:
            fin = abi.TblFields()
            for f in ("u", "v", "w", "p"):
                a = dL_dfinal.get(f)
                if a is not None:
                    a = np.asfortranarray(a, dtype=np.float64)
                    assert a.shape == (nx, ny, nz)
                    keep.append(a)
                    setattr(fin, f, abi.dptr(a))
        init, out = None, None
        if want_initial:
            out = {f: np.zeros((nx, ny, nz), order="F") for f in ("u", "v", "w", "p")}
            init = abi.TblFields(*(abi.dptr(out[f]) for f in ("u", "v", "w", "p")))
        gc = np.zeros((nx, ny - 2), order="F")
        ast = abi.TblAdjointStats()
        st = self.lib.tbl_backward_window(self._h, float(dL_dJ), C.byref(fin) if fin is not None else None,
                                          abi.dptr(gc), C.byref(init) if init is not None else None, C.byref(ast))
        if st != abi.TBL_OK:
            raise TblError(st, "tbl_backward_window")
        return gc, out, ast.as_dict()
