"""ctypes binding of the C++ oracle (test infrastructure only)."""
import ctypes as C

import numpy as np

from turbulentbl_gb300.runner import AbiRunner
from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build())
        _lib.orc_apply_lap.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.orc_apply_ssor.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.orc_solve_ppe.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_int32)]
        _lib.orc_flux_shear.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.orc_thicknesses.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 6
    return _lib


class OracleRunner(AbiRunner):
    def __init__(self, mesh, rp):
        super().__init__(lib(), "orc_", mesh, rp)

    def apply_lap(self, x):
        x = np.asfortranarray(x, dtype=np.float64)
        y = np.zeros_like(x, order="F")
        lib().orc_apply_lap(self._h, x.ctypes.data_as(C.POINTER(C.c_double)), y.ctypes.data_as(C.POINTER(C.c_double)))
        return y

    def solve_ppe(self, rhs):
        rhs = np.asfortranarray(rhs, dtype=np.float64)
        x = np.zeros_like(rhs, order="F")
        it = C.c_int32(0)
        st = lib().orc_solve_ppe(self._h, rhs.ctypes.data_as(C.POINTER(C.c_double)),
                                 x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(it))
        return st, x, it.value

    def apply_ssor(self, x):
        x = np.asfortranarray(x, dtype=np.float64)
        y = np.zeros_like(x, order="F")
        lib().orc_apply_ssor(self._h, x.ctypes.data_as(C.POINTER(C.c_double)), y.ctypes.data_as(C.POINTER(C.c_double)))
        return y

    def flux_shear(self):
        """Mass flux at the five planes and per-column span sums of the wall
        shear of the current state (not accumulated)."""
        ub = np.zeros(5)
        tau = np.zeros(self.mesh.nx)
        lib().orc_flux_shear(self._h, ub.ctypes.data_as(C.POINTER(C.c_double)),
                             tau.ctypes.data_as(C.POINTER(C.c_double)))
        return ub, tau

    def thicknesses(self, usum2):
        """bltkns, deltastar, theta, H, Re_theta (each nx) of the rescaling
        bookkeeping for the time-mean streamwise velocity usum2 (nx x nz);
        bltkns starts from the handle's current value."""
        u = np.asfortranarray(usum2, dtype=np.float64)
        outs = [np.zeros(self.mesh.nx) for _ in range(5)]
        dp = C.POINTER(C.c_double)
        st = lib().orc_thicknesses(self._h, u.ctypes.data_as(dp), *[x.ctypes.data_as(dp) for x in outs])
        assert st == 0
        return outs
