"""ctypes mirror of include/tbl_gpu.h (the C ABI of the time-step library).

The same structs describe the GPU library (libtblgpu.so, symbols ``tbl_*``)
and are reused by the test harness for the CPU restatement in oracle/.
"""
import ctypes as C

import numpy as np

TBL_OK = 0
TBL_ERR_CUDA = -1
TBL_ERR_BAD_ARG = -2
TBL_ERR_NOT_CONVERGED = -3
TBL_ERR_NAN = -4
TBL_ERR_BLOWUP = -5
TBL_ERR_TIMEOUT = -6
TBL_ERR_NO_DEVICE = -7
TBL_ERR_REPLAY = -8
TBL_ERR_ZERO_RHS = -9
TBL_ERR_TOO_LARGE = -10
TBL_ERR_IO = -11

STATUS_NAMES = {
    TBL_OK: "OK",
    TBL_ERR_CUDA: "CUDA_ERROR",
    TBL_ERR_BAD_ARG: "BAD_ARG",
    TBL_ERR_NOT_CONVERGED: "NOT_CONVERGED",
    TBL_ERR_NAN: "NAN",
    TBL_ERR_BLOWUP: "BLOWUP",
    TBL_ERR_TIMEOUT: "TIMEOUT",
    TBL_ERR_NO_DEVICE: "NO_DEVICE",
    TBL_ERR_REPLAY: "REPLAY",
    TBL_ERR_ZERO_RHS: "ZERO_RHS",
    TBL_ERR_TOO_LARGE: "TOO_LARGE",
    TBL_ERR_IO: "IO",
}

TBL_TP_DNSTBL2 = 0
TBL_TP_ORIGINAL = 1
TBL_TP_DNSSETBL = 2

TBL_PREC_FP64 = 0
TBL_PREC_MIXED = 1

TBL_FLAG_REPLAY = 1
TBL_FLAG_PPE_RESIDUAL = 2
TBL_FLAG_DIAGNOSTICS = 4
TBL_FLAG_RB_ORDER = 8
TBL_FLAG_RB_PRECOND = 16
TBL_FLAG_SSOR_SPAN_BLOCKS = 32
TBL_FLAG_SSOR_STREAM_BLOCKS = 64

TBL_VARIANT_DNSTBL2 = 0
TBL_VARIANT_ORIGINAL = 1
TBL_VARIANT_DNSSETBL = 2

TBL_BRANCH_FREE = 0
TBL_BRANCH_RECORD = 1
TBL_BRANCH_REPLAY = 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class TblConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nproc", C.c_int32), ("irec", C.c_int32), ("cum", C.c_int32),
        ("istat", C.c_int32), ("recycle_after", C.c_int32), ("kmax", C.c_int32),
        ("mmax", C.c_int32), ("precision", C.c_int32), ("flags", C.c_int32),
        ("mixed_kmax", C.c_int32), ("mixed_max_outer", C.c_int32),
        ("dt", C.c_double), ("re", C.c_double), ("ue", C.c_double),
        ("dx", C.c_double), ("dy", C.c_double), ("dxi", C.c_double),
        ("omega", C.c_double), ("errtol", C.c_double), ("errorstop", C.c_double),
        ("mixed_inner_tol", C.c_double), ("mixed_outer_tol", C.c_double), ("mixed_true_tol", C.c_double),
        ("variant", C.c_int32), ("reserved_", C.c_int32),
    ]


class TblMesh(C.Structure):
    _fields_ = [("x1", _dp), ("x2", _dp), ("x3", _dp), ("jac", _dp), ("jac2", _dp)]


class TblState(C.Structure):
    _fields_ = [
        ("u", _dp), ("v", _dp), ("w", _dp), ("p", _dp), ("pcorr", _dp),
        ("usum2", _dp), ("vsum2", _dp), ("wsum2", _dp), ("wt", _dp),
        ("uf", _dp), ("vf", _dp), ("wf", _dp), ("newk", _ip), ("ume1", _dp),
        ("bltkns", _dp),
        ("lamda", C.c_double), ("time", C.c_double),
        ("nstep", C.c_int32), ("cont", C.c_int32), ("ksep", C.c_int32), ("cnt2", C.c_int32),
    ]


class TblStepStats(C.Structure):
    _fields_ = [
        ("nstep", C.c_int32), ("status", C.c_int32), ("gs_sweeps", C.c_int32 * 3),
        ("gmres_restarts", C.c_int32), ("gmres_iters", C.c_int32), ("cum_step", C.c_int32),
        ("outer_iters", C.c_int32), ("pad_", C.c_int32),
        ("gs_resid", C.c_double * 3), ("gmres_resid", C.c_double),
        ("ppe_rel_resid", C.c_double), ("div_diag", C.c_double), ("ke", C.c_double),
        ("lamda", C.c_double), ("time", C.c_double),
    ]

    def as_dict(self):
        return {
            "nstep": self.nstep, "status": self.status,
            "gs_sweeps": list(self.gs_sweeps), "gmres_restarts": self.gmres_restarts,
            "gmres_iters": self.gmres_iters, "cum_step": self.cum_step,
            "outer_iters": self.outer_iters,
            "gs_resid": list(self.gs_resid), "gmres_resid": self.gmres_resid,
            "ppe_rel_resid": self.ppe_rel_resid, "div_diag": self.div_diag,
            "ke": self.ke, "lamda": self.lamda, "time": self.time,
        }


class TblStatsOut(C.Structure):
    _fields_ = [
        ("usum", _dp), ("vsum", _dp), ("wsum", _dp), ("uusum", _dp), ("vvsum", _dp),
        ("wwsum", _dp), ("uvsum", _dp), ("uwsum", _dp), ("vwsum", _dp),
        ("deltastar", _dp), ("theta", _dp), ("ht", _dp), ("reth", _dp),
        ("tauw_sum", _dp), ("ubulk", _dp),
        ("lamda03", C.c_double), ("nstat", C.c_int32), ("pad_", C.c_int32),
        ("tauw_window", _dp),
    ]


class TblWindowConfig(C.Structure):
    _fields_ = [("x_lo", C.c_double), ("x_hi", C.c_double), ("ckpt_every", C.c_int32), ("branch_mode", C.c_int32)]


class TblFields(C.Structure):
    _fields_ = [("u", _dp), ("v", _dp), ("w", _dp), ("p", _dp)]


class TblAdjointStats(C.Structure):
    _fields_ = [
        ("steps", C.c_int32), ("recomputed_steps", C.c_int32), ("adj_gs_sweeps", C.c_int32),
        ("adj_gmres_iters", C.c_int32), ("status", C.c_int32), ("pad_", C.c_int32),
        ("max_gs_resid", C.c_double), ("max_gmres_resid", C.c_double),
        ("forward_ms", C.c_double), ("backward_ms", C.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad_"}


STATS_FIELDS = ["usum", "vsum", "wsum", "uusum", "vvsum", "wwsum", "uvsum", "uwsum", "vwsum"]
STATE_FIELDS_3D = ["u", "v", "w", "p", "pcorr", "uf", "vf", "wf"]
STATE_FIELDS_2D = ["usum2", "vsum2", "wsum2", "wt"]


def dptr(a):
    """Pointer to a contiguous float64 numpy array (Fortran-ordered 3-D arrays pass as-is)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.flags.c_contiguous)
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32
    return a.ctypes.data_as(_ip)


def declare(lib, prefix, handle_t=C.c_void_p):
    """Declare argtypes/restypes of the ABI functions with the given prefix."""
    H = handle_t
    f = getattr(lib, prefix + "create")
    f.argtypes = [C.POINTER(TblConfig), C.POINTER(TblMesh), C.POINTER(H)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "upload_state")
    f.argtypes = [H, C.POINTER(TblState)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "step")
    f.argtypes = [H, C.c_int32, C.POINTER(TblStepStats)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "download_state")
    f.argtypes = [H, C.POINTER(TblState)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "download_stats")
    f.argtypes = [H, C.POINTER(TblStatsOut)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "download_averages")
    f.argtypes = [H, C.POINTER(C.c_double)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "set_replay")
    f.argtypes = [H, _ip, C.c_int64]
    f.restype = C.c_int
    f = getattr(lib, prefix + "last_counts")
    f.argtypes = [H, _ip, C.c_int32]
    f.restype = C.c_int
    f = getattr(lib, prefix + "destroy")
    f.argtypes = [H]
    f.restype = None
