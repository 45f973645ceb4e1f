"""The reference's monitor files from a run, through the library's C ABI.

``Monitor`` steps a runner (``TblGpu``, or any ``AbiRunner``) one step at a
time and writes the files that dnstbl2's rank 0 writes, on its schedule
(dnstbl2/dnstbl.f90):

====================================  =======================================
when                                  files
====================================  =======================================
every disp1-th step (disp1 = 1)       massflow.xy (:1526, :1613-1615)
at the end of a wall-shear window     numrcltauwall.xy (:1670-1681; 500 steps,
                                      originalTBL 1000)
every step after the fifth            kineticenergy.dat (:1707, :1718-1721;
                                      after recycle_after steps)
every rescaling (cont % cum == 0)     means, medians, taustress,
                                      Umeanvalues.dat, lamda.dat, W.dat,
                                      boundarylthickness.dat (:1974-2267)
a rescaling at a multiple of 100      k.dat, meanvalues.dat (:2286-2302)
====================================  =======================================

Files the reference appends to are appended to; the others are rewritten.
The records are written by the C++ writers of libtblgpu.so
(``tbl_monitor_*`` in csrc/tbl_restart.cpp) in the reference's edit
descriptors.  A rescaling's values are read back after its step: the device
keeps the averaged sums of the last rescaling (``tbl_download_averages``),
since the running sums are reset in the same step.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_declared = False


def _lib():
    global _declared
    from .lib import load
    lib = load()
    if not _declared:
        I, D, S = C.c_int32, C.c_double, C.c_char_p
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        sigs = {
            "tbl_monitor_massflow": [S, D, dp],
            "tbl_monitor_tauwall": [S, D, I, I, D, dp, dp],
            "tbl_monitor_kinetic_energy": [S, D, D],
            "tbl_monitor_lamda": [S, D, D, D],
            "tbl_monitor_blend": [S, I, I, dp, dp, dp],
            "tbl_monitor_bl_thickness": [S, D, I, dp, dp, dp, dp, dp, dp],
            "tbl_monitor_knew": [S, I, ip, dp],
            "tbl_monitor_meanvalues": [S, I, I, dp, dp, dp, dp, dp],
            "tbl_monitor_umeanvalues": [S, I, I, dp, dp, dp, dp, dp, D],
            "tbl_monitor_averages": [S, I, I, dp, dp, dp],
        }
        for name, args in sigs.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int
        _declared = True
    return lib


def _d(a):
    return abi.dptr(np.asfortranarray(a, dtype=np.float64))


def _call(name, *args):
    from .runner import TblError
    st = getattr(_lib(), name)(*args)
    if st != abi.TBL_OK:
        raise TblError(st, name)


class Monitor:
    """Steps ``runner`` and writes the monitor files into ``dirname``."""

    FILES = ("massflow.xy", "numrcltauwall.xy", "kineticenergy.dat", "means", "medians", "taustress",
             "Umeanvalues.dat", "lamda.dat", "W.dat", "boundarylthickness.dat", "k.dat", "meanvalues.dat")

    def __init__(self, runner, dirname, disp1=1):
        self.r = runner
        self.dir = os.fspath(dirname)
        self.disp1 = int(disp1)
        m, rp = runner.mesh, runner.rp
        self.nx, self.ny, self.nz = m.nx, m.ny, m.nz
        self.x1 = np.ascontiguousarray(m.x1, dtype=np.float64)
        self.x3 = np.ascontiguousarray(m.x3, dtype=np.float64)
        self.window = 1000 if rp.variant == 1 else 500
        # eta(k) of the rescaling's inner/outer split; eta(nz) is never
        # assigned by the reference and stays at its initial zero
        self.eta = np.zeros(self.nz)

    def path(self, name):
        return os.path.join(self.dir, name).encode()

    def step(self, nsteps=1, check=True):
        """Runs nsteps steps one at a time, writing each step's records."""
        recs = []
        st = abi.TBL_OK
        for _ in range(int(nsteps)):
            st, rec = self.r.step(1, check=check)
            recs.extend(rec)
            if st != abi.TBL_OK:
                break
            self.record(rec[0])
        return st, recs

    def _stats_subset(self, ubulk=None, tauw_window=None, bl=None):
        o = abi.TblStatsOut()
        if ubulk is not None:
            o.ubulk = abi.dptr(ubulk)
        if tauw_window is not None:
            o.tauw_window = abi.dptr(tauw_window)
        if bl is not None:
            o.deltastar, o.theta, o.ht, o.reth = (abi.dptr(a) for a in bl)
        st = self.r._fn("download_stats")(self.r._h, C.byref(o))
        if st != abi.TBL_OK:
            from .runner import TblError
            raise TblError(st, self.r.prefix + "download_stats")
        return o

    def record(self, rec):
        """Writes the records of one completed step (its tbl_step_stats)."""
        n, t = int(rec["nstep"]), float(rec["time"])
        nx, ny, nz = self.nx, self.ny, self.nz
        if n % self.disp1 == 0:
            ub = np.zeros(5)
            self._stats_subset(ubulk=ub)
            _call("tbl_monitor_massflow", self.path("massflow.xy"), t, abi.dptr(ub))
        if n % self.window == 0:
            tw = np.zeros(nx)
            self._stats_subset(tauw_window=tw)
            _call("tbl_monitor_tauwall", self.path("numrcltauwall.xy"), t, nx, ny, float(self.r.rp.ue),
                  abi.dptr(self.x1), abi.dptr(tw))
        if n > self.r.rp.recycle_after:  # the reference's nstep > 5 (recycling starts after step 5)
            _call("tbl_monitor_kinetic_energy", self.path("kineticenergy.dat"), t, float(rec["ke"]))
        if rec["cum_step"]:
            self._rescaling(n, t, float(rec["lamda"]))

    def _rescaling(self, n, t, lamda):
        nx, nz = self.nx, self.nz
        avg = self.r.download_averages()
        for name, keys in (("means", ("u", "v", "w")), ("medians", ("uu", "vv", "ww")),
                           ("taustress", ("uv", "uw", "vw"))):
            _call("tbl_monitor_averages", self.path(name), nx, nz, *(_d(avg[q]) for q in keys))
        s = self.r.download(fields=("usum2", "vsum2", "wsum2", "wt"))
        bl = [np.zeros(nx) for _ in range(4)]
        o = self._stats_subset(bl=bl)
        lamda03 = float(o.lamda03)
        x1, x3 = abi.dptr(self.x1), abi.dptr(self.x3)
        means = [_d(s[q]) for q in ("usum2", "vsum2", "wsum2")]
        _call("tbl_monitor_umeanvalues", self.path("Umeanvalues.dat"), nx, nz, x1, x3, *means,
              float(self.r.rp.re))
        _call("tbl_monitor_lamda", self.path("lamda.dat"), t, lamda, lamda03)
        _call("tbl_monitor_blend", self.path("W.dat"), nx, nz, x1, x3, _d(s["wt"]))
        _call("tbl_monitor_bl_thickness", self.path("boundarylthickness.dat"), t, nx, x1,
              _d(s["bltkns"]), *(abi.dptr(a) for a in bl))
        wt_rec = np.asarray(s["wt"])[self.r.rp.irec - 1, :]
        for k in range(nz - 1):  # :2195-2204
            self.eta[k] = lamda if wt_rec[k] <= 0.99 else lamda03
        if n % 100 == 0:
            newk = np.ascontiguousarray(s["newk"], dtype=np.int32)
            _call("tbl_monitor_knew", self.path("k.dat"), nz, abi.iptr(newk), abi.dptr(self.eta))
            _call("tbl_monitor_meanvalues", self.path("meanvalues.dat"), nx, nz, x1, x3, *means)
