"""Host-side driver over the C ABI (create / upload / step / download).

``AbiRunner`` drives any library exporting the tbl_gpu.h entry points under a
symbol prefix.  The product uses it with libtblgpu.so (prefix ``tbl_``);
the test harness reuses it for the CPU restatement in oracle/.
"""
import ctypes as C

import numpy as np

from . import abi
from .mesh import make_config, make_mesh_struct


class TblError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__(f"{what} failed: {abi.STATUS_NAMES.get(status, status)} ({status})")


class AbiRunner:
    def __init__(self, lib, prefix, mesh, rp):
        self.lib = lib
        self.prefix = prefix
        self.mesh = mesh
        self.rp = rp
        self.n3d = (mesh.nx, mesh.ny, mesh.nz)
        abi.declare(lib, prefix)
        self._cfg = make_config(mesh, rp)
        self._mesh_struct = make_mesh_struct(mesh)
        self._h = C.c_void_p()
        st = self._fn("create")(C.byref(self._cfg), C.byref(self._mesh_struct), C.byref(self._h))
        if st != abi.TBL_OK:
            raise TblError(st, prefix + "create")

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def close(self):
        if self._h:
            self._fn("destroy")(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ state
    def upload(self, state):
        nx, ny, nz = self.n3d
        keep = {}
        s = abi.TblState()
        for name in abi.STATE_FIELDS_3D:
            a = state.get(name)
            if a is not None:
                a = np.asfortranarray(a, dtype=np.float64)
                assert a.shape == (nx, ny, nz), (name, a.shape)
                keep[name] = a
                setattr(s, name, abi.dptr(a))
        for name in abi.STATE_FIELDS_2D:
            a = np.asfortranarray(state[name], dtype=np.float64)
            assert a.shape == (nx, nz)
            keep[name] = a
            setattr(s, name, abi.dptr(a))
        newk = np.ascontiguousarray(state["newk"], dtype=np.int32)
        ume1 = np.ascontiguousarray(state["ume1"], dtype=np.float64)
        keep["newk"], keep["ume1"] = newk, ume1
        s.newk = abi.iptr(newk)
        s.ume1 = abi.dptr(ume1)
        if state.get("bltkns") is not None:
            bl = np.ascontiguousarray(state["bltkns"], dtype=np.float64)
            keep["bltkns"] = bl
            s.bltkns = abi.dptr(bl)
        s.lamda = float(state.get("lamda", 1.0))
        s.time = float(state.get("time", 0.0))
        s.nstep = int(state.get("nstep", 0))
        s.cont = int(state.get("cont", 0))
        s.ksep = int(state.get("ksep", 0))
        s.cnt2 = int(state.get("cnt2", 0))
        st = self._fn("upload_state")(self._h, C.byref(s))
        if st != abi.TBL_OK:
            raise TblError(st, self.prefix + "upload_state")

    def download(self, fields=None):
        nx, ny, nz = self.n3d
        out = {}
        s = abi.TblState()
        want3 = abi.STATE_FIELDS_3D if fields is None else [f for f in abi.STATE_FIELDS_3D if f in fields]
        want2 = abi.STATE_FIELDS_2D if fields is None else [f for f in abi.STATE_FIELDS_2D if f in fields]
        for name in want3:
            a = np.zeros((nx, ny, nz), order="F")
            out[name] = a
            setattr(s, name, abi.dptr(a))
        for name in want2:
            a = np.zeros((nx, nz), order="F")
            out[name] = a
            setattr(s, name, abi.dptr(a))
        newk = np.zeros(nz, dtype=np.int32)
        ume1 = np.zeros(nz)
        bl = np.zeros(nx)
        s.newk, s.ume1, s.bltkns = abi.iptr(newk), abi.dptr(ume1), abi.dptr(bl)
        st = self._fn("download_state")(self._h, C.byref(s))
        if st != abi.TBL_OK:
            raise TblError(st, self.prefix + "download_state")
        out.update(newk=newk, ume1=ume1, bltkns=bl, lamda=s.lamda, time=s.time, nstep=s.nstep,
                   cont=s.cont, ksep=s.ksep, cnt2=s.cnt2)
        return out

    def download_stats(self):
        nx, ny, nz = self.n3d
        o = abi.TblStatsOut()
        out = {}
        for name in abi.STATS_FIELDS:
            a = np.zeros((nx, nz), order="F")
            out[name] = a
            setattr(o, name, abi.dptr(a))
        for name in ("deltastar", "theta", "ht", "reth", "tauw_sum", "tauw_window"):
            a = np.zeros(nx)
            out[name] = a
            setattr(o, name, abi.dptr(a))
        ub = np.zeros(5)
        out["ubulk"] = ub
        o.ubulk = abi.dptr(ub)
        st = self._fn("download_stats")(self._h, C.byref(o))
        if st != abi.TBL_OK:
            raise TblError(st, self.prefix + "download_stats")
        out["lamda03"] = o.lamda03
        out["nstat"] = o.nstat
        return out

    AVERAGES = ("u", "v", "w", "uu", "vv", "ww", "uv", "uw", "vw")

    def download_averages(self):
        """The running sums divided by cum at the last rescaling, before the
        reset: {"u", "v", "w", "uu", ..., "vw"} -> (nx, nz) arrays."""
        nx, ny, nz = self.n3d
        a = np.zeros(9 * nx * nz)
        st = self._fn("download_averages")(self._h, abi.dptr(a))
        if st != abi.TBL_OK:
            raise TblError(st, self.prefix + "download_averages")
        return {name: a[q * nx * nz:(q + 1) * nx * nz].reshape((nx, nz), order="F")
                for q, name in enumerate(self.AVERAGES)}

    # ------------------------------------------------------------------- step
    def step(self, nsteps=1, check=True):
        arr = (abi.TblStepStats * max(nsteps, 1))()
        st = self._fn("step")(self._h, int(nsteps), arr)
        recs = [arr[q].as_dict() for q in range(nsteps)]
        if check and st not in (abi.TBL_OK,):
            raise TblError(st, self.prefix + "step")
        return st, recs

    def last_counts(self):
        buf = (C.c_int32 * 4096)()
        n = self._fn("last_counts")(self._h, buf, 4096)
        if n < 0:
            raise TblError(n, self.prefix + "last_counts")
        return [buf[q] for q in range(n)]

    def set_replay(self, rec):
        a = np.ascontiguousarray(rec, dtype=np.int32)
        self._replay_keep = a
        st = self._fn("set_replay")(self._h, abi.iptr(a), int(a.size))
        if st != abi.TBL_OK:
            raise TblError(st, self.prefix + "set_replay")
