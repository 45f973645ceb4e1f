"""The reference's restart and counter files, through the library's C ABI.

The readers and writers are the C++ ones in libtblgpu.so
(csrc/tbl_restart.cpp: tbl_tp_write, tbl_tp_write_ranks, tbl_tp_merge,
tbl_tp_read, tbl_counters_*, tbl_statdata_*, tbl_inflow_profile_*); they
touch no device.  Formats
(``fmt``): 0 dnstbl2's 15 columns (x y z U V W P Um Vm Wm Uf Vf Wf Wt Nk),
1 originalTBL's 8 (x y z U V W T P), 2 dnssetbl's 7 (x y z U V W P).

Values carry 15 significant digits (E22.15), as the reference writes them,
so a restart through these files is not bit-exact in FP64.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .runner import TblError

_declared = False


def _lib():
    global _declared
    from .lib import load
    lib = load()
    if not _declared:
        I, P, S = C.c_int32, C.c_void_p, C.c_char_p
        Mp, Sp = C.POINTER(abi.TblMesh), C.POINTER(abi.TblState)
        ip = C.POINTER(C.c_int32)
        dp = C.POINTER(C.c_double)
        sigs = {
            "tbl_tp_write": [S, I, Mp, Sp, I, I, I, I, I, I, I, I, I],
            "tbl_tp_write_ranks": [S, I, Mp, Sp, I, I, I, I],
            "tbl_tp_merge": [S, I, I, I, S],
            "tbl_tp_read": [S, I, I, I, I, dp, dp, dp, Sp],
            "tbl_counters_write": [S, I, I, I, I],
            "tbl_counters_read": [S, ip, ip, ip, ip],
            "tbl_statdata_write": [S, I, I, I, Sp],
            "tbl_statdata_read": [S, I, I, I, Sp],
            "tbl_inflow_profile_read": [S, I, dp],
            "tbl_inflow_profile_write": [S, I, dp, dp],
        }
        for name, args in sigs.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int
        _declared = True
    return lib


def _check(st, what):
    if st != abi.TBL_OK:
        raise TblError(st, what)


def _mesh_struct(mesh):
    m = abi.TblMesh()
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (mesh.x1, mesh.x2, mesh.x3)]
    m.x1, m.x2, m.x3 = (abi.dptr(a) for a in keep)
    return m, keep


def _state_struct(st, time, nstep):
    s = abi.TblState()
    keep = []
    for name in ("u", "v", "w", "p", "uf", "vf", "wf"):
        if st.get(name) is not None:
            a = np.asfortranarray(st[name], dtype=np.float64)
            keep.append(a)
            setattr(s, name, abi.dptr(a))
    for name in ("usum2", "vsum2", "wsum2", "wt"):
        if st.get(name) is not None:
            a = np.asfortranarray(st[name], dtype=np.float64)
            keep.append(a)
            setattr(s, name, abi.dptr(a))
    if st.get("newk") is not None:
        nk = np.ascontiguousarray(st["newk"], dtype=np.int32)
        keep.append(nk)
        s.newk = abi.iptr(nk)
    s.time, s.nstep = float(time), int(nstep)
    return s, keep


def _b(path):
    return os.fsencode(str(path))


def write_tp(path, mesh, st, time, nstep, j_range=None, k_range=None, header=1, fmt=0, nproc=0):
    """One file of points i = all, j in j_range, k in k_range (0-based
    inclusive; default every j and k).  header: 0 none, 1 the program's own
    writer, 2 the merger's."""
    j0, j1 = j_range if j_range is not None else (0, mesh.ny - 1)
    k0, k1 = k_range if k_range is not None else (0, mesh.nz - 1)
    m, km = _mesh_struct(mesh)
    s, ks = _state_struct(st, time, nstep)
    _check(_lib().tbl_tp_write(_b(path), fmt, C.byref(m), C.byref(s), mesh.nx, mesh.ny, mesh.nz, j0 + 1, j1 + 1,
                               k0 + 1, k1 + 1, header, nproc), "tbl_tp_write")


def write_rank_files(dirname, mesh, st, time, nstep, nproc, fmt=0):
    """The per-rank files 3D%03d.tp (3D%03d.dat for dnssetbl): j = 2..ny-1 and
    each rank's k range."""
    m, km = _mesh_struct(mesh)
    s, ks = _state_struct(st, time, nstep)
    _check(_lib().tbl_tp_write_ranks(_b(dirname), fmt, C.byref(m), C.byref(s), mesh.nx, mesh.ny, mesh.nz, nproc),
           "tbl_tp_write_ranks")


def merge_rank_files(dirname, nz, nproc, out_name="3D.tp", fmt=0):
    """Merge the per-rank files into one with every j (the restart mergers)."""
    _check(_lib().tbl_tp_merge(_b(dirname), fmt, nz, nproc, _b(os.path.join(str(dirname), out_name))),
           "tbl_tp_merge")


def read_tp(path, nx, ny, nz, fmt=0):
    """Read a merged file.  Returns (state dict, time, nstep); the state has
    x1, x2, x3, u, v, w, p and, for the 15-column format, the recycling and
    statistics columns."""
    out = {"x1": np.zeros(nx), "x2": np.zeros(ny), "x3": np.zeros(nz)}
    names = ["u", "v", "w", "p"] + (["uf", "vf", "wf"] if fmt == 0 else [])
    for n in names:
        out[n] = np.zeros((nx, ny, nz), order="F")
    if fmt == 0:
        for n in ("usum2", "vsum2", "wsum2", "wt"):
            out[n] = np.zeros((nx, nz), order="F")
        out["newk"] = np.zeros(nz, dtype=np.int32)
    s, _ = _state_struct(out, 0.0, 0)
    _check(_lib().tbl_tp_read(_b(path), fmt, nx, ny, nz, abi.dptr(out["x1"]), abi.dptr(out["x2"]),
                              abi.dptr(out["x3"]), C.byref(s)), "tbl_tp_read")
    return out, s.time, s.nstep


def write_counters(dirname, nz, cnt, nproc, cnt2):
    _check(_lib().tbl_counters_write(_b(dirname), nz, cnt, nproc, cnt2), "tbl_counters_write")


def read_counters(dirname):
    v = [C.c_int32() for _ in range(4)]
    _check(_lib().tbl_counters_read(_b(dirname), *[C.byref(x) for x in v]), "tbl_counters_read")
    return tuple(int(x.value) for x in v)


def write_statdata(path, st, irec):
    """dnssetbl's statData.dat: the recycling means at irec, Wt(1,k), new(k)."""
    nx, nz = st["usum2"].shape
    s, ks = _state_struct(st, 0.0, 0)
    _check(_lib().tbl_statdata_write(_b(path), nx, nz, irec, C.byref(s)), "tbl_statdata_write")


def read_statdata(path, st, irec):
    """Fill st's usum2/vsum2/wsum2 at irec, wt(1,:) and newk from statData.dat
    (st's arrays are updated in place; they must be float64 Fortran arrays)."""
    nx, nz = st["usum2"].shape
    for n in ("usum2", "vsum2", "wsum2", "wt"):
        assert st[n].dtype == np.float64 and st[n].flags.f_contiguous
    assert st["newk"].dtype == np.int32
    s = abi.TblState()
    s.usum2, s.vsum2, s.wsum2, s.wt = (abi.dptr(st[n]) for n in ("usum2", "vsum2", "wsum2", "wt"))
    s.newk = abi.iptr(st["newk"])
    _check(_lib().tbl_statdata_read(_b(path), nx, nz, irec, C.byref(s)), "tbl_statdata_read")


def read_inflow_profile(path, nz):
    """The inflow mean profile Ume1 (nz values) from U_innerdns.dat: 37
    records FORMAT(24X,E18.8), record 37 repeated above plane 37."""
    u = np.zeros(nz)
    _check(_lib().tbl_inflow_profile_read(_b(path), nz, abi.dptr(u)), "tbl_inflow_profile_read")
    return u


def write_inflow_profile(path, x3, ume1):
    """U_innerdns.dat for a profile (nz >= 37): k and x3(k) in the skipped
    columns, Ume1(k) in E18.8, the 37 records the reference reads."""
    x3 = np.ascontiguousarray(x3, dtype=np.float64)
    u = np.ascontiguousarray(ume1, dtype=np.float64)
    _check(_lib().tbl_inflow_profile_write(_b(path), len(u), abi.dptr(x3), abi.dptr(u)),
           "tbl_inflow_profile_write")
