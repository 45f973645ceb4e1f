"""Checkpoint/resume of the GPU time step through the reference's files.

A GPU run of 3 steps is downloaded and written the way the reference writes
its restart: per-rank 3D%03d.tp files (dnstbl2/dnstbl.f90:2357-2377), merged
into 3D.tp (dnstbl/restart.f90:17-86), the counters cnt and cnt2, and the
inflow profile file U_innerdns.dat.  A fresh GPU handle then reads them back
(:147-159, :322-358) and runs 3 more steps.  A restart starts a new program
run (PCorr, lamda, cont and the statistics sums start afresh), so the
reference for the resumed run is (a) the oracle resumed from the same files,
to 1e-12, and (b) the GPU resumed from the in-memory arrays with the same
fresh-run values, to the files' 15 significant digits (1e-9).
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi, tpfile
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("P", [2, 3])
def test_gpu_restart_through_files_continues_the_run(tmp_path, P):
    from turbulentbl_gb300.lib import TblGpu
    wl = small_workload(nx=24, nz_span=12, ny_wall=40, kmax=20)
    mesh, rp, st = make_state(wl, nproc=P)
    rp.cum = 4
    g = TblGpu(mesh, rp)
    g.upload(st)
    g.step(3)
    d = g.download()
    g.close()
    d["ume1"], d["bltkns"] = st["ume1"], st["bltkns"]
    tpfile.write_rank_files(tmp_path, mesh, d, d["time"], d["nstep"], nproc=P)
    tpfile.merge_rank_files(tmp_path, mesh.nz, P)
    tpfile.write_counters(tmp_path, mesh.nz, 1, P, d["cnt2"])
    tpfile.write_inflow_profile(tmp_path / "U_innerdns.dat", mesh.x3, st["ume1"])
    back, t, n = tpfile.read_tp(tmp_path / "3D.tp", mesh.nx, mesh.ny, mesh.nz)
    nz_, cnt, nproc, cnt2 = tpfile.read_counters(tmp_path)
    ume1 = tpfile.read_inflow_profile(tmp_path / "U_innerdns.dat", mesh.nz)
    assert (n, nz_, nproc, cnt2) == (d["nstep"], mesh.nz, P, 3)
    fresh = dict(lamda=1.0, cont=0, pcorr=None, ume1=ume1, bltkns=st["bltkns"], ksep=d["ksep"])
    from_files = dict(back, time=t, nstep=n, cnt2=cnt2, **fresh)
    runs = {}
    for name, src, cls in (("gpu_files", from_files, TblGpu), ("oracle_files", from_files, OracleRunner),
                           ("gpu_memory", dict(d, **fresh), TblGpu)):
        r = cls(mesh, rp)
        r.upload(src)
        status, _ = r.step(3, check=False)
        assert status == abi.TBL_OK, (name, status)
        runs[name] = (r.download(), r.last_counts())
        if cls is TblGpu:
            r.close()
    (gf, cg), (of, co), (gm, _) = runs["gpu_files"], runs["oracle_files"], runs["gpu_memory"]
    assert cg == co
    for f in ("u", "v", "w", "p"):
        assert rel(gf[f], of[f]) <= 1e-12, (f, rel(gf[f], of[f]))
        assert rel(gf[f], gm[f]) <= 1e-9, (f, rel(gf[f], gm[f]))
    assert gf["nstep"] == of["nstep"] == d["nstep"] + 3
    assert gf["cnt2"] == cnt2 + 3
