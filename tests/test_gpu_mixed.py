"""Mixed precision (FP32 fields, stencils and inner GMRES inside FP64
iterative refinement) against the FP64 oracle.

Tolerances stated here: per step the velocity fields agree with the FP64
oracle to 1e-5 relative L2 (FP32 storage), the pressure to 1e-4, and the
relative pressure-Poisson residual ||L7 p' - Q8|| / ||Q8|| of the mixed solve
is <= 1e-8.
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def pair(nx=24, nzs=12, nyw=20, P=2, kmax=20):
    from turbulentbl_gb300.lib import TblGpu
    wl = small_workload(nx=nx, nz_span=nzs, ny_wall=nyw, kmax=kmax, errtol=1e-10)
    mesh, rp, st = make_state(wl, nproc=P)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    rp.precision = abi.TBL_PREC_MIXED
    rp.mixed_kmax = kmax
    rp.mixed_outer_tol = 1e-10
    rp.mixed_inner_tol = 1e-5
    rp.flags = abi.TBL_FLAG_PPE_RESIDUAL
    g = TblGpu(mesh, rp)
    g.upload(st)
    return o, g


@pytest.mark.parametrize("shape", [(24, 12, 20, 2), (30, 10, 26, 3)])
def test_mixed_step_tracks_fp64(shape):
    o, g = pair(*shape)
    for s in range(6):
        o.step(1)
        st, rec = g.step(1)
        assert st == abi.TBL_OK
        a, b = o.download(), g.download()
        for f in ("u", "v", "w"):
            assert rel(b[f], a[f]) < 1e-5, (s, f, rel(b[f], a[f]))
        assert rel(b["p"], a["p"]) < 1e-4, (s, rel(b["p"], a["p"]))
        assert rec[0]["ppe_rel_resid"] <= 1e-8, rec[0]
        assert rec[0]["outer_iters"] >= 1


def test_mixed_statistics_close():
    o, g = pair()
    for _ in range(7):
        o.step(1)
        g.step(1)
    a, b = o.download_stats(), g.download_stats()
    for f in ("usum", "uusum", "uvsum"):
        assert rel(b[f], a[f]) < 1e-5, f
    sa, sb = o.download(), g.download()
    assert rel(sb["usum2"], sa["usum2"]) < 1e-5
