"""Red-black throughput mode (TBL_FLAG_RB_ORDER) against the oracle.

The mode changes the order of the implicit-diffusion Gauss-Seidel sweeps
(and, with TBL_FLAG_RB_PRECOND, of the SSOR preconditioner): not the
reference's sweep order, so iteration counts differ, but the converged solves
are the same.  With tight solver tolerances the fields
after a few steps agree with the oracle (reference ordering) to 1e-8 in FP64
and to the mixed-precision tolerances in mixed mode.
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _pair(precision, flags=abi.TBL_FLAG_RB_ORDER, nx=24):
    """FP64: tight tolerances on both sides.  Mixed: the settings of the
    mixed-precision tests (an FP32 Gauss-Seidel cannot reach 1e-12)."""
    from turbulentbl_gb300.lib import TblGpu
    fp64 = precision == abi.TBL_PREC_FP64
    wl = small_workload(nx=nx, nz_span=12, ny_wall=20, kmax=20, errtol=1e-12 if fp64 else 1e-10)
    mesh, rp, st = make_state(wl, nproc=2)
    if fp64:
        rp.errorstop = 1e-12
    rp.mmax = 3000
    o = OracleRunner(mesh, rp)
    o.upload(st)
    rp.flags = flags | abi.TBL_FLAG_PPE_RESIDUAL
    if precision == abi.TBL_PREC_MIXED:
        rp.precision = abi.TBL_PREC_MIXED
        rp.mixed_kmax = 20
        rp.mixed_outer_tol = 1e-10
        rp.mixed_inner_tol = 1e-5
    g = TblGpu(mesh, rp)
    g.upload(st)
    return o, g


RB_GS = abi.TBL_FLAG_RB_ORDER
RB_ALL = abi.TBL_FLAG_RB_ORDER | abi.TBL_FLAG_RB_PRECOND


@pytest.mark.parametrize("flags,nx", [(RB_GS, 24), (RB_ALL, 24), (RB_GS, 25), (RB_ALL, 25)])
@pytest.mark.parametrize("precision,tol_uvw,tol_p", [(abi.TBL_PREC_FP64, 1e-8, 1e-7), (abi.TBL_PREC_MIXED, 1e-5, 1e-4)])
def test_red_black_steps_track_the_oracle(precision, tol_uvw, tol_p, flags, nx):
    """Red-black diffusion sweeps (and, with RB_PRECOND, the red-black SSOR
    preconditioner); odd and even interior row lengths."""
    o, g = _pair(precision, flags, nx)
    for s in range(3):
        o.step(1, check=False)
        _, rec = g.step(1)
        a, b = o.download(), g.download()
        for f, tol in (("u", tol_uvw), ("v", tol_uvw), ("w", tol_uvw), ("p", tol_p)):
            assert rel(b[f], a[f]) <= tol, (s, f, rel(b[f], a[f]))
        assert rec[0]["ppe_rel_resid"] <= 1e-8, rec[0]
        assert rec[0]["gmres_iters"] > 0 and min(rec[0]["gs_sweeps"]) > 0


def test_red_black_needs_an_even_number_of_span_rows():
    from turbulentbl_gb300.lib import TblGpu
    from turbulentbl_gb300.runner import TblError
    wl = small_workload(nx=24, nz_span=11, ny_wall=20)
    mesh, rp, st = make_state(wl, nproc=2)
    rp.flags = abi.TBL_FLAG_RB_ORDER
    with pytest.raises(TblError):
        TblGpu(mesh, rp)


def test_red_black_preconditioner_needs_red_black_sweeps():
    from turbulentbl_gb300.lib import TblGpu
    from turbulentbl_gb300.runner import TblError
    wl = small_workload(nx=24, nz_span=12, ny_wall=20)
    mesh, rp, st = make_state(wl, nproc=2)
    rp.flags = abi.TBL_FLAG_RB_PRECOND
    with pytest.raises(TblError):
        TblGpu(mesh, rp)
