"""Failure detection on the GPU without a GPU fault.

Every failure is made on the host (bad input, an unreachable tolerance) or is
a bounded wait on a flag that nothing sets; the library reports it as a
status code and the device stays usable.  NaN input, a zero Poisson
right-hand side (the reference divides by zero there, dnstbl2/dnstbl.f90:1056),
Gauss-Seidel and GMRES stopping at mmax (:777, :956) and the u' > 25 blow-up
test (:1754-1772) must give the same status as the oracle.
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu


def _case(**rp_kw):
    wl = small_workload(nx=16, nz_span=8, ny_wall=14, kmax=10)
    mesh, rp, st = make_state(wl, nproc=2)
    for k, v in rp_kw.items():
        setattr(rp, k, v)
    return mesh, rp, dict(st)


def _both(mesh, rp, st):
    from turbulentbl_gb300.lib import TblGpu
    o = OracleRunner(mesh, rp)
    o.upload(st)
    g = TblGpu(mesh, rp)
    g.upload(st)
    so, _ = o.step(1, check=False)
    sg, rec = g.step(1, check=False)
    return so, sg, g, rec


def _still_usable(g, mesh, rp):
    _, _, clean = _case()
    g.upload(clean)
    sg, _ = g.step(1, check=False)
    return sg


def test_nan_input_reports_nan():
    mesh, rp, st = _case(mmax=20)
    st["u"] = np.asfortranarray(st["u"].copy())
    st["u"][5, 5, 5] = np.nan
    so, sg, g, _ = _both(mesh, rp, st)
    assert so == sg == abi.TBL_ERR_NAN
    assert _still_usable(g, mesh, rp) != abi.TBL_ERR_CUDA


def test_zero_poisson_rhs_reports_zero_rhs():
    mesh, rp, st = _case(mmax=6, recycle_after=10 ** 6)
    for f in ("u", "v", "w", "p", "pcorr", "uf", "vf", "wf"):
        st[f] = np.zeros_like(st[f], order="F")
    for f in ("usum2", "vsum2", "wsum2"):
        st[f] = np.zeros_like(st[f], order="F")
    so, sg, g, _ = _both(mesh, rp, st)
    assert so == sg == abi.TBL_ERR_ZERO_RHS
    # mmax = 6 stays in force, so Gauss-Seidel may stop at its cap on a real field
    assert _still_usable(g, mesh, rp) in (abi.TBL_OK, abi.TBL_ERR_NOT_CONVERGED)


def test_unreachable_tolerances_report_not_converged():
    mesh, rp, st = _case(mmax=4, errorstop=1e-300, errtol=1e-300)
    so, sg, g, rec = _both(mesh, rp, st)
    assert so == sg == abi.TBL_ERR_NOT_CONVERGED
    assert rec[0]["gs_sweeps"] == [4, 4, 4]
    d = g.download()
    assert all(np.isfinite(d[f]).all() for f in ("u", "v", "w", "p"))


def test_large_fluctuation_reports_blowup():
    mesh, rp, st = _case()
    st["nstep"] = 10  # past the recycling start: the fluctuation test runs
    st["u"] = np.asfortranarray(st["u"].copy())
    st["u"][8, 6, 6] += 60.0
    so, sg, g, _ = _both(mesh, rp, st)
    assert so == sg == abi.TBL_ERR_BLOWUP
    assert _still_usable(g, mesh, rp) == abi.TBL_OK


def test_bounded_wait_gives_up_and_the_device_stays_usable():
    import ctypes as C
    from turbulentbl_gb300.lib import load
    lib = load()
    lib.tbl_selftest_bounded_wait.argtypes = [C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    lib.tbl_selftest_bounded_wait.restype = C.c_int
    obs, secs = C.c_int32(0), C.c_double(0.0)
    assert lib.tbl_selftest_bounded_wait(C.byref(obs), C.byref(secs)) == abi.TBL_OK
    assert obs.value == abi.TBL_ERR_TIMEOUT
    assert 0.05 < secs.value < 60.0
    mesh, rp, st = _case()
    from turbulentbl_gb300.lib import TblGpu
    g = TblGpu(mesh, rp)
    g.upload(st)
    assert g.step(1, check=False)[0] == abi.TBL_OK
