"""Failure detection in the host logic (CPU): the oracle reports NaN input,
a zero Poisson right-hand side and unreachable tolerances with the status
codes the library uses; corrupt restart files are covered in test_tpfile.py."""
import numpy as np

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner


def _run(mutate, **rp_kw):
    wl = small_workload(nx=16, nz_span=8, ny_wall=14, kmax=10)
    mesh, rp, st = make_state(wl, nproc=2)
    for k, v in rp_kw.items():
        setattr(rp, k, v)
    st = dict(st)
    mutate(st)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    s, rec = o.step(1, check=False)
    return s, rec


def test_nan():
    def m(st):
        st["u"] = np.asfortranarray(st["u"].copy())
        st["u"][5, 5, 5] = np.nan
    assert _run(m, mmax=20)[0] == abi.TBL_ERR_NAN


def test_zero_rhs():
    def m(st):
        for f in ("u", "v", "w", "p", "pcorr", "uf", "vf", "wf", "usum2", "vsum2", "wsum2"):
            st[f] = np.zeros_like(st[f], order="F")
    assert _run(m, mmax=6, recycle_after=10 ** 6)[0] == abi.TBL_ERR_ZERO_RHS


def test_not_converged():
    s, rec = _run(lambda st: None, mmax=4, errorstop=1e-300, errtol=1e-300)
    assert s == abi.TBL_ERR_NOT_CONVERGED
    assert rec[0]["gs_sweeps"] == [4, 4, 4]
