"""Block SSOR preconditioners on span blocks (TBL_FLAG_SSOR_SPAN_BLOCKS) and
streamwise blocks (TBL_FLAG_SSOR_STREAM_BLOCKS) against the oracle.

Throughput modes: the block SSOR of GMRES also splits every slab into blocks
of 32 span rows and/or two streamwise halves, which changes the
preconditioner (and the iteration counts), not the systems solved.  With tight solver tolerances the fields after a few
steps agree with the oracle (the reference's preconditioner) to 1e-8 in FP64
and to the mixed-precision tolerances in mixed mode.  The span of 40 rows
gives a full block of 32 and a partial one.
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


SPAN, STREAM = abi.TBL_FLAG_SSOR_SPAN_BLOCKS, abi.TBL_FLAG_SSOR_STREAM_BLOCKS


@pytest.mark.parametrize("blocks,nx", [(SPAN, 24), (STREAM, 24), (STREAM, 30), (SPAN | STREAM, 31)])
@pytest.mark.parametrize("extra", [0, abi.TBL_FLAG_RB_ORDER])
@pytest.mark.parametrize("precision,tol_uvw,tol_p", [(abi.TBL_PREC_FP64, 1e-8, 1e-7), (abi.TBL_PREC_MIXED, 1e-5, 1e-4)])
def test_block_preconditioners_track_the_oracle(precision, tol_uvw, tol_p, extra, blocks, nx):
    from turbulentbl_gb300.lib import TblGpu
    fp64 = precision == abi.TBL_PREC_FP64
    wl = small_workload(nx=nx, nz_span=40, ny_wall=20, kmax=20, errtol=1e-12 if fp64 else 1e-10)
    mesh, rp, st = make_state(wl, nproc=2)
    if fp64:
        rp.errorstop = 1e-12
    rp.mmax = 3000
    o = OracleRunner(mesh, rp)
    o.upload(st)
    rp.flags = blocks | abi.TBL_FLAG_PPE_RESIDUAL | extra
    if not fp64:
        rp.precision = abi.TBL_PREC_MIXED
        rp.mixed_kmax = 20
        rp.mixed_outer_tol = 1e-10
        rp.mixed_inner_tol = 1e-5
    g = TblGpu(mesh, rp)
    g.upload(st)
    for s in range(3):
        o.step(1, check=False)
        sg, rec = g.step(1, check=False)
        assert sg == abi.TBL_OK
        a, b = o.download(), g.download()
        for f, tol in (("u", tol_uvw), ("v", tol_uvw), ("w", tol_uvw), ("p", tol_p)):
            assert rel(b[f], a[f]) <= tol, (s, f, rel(b[f], a[f]))
        assert rec[0]["ppe_rel_resid"] <= 1e-8, rec[0]
