"""GPU time step of the reference's other two programs (tbl_config.variant)
against the CPU oracle: originalTBL/fnldnstbl.f90 (1) and dnssetbl/dnssetbl.f90
(2).  The recycling start, cum and the state's counters are set so that the
inflow ramp, the rescaling and (dnssetbl) the fluctuation/KE guard switch on
within a few steps; P = 3 exercises dnssetbl's uneven slab partition.

Tolerances as for the default program: relative L2 <= 1e-12 for u, v, w, p
each step in FP64, statistics and diagnostics to 1e-12; the mixed-precision
path to its usual 1e-5 (velocities) and 1e-4 (pressure).
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu
VARIANTS = [abi.TBL_VARIANT_ORIGINAL, abi.TBL_VARIANT_DNSSETBL]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def pair(variant, P=3, nx=24, nzs=12, nyw=20, precision=abi.TBL_PREC_FP64, recycle_after=2, cum=3):
    from turbulentbl_gb300.lib import TblGpu
    wl = small_workload(nx=nx, nz_span=nzs, ny_wall=nyw, kmax=20, errtol=1e-10)
    mesh, rp, st = make_state(wl, nproc=P)
    rp.variant = variant
    rp.recycle_after, rp.cum = recycle_after, cum
    st = dict(st, cnt2=5000, nstep=4000 if variant == abi.TBL_VARIANT_DNSSETBL else 0)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    if precision == abi.TBL_PREC_MIXED:
        rp.precision = abi.TBL_PREC_MIXED
        rp.mixed_kmax = 20
        rp.mixed_outer_tol = 1e-10
        rp.mixed_inner_tol = 1e-5
    g = TblGpu(mesh, rp)
    g.upload(st)
    return o, g, st


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("P", [2, 3])
def test_variant_steps_match_the_oracle(variant, P):
    o, g, st = pair(variant, P=P)
    lam = set()
    for s in range(8):
        so, ro = o.step(1, check=False)
        sg, rg = g.step(1, check=False)
        assert so == sg == abi.TBL_OK, (s, so, sg)
        assert g.last_counts() == o.last_counts(), s
        a, b = o.download(), g.download()
        for f in ("u", "v", "w", "p"):
            assert rel(b[f], a[f]) <= 1e-12, (s, f, rel(b[f], a[f]))
        assert np.array_equal(a["newk"], b["newk"])
        assert a["lamda"] == pytest.approx(b["lamda"], rel=1e-12)
        assert a["cnt2"] == b["cnt2"] == st["cnt2"] + s + 1
        assert rg[0]["cum_step"] == ro[0]["cum_step"]
        assert rg[0]["div_diag"] == pytest.approx(ro[0]["div_diag"], rel=1e-8, abs=1e-300)
        assert rg[0]["ke"] == pytest.approx(ro[0]["ke"], rel=1e-10, abs=1e-300)
        lam.add(a["lamda"])
    assert len(lam) > 1
    sa, sb = o.download_stats(), g.download_stats()
    for f in ("usum", "vsum", "wsum", "uusum", "uvsum", "deltastar", "theta", "ubulk"):
        assert rel(sb[f], sa[f]) <= 1e-12, f


@pytest.mark.parametrize("variant", VARIANTS)
def test_variant_mixed_precision_tracks_the_oracle(variant):
    o, g, _ = pair(variant, P=2, precision=abi.TBL_PREC_MIXED)
    for s in range(4):
        o.step(1, check=False)
        sg, _ = g.step(1, check=False)
        assert sg == abi.TBL_OK
        a, b = o.download(), g.download()
        for f, tol in (("u", 1e-5), ("v", 1e-5), ("w", 1e-5), ("p", 1e-4)):
            assert rel(b[f], a[f]) <= tol, (s, f, rel(b[f], a[f]))


def test_variant_rejections():
    from turbulentbl_gb300.lib import TblGpu
    from turbulentbl_gb300.runner import TblError
    wl = small_workload(nx=24, nz_span=12, ny_wall=20)
    mesh, rp, st = make_state(wl, nproc=2)
    rp.variant = 3
    with pytest.raises(TblError):
        TblGpu(mesh, rp)
    rp.variant = abi.TBL_VARIANT_DNSSETBL
    rp.nproc = 8  # 20 planes in 8 dnssetbl slabs: rank 0 keeps only 1 after the wall plane
    with pytest.raises(TblError):
        TblGpu(mesh, rp)
    rp.nproc = 2
    rp.cum = 10 ** 6
    g = TblGpu(mesh, rp)
    g.upload(st)
    with pytest.raises(TblError):  # adjoint windows follow dnstbl2 only
        g.forward_window(2, 0.3, 1.5, 1)
    rp.variant = abi.TBL_VARIANT_DNSTBL2
    for flag in (abi.TBL_FLAG_SSOR_SPAN_BLOCKS, abi.TBL_FLAG_SSOR_STREAM_BLOCKS, abi.TBL_FLAG_RB_ORDER):
        rp.flags = flag
        g = TblGpu(mesh, rp)
        g.upload(st)
        with pytest.raises(TblError):  # and the reference's orderings and preconditioner
            g.forward_window(2, 0.3, 1.5, 1)
