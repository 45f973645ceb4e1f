"""GPU time step against the CPU oracle (parity tests proper).

Tolerance: relative L2 <= 1e-12 for u, v, w, p after each step (the target
the reference's FP64 path is held to).  Both run free (each picks its own GS
and GMRES iteration counts, which must coincide) or with the oracle's counts
replayed on the GPU.
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def pair(nx, nzs, nyw, P, kmax=20, cum=5, flags=0, seed=0):
    from turbulentbl_gb300.lib import TblGpu
    wl = small_workload(nx=nx, nz_span=nzs, ny_wall=nyw, kmax=kmax, seed=seed)
    mesh, rp, st = make_state(wl, nproc=P)
    rp.cum = cum
    rp.flags = flags
    o = OracleRunner(mesh, rp)
    g = TblGpu(mesh, rp)
    o.upload(st)
    g.upload(st)
    return o, g, st


def compare(o, g, fields=("u", "v", "w", "p", "pcorr")):
    a, b = o.download(), g.download()
    return {f: rel(b[f], a[f]) for f in fields}, a, b


@pytest.mark.parametrize("nx,nzs,nyw,P", [(24, 12, 20, 2), (30, 10, 26, 3), (21, 7, 17, 1), (40, 34, 33, 4),
                                          (20, 4, 16, 2), (22, 5, 16, 2), (26, 70, 12, 2), (24, 12, 40, 3),
                                          (24, 12, 40, 1)])
def test_free_running_steps_match(nx, nzs, nyw, P):
    """Grids with 4 span rows or fewer sweep with a row lag of a whole chunk
    (the Gauss-Seidel wrap row would otherwise share a step with row 1); 5
    rows is the smallest grid with the one-position lag; 70 rows span three
    32-row blocks.  The sweeps' plane groups of a slab column run as one
    thread-block cluster when they are 2..8: 40 planes in 3 slabs (13, 13 and
    12 planes: 4 plane groups, the last slab's top CTA idle) take that path,
    40 planes in one slab (10 plane groups) the cooperative launch with
    global flags."""
    o, g, _ = pair(nx, nzs, nyw, P)
    for s in range(7):
        so, _ = o.step(1, check=False)
        sg, rg = g.step(1, check=False)
        assert so == sg == abi.TBL_OK
        assert g.last_counts() == o.last_counts(), s
        errs, a, b = compare(o, g)
        for f in ("u", "v", "w", "p"):
            assert errs[f] <= TOL, (s, f, errs[f])
        assert np.array_equal(a["newk"], b["newk"])
        assert a["lamda"] == pytest.approx(b["lamda"], rel=1e-12)


def test_replayed_counts_match():
    o, g, _ = pair(24, 12, 20, 2, flags=abi.TBL_FLAG_REPLAY)
    # the oracle runs free (replay flag set but no record: derive counts first with a free oracle)
    o2, _, st = pair(24, 12, 20, 2)
    recs = []
    for _ in range(6):
        o2.step(1)
        recs += o2.last_counts()
    o.set_replay(recs)
    g.set_replay(recs)
    for s in range(6):
        o.step(1)
        g.step(1)
        errs, _, _ = compare(o, g)
        assert max(errs[f] for f in ("u", "v", "w", "p")) <= TOL, (s, errs)


def test_statistics_and_rescaling_match():
    o, g, _ = pair(24, 12, 20, 2, cum=3)
    for _ in range(7):
        o.step(1)
        g.step(1)
    a, b = o.download_stats(), g.download_stats()
    for f in ("usum", "vsum", "wsum", "uusum", "vvsum", "wwsum", "uvsum", "uwsum", "vwsum"):
        assert rel(b[f], a[f]) <= 1e-12, f
    for f in ("deltastar", "theta", "ht", "reth", "tauw_sum", "ubulk"):
        assert rel(b[f], a[f]) <= 1e-12, f
    assert np.abs(a["tauw_sum"]).max() > 0 and np.abs(a["ubulk"]).max() > 0
    assert b["lamda03"] == pytest.approx(a["lamda03"], rel=1e-12)
    sa, sb = o.download(), g.download()
    for f in ("usum2", "vsum2", "wsum2", "wt", "uf", "vf", "wf"):
        assert rel(sb[f], sa[f]) <= 1e-12, f
    assert np.array_equal(sa["newk"], sb["newk"])


def test_wall_shear_window_closes_like_the_oracle():
    """The 500-step wall-shear window (:1670-1681) closes at nstep = 500."""
    o, g, st = pair(24, 12, 20, 2, cum=10 ** 6)
    st = dict(st, nstep=497)
    o.upload(st)
    g.upload(st)
    for _ in range(5):
        o.step(1)
        g.step(1)
    a, b = o.download_stats(), g.download_stats()
    assert np.abs(a["tauw_window"]).max() > 0
    assert rel(b["tauw_window"], a["tauw_window"]) <= 1e-12
    assert rel(b["tauw_sum"], a["tauw_sum"]) <= 1e-12  # two steps into the next window
    assert rel(b["ubulk"], a["ubulk"]) <= 1e-12


def test_ppe_residual_reported():
    o, g, _ = pair(24, 12, 20, 2, flags=abi.TBL_FLAG_PPE_RESIDUAL)
    _, ro = o.step(1)
    _, rg = g.step(1)
    assert rg[0]["ppe_rel_resid"] == pytest.approx(ro[0]["ppe_rel_resid"], rel=1e-6)
    assert 0 < rg[0]["ppe_rel_resid"] < 1e-3


def test_reference_config1_box_one_step():
    """The 128 x 64 x 64 box of the FP64 parity case (restart 30, tol 1e-8), two steps."""
    from turbulentbl_gb300.synth import WORKLOADS
    from turbulentbl_gb300.lib import TblGpu
    wl = WORKLOADS["box128_fp64"]
    mesh, rp, st = make_state(wl, nproc=8)
    o = OracleRunner(mesh, rp)
    g = TblGpu(mesh, rp)
    o.upload(st)
    g.upload(st)
    for s in range(2):
        o.step(1)
        g.step(1)
        assert g.last_counts() == o.last_counts()
        errs, _, _ = compare(o, g)
        assert max(errs[f] for f in ("u", "v", "w", "p")) <= TOL, errs


def test_launch_count_reported():
    _, g, _ = pair(24, 12, 20, 2)
    n0 = g.launches()
    g.step(1)
    assert g.launches() > n0 + 10
