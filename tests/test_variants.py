"""The reference's other two programs of the method (tbl_config.variant) on
the CPU: the C++ oracle against the NumPy restatement with each variant's
switches active (recycling, eps ramp, rescaling and the slab partition all
exercised within a few steps), plus known answers for the switched pieces.

Variant 1 follows originalTBL/fnldnstbl.f90, variant 2 dnssetbl/dnssetbl.f90.
"""
import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner
from oracle.np_oracle import NpOracle


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def variant_case(variant, nx=16, nzs=8, nyw=14, P=3, kmax=10, recycle_after=2, cum=3):
    wl = small_workload(nx=nx, nz_span=nzs, ny_wall=nyw, kmax=kmax)
    mesh, rp, st = make_state(wl, nproc=P)
    rp.variant = variant
    rp.recycle_after, rp.cum = recycle_after, cum
    st = dict(st, cnt2=5000, nstep=4000 if variant == 2 else 0)  # eps = 0.25 (cnt2) / 0.2 (nstep)
    return mesh, rp, st


def dnssetbl_partition(nz, P):
    """dnssetbl.f90:78-92 as written (1-based b, e, bn, en)."""
    it1 = nz // P
    it2 = P - nz % P
    b, e = [0] * (P + 1), [0] * P
    b[0] = 1
    for i in range(P):
        if i == it2:
            it1 += 1
        e[i] = b[i] + it1 - 1
        b[i + 1] = e[i] + 1
    bn, en = b[:P], list(e)
    bn[0] = b[0] + 1
    en[P - 1] = e[P - 1] - 1
    return bn, en


@pytest.mark.parametrize("variant", [abi.TBL_VARIANT_ORIGINAL, abi.TBL_VARIANT_DNSSETBL])
@pytest.mark.parametrize("P", [2, 3])
def test_cpp_equals_numpy(variant, P):
    mesh, rp, st = variant_case(variant, P=P)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    n = NpOracle(mesh, rp)
    n.upload(st)
    lam = []
    for s in range(7):
        o.step(1)
        counts = o.last_counts()
        assert n.step(counts) == counts
        d = o.download()
        for f, x in (("u", n.U[0]), ("v", n.U[1]), ("w", n.U[2]), ("p", n.P), ("pcorr", n.PC)):
            assert rel(x, d[f]) < 1e-12, (s, f, rel(x, d[f]))
        assert np.array_equal(d["newk"], n.newk)
        assert d["lamda"] == pytest.approx(n.lamda, rel=1e-13)
        assert d["cnt2"] == st["cnt2"] + s + 1
        lam.append(d["lamda"])
    assert len(set(lam)) > 1  # rescaling ran and changed lamda


@pytest.mark.parametrize("nz,P", [(14, 3), (14, 4), (20, 8), (50, 8), (17, 2)])
def test_dnssetbl_partition(nz, P):
    bn, en = dnssetbl_partition(nz, P)
    wl = small_workload(nx=12, nz_span=6, ny_wall=nz)
    mesh, rp, st = make_state(wl, nproc=P)
    assert mesh.nz == nz
    rp.variant = abi.TBL_VARIANT_DNSSETBL
    n = NpOracle(mesh, rp)
    assert [(a - 1, b - 1) for a, b in zip(bn, en)] == n.slabs
    assert bn[0] == 2 and en[-1] == nz - 1
    assert all(bn[r + 1] == en[r] + 1 for r in range(P - 1))


def test_variant_differences_change_the_step():
    """Each variant's switches are live: one step from the same state differs."""
    out = {}
    for v in (0, 1, 2):
        mesh, rp, st = variant_case(v, P=2)
        o = OracleRunner(mesh, rp)
        o.upload(st)
        o.step(3)
        out[v] = o.download()["u"]
    assert rel(out[1], out[0]) > 1e-8 and rel(out[2], out[0]) > 1e-8 and rel(out[2], out[1]) > 1e-8


@pytest.mark.parametrize("variant", [abi.TBL_VARIANT_ORIGINAL, abi.TBL_VARIANT_DNSSETBL])
def test_inflow_ramp_known_answer(variant):
    """With zero recycled fluctuations, u(1,j,k) = eps usum2(irec,new(k)) +
    (1-eps) Ume1(k) (fnldnstbl.f90:577, dnssetbl.f90:268); dnssetbl's v mean is
    lamda vsum2(irec,new(k)) (dnssetbl.f90:271)."""
    mesh, rp, st = variant_case(variant, P=2)
    ir = rp.irec - 1
    st = dict(st, lamda=1.3)
    st["usum2"] = np.asfortranarray(np.full_like(st["usum2"], 0.5))
    st["vsum2"] = np.asfortranarray(np.full_like(st["vsum2"], 0.02))
    for f in ("uf", "vf", "wf"):
        st[f] = np.zeros_like(st[f])
    for f, m in (("u", "usum2"), ("v", "vsum2"), ("w", "wsum2")):
        st[f] = np.asfortranarray(st[f].copy())
        st[f][ir, 1:-1, :] = st[m][ir][None, :]
    n = NpOracle(mesh, rp)
    n.upload(st)
    n.nstep += 1
    n.inflow()
    eps = 0.25 if variant == abi.TBL_VARIANT_ORIGINAL else 4001 * 5e-5
    k = np.arange(1, mesh.nz - 1)
    expect_u = eps * 0.5 + (1 - eps) * st["ume1"][k]
    assert np.allclose(n.U[0][0, 1:-1, 1:-1], expect_u[None, :], rtol=1e-14)
    expect_v = 1.3 * 0.02 if variant == abi.TBL_VARIANT_DNSSETBL else 0.02
    assert np.allclose(n.U[1][0, 1:-1, 1:-1], expect_v, rtol=1e-14)


def test_dnssetbl_span_boundary_rows_are_central():
    """dnssetbl's y convection on the first/last unique rows is the
    second-order central v (F(j+1) - F(j-1)) / (2 dy) with the periodic wrap
    (dnssetbl.f90:325-326); dnstbl2 is first-order upwind there (:670-677)."""
    for variant in (0, 2):
        mesh, rp, st = variant_case(variant, P=2)
        rng = np.random.default_rng(4)
        nx, ny, nz = st["u"].shape
        f = rng.normal(size=ny)
        f[0], f[-1] = f[ny - 2], f[1]  # periodic ghosts
        F = np.asfortranarray(np.broadcast_to(f[None, :, None], (nx, ny, nz)).copy())  # w = F(j): no x, xi terms
        st = dict(st, u=np.zeros_like(F), v=np.full_like(F, 0.3), w=np.zeros_like(F), p=np.zeros_like(F))
        n = NpOracle(mesh, rp)
        n.upload(st)
        n.U[2] = F.copy()
        n.conv_q()
        conv = (n.U[2] - n.Q[2]) / rp.dt
        for j, jm, jp in ((1, ny - 2, 2), (ny - 2, ny - 3, 1)):
            got = conv[1:-1, j, 1:-1]
            if variant == 2:
                want = 0.3 * (F[1:-1, jp, 1:-1] - F[1:-1, jm, 1:-1]) * (0.5 / mesh.dy)
            else:
                want = 0.3 * (F[1:-1, j, 1:-1] - F[1:-1, jm, 1:-1]) / mesh.dy
            assert np.allclose(got, want, rtol=1e-12, atol=1e-12), (variant, j)
