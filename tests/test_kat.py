"""Known-answer tests of the restated operators (CPU).

The reference ships no tests or golden data, so these pin the restatement
to the mathematics it discretises and to its own ordering semantics:
manufactured solutions for the stretched-grid Laplacian, the GMRES/SSOR
solve against a direct sparse solve, exactness of the convection stencils on
polynomials, the lexicographic Gauss-Seidel against a hyperplane-ordered one
(the ordering the GPU wavefront uses), the recycling index map, and the
boundary-layer, displacement and momentum thicknesses of the rescaling.
"""
import numpy as np
import pytest

from turbulentbl_gb300.mesh import make_mesh, RunParams, make_config
from turbulentbl_gb300.synth import small_workload, make_state, rescaling_state
from oracle.bind import OracleRunner
from oracle.np_oracle import NpOracle


def runner(nx, ny, nz, P=2, kmax=20, errtol=1e-12, lx=3.0, lz=2.0, ly=2.0, beta=2.0):
    mesh = make_mesh(nx, ny, nz, lx, lz, ly, beta)
    rp = RunParams(dt=1e-3, re=1000.0, ue=1.0, nproc=P, irec=max(2, nx // 2), kmax=kmax, errtol=errtol)
    return mesh, rp, OracleRunner(mesh, rp)


def grids(mesh):
    return np.meshgrid(mesh.x1, mesh.x2, mesh.x3, indexing="ij")


@pytest.mark.parametrize("beta", [1.5, 2.4])
def test_laplacian_second_order_on_stretched_grid(beta):
    errs = []
    for n in (16, 32):
        mesh, rp, o = runner(n, n // 2 + 2, n, beta=beta)
        X, Y, Z = grids(mesh)
        Ly = (mesh.ny - 2) * mesh.dy  # spanwise period
        ky, kx = 2 * np.pi / Ly, np.pi / 3.0
        p = np.sin(ky * Y) * np.cos(kx * X) * Z ** 2
        exact = np.sin(ky * Y) * np.cos(kx * X) * (2.0 - (kx ** 2 + ky ** 2) * Z ** 2)
        lap = o.apply_lap(p)
        s = (slice(2, -2), slice(1, -1), slice(2, -2))
        errs.append(np.abs(lap[s] - exact[s]).max() / np.abs(exact[s]).max())
    order = np.log2(errs[0] / errs[1])
    assert order > 1.8, (errs, order)


def test_gmres_matches_direct_solve():
    scipy = pytest.importorskip("scipy.sparse.linalg")
    import scipy.sparse as sp
    mesh, rp, o = runner(10, 8, 12, P=2, kmax=20, errtol=1e-13)
    nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
    interior = [(i, j, k) for k in range(1, nz - 1) for j in range(1, ny - 1) for i in range(1, nx - 1)]
    index = {q: n for n, q in enumerate(interior)}
    rows, cols, vals = [], [], []
    for n, (i, j, k) in enumerate(interior):
        e = np.zeros((nx, ny, nz), order="F")
        e[i, j, k] = 1.0
        col = o.apply_lap(e)
        for m, (a, b, c) in enumerate(interior):
            v = col[a, b, c]
            if v != 0.0:
                rows.append(m)
                cols.append(n)
                vals.append(v)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(len(interior), len(interior)))
    rng = np.random.default_rng(5)
    rhs = np.zeros((nx, ny, nz), order="F")
    b = rng.standard_normal(len(interior))
    for n, q in enumerate(interior):
        rhs[q] = b[n]
    xd = scipy.spsolve(A.tocsc(), b)
    st, x, it = o.solve_ppe(rhs)
    xg = np.array([x[q] for q in interior])
    assert st == 0 and it > 0
    assert np.linalg.norm(xg - xd) / np.linalg.norm(xd) < 1e-8


def test_convection_exact_for_cubics():
    """4th-order central differences are exact for cubics: Q = U - dt*u*dF/dx."""
    wl = small_workload(nx=16, nz_span=8, ny_wall=12)
    mesh, rp, st = make_state(wl, nproc=2)
    n = NpOracle(mesh, rp)
    X, Y, Z = grids(mesh)
    c = 3.0  # Pe = Re*c*dx well above 50: the central branch
    st = dict(st)
    st["u"] = np.full_like(X, c)
    st["v"] = np.zeros_like(X)
    st["w"] = np.zeros_like(X)
    st["p"] = np.zeros_like(X)
    n.upload(st)
    F = (X - 0.3) ** 3
    n.U[1] = np.asfortranarray(F)
    n.conv_q()
    conv = (n.U[1] - n.Q[1]) / rp.dt
    exact = c * 3 * (X - 0.3) ** 2
    s = (slice(2, -2), slice(1, -1), slice(1, -1))  # 4th-order columns
    assert np.allclose(conv[s], exact[s], rtol=1e-9, atol=1e-9)


def _gs_sweep(F, Q, order, coef):
    cE, cW, cN, cS, cT, cB, d = coef
    nx, ny, nz = F.shape
    jm = lambda j: ny - 2 if j == 1 else j - 1
    jp = lambda j: 1 if j == ny - 2 else j + 1
    for (i, j, k) in order:
        F[i, j, k] = (Q[i, j, k] - cE * F[i + 1, j, k] - cW * F[i - 1, j, k] - cN * F[i, jp(j), k]
                      - cS * F[i, jm(j), k] - cT * F[i, j, k + 1] - cB * F[i, j, k - 1]) / d


def test_gs_hyperplane_order_is_bitwise_lexicographic():
    """Any order respecting (i-1, j-1, k-1) -> (i,j,k) gives the same GS sweep,
    including the periodic wrap in j; the GPU wavefront relies on this."""
    rng = np.random.default_rng(1)
    nx, ny, nz = 9, 8, 7
    F0 = rng.standard_normal((nx, ny, nz))
    Q = rng.standard_normal((nx, ny, nz))
    coef = (-0.1, -0.12, -0.2, -0.21, -0.3, -0.33, 2.7)
    pts = [(i, j, k) for k in range(1, nz - 1) for j in range(1, ny - 1) for i in range(1, nx - 1)]
    lex = F0.copy()
    _gs_sweep(lex, Q, pts, coef)
    hyp = F0.copy()
    _gs_sweep(hyp, Q, sorted(pts, key=lambda p: (p[0] + p[1] + p[2], p[1], p[0])), coef)
    assert np.array_equal(lex, hyp)
    # a chunked schedule like the GPU's: chunk c of line (j,k) at step c + j + k
    ch = 4
    chk = F0.copy()
    sched = sorted(pts, key=lambda p: ((p[0] // ch) + p[1] + p[2], p[1], p[2], p[0]))
    _gs_sweep(chk, Q, sched, coef)
    assert np.array_equal(lex, chk)
    # an order that breaks the dependencies does not reproduce it
    bad = F0.copy()
    _gs_sweep(bad, Q, list(reversed(pts)), coef)
    assert not np.array_equal(lex, bad)


def test_recycling_map_identity_when_no_rescaling():
    """With lamda = lamda03 = 1 the recycling map is the identity (new(k) = k)."""
    nx, nz = 12, 20
    x3 = np.linspace(0.0, 3.0, nz) ** 1.3
    usum2 = np.minimum(x3[None, :] / 1.0, 1.0) * np.ones((nx, 1))
    bl, wt, newk, ksep = rescaling_state(usum2, x3, 1.0, irec=6, lamda=1.0)
    assert np.allclose(bl, x3[np.argmax(x3 >= 0.99)])
    assert list(newk[:nz - 1]) == list(range(1, nz))
    assert newk[nz - 1] == nz - 1
    # Wt rises monotonically from ~0 at the wall to ~1 above the layer
    assert np.all(np.diff(wt[0]) >= 0) and wt[0, 0] < 0.05 and wt[0, -1] > 0.99
    assert 1 <= ksep < nz


def test_recycling_map_outer_stretch_is_monotone():
    nx, nz = 12, 24
    x3 = np.linspace(0.0, 3.0, nz)
    dl = np.linspace(1.0, 1.3, nx)
    usum2 = np.minimum(x3[None, :] / dl[:, None], 1.0)
    bl, wt, newk, ksep = rescaling_state(usum2, x3, 1.0, irec=10, lamda=1.05)
    k = newk[:nz - 1]
    assert np.all(np.diff(k) >= 0) and k.min() >= 1 and k.max() <= nz - 1


def test_mass_flux_and_wall_shear_known_answers():
    """Mass flux (:1578-1594) and wall shear (:1616-1668) on fields with known
    answers.  u = U0 + s x gives, at each plane i_p, (U0 + s x(i_p)) times
    (ny-2)/(ny-3): the reference divides the flux through the ny-2 unique span
    cells by an area spanning only x2(ny-1) - x2(2) = (ny-3) dy.  u = a z + e z^2
    near the wall and w(wall) = b x give the span sum (ny-2)(a + b)/Re in every
    column (both stencils are exact there)."""
    wl = small_workload(nx=24, nz_span=10, ny_wall=14)
    mesh, rp, st = make_state(wl, nproc=2)
    o = OracleRunner(mesh, rp)
    X, Y, Z = grids(mesh)
    assert mesh.x3[0] == 0.0
    U0, s = 0.7, 0.05
    st = dict(st, u=np.asfortranarray(U0 + s * X), v=np.zeros_like(X), w=np.zeros_like(X), p=np.zeros_like(X))
    o.upload(st)
    ub, _ = o.flux_shear()
    ratio = (mesh.ny - 2) / (mesh.ny - 3)
    for q, plane in enumerate((5, 20, 40, 60, 85)):
        ip = min(plane, mesh.nx - 1) - 1
        assert ub[q] == pytest.approx((U0 + s * mesh.x1[ip]) * ratio, rel=1e-12)
    a, e, b = 2.0, -3.0, 0.4
    w = np.zeros_like(X)
    w[:, :, 0] = b * X[:, :, 0]
    st = dict(st, u=np.asfortranarray(a * Z + e * Z * Z), w=np.asfortranarray(w))
    o.upload(st)
    _, tau = o.flux_shear()
    expect = (mesh.ny - 2) * (a + b) / rp.re
    assert np.allclose(tau[1:-1], expect, rtol=1e-10)
    assert tau[0] == 0.0 and tau[-1] == 0.0


def _uniform_x3_runner(nx=8, nz=40, h=0.05, ue=1.0, re=1000.0):
    mesh = make_mesh(nx, 6, nz, 3.0, 2.0, 2.0, 2.0)
    mesh.x3 = np.ascontiguousarray(h * np.arange(nz, dtype=np.float64))
    rp = RunParams(dt=1e-3, re=re, ue=ue, nproc=2, irec=max(2, nx // 2))
    return mesh, rp, OracleRunner(mesh, rp)


@pytest.mark.parametrize("ue", [1.0, 19.798])
def test_integral_thicknesses_of_linear_profiles(ue):
    """u = Ue min(x3/delta, 1) on a uniform x3 (spacing h, delta = m h,
    m < 100) has bltkns = delta (the first point at or above 0.99 Ue), and the
    reference's left sums (dnstbl2/dnstbl.f90:2234-2256) give
    delta* = h (m+1)/2, theta = h (m+1)(m-1)/(6m), H = 3m/(m-1) and
    Re_theta = theta Re Ue."""
    h, re = 0.05, 1000.0
    mesh, rp, o = _uniform_x3_runner(h=h, ue=ue, re=re)
    ms = np.array([3, 5, 8, 12, 17, 23, 30, 38])
    u = ue * np.minimum(mesh.x3[None, :] / (ms[:, None] * h), 1.0)
    bl, ds, th, ht, rt = o.thicknesses(u)
    assert np.array_equal(bl, mesh.x3[ms])
    assert np.allclose(ds, h * (ms + 1) / 2, rtol=1e-13, atol=0)
    assert np.allclose(th, h * (ms + 1) * (ms - 1) / (6 * ms), rtol=1e-13, atol=0)
    assert np.allclose(ht, 3 * ms / (ms - 1), rtol=1e-13, atol=0)
    assert np.allclose(rt, th * re * ue, rtol=1e-15, atol=0)


def test_integral_thicknesses_keep_the_previous_edge():
    """When no point reaches 0.99 Ue, bltkns keeps its previous value
    (dnstbl2/dnstbl.f90:2150-2158).  The displacement sum stops after the
    cell that starts exactly at bltkns (:2237), the momentum sum after the
    first cell starting at or above it (:2245): with an edge between two grid
    points (a value from the restart state) the displacement sum runs over
    every cell and the momentum sum stops at the next point above the edge."""
    wl = small_workload(nx=10, nz_span=6, ny_wall=24)
    mesh, rp, st = make_state(wl, nproc=2)
    o = OracleRunner(mesh, rp)
    x3 = mesh.x3
    edge = 0.5 * (x3[10] + x3[11])
    o.upload(dict(st, bltkns=np.full(mesh.nx, edge)))
    r = 0.5 * x3 / x3[-1]  # u / Ue, never reaches 0.99
    bl, ds, th, _, _ = o.thicknesses(np.tile(rp.ue * r, (mesh.nx, 1)))
    assert np.all(bl == edge)
    dz = np.diff(x3)
    assert np.allclose(ds, np.sum((1 - r[:-1]) * dz), rtol=1e-13, atol=0)
    assert np.allclose(th, np.sum((r * (1 - r))[:12] * dz[:12]), rtol=1e-13, atol=0)
    # a new edge on a grid point ends both sums at that point's cell
    bl, ds, th, _, _ = o.thicknesses(np.tile(rp.ue * np.minimum(x3 / x3[7], 1.0), (mesh.nx, 1)))
    r = np.minimum(x3 / x3[7], 1.0)
    assert np.all(bl == x3[7])
    assert np.allclose(ds, np.sum((1 - r[:8]) * dz[:8]), rtol=1e-13, atol=0)
    assert np.allclose(th, np.sum((r * (1 - r))[:8] * dz[:8]), rtol=1e-13, atol=0)
