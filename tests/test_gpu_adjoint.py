"""Discrete adjoint of a window of steps (tbl_forward_window / tbl_backward_window).

References: oracle/torch_step.py, a float64 torch restatement of the step with
exact solves whose autograd gives the exact vjp (adjoint) and jvp
(tangent-linear) of the map the library differentiates, and central finite
differences of the library's own forward window.  Solver tolerances are tight
(GS 1e-13, GMRES 1e-13) so that the iterative forward matches the exact-solve
map to ~1e-12.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

W = 4              # window length (steps)
PATCH = (0.3, 1.5)  # streamwise extent of the wall-shear patch
TOL_TORCH = 1e-7   # library adjoint vs exact autograd (max-norm relative)
TOL_FD = 1e-4      # directional derivative vs central differences (relative)


def _case(seed=3):
    from turbulentbl_gb300.synth import small_workload, make_state
    from turbulentbl_gb300.lib import TblGpu

    wl = small_workload(nx=14, nz_span=8, ny_wall=12, kmax=30, errtol=1e-13)
    mesh, rp, st = make_state(wl, nproc=2)
    rp.errorstop = 1e-13
    rp.cum = 10 ** 6
    rp.mmax = 3000
    st["nstep"] = 10
    g = TblGpu(mesh, rp)
    g.upload(st)
    rng = np.random.default_rng(seed)
    c = rng.normal(0.0, 1e-3, (mesh.nx, mesh.ny - 2))
    g.set_wall_control(c)
    g.step(1)  # the live recycling plane now comes from the state itself
    x0 = g.download()
    return mesh, rp, g, x0, c


def _torch_ref(mesh, rp, x0):
    from oracle.torch_step import TorchStep

    P = rp.nproc
    loc = (mesh.nz - 1) // P
    slabs = [(1 + r * loc, (1 + r * loc + loc - 1) if r < P - 1 else mesh.nz - 2) for r in range(P)]
    ir = rp.irec - 1
    rc = dict(usum2=x0["usum2"], vsum2=x0["vsum2"], wsum2=x0["wsum2"], wt=x0["wt"], newk=x0["newk"],
              ume1=x0["ume1"], lamda=x0["lamda"], slabs=slabs, fl_file=[x0[f][ir] for f in ("uf", "vf", "wf")])
    return TorchStep(mesh, rp, rc)


def _torch_window(ts, x0, c_full, nsteps):
    U = [torch.tensor(x0[f]) for f in ("u", "v", "w")]
    P = torch.tensor(x0["p"])
    cols = ts.patch_columns(*PATCH)
    J = 0.0
    for s in range(nsteps):
        U, P = ts.step(U, P, c_full, x0["nstep"] + 1 + s)
        J = J + ts.wall_shear(U, cols)
    return J / nsteps, U, P


def _full(c, ny):
    cf = torch.zeros(c.shape[0], ny, dtype=torch.float64)
    cf[:, 1:ny - 1] = torch.as_tensor(c)
    return cf


def _gpu_J(g, x0, c, nsteps=W, ckpt=2):
    g.upload(x0)
    g.set_wall_control(c)
    J, _ = g.forward_window(nsteps, PATCH[0], PATCH[1], ckpt)
    return J


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def case():
    mesh, rp, g, x0, c = _case()
    ts = _torch_ref(mesh, rp, x0)
    ct = _full(c, mesh.ny).requires_grad_(True)
    Jt, _, _ = _torch_window(ts, x0, ct, W)
    (gt,) = torch.autograd.grad(Jt, ct)
    return dict(mesh=mesh, rp=rp, g=g, x0=x0, c=c, ts=ts, Jt=float(Jt.detach()), gt=gt[:, 1:mesh.ny - 1].numpy())


def test_window_objective_and_gradient_match_autograd(case):
    g = case["g"]
    J = _gpu_J(g, case["x0"], case["c"], ckpt=2)
    gc, _, ast = g.backward_window(1.0)
    assert abs(J - case["Jt"]) <= 1e-10 * abs(case["Jt"])
    assert _rel(gc, case["gt"]) <= TOL_TORCH, _rel(gc, case["gt"])
    assert ast["steps"] == W and ast["recomputed_steps"] == 2
    assert ast["adj_gmres_iters"] > 0 and ast["adj_gs_sweeps"] > 0


def test_checkpoint_recompute_is_bitwise(case):
    g = case["g"]
    _gpu_J(g, case["x0"], case["c"], ckpt=1)
    g1, _, a1 = g.backward_window(1.0)
    _gpu_J(g, case["x0"], case["c"], ckpt=W)
    g2, _, a2 = g.backward_window(1.0)
    assert a1["recomputed_steps"] == W - 1 and a2["recomputed_steps"] == 0
    assert np.array_equal(g1, g2)


def test_state_after_backward_is_end_of_window(case):
    g = case["g"]
    _gpu_J(g, case["x0"], case["c"], ckpt=2)
    end = g.download()
    g.backward_window(1.0)
    again = g.download()
    for f in ("u", "v", "w", "p", "pcorr"):
        assert np.array_equal(end[f], again[f]), f
    assert end["nstep"] == again["nstep"] and end["time"] == again["time"]
    # and stepping on from there matches stepping on without the adjoint
    g.step(1)
    a = g.download()
    _gpu_J(g, case["x0"], case["c"], ckpt=2)
    g.step(1)
    b = g.download()
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(a[f], b[f]), f


def test_single_step_vjp_all_inputs(case):
    """One step, loss = dL_dJ * J + <lam, X1>: dL/dc and dL/dX0 against autograd."""
    mesh, g, x0, c, ts = case["mesh"], case["g"], case["x0"], case["c"], case["ts"]
    rng = np.random.default_rng(11)
    lam = {f: rng.normal(size=(mesh.nx, mesh.ny, mesh.nz)) for f in ("u", "v", "w", "p")}
    gJ = 0.7
    _gpu_J(g, x0, c, nsteps=1, ckpt=1)
    gc, gi, _ = g.backward_window(gJ, lam, want_initial=True)
    U0 = [torch.tensor(x0[f], requires_grad=True) for f in ("u", "v", "w")]
    P0 = torch.tensor(x0["p"], requires_grad=True)
    ct = _full(c, mesh.ny).requires_grad_(True)
    U1, P1 = ts.step(U0, P0, ct, x0["nstep"] + 1)
    L = gJ * ts.wall_shear(U1, ts.patch_columns(*PATCH))
    for f, X in zip(("u", "v", "w", "p"), list(U1) + [P1]):
        L = L + (X * torch.tensor(lam[f])).sum()
    grads = torch.autograd.grad(L, U0 + [P0, ct])
    assert _rel(gc, grads[4][:, 1:mesh.ny - 1].numpy()) <= TOL_TORCH
    # the first step after an upload reads the recycling plane as uploaded
    # data, so the plane i = irec carries no gradient in the library
    ir = case["rp"].irec - 1
    for q, f in enumerate(("u", "v", "w", "p")):
        ref = grads[q].numpy().copy()
        got = gi[f].copy()
        ref[ir] = 0.0
        got[ir] = 0.0
        assert _rel(got, ref) <= TOL_TORCH, (f, _rel(got, ref))


def test_directional_derivatives_fd_and_tangent_linear(case):
    """16 seeded directions: <dJ/dc, d> against central differences of the
    library's forward window and against the torch tangent-linear (jvp)."""
    mesh, g, x0, c, ts = case["mesh"], case["g"], case["x0"], case["c"], case["ts"]
    _gpu_J(g, x0, c, ckpt=2)
    gc, _, _ = g.backward_window(1.0)
    rng = np.random.default_rng(2024)
    ct = _full(c, mesh.ny)
    worst_fd = worst_tl = 0.0
    for _ in range(16):
        d = rng.normal(0.0, 1e-3, c.shape)
        eps = 1e-3
        fd = (_gpu_J(g, x0, c + eps * d) - _gpu_J(g, x0, c - eps * d)) / (2 * eps)
        ad = float((gc * d).sum())
        worst_fd = max(worst_fd, abs(fd - ad) / abs(ad))
        _, tl = torch.autograd.functional.jvp(lambda cc: _torch_window(ts, x0, cc, W)[0], ct,
                                              _full(d, mesh.ny))
        worst_tl = max(worst_tl, abs(float(tl) - ad) / abs(ad))
    assert worst_fd <= TOL_FD, worst_fd
    assert worst_tl <= TOL_TORCH, worst_tl


def test_frozen_branch_record_is_the_free_run_and_replay_fd_is_exact(case):
    """TBL_BRANCH_RECORD reproduces the free run; finite differences through
    TBL_BRANCH_REPLAY (the recorded Peclet/sign decisions) follow exactly the
    map the adjoint differentiates."""
    from turbulentbl_gb300 import abi
    g, x0, c = case["g"], case["x0"], case["c"]
    J0 = _gpu_J(g, x0, c)
    s0 = g.download()
    g.upload(x0)
    g.set_wall_control(c)
    J1, _ = g.forward_window(W, PATCH[0], PATCH[1], 2, abi.TBL_BRANCH_RECORD)
    s1 = g.download()
    assert abs(J1 - J0) <= 1e-14 * abs(J0)
    for f in ("u", "v", "w", "p"):
        assert np.abs(s1[f] - s0[f]).max() <= 1e-13 * np.abs(s0[f]).max(), f
    gc, _, _ = g.backward_window(1.0)
    assert _rel(gc, case["gt"]) <= TOL_TORCH
    rng = np.random.default_rng(77)
    for _ in range(4):
        d = rng.normal(0.0, 1e-3, c.shape)
        eps = 1e-2
        Jp = Jm = None
        for sgn in (1, -1):
            g.upload(x0)
            g.set_wall_control(c + sgn * eps * d)
            J, _ = g.forward_window(W, PATCH[0], PATCH[1], 2, abi.TBL_BRANCH_REPLAY)
            if sgn > 0:
                Jp = J
            else:
                Jm = J
        fd = (Jp - Jm) / (2 * eps)
        ad = float((gc * d).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


class _WindowObjective(torch.autograd.Function):
    """torch.autograd wrapper over the C ABI: J(c) forward, dJ/dc backward."""

    @staticmethod
    def forward(ctx, c, g, x0, nsteps, ckpt):
        J = _gpu_J(g, x0, c.detach().numpy(), nsteps=nsteps, ckpt=ckpt)
        ctx.g = g
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        gc, _, _ = ctx.g.backward_window(float(gJ))
        return torch.tensor(gc), None, None, None, None


def test_autograd_function_wrapper(case):
    c = torch.tensor(case["c"], requires_grad=True)
    J = _WindowObjective.apply(c, case["g"], case["x0"], W, 2)
    (2.5 * J).backward()
    assert abs(float(J) - case["Jt"]) <= 1e-10 * abs(case["Jt"])
    assert _rel(c.grad.numpy(), 2.5 * case["gt"]) <= TOL_TORCH


def test_window_rejects_rescaling_step_and_mixed(case):
    from turbulentbl_gb300.runner import TblError
    from turbulentbl_gb300.synth import small_workload, make_state
    from turbulentbl_gb300.lib import TblGpu

    wl = small_workload(nx=14, nz_span=8, ny_wall=12)
    mesh, rp, st = make_state(wl, nproc=2)
    rp.cum = 3
    g = TblGpu(mesh, rp)
    g.upload(st)
    with pytest.raises(TblError):
        g.forward_window(5, PATCH[0], PATCH[1], 2)
    with pytest.raises(TblError):  # no window recorded
        g.backward_window(1.0)
