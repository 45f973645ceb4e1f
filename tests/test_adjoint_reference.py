"""Pins the adjoint reference (oracle/torch_step.py) on the CPU.

1. Its forward step (exact solves) agrees with the C++ oracle run to tight
   solver tolerances, with the reference's wall condition w = 0.
2. Its autograd derivatives agree with central differences of itself, and
   the tangent-linear (jvp) and adjoint (vjp) satisfy <J'd, l> = <d, J'^T l>.
"""
import numpy as np
import pytest
import torch

from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner
from oracle.torch_step import TorchStep


def _setup():
    wl = small_workload(nx=14, nz_span=8, ny_wall=12, kmax=30, errtol=1e-14)
    mesh, rp, st = make_state(wl, nproc=2)
    rp.errorstop = 1e-15
    rp.cum = 10 ** 6
    rp.mmax = 3000
    st["nstep"] = 10
    P = rp.nproc
    loc = (mesh.nz - 1) // P
    slabs = [(1 + r * loc, (1 + r * loc + loc - 1) if r < P - 1 else mesh.nz - 2) for r in range(P)]
    ir = rp.irec - 1
    rc = dict(usum2=st["usum2"], vsum2=st["vsum2"], wsum2=st["wsum2"], wt=st["wt"], newk=st["newk"],
              ume1=st["ume1"], lamda=st["lamda"], slabs=slabs, fl_file=[st[f][ir] for f in ("uf", "vf", "wf")])
    return mesh, rp, st, TorchStep(mesh, rp, rc)


def test_torch_step_matches_cpp_oracle():
    mesh, rp, st, ts = _setup()
    o = OracleRunner(mesh, rp)
    o.upload(st)
    U = [torch.tensor(st[f]) for f in ("u", "v", "w")]
    P = torch.tensor(st["p"])
    c = torch.zeros(mesh.nx, mesh.ny, dtype=torch.float64)
    for s in range(3):
        U, P = ts.step(U, P, c, st["nstep"] + 1 + s)
        o.step(1, check=False)  # GS at errorstop 1e-15 may stop at mmax, ~1e-15 from converged
        d = o.download()
        for f, x in zip(("u", "v", "w", "p"), list(U) + [P]):
            x = x.numpy()
            err = np.linalg.norm(x - d[f]) / np.linalg.norm(d[f])
            assert err < (1e-12 if f != "p" else 1e-11), (s, f, err)


def _J(ts, st, c, nsteps=2):
    U = [torch.tensor(st[f]) for f in ("u", "v", "w")]
    P = torch.tensor(st["p"])
    cols = ts.patch_columns(0.3, 1.5)
    J = 0.0
    for s in range(nsteps):
        U, P = ts.step(U, P, c, st["nstep"] + 1 + s)
        J = J + ts.wall_shear(U, cols)
    return J / nsteps


def test_torch_adjoint_fd_and_dot_product():
    mesh, rp, st, ts = _setup()
    rng = np.random.default_rng(5)
    c0 = np.zeros((mesh.nx, mesh.ny))
    c0[:, 1:-1] = rng.normal(0, 1e-3, (mesh.nx, mesh.ny - 2))
    c = torch.tensor(c0, requires_grad=True)
    J = _J(ts, st, c)
    (g,) = torch.autograd.grad(J, c)
    for q in range(3):
        d = np.zeros_like(c0)
        d[:, 1:-1] = rng.normal(0, 1e-3, (mesh.nx, mesh.ny - 2))
        dt = torch.tensor(d)
        eps = 1e-2
        with torch.no_grad():
            fd = (float(_J(ts, st, torch.tensor(c0) + eps * dt)) - float(_J(ts, st, torch.tensor(c0) - eps * dt))) / (2 * eps)
        ad = float((g * dt).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (q, fd, ad)
        _, tl = torch.autograd.functional.jvp(lambda cc: _J(ts, st, cc), torch.tensor(c0), dt)
        assert abs(float(tl) - ad) <= 1e-12 * abs(ad)
