"""Seeded synthetic inputs standing in for the reference's missing input files.

The reference reads cnt, cnt2, 3D.tp and U_innerdns.dat
(dnstbl2/dnstbl.f90:147-159, :323-358), none of which ship with it.  This
module builds an equivalent restart state from a named workload:

  * mean profile U = Ue * min((x3/delta0)^(1/7), 1) (1/7 power law, delta0=1,
    Ue=1), also used as the fixed inflow mean Ume1 (the U_innerdns.dat role);
  * Re = Re_theta / theta0 with theta0 = 7/72 (momentum thickness of the
    1/7 law with delta0 = 1);
  * a divergence-free perturbation: the curl of a seeded, smoothed Gaussian
    vector potential damped to zero at the wall, scaled to a given rms;
  * recycling state (usum2, vsum2, wsum2, Wt, new, bltkns) from the spanwise
    means of that field through the same rescaling formulas the library uses
    (dnstbl2/dnstbl.f90:2173-2252) with lamda = 1;
  * Ufluc = U - usum2 (the restart file's fluctuation columns);
  * dt from a CFL number on the initial field.
"""
from dataclasses import dataclass

import numpy as np

from .mesh import make_mesh, RunParams, recycle_plane

THETA0 = 7.0 / 72.0


@dataclass
class Workload:
    name: str
    nx: int        # streamwise points
    ny_wall: int   # wall-normal points (reference nz)
    nz_span: int   # unique spanwise points (reference ny - 2)
    lx: float
    ly_wall: float
    lz_span: float
    beta: float
    re_theta: float
    seed: int
    cfl: float
    kmax: int
    errtol: float
    steps: int
    precision: int = 0

    @property
    def n3d(self):
        return (self.nx, self.nz_span + 2, self.ny_wall)

    @property
    def points(self):
        return self.nx * self.ny_wall * self.nz_span


# The seeded synthetic boxes (grid nx x ny(wall) x nz(span)).
WORKLOADS = {
    "box128_fp64": Workload("box128_fp64", 128, 64, 64, 20.0, 3.0, 4.0, 2.0, 300.0, 0, 0.3, 30, 1e-8, 200),
    "box512_fp64": Workload("box512_fp64", 512, 128, 128, 40.0, 3.0, 6.0, 2.2, 300.0, 0, 0.3, 40, 1e-10, 2000),
    "box512_mixed": Workload("box512_mixed", 512, 128, 128, 40.0, 3.0, 6.0, 2.2, 300.0, 0, 0.3, 40, 1e-10, 2000, 1),
    "box1024_mixed": Workload("box1024_mixed", 1024, 192, 256, 60.0, 3.5, 8.0, 2.4, 400.0, 7, 0.3, 30, 1e-10, 1000, 1),
    "box256_adjoint": Workload("box256_adjoint", 256, 96, 96, 20.0, 3.0, 4.0, 2.0, 300.0, 3, 0.3, 30, 1e-10, 50),
}


def _smooth_noise(rng, shape, width):
    """Gaussian random field smoothed with a Gaussian kernel of `width` cells (FFT)."""
    a = rng.standard_normal(shape)
    F = np.fft.rfftn(a)
    ks = [np.fft.fftfreq(n) for n in shape[:-1]] + [np.fft.rfftfreq(shape[-1])]
    K = np.meshgrid(*ks, indexing="ij")
    k2 = sum(k * k for k in K)
    F *= np.exp(-2.0 * (np.pi * width) ** 2 * k2)
    return np.fft.irfftn(F, s=shape, axes=tuple(range(len(shape))))


def _ddx(f, h, axis):
    """Central difference, one-sided 2nd order at the ends."""
    g = np.empty_like(f)
    sl = lambda a, b: tuple(slice(a, b) if d == axis else slice(None) for d in range(f.ndim))
    g[sl(1, -1)] = (f[sl(2, None)] - f[sl(0, -2)]) / (2 * h)
    g[sl(0, 1)] = (-3 * f[sl(0, 1)] + 4 * f[sl(1, 2)] - f[sl(2, 3)]) / (2 * h)
    g[sl(-1, None)] = (3 * f[sl(-1, None)] - 4 * f[sl(-2, -1)] + f[sl(-3, -2)]) / (2 * h)
    return g


def rescaling_state(usum2, x3, ue, irec, lamda=1.0, ksep0=0, bl_prev=None):
    """bltkns, Wt, new(k) (1-based), ksep from the means (dnstbl2/dnstbl.f90:2173-2252).

    A column whose mean never reaches 0.99 Ue keeps its previous thickness
    (bl_prev, zero when absent), as the reference's search loop does.
    """
    nx, nz = usum2.shape
    bl = np.zeros(nx) if bl_prev is None else np.array(bl_prev, dtype=np.float64)
    for i in range(nx):
        for k in range(nz):
            if usum2[i, k] >= 0.99 * ue:
                bl[i] = x3[k]
                break
    lam03 = bl[irec - 1] / bl[0]
    xb = x3[None, :] / bl[:, None]
    wt = 0.5 * (1 + (np.tanh((4.0 * (xb - 0.2)) / ((1 - 2.0 * 0.2) * xb + 0.2)) / np.tanh(4.0)))
    newk = np.full(nz, nz - 1, dtype=np.int32)
    eta = np.zeros(nz + 1)
    ksep = ksep0
    for k in range(1, nz):
        if wt[irec - 1, k - 1] <= 0.99:
            ksep = k
            eta[k] = lamda
        else:
            eta[k] = lam03
    zrecy = np.zeros(nz + 1)
    for k in range(1, nz):
        zrecy[k] = eta[k] * x3[k - 1]
    counter = 1
    for k in range(1, nz):
        if counter <= ksep and x3[k - 1] >= zrecy[counter]:
            newk[counter - 1] = k
            counter += 1
    counter = ksep + 1
    for k in range(ksep + 1, nz):
        if counter <= nz - 1 and x3[k - 1] >= zrecy[counter]:
            newk[counter - 1] = k
            counter += 1
    return bl, wt, newk, ksep


def spanwise_mean(f):
    """Mean over the unique spanwise rows j=2..ny-1 of an (nx,ny,nz) array -> (nx,nz)."""
    return f[:, 1:-1, :].mean(axis=1)


def cfl_dt(u, v, w, mesh, cfl):
    dz = np.diff(mesh.x3)
    dzl = np.minimum(np.r_[dz[0], dz], np.r_[dz, dz[-1]])
    s = (np.abs(u) / mesh.dx + np.abs(v) / mesh.dy + np.abs(w) / dzl[None, None, :])
    return cfl / float(s[1:-1, 1:-1, 1:-1].max())


def make_state(wl, nproc=8, rms=0.05, dt=None):
    """Build (mesh, RunParams, state dict) for a workload."""
    nx, ny, nz = wl.n3d
    mesh = make_mesh(nx, ny, nz, wl.lx, wl.lz_span, wl.ly_wall, wl.beta)
    ue = 1.0
    re = wl.re_theta / THETA0
    x3 = mesh.x3
    ume1 = ue * np.minimum(np.maximum(x3, 0.0) ** (1.0 / 7.0), 1.0)
    rng = np.random.default_rng(wl.seed)
    shape = (nx, ny - 2, nz)
    width = 2.0
    A = [_smooth_noise(rng, shape, width) for _ in range(3)]
    damp = (x3 / 1.0) ** 2 * np.exp(-((x3 / 1.0) ** 2))
    A = [a * damp[None, None, :] for a in A]
    # curl with periodic span (axis 1), streamwise axis 0, wall-normal via x3(xi)
    def dspan(f):
        return (np.roll(f, -1, axis=1) - np.roll(f, 1, axis=1)) / (2 * mesh.dy)
    def dwall(f):
        return _ddx(f, mesh.dxi, 2) / mesh.jac[None, None, :]
    def dstream(f):
        return _ddx(f, mesh.dx, 0)
    up = dspan(A[2]) - dwall(A[1])
    vp = dwall(A[0]) - dstream(A[2])
    wp = dstream(A[1]) - dspan(A[0])
    s = np.sqrt((up ** 2 + vp ** 2 + wp ** 2).mean() / 3.0)
    up, vp, wp = (rms * ue / s) * up, (rms * ue / s) * vp, (rms * ue / s) * wp
    u = np.zeros((nx, ny, nz))
    v = np.zeros((nx, ny, nz))
    w = np.zeros((nx, ny, nz))
    u[:, 1:-1, :] = ume1[None, None, :] + up
    v[:, 1:-1, :] = vp
    w[:, 1:-1, :] = wp
    for f in (u, v, w):
        f[:, :, 0] = 0.0                     # no-slip wall
        f[:, 0, :] = f[:, ny - 2, :]         # periodic ghosts
        f[:, ny - 1, :] = f[:, 1, :]
    u = np.asfortranarray(u)
    v = np.asfortranarray(v)
    w = np.asfortranarray(w)
    usum2 = np.asfortranarray(spanwise_mean(u))
    vsum2 = np.asfortranarray(spanwise_mean(v))
    wsum2 = np.asfortranarray(spanwise_mean(w))
    irec = recycle_plane(nx)
    bl, wt, newk, ksep = rescaling_state(usum2, x3, ue, irec)
    uf = np.zeros((nx, ny, nz), order="F")
    vf = np.zeros((nx, ny, nz), order="F")
    wf = np.zeros((nx, ny, nz), order="F")
    uf[:, 1:-1, :] = u[:, 1:-1, :] - usum2[:, None, :]
    vf[:, 1:-1, :] = v[:, 1:-1, :] - vsum2[:, None, :]
    wf[:, 1:-1, :] = w[:, 1:-1, :] - wsum2[:, None, :]
    if dt is None:
        dt = cfl_dt(u, v, w, mesh, wl.cfl)
    rp = RunParams(dt=dt, re=re, ue=ue, nproc=nproc, irec=irec, kmax=wl.kmax, errtol=wl.errtol,
                   precision=wl.precision, mixed_kmax=wl.kmax, mixed_outer_tol=wl.errtol)
    state = dict(u=u, v=v, w=w, p=np.zeros((nx, ny, nz), order="F"), pcorr=np.zeros((nx, ny, nz), order="F"),
                 usum2=usum2, vsum2=vsum2, wsum2=wsum2, wt=np.asfortranarray(wt), uf=uf, vf=vf, wf=wf,
                 newk=newk, ume1=ume1.copy(), bltkns=bl, lamda=1.0, time=0.0, nstep=0, cont=0, ksep=ksep)
    return mesh, rp, state


def small_workload(nx=24, nz_span=12, ny_wall=20, seed=0, kmax=20, errtol=1e-8):
    """A tiny box for tests (same recipe, reduced size)."""
    return Workload("tiny", nx, ny_wall, nz_span, 20.0 * nx / 128, 3.0, 4.0 * nz_span / 64, 2.0, 300.0,
                    seed, 0.3, kmax, errtol, 5)
