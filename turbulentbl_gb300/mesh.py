"""Mesh and run-parameter setup (host side, computed once).

Restates dnstbl2/dnstbl.f90:392-426 (uniform x1, x2, tanh-stretched x3 and its
Jacobians) and the parameter literals of :20-140.  The reference hard-codes
Lx=12, Lz_span=2, Ly_wall=3.4 and delta=1.95; here they are arguments.  The
``reference_literals`` switch reproduces the reference exactly, including its
REAL(4) literals (3.4 and 1.7 inside the tanh/cosh arguments, :423-425, and
w = 1.835, :140) promoted to double.
"""
from dataclasses import dataclass, field

import numpy as np

F32 = lambda v: float(np.float32(v))  # a Fortran REAL(4) literal promoted to DOUBLE

OMEGA_REF = F32(1.835)  # dnstbl2/dnstbl.f90:140  w = 1.835 (default REAL)


@dataclass
class Mesh:
    nx: int
    ny: int
    nz: int
    x1: np.ndarray
    x2: np.ndarray
    x3: np.ndarray
    jac: np.ndarray   # dx3/dxi, NOT inverted
    jac2: np.ndarray  # d2x3/dxi2
    dx: float
    dy: float
    dxi: float
    lx: float = 0.0
    lz_span: float = 0.0
    ly_wall: float = 0.0
    beta: float = 0.0


def make_mesh(nx, ny, nz, lx, lz_span, ly_wall, beta, reference_literals=False):
    """Build the mesh.

    nx, ny, nz are the reference's n3d (ny includes the two periodic ghost
    rows).  The spanwise period is (ny-2)*dy; x2(ny) = lz_span*(ny-1)/(ny-2)
    makes it equal lz_span.  ``reference_literals`` reproduces
    dnstbl2/dnstbl.f90:392-426 with its literal domain (lx=12, x2(ny)=2,
    ly_wall=3.4, beta=delta=1.95) and REAL(4) literals.
    """
    x1 = np.zeros(nx)
    x2 = np.zeros(ny)
    xi = np.zeros(nz)
    if reference_literals:
        lx_, x2n, L, d = 12.0, 2.0, 3.4, 1.95
    else:
        lx_, x2n, L, d = float(lx), float(lz_span) * (ny - 1) / (ny - 2), float(ly_wall), float(beta)
    x1[nx - 1] = lx_
    x2[ny - 1] = x2n
    dx = x1[nx - 1] / float(nx - 1)
    dy = x2[ny - 1] / float(ny - 1)
    dxi = L / float(nz - 1)
    # accumulated coordinates (:405-415)
    for i in range(nx - 1):
        x1[i + 1] = x1[i] + dx
    for j in range(ny - 1):
        x2[j + 1] = x2[j] + dy
    for k in range(nz - 1):
        xi[k + 1] = xi[k] + dxi
    x3 = np.zeros(nz)
    jac = np.zeros(nz)
    jac2 = np.zeros(nz)
    if reference_literals:
        s34 = F32(3.4)
        s17 = F32(1.7)
        for k in range(nz):
            a = d * 0.5 * (xi[k] - s34)
            x3[k] = 3.4 + 3.4 * np.tanh(a) / (np.tanh(1.7 * d))
            c2 = np.cosh(0.5 * d * (xi[k] - s34)) ** 2
            jac[k] = 1.7 * d / (np.tanh(s17 * d) * c2)
            jac2[k] = -1.7 * d ** 2 * np.tanh(0.5 * d * (xi[k] - s34)) / (np.tanh(s17 * d) * c2)
    else:
        th = np.tanh(0.5 * d * L)
        for k in range(nz):
            a = 0.5 * d * (xi[k] - L)
            x3[k] = L + L * np.tanh(a) / th
            c2 = np.cosh(a) ** 2
            jac[k] = 0.5 * L * d / (th * c2)
            jac2[k] = -0.5 * L * d * d * np.tanh(a) / (th * c2)
    return Mesh(nx, ny, nz, x1, x2, x3, jac, jac2, dx, dy, dxi, lx_, x2n * (ny - 2) / (ny - 1), L, d)


@dataclass
class RunParams:
    """Everything tbl_config carries besides the grid."""
    dt: float = 1.0e-4
    re: float = 150.92
    ue: float = 19.798
    nproc: int = 8
    irec: int = 68
    cum: int = 5
    istat: int = 1
    recycle_after: int = 5
    kmax: int = 50
    mmax: int = 1000
    omega: float = OMEGA_REF
    errtol: float = 1.0e-5
    errorstop: float = 1.0e-6
    precision: int = 0
    flags: int = 0
    mixed_kmax: int = 40
    mixed_max_outer: int = 20
    mixed_inner_tol: float = 1.0e-5
    mixed_outer_tol: float = 1.0e-10
    mixed_true_tol: float = 1.0e-8   # divergence target of the mixed solve (true relative PPE residual)
    variant: int = 0                 # TBL_VARIANT_*: dnstbl2 (0), originalTBL (1), dnssetbl (2)

    def use_variant(self, variant):
        """Switch to one of the reference's programs with its own cum and
        recycling start: originalTBL cum = 1000, recycling after step 1000
        (fnldnstbl.f90:115, :567); dnssetbl freqTimAvg = 500 for both
        (dnssetbl.f90:20, :264, :986)."""
        self.variant = variant
        if variant == 1:
            self.cum, self.recycle_after = 1000, 1000
        elif variant == 2:
            self.cum, self.recycle_after = 500, 500
        else:
            self.cum, self.recycle_after = 5, 5
        return self


def recycle_plane(nx):
    """Recycling plane at x = 0.8 Lx, 1-based: nint(0.8 (nx-1)) + 1."""
    return int(np.floor(0.8 * (nx - 1) + 0.5)) + 1


def make_config(mesh, rp):
    from .abi import TblConfig
    c = TblConfig()
    c.nx, c.ny, c.nz = mesh.nx, mesh.ny, mesh.nz
    c.nproc = rp.nproc
    c.irec = rp.irec
    c.cum = rp.cum
    c.istat = rp.istat
    c.recycle_after = rp.recycle_after
    c.kmax = rp.kmax
    c.mmax = rp.mmax
    c.precision = rp.precision
    c.flags = rp.flags
    c.mixed_kmax = rp.mixed_kmax
    c.mixed_max_outer = rp.mixed_max_outer
    c.dt = rp.dt
    c.re = rp.re
    c.ue = rp.ue
    c.dx, c.dy, c.dxi = mesh.dx, mesh.dy, mesh.dxi
    c.omega = rp.omega
    c.errtol = rp.errtol
    c.errorstop = rp.errorstop
    c.mixed_inner_tol = rp.mixed_inner_tol
    c.mixed_outer_tol = rp.mixed_outer_tol
    c.mixed_true_tol = rp.mixed_true_tol
    c.variant = rp.variant
    return c


def make_mesh_struct(mesh):
    """TblMesh pointing into the Mesh arrays (keep ``mesh`` alive)."""
    from .abi import TblMesh, dptr
    m = TblMesh()
    for name in ("x1", "x2", "x3", "jac", "jac2"):
        arr = getattr(mesh, name)
        assert arr.flags.c_contiguous and arr.dtype == np.float64
        setattr(m, name, dptr(arr))
    return m
