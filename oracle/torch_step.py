"""Differentiable FP64 restatement of one turbulentBL time step (tiny grids).

TEST INFRASTRUCTURE ONLY: the tangent-linear / adjoint reference the GPU
adjoint is checked against.  It restates the same step as np_oracle.py
(dnstbl2/dnstbl.f90:538-1469) in torch float64 with two changes that define
the map the adjoint differentiates:
  * the Gauss-Seidel and GMRES solves are replaced by exact dense solves of
    the same linear systems (the converged solution; the adjoint of a solve is
    the solve with the transposed operator);
  * the branch decisions (Peclet windows, upwind direction, |u|) are those of
    the current state, so the step is piecewise polynomial and torch autograd
    gives its exact Jacobian (jvp = tangent-linear, vjp = adjoint).
The control is the wall-normal velocity at the wall, w(:, j, k=1) = c(:, j)
(the reference's wall condition w = 0 at :1317-1319 with blowing/suction).
Statistics and the recycling parameters are held at the values supplied
(frozen within the window).
"""
import numpy as np
import torch

D = torch.float64


class TorchStep:
    def __init__(self, mesh, rp, recycle):
        """recycle: dict with usum2, vsum2, wsum2, wt (nx,nz), newk (nz, 1-based),
        ume1 (nz), lamda, slabs [(bn,en)] 0-based, fl_file (3 x (ny,nz)) and
        the step counter nstep0 of the first step."""
        self.m, self.rp = mesh, rp
        nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dx, self.dy, self.dxi = mesh.dx, mesh.dy, mesh.dxi
        J = mesh.jac
        self.jinv = torch.tensor(1.0 / J, dtype=D)
        self.jac2 = torch.tensor(mesh.jac2, dtype=D)
        self.x3 = torch.tensor(mesh.x3, dtype=D)
        a = 1.0 / (self.dxi * self.dxi * J * J)
        b = mesh.jac2 / (2.0 * self.dxi * J * J * J)
        self.Ab, self.At = a + b, a - b
        self.Ap = -2.0 * ((1.0 / self.dx ** 2) + (1.0 / self.dy ** 2) + a)
        self.aw, self.as_ = 1.0 / self.dx ** 2, 1.0 / self.dy ** 2
        j = np.arange(ny)
        self.jm1 = torch.tensor(np.where(j == 1, ny - 2, j - 1))
        self.jp1 = torch.tensor(np.where(j == ny - 2, 1, j + 1))
        self.jm2 = torch.tensor(np.where(j == 2, ny - 2, np.where(j == 1, ny - 3, j - 2)))
        self.jp2 = torch.tensor(np.where(j == ny - 3, 1, np.where(j == ny - 2, 2, j + 2)))
        self.rc = recycle
        self._build_systems()

    # ---------------------------------------------------------- linear systems
    def _build_systems(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        I = [(i, j, k) for k in range(1, nz - 1) for j in range(1, ny - 1) for i in range(1, nx - 1)]
        self.int_idx = torch.tensor([i + nx * (j + ny * k) for (i, j, k) in I])
        pos = {q: n for n, q in enumerate(I)}
        nI = len(I)
        t = -self.rp.dt / self.rp.re
        L = np.zeros((nI, nI))
        Ab_ = np.zeros((nI, nx * ny * nz))  # coupling of the GS system to boundary values
        A = np.zeros((nI, nI))
        for n, (i, j, k) in enumerate(I):
            nb = [((i - 1, j, k), self.aw), ((i + 1, j, k), self.aw),
                  ((i, int(self.jm1[j]), k), self.as_), ((i, int(self.jp1[j]), k), self.as_),
                  ((i, j, k - 1), self.Ab[k]), ((i, j, k + 1), self.At[k])]
            L[n, n] = self.Ap[k]
            A[n, n] = 1.0 + t * self.Ap[k]
            for q, cf in nb:
                if q in pos:
                    L[n, pos[q]] += cf
                    A[n, pos[q]] += t * cf
                else:
                    Ab_[n, q[0] + nx * (q[1] + ny * q[2])] += t * cf
        self.L = torch.tensor(L, dtype=D)
        self.A = torch.tensor(A, dtype=D)
        self.AB = torch.tensor(Ab_, dtype=D)

    def flat(self, X):
        return X.permute(2, 1, 0).reshape(-1)  # i fastest

    def unflat(self, x):
        return x.reshape(self.nz, self.ny, self.nx).permute(2, 1, 0)

    # --------------------------------------------------------------- the step
    def step(self, U, P, c, nstep):
        """U: list of 3 (nx,ny,nz) tensors, P: (nx,ny,nz), c: (nx,ny) wall-normal
        wall velocity.  Returns the new (U, P)."""
        nx, ny, nz, dt, re = self.nx, self.ny, self.nz, self.rp.dt, self.rp.re
        U = [u.clone() for u in U]
        P = P.clone()
        uold1 = U[0][0].clone()
        rc = self.rc
        # a1 inflow (:557-618)
        if nstep > self.rp.recycle_after:
            ir = self.rp.irec - 1
            for k in range(1, nz - 1):
                bn, en = next(s for s in rc["slabs"] if s[0] <= k <= s[1])
                if rc["usum2"][ir, k] < 0.99 * self.rp.ue:
                    nk = int(rc["newk"][k]) - 1
                    wt = float(rc["wt"][nx - 2, k])
                    means = (float(rc["ume1"][k]), float(rc["vsum2"][ir, nk]), float(rc["wsum2"][ir, nk]))
                    mean2 = (rc["usum2"], rc["vsum2"], rc["wsum2"])
                    for cc in range(3):
                        if bn <= nk <= en:  # live plane: U(irec) - mean, from the current state
                            fl = U[cc][ir, 1:ny - 1, nk] - float(mean2[cc][ir, nk])
                        else:
                            fl = torch.tensor(rc["fl_file"][cc][1:ny - 1, nk], dtype=D)
                        f = rc["lamda"] * fl
                        U[cc] = U[cc].index_put((torch.tensor([0]), torch.arange(1, ny - 1), torch.tensor([k])),
                                                ((means[cc] + f) * (1.0 - wt) + (means[cc] + f) * wt))
                else:
                    for cc, s2 in enumerate((rc["usum2"], rc["vsum2"], rc["wsum2"])):
                        U[cc] = U[cc].index_put((torch.tensor([0]), torch.arange(1, ny - 1), torch.tensor([k])),
                                                torch.full((ny - 2,), float(s2[ir, k]), dtype=D))
        self.last_u1 = [u.detach().clone() for u in U]  # velocities after the inflow
        # a2, a3 convection and Q (:621-768)
        Q = self._conv_q(U, P)
        # a4 implicit diffusion: exact solve of (1 - dt/Re L7) U* = Q
        Us = []
        for cc in range(3):
            rhs = self.flat(Q[cc])[self.int_idx] - self.AB @ self.flat(U[cc])
            xi = torch.linalg.solve(self.A, rhs)
            f = self.flat(U[cc]).clone()
            f = f.index_put((self.int_idx,), xi)
            Us.append(self.unflat(f))
        U = Us
        # a5 Q8 (:905-935)
        Q8 = self._div(U)
        # a6 exact Poisson solve, p' = 0 on the faces
        pci = torch.linalg.solve(self.L, self.flat(Q8)[self.int_idx])
        PC = self.unflat(torch.zeros(nx * ny * nz, dtype=D).index_put((self.int_idx,), pci))
        # a7, a8 (:1245-1469)
        U, P = self._project_bcs(U, P, PC, uold1, c)
        return U, P

    def _conv_q(self, U, P):
        nx, ny, nz, re, dt = self.nx, self.ny, self.nz, self.rp.re, self.rp.dt
        ii, jj, kk = torch.meshgrid(torch.arange(1, nx - 1), torch.arange(1, ny - 1), torch.arange(1, nz - 1),
                                    indexing="ij")
        u, v, w = U
        uc, vc, wc = u[ii, jj, kk], v[ii, jj, kk], w[ii, jj, kk]
        sg = lambda x: torch.where(torch.ceil(x.detach()) >= 0, 1.0, -1.0).to(D)
        dz = self.x3[kk + 1] - self.x3[kk]
        c12 = 1.0 / 12.0
        conv = []
        for F in U:
            f0 = F[ii, jj, kk]
            fm1, fp1 = F[ii - 1, jj, kk], F[ii + 1, jj, kk]
            fm2, fp2 = F[torch.clamp(ii - 2, min=0), jj, kk], F[torch.clamp(ii + 2, max=nx - 1), jj, kk]
            Pe = sg(uc) * re * uc.detach() * self.dx
            near = (ii <= 1) | (ii >= nx - 2)
            dn = uc * (fp1 - fm1) / (2.0 * self.dx)
            t1 = torch.abs(uc) * (fp2 - 4 * fp1 + 6 * f0 - 4 * fm1 + fm2) * (0.25 / self.dx)
            t2 = uc * (-fp2 + 8 * fp1 - 8 * fm1 + fm2) * (c12 / self.dx)
            cen = uc * ((fm2 - 8 * fm1 + 8 * fp1 - fp2) * (c12 / self.dx))
            d1 = torch.where(near, dn, torch.where((Pe > 2) & (Pe < 50), t1 + t2, cen))
            gm1, gp1 = F[ii, self.jm1[jj], kk], F[ii, self.jp1[jj], kk]
            gm2, gp2 = F[ii, self.jm2[jj], kk], F[ii, self.jp2[jj], kk]
            Pe = sg(vc) * re * vc.detach() * self.dy
            near = (jj == 1) | (jj == ny - 2)
            up = torch.clamp(vc, min=0.0) * ((f0 - gm1) / self.dy) + torch.clamp(vc, max=0.0) * ((gp1 - f0) / self.dy)
            t1 = torch.abs(vc) * (gp2 - 4 * gp1 + 6 * f0 - 4 * gm1 + gm2) * (0.25 / self.dy)
            t2 = vc * (-gp2 + 8 * gp1 - 8 * gm1 + gm2) * (c12 / self.dy)
            cen = vc * ((gm2 - 8 * gm1 + 8 * gp1 - gp2) * (c12 / self.dy))
            d2 = torch.where(near, up, torch.where((Pe > 2) & (Pe < 50), t1 + t2, cen))
            hm1, hp1 = F[ii, jj, kk - 1], F[ii, jj, kk + 1]
            hm2, hp2 = F[ii, jj, torch.clamp(kk - 2, min=0)], F[ii, jj, torch.clamp(kk + 2, max=nz - 1)]
            Pe = sg(wc) * re * wc.detach() * dz
            near = (kk <= 1) | (kk >= nz - 2)
            dn = wc * (hp1 - hm1) * (0.5 / self.dxi)
            t1 = torch.abs(wc) * (hp2 - 4 * hp1 + 6 * f0 - 4 * hm1 + hm2) * (0.25 / self.dxi)
            t2 = wc * (-hp2 + 8 * hp1 - 8 * hm1 + hm2) * (c12 / self.dxi)
            cen = wc * ((hm2 - 8 * hm1 + 8 * hp1 - hp2) * (c12 / self.dxi))
            d3 = torch.where(near, dn, torch.where((Pe > 2) & (Pe < 5), t1 + t2, cen))
            conv.append(d1 + d2 + d3 * self.jinv[kk])
        g1 = 0.5 * (P[ii + 1, jj, kk] - P[ii - 1, jj, kk]) / self.dx
        g2 = 0.5 * (P[ii, self.jp1[jj], kk] - P[ii, self.jm1[jj], kk]) / self.dy
        g3 = 0.5 * (P[ii, jj, kk + 1] - P[ii, jj, kk - 1]) * (self.jinv[kk] / self.dxi)
        Q = []
        for cc, gc in enumerate((g1, g2, g3)):
            q = torch.zeros_like(U[cc])
            Q.append(q.index_put((ii, jj, kk), U[cc][ii, jj, kk] - dt * conv[cc] - dt * gc))
        return Q

    def _div(self, U):
        nx, ny, nz = self.nx, self.ny, self.nz
        u, v, w = U
        ii, jj, kk = torch.meshgrid(torch.arange(1, nx - 1), torch.arange(1, ny - 1), torch.arange(1, nz - 1),
                                    indexing="ij")
        d1 = (((u[ii + 1, jj, kk] + u[ii, jj, kk]) * 0.5) - ((u[ii, jj, kk] + u[ii - 1, jj, kk]) * 0.5)) / self.dx
        d2 = (((v[ii, self.jp1[jj], kk] + v[ii, jj, kk]) * 0.5) - ((v[ii, jj, kk] + v[ii, self.jm1[jj], kk]) * 0.5)) / self.dy
        d3 = 2.0 * (((w[ii, jj, kk + 1] + w[ii, jj, kk]) * 0.5) - ((w[ii, jj, kk] + w[ii, jj, kk - 1]) * 0.5)) / \
            (self.x3[kk + 1] - self.x3[kk - 1])
        return torch.zeros_like(u).index_put((ii, jj, kk), (d1 + d2 + d3) / self.rp.dt)

    def _project_bcs(self, U, P, PC, uold1, c):
        nx, ny, nz, dt, re = self.nx, self.ny, self.nz, self.rp.dt, self.rp.re
        PC = PC.clone()
        J = slice(1, ny - 1)
        PC[:, J, 0] = (4.0 * PC[:, J, 1] - PC[:, J, 2]) / 3.0
        PC[:, J, nz - 1] = (5.0 * PC[:, J, nz - 2] + (-4.0 * PC[:, J, nz - 3] + PC[:, J, nz - 4])) / 2.0
        PC[:, 0, :] = PC[:, ny - 2, :]
        PC[:, ny - 1, :] = PC[:, 1, :]
        PC[0, J, :] = (4.0 * PC[1, J, :] - PC[2, J, :]) / 3.0
        PC[nx - 1, J, :] = (5.0 * PC[nx - 2, J, :] + (-4.0 * PC[nx - 3, J, :] + PC[nx - 4, J, :])) / 2.0
        ii, jj, kk = torch.meshgrid(torch.arange(1, nx - 1), torch.arange(1, ny - 1), torch.arange(1, nz - 1),
                                    indexing="ij")
        P = P.index_put((ii, jj, kk), P[ii, jj, kk] + PC[ii, jj, kk])
        g = (0.5 * (PC[ii + 1, jj, kk] - PC[ii - 1, jj, kk]) / self.dx,
             0.5 * (PC[ii, self.jp1[jj], kk] - PC[ii, self.jm1[jj], kk]) / self.dy,
             0.5 * (PC[ii, jj, kk + 1] - PC[ii, jj, kk - 1]) * (self.jinv[kk] / self.dxi))
        U = [U[cc].index_put((ii, jj, kk), U[cc][ii, jj, kk] - dt * g[cc]) for cc in range(3)]
        U = [u.clone() for u in U]
        for cc in range(3):
            U[cc][:, J, 0] = c[:, J] if cc == 2 else 0.0
            U[cc][:, J, nz - 1] = (4.0 * U[cc][:, J, nz - 2] - U[cc][:, J, nz - 3]) / 3.0
        for cc in range(3):
            U[cc][nx - 1, J, :] = (4.0 * U[cc][nx - 2, J, :] - U[cc][nx - 3, J, :]) / 3.0
        u, v, w = U
        P = P.clone()
        x3 = self.x3
        df1, df2 = x3[1] - x3[0], x3[2] - x3[0]
        I2 = slice(1, nx - 1)
        wi = lambda a, b, k: w[a, b, k]
        fder = (w[I2, J, 1] - w[I2, J, 0]) / df1
        d3 = w[I2, J, 0] * fder
        g1 = (w[0:nx - 2, J, 0] + w[2:nx, J, 0] - 2 * w[I2, J, 0]) / (self.dx * self.dx)
        g2 = (w[I2, 0:ny - 2, 0] + w[I2, 2:ny, 0] - 2 * w[I2, J, 0]) / (self.dy * self.dy)
        g3 = (2 * df1 * w[I2, J, 2] - 2 * df2 * w[I2, J, 1] + 2 * (df2 - df1) * w[I2, J, 0]) / \
            (df1 * df2 ** 2 - df2 * df1 ** 2)
        P[I2, J, 0] = P[I2, J, 1] - (-d3 + (g1 + g2 + g3) / re) * df1
        fder = (11.0 * w[I2, J, nz - 1] - 18.0 * w[I2, J, nz - 2] + 9.0 * w[I2, J, nz - 3] - 2.0 * w[I2, J, nz - 4]) / \
            (6.0 * self.dxi)
        P[I2, J, nz - 1] = fder * self.jinv[nz - 1] / re
        K = slice(1, nz - 1)
        P[nx - 1, J, K] = (3.0 * u[nx - 1, J, K] - 4.0 * u[nx - 2, J, K] + u[nx - 3, J, K]) / (2.0 * self.dx * re)
        u0 = u[0, J, K]
        Jk = self.jinv[1:nz - 1][None, :]
        d1 = u0 * ((u[1, J, K] - u0) / self.dx)
        d2 = v[0, J, K] * ((u[0, 2:ny, K] - u[0, 0:ny - 2, K]) / (2.0 * self.dy))
        d3 = w[0, J, K] * ((u[0, J, 2:nz] - u[0, J, 0:nz - 2]) / (2.0 * self.dxi))
        g1 = (u0 + u[2, J, K] - 2 * u[1, J, K]) / (self.dx * self.dx)
        g2 = (u[0, 2:ny, K] + u[0, 0:ny - 2, K] - 2 * u0) / (self.dy * self.dy)
        fder = (u[0, J, 2:nz] - u[0, J, 0:nz - 2]) / (2.0 * self.dxi)
        g3 = (-2 * u0 + u[0, J, 2:nz] + u[0, J, 0:nz - 2]) / (self.dxi * self.dxi)
        # first and last interior planes use one-sided forms (:1444-1450)
        fder = fder.clone()
        g3 = g3.clone()
        fder[:, 0] = (u[0, J, 2] - u[0, J, 1]) / self.dxi
        g3[:, 0] = (u[0, J, 3] - 2.0 * u[0, J, 2] + u[0, J, 1]) / (self.dxi * self.dxi)
        fder[:, -1] = (u[0, J, nz - 2] - u[0, J, nz - 3]) / self.dxi
        g3[:, -1] = (u[0, J, nz - 4] - 2.0 * u[0, J, nz - 3] + u[0, J, nz - 2]) / (self.dxi * self.dxi)
        g3 = g3 * (Jk * Jk) - (self.jac2[1:nz - 1][None, :] * fder) * (Jk * Jk * Jk)
        fder2 = (u0 - uold1[J, K]) / dt
        P[0, J, K] = ((2 * self.dx * ((fder2 + d1 + d2 + d3 * Jk) - ((g1 + g2 + g3) / re))) - 0.0 - P[2, J, K] +
                      4 * P[1, J, K]) / 3.0
        out = []
        for F in (u, v, w, P):
            F = F.clone()
            F[:, 0, :] = F[:, ny - 2, :]
            F[:, ny - 1, :] = F[:, 1, :]
            out.append(F)
        return out[:3], out[3]

    # ------------------------------------------------------------- objective
    def patch_columns(self, x0, x1):
        x = self.m.x1
        return [i for i in range(1, self.nx - 1) if x0 <= x[i] <= x1]

    def wall_shear(self, U, cols):
        """Mean wall shear over the patch columns (:1636-1660): (dw/dx + du/dz)/Re
        at the wall, averaged over the patch and the span."""
        u, w = U[0], U[2]
        nx, ny = self.nx, self.ny
        x3 = self.m.x3
        df1, df2 = x3[1] - x3[0], x3[2] - x3[0]
        J = slice(1, ny - 1)
        tot = 0.0
        for i in cols:
            if i <= 2 or i >= nx - 3:
                mfb1 = (w[i + 1, J, 0] - w[i - 1, J, 0]) / (2.0 * self.dx)
            else:
                mfb1 = (-w[i - 3, J, 0] + 9.0 * w[i - 2, J, 0] - 45.0 * w[i - 1, J, 0] + 45.0 * w[i + 1, J, 0] -
                        9.0 * w[i + 2, J, 0] + w[i + 3, J, 0]) / (60.0 * self.dx)
            mfb2 = ((u[i, J, 2] - u[i, J, 0]) * df1 ** 2 + (u[i, J, 0] - u[i, J, 1]) * df2 ** 2) / \
                (df2 * df1 ** 2 - df2 ** 2 * df1)
            tot = tot + ((mfb1 + mfb2) / self.rp.re).sum()
        return tot / (len(cols) * (ny - 2))
