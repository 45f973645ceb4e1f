"""Independent NumPy restatement of one turbulentBL time step (tiny grids).

TEST INFRASTRUCTURE ONLY: cross-checks the C++ oracle (tbl_oracle.cpp) so
that the restatement does not rest on a single reading of the reference.  It
is written separately from the C++ code (array slicing for the stencils,
explicit loops only where the reference is sequential: GS, SSOR, the
rescaling scans).  Follows theparvezahmad/turbulentBL dnstbl2/dnstbl.f90; the
line ranges are cited per function.  Arrays are indexed [i, j, k] 0-based.
``rp.variant`` switches to the differences of originalTBL/fnldnstbl.f90 (1)
and dnssetbl/dnssetbl.f90 (2), cited where applied.
Parity status: unpinned against the reference binary (no Fortran compiler).
"""
import numpy as np


class NpOracle:
    def __init__(self, mesh, rp):
        self.m = mesh
        self.rp = rp
        nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
        self.nx, self.ny, self.nz = nx, ny, nz
        P = rp.nproc
        self.var = getattr(rp, "variant", 0)
        self.slabs = []
        if self.var == 2:
            # dnssetbl.f90:78-92: sizes nz//P, the last nz % P ranks one more,
            # from the first plane; the wall and top planes are then dropped
            sizes = [nz // P + (1 if r >= P - nz % P else 0) for r in range(P)]
            starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
            for r in range(P):
                self.slabs.append((int(starts[r]) + (1 if r == 0 else 0),
                                   int(starts[r] + sizes[r] - 1) - (1 if r == P - 1 else 0)))
        else:
            loc = (nz - 1) // P
            # 0-based slabs [bn, en] (dnstbl2/dnstbl.f90:469-475)
            for r in range(P):
                bn = 1 + r * loc
                en = bn + loc - 1 if r < P - 1 else nz - 2
                self.slabs.append((bn, en))
        self.dx, self.dy, self.dxi = mesh.dx, mesh.dy, mesh.dxi
        J = mesh.jac
        self.jinv = 1.0 / J
        a = 1.0 / (self.dxi * self.dxi * J * J)
        b = mesh.jac2 / (2.0 * self.dxi * J * J * J)
        self.Ab = a + b
        self.At = a - b
        self.Ap = -2.0 * ((1.0 / (self.dx * self.dx)) + (1.0 / (self.dy * self.dy)) + a)
        self.Aw = 1.0 / (self.dx * self.dx)
        self.As = 1.0 / (self.dy * self.dy)
        j = np.arange(ny)
        self.jm1 = np.where(j == 1, ny - 2, j - 1)
        self.jp1 = np.where(j == ny - 2, 1, j + 1)
        self.jm2 = np.where(j == 2, ny - 2, self.jm1 - 1)
        self.jp2 = np.where(j == ny - 3, 1, self.jp1 + 1)

    def upload(self, st):
        self.U = [np.array(st[c], dtype=np.float64) for c in ("u", "v", "w")]
        self.P = np.array(st["p"], dtype=np.float64)
        self.PC = np.array(st["pcorr"], dtype=np.float64) if st.get("pcorr") is not None else np.zeros_like(self.P)
        self.usum2 = np.array(st["usum2"]); self.vsum2 = np.array(st["vsum2"]); self.wsum2 = np.array(st["wsum2"])
        self.Wt = np.array(st["wt"])
        self.newk = np.array(st["newk"], dtype=np.int64)
        self.ume1 = np.array(st["ume1"])
        self.bltkns = np.array(st["bltkns"]) if st.get("bltkns") is not None else np.zeros(self.nx)
        ir = self.rp.irec - 1
        uf = [st.get(c) for c in ("uf", "vf", "wf")]
        means = [self.usum2, self.vsum2, self.wsum2]
        self.fl_file = [np.array(uf[c][ir]) if uf[c] is not None else self.U[c][ir] - means[c][ir][None, :]
                        for c in range(3)]
        self.fl_live = [f.copy() for f in self.fl_file]
        if self.var == 2:  # computed on each rank's own slab only (dnssetbl.f90:141-149)
            self.fl_file = [np.zeros_like(f) for f in self.fl_file]
        self.cnt2 = st.get("cnt2", 0)
        self.lamda = st.get("lamda", 1.0)
        self.nstep = st.get("nstep", 0)
        self.cont = st.get("cont", 0)
        self.ksep = st.get("ksep", 0)
        nxz = (self.nx, self.nz)
        self.sums = {k: np.zeros(nxz) for k in ("u", "v", "w", "uu", "vv", "ww", "uv", "uw", "vw")}

    def slab_of(self, k):
        for r, (bn, en) in enumerate(self.slabs):
            if bn <= k <= en:
                return r
        return -1

    # a1: inflow (:557-618)
    def inflow(self):
        ir, ue, nx, ny = self.rp.irec - 1, self.rp.ue, self.nx, self.ny
        for k in range(1, self.nz - 1):
            r = self.slab_of(k)
            bn, en = self.slabs[r]
            if self.usum2[ir, k] < 0.99 * ue:
                nk = self.newk[k] - 1
                src = self.fl_live if bn <= nk <= en else self.fl_file
                wt = self.Wt[0 if self.var == 2 else nx - 2, k]  # dnssetbl: Wt(1,k) (dnssetbl.f90:291)
                um = self.ume1[k]
                if self.var:  # eps ramp (fnldnstbl.f90:561-587, dnssetbl.f90:259-274)
                    eps = min((self.cnt2 if self.var == 1 else self.nstep) * 5.0e-5, 1.0)
                    um = eps * self.usum2[ir, nk] + (1 - eps) * self.ume1[k]
                vm = self.lamda * self.vsum2[ir, nk] if self.var == 2 else self.vsum2[ir, nk]
                means = (um, vm, self.wsum2[ir, nk])
                for c in range(3):
                    f = self.lamda * src[c][1:ny - 1, nk]
                    self.U[c][0, 1:ny - 1, k] = (means[c] + f) * (1.0 - wt) + (means[c] + f) * wt
            else:
                for c, s in enumerate((self.usum2, self.vsum2, self.wsum2)):
                    self.U[c][0, 1:ny - 1, k] = s[ir, k]

    def _win(self, Pe, hi):
        """Peclet window: 2 < Pe < hi; originalTBL Pe > 2 (fnldnstbl.f90:665);
        dnssetbl |Pe| > 2 (dnssetbl.f90:311)."""
        if self.var == 2:
            return np.abs(Pe) > 2
        if self.var == 1:
            return Pe > 2
        return (Pe > 2) & (Pe < hi)

    # a2, a3: convection and Q (:621-768)
    def conv_q(self):
        nx, ny, nz, re, dt = self.nx, self.ny, self.nz, self.rp.re, self.rp.dt
        I = slice(2, nx - 2)  # interior minus the near-boundary columns
        u, v, w = self.U
        c12 = 1.0 / 12.0
        idx_i = np.arange(1, nx - 1)
        idx_j = np.arange(1, ny - 1)
        idx_k = np.arange(1, nz - 1)
        ii, jj, kk = np.meshgrid(idx_i, idx_j, idx_k, indexing="ij")
        U0 = lambda F, a, b, c: F[a, b, c]
        uc, vc, wc = u[ii, jj, kk], v[ii, jj, kk], w[ii, jj, kk]
        sg = lambda x: np.where(np.ceil(x) >= 0, 1.0, -1.0)
        dz = self.m.x3[kk + 1] - self.m.x3[kk]
        conv = []
        for F in self.U:
            f0 = F[ii, jj, kk]
            # x
            fm1, fp1 = F[ii - 1, jj, kk], F[ii + 1, jj, kk]
            fm2 = F[np.maximum(ii - 2, 0), jj, kk]
            fp2 = F[np.minimum(ii + 2, nx - 1), jj, kk]
            Pe = sg(uc) * re * uc * self.dx
            near = (ii <= 1) | (ii >= nx - 2)
            dn = uc * (fp1 - fm1) / (2.0 * self.dx)
            t1 = np.abs(uc) * (fp2 - 4 * fp1 + 6 * f0 - 4 * fm1 + fm2) * (0.25 / self.dx)
            t2 = uc * (-fp2 + 8 * fp1 - 8 * fm1 + fm2) * (c12 / self.dx)
            cen = uc * ((fm2 - 8 * fm1 + 8 * fp1 - fp2) * (c12 / self.dx))
            d1 = np.where(near, dn, np.where(self._win(Pe, 50), t1 + t2, cen))
            # y (periodic, first-order upwind on the first/last unique rows)
            gm1, gp1 = F[ii, self.jm1[jj], kk], F[ii, self.jp1[jj], kk]
            gm2, gp2 = F[ii, self.jm2[jj], kk], F[ii, self.jp2[jj], kk]
            Pe = sg(vc) * re * vc * self.dy
            near = (jj == 1) | (jj == ny - 2)
            up = np.maximum(vc, 0.0) * ((f0 - gm1) / self.dy) + np.minimum(vc, 0.0) * ((gp1 - f0) / self.dy)
            t1 = np.abs(vc) * (gp2 - 4 * gp1 + 6 * f0 - 4 * gm1 + gm2) * (0.25 / self.dy)
            t2 = vc * (-gp2 + 8 * gp1 - 8 * gm1 + gm2) * (c12 / self.dy)
            cen = vc * ((gm2 - 8 * gm1 + 8 * gp1 - gp2) * (c12 / self.dy))
            if self.var == 2:  # central on the first/last rows (dnssetbl.f90:325-326)
                up = vc * (gp1 - gm1) * (0.5 / self.dy)
            d2 = np.where(near, up, np.where(self._win(Pe, 50), t1 + t2, cen))
            # xi
            hm1, hp1 = F[ii, jj, kk - 1], F[ii, jj, kk + 1]
            hm2 = F[ii, jj, np.maximum(kk - 2, 0)]
            hp2 = F[ii, jj, np.minimum(kk + 2, nz - 1)]
            Pe = sg(wc) * re * wc * dz
            near = (kk <= 1) | (kk >= nz - 2)
            dn = wc * (hp1 - hm1) * (0.5 / self.dxi)
            t1 = np.abs(wc) * (hp2 - 4 * hp1 + 6 * f0 - 4 * hm1 + hm2) * (0.25 / self.dxi)
            t2 = wc * (-hp2 + 8 * hp1 - 8 * hm1 + hm2) * (c12 / self.dxi)
            cen = wc * ((hm2 - 8 * hm1 + 8 * hp1 - hp2) * (c12 / self.dxi))
            d3 = np.where(near, dn, np.where(self._win(Pe, 5), t1 + t2, cen))
            conv.append(d1 + d2 + d3 * self.jinv[kk])
        P = self.P
        g1 = 0.5 * (P[ii + 1, jj, kk] - P[ii - 1, jj, kk]) / self.dx
        g2 = 0.5 * (P[ii, self.jp1[jj], kk] - P[ii, self.jm1[jj], kk]) / self.dy
        g3 = 0.5 * (P[ii, jj, kk + 1] - P[ii, jj, kk - 1]) * (self.jinv[kk] / self.dxi)
        self.Q = [np.zeros_like(u) for _ in range(3)]
        for c, gc in enumerate((g1, g2, g3)):
            self.Q[c][ii, jj, kk] = self.U[c][ii, jj, kk] - dt * conv[c] - dt * gc

    # a4: block Gauss-Seidel (:771-896)
    def gs(self, target=None):
        t = -self.rp.dt / self.rp.re
        nx, ny = self.nx, self.ny
        sweeps = []
        for c in range(3):
            F, Q = self.U[c], self.Q[c]
            n = 0
            sumnor = 0.0
            for it in range(1, self.rp.mmax + 1):
                if it % 2 == 1:
                    diver = 0.0
                    for (bn, en) in self.slabs:
                        tmp = 0.0
                        for k in range(bn, en + 1):
                            d = 1.0 + t * self.Ap[k]
                            for j in range(1, ny - 1):
                                i = np.arange(1, nx - 1)
                                res = (Q[i, j, k] - d * F[i, j, k] - t * self.Aw * F[i + 1, j, k] - t * self.Aw * F[i - 1, j, k]
                                       - t * self.As * F[i, self.jp1[j], k] - t * self.As * F[i, self.jm1[j], k]
                                       - t * self.At[k] * F[i, j, k + 1] - t * self.Ab[k] * F[i, j, k - 1])
                                tmp += float(np.abs(res).sum())
                        diver += tmp
                    if it == 1:
                        sumnor = 1.0 / diver
                    sumav = diver * sumnor
                    stop = (n >= target[c]) if target is not None else (
                        sumav < self.rp.errorstop or (self.var == 2 and diver < float(np.float32(1e-12))))
                    if stop:
                        break
                old = F.copy()  # neighbours' halo planes as of the previous sweep
                for r, (bn, en) in enumerate(self.slabs):
                    for k in range(bn, en + 1):
                        d = 1.0 + t * self.Ap[k]
                        lo = old if (k == bn and r > 0) else F
                        hi = old if (k == en and r < len(self.slabs) - 1) else F
                        for j in range(1, ny - 1):
                            for i in range(1, nx - 1):
                                F[i, j, k] = (Q[i, j, k] - t * self.Aw * F[i + 1, j, k] - t * self.Aw * F[i - 1, j, k]
                                              - t * self.As * F[i, self.jp1[j], k] - t * self.As * F[i, self.jm1[j], k]
                                              - t * self.At[k] * hi[i, j, k + 1] - t * self.Ab[k] * lo[i, j, k - 1]) / d
                n += 1
            sweeps.append(n)
        return sweeps

    # a5: Q8 (:905-935)
    def div(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        u, v, w = self.U
        ii, jj, kk = np.meshgrid(np.arange(1, nx - 1), np.arange(1, ny - 1), np.arange(1, nz - 1), indexing="ij")
        d1 = (((u[ii + 1, jj, kk] + u[ii, jj, kk]) * 0.5) - ((u[ii, jj, kk] + u[ii - 1, jj, kk]) * 0.5)) / self.dx
        d2 = (((v[ii, self.jp1[jj], kk] + v[ii, jj, kk]) * 0.5) - ((v[ii, jj, kk] + v[ii, self.jm1[jj], kk]) * 0.5)) / self.dy
        x3 = self.m.x3
        d3 = 2.0 * (((w[ii, jj, kk + 1] + w[ii, jj, kk]) * 0.5) - ((w[ii, jj, kk] + w[ii, jj, kk - 1]) * 0.5)) / (x3[kk + 1] - x3[kk - 1])
        self.Q8 = np.zeros_like(u)
        self.Q8[ii, jj, kk] = (d1 + d2 + d3) / self.rp.dt

    def lap(self, X):
        nx, ny, nz = self.nx, self.ny, self.nz
        Y = np.zeros_like(X)
        ii, jj, kk = np.meshgrid(np.arange(1, nx - 1), np.arange(1, ny - 1), np.arange(1, nz - 1), indexing="ij")
        Y[ii, jj, kk] = (self.Aw * X[ii - 1, jj, kk] + self.Aw * X[ii + 1, jj, kk] + self.As * X[ii, self.jm1[jj], kk]
                         + self.As * X[ii, self.jp1[jj], kk] + self.Ab[kk] * X[ii, jj, kk - 1]
                         + self.At[kk] * X[ii, jj, kk + 1] + self.Ap[kk] * X[ii, jj, kk])
        return Y

    # block SSOR (:1011-1042), zero halos per slab, no periodic wrap
    def ssor(self, R):
        w = self.rp.omega
        nx, ny = self.nx, self.ny
        out = np.zeros_like(R)
        for (bn, en) in self.slabs:
            x = np.zeros((nx, ny, en - bn + 3))
            for k in range(bn, en + 1):
                kl = k - bn + 1
                for j in range(1, ny - 1):
                    for i in range(1, nx - 1):
                        x[i, j, kl] = -w * (R[i, j, k] + self.Aw * x[i - 1, j, kl] + self.As * x[i, j - 1, kl]
                                            + self.Ab[k] * x[i, j, kl - 1]) / self.Ap[k]
            for k in range(bn, en + 1):
                x[1:nx - 1, 1:ny - 1, k - bn + 1] *= ((2 - w) / w) * self.Ap[k]
            for k in range(en, bn - 1, -1):
                kl = k - bn + 1
                for j in range(ny - 2, 0, -1):
                    for i in range(nx - 2, 0, -1):
                        x[i, j, kl] = -w * (x[i, j, kl] + self.Aw * x[i + 1, j, kl] + self.As * x[i, j + 1, kl]
                                            + self.At[k] * x[i, j, kl + 1]) / self.Ap[k]
            out[1:nx - 1, 1:ny - 1, bn:en + 1] = x[1:nx - 1, 1:ny - 1, 1:en - bn + 2]
        return out

    # a6: GMRES (:940-1208)
    def gmres(self, rec=None):
        nx, ny, nz = self.nx, self.ny, self.nz
        PC = self.PC
        PC[0, :, :] = 0; PC[nx - 1, :, :] = 0; PC[:, 0, :] = 0; PC[:, ny - 1, :] = 0
        PC[:, :, 0] = 0; PC[:, :, nz - 1] = 0
        kmax, tol = self.rp.kmax, self.rp.errtol
        interior = (slice(1, nx - 1), slice(1, ny - 1), slice(1, nz - 1))
        dot = lambda a, b: float(np.sum(a[interior] * b[interior]))
        sumav, m = 1.0, 0
        kits = []
        nr = rec[0] if rec is not None else 0
        while (m < nr) if rec is not None else (sumav > tol and m < self.rp.mmax):
            m += 1
            r = self.Q8 - self.lap(PC)
            r = self.ssor(r)
            rho = np.sqrt(dot(r, r))
            if m == 1:
                sumnor = rho
            sumav = rho / sumnor
            V = [r / rho]
            H = np.zeros((kmax + 1, kmax + 1))
            g = np.zeros(kmax + 1); cs = np.zeros(kmax + 1); sn = np.zeros(kmax + 1)
            g[0] = rho
            kit = 0
            tgt = rec[m] if rec is not None else 0
            while (kit < tgt) if rec is not None else (sumav > tol and kit < kmax):
                kit += 1
                wv = self.ssor(self.lap(V[kit - 1]))
                for q in range(kit):
                    H[q, kit - 1] = dot(V[q], wv)
                    wv = wv - H[q, kit - 1] * V[q]
                H[kit, kit - 1] = np.sqrt(dot(wv, wv))
                if H[kit, kit - 1] != 0:
                    wv = wv / H[kit, kit - 1]
                V.append(wv)
                for q in range(kit - 1):
                    a, b = H[q, kit - 1], H[q + 1, kit - 1]
                    H[q, kit - 1] = cs[q] * a - sn[q] * b
                    H[q + 1, kit - 1] = sn[q] * a + cs[q] * b
                nu = np.sqrt(H[kit - 1, kit - 1] ** 2 + H[kit, kit - 1] ** 2)
                if nu > 0:
                    cs[kit - 1] = H[kit - 1, kit - 1] / nu
                    sn[kit - 1] = -H[kit, kit - 1] / nu
                    H[kit - 1, kit - 1] = cs[kit - 1] * H[kit - 1, kit - 1] - sn[kit - 1] * H[kit, kit - 1]
                    H[kit, kit - 1] = 0.0
                    gk = cs[kit - 1] * g[kit - 1] - sn[kit - 1] * g[kit]
                    gkp = sn[kit - 1] * g[kit - 1] + cs[kit - 1] * g[kit]
                    g[kit - 1], g[kit] = gk, gkp
                sumav = abs(g[kit]) / sumnor
            kits.append(kit)
            if kit > 0:
                y = np.zeros(kit)
                for q in range(kit - 1, -1, -1):
                    y[q] = (g[q] - np.dot(H[q, q + 1:kit], y[q + 1:kit])) / H[q, q]
                for q in range(kit):
                    PC[interior] = PC[interior] + V[q][interior] * y[q]
        return kits

    # a7, a8 (:1245-1469)
    def project_bcs(self, uold1):
        nx, ny, nz, dt, re = self.nx, self.ny, self.nz, self.rp.dt, self.rp.re
        PC, P = self.PC, self.P
        PC[:, 1:ny - 1, 0] = (4.0 * PC[:, 1:ny - 1, 1] - PC[:, 1:ny - 1, 2]) / 3.0
        PC[:, 1:ny - 1, nz - 1] = (5.0 * PC[:, 1:ny - 1, nz - 2] + (-4.0 * PC[:, 1:ny - 1, nz - 3] + PC[:, 1:ny - 1, nz - 4])) / 2.0
        PC[:, 0, :] = PC[:, ny - 2, :]
        PC[:, ny - 1, :] = PC[:, 1, :]
        PC[0, 1:ny - 1, :] = (4.0 * PC[1, 1:ny - 1, :] - PC[2, 1:ny - 1, :]) / 3.0
        PC[nx - 1, 1:ny - 1, :] = (5.0 * PC[nx - 2, 1:ny - 1, :] + (-4.0 * PC[nx - 3, 1:ny - 1, :] + PC[nx - 4, 1:ny - 1, :])) / 2.0
        ii, jj, kk = np.meshgrid(np.arange(1, nx - 1), np.arange(1, ny - 1), np.arange(1, nz - 1), indexing="ij")
        P[ii, jj, kk] = P[ii, jj, kk] + PC[ii, jj, kk]
        g1 = 0.5 * (PC[ii + 1, jj, kk] - PC[ii - 1, jj, kk]) / self.dx
        g2 = 0.5 * (PC[ii, self.jp1[jj], kk] - PC[ii, self.jm1[jj], kk]) / self.dy
        g3 = 0.5 * (PC[ii, jj, kk + 1] - PC[ii, jj, kk - 1]) * (self.jinv[kk] / self.dxi)
        for c, gc in enumerate((g1, g2, g3)):
            self.U[c][ii, jj, kk] = self.U[c][ii, jj, kk] - dt * gc
        for F in self.U:
            F[:, 1:ny - 1, 0] = 0.0
            F[:, 1:ny - 1, nz - 1] = (4.0 * F[:, 1:ny - 1, nz - 2] - F[:, 1:ny - 1, nz - 3]) / 3.0
        for F in self.U:
            F[nx - 1, 1:ny - 1, :] = (4.0 * F[nx - 2, 1:ny - 1, :] - F[nx - 3, 1:ny - 1, :]) / 3.0
        u, v, w = self.U
        x3 = self.m.x3
        df1, df2 = x3[1] - x3[0], x3[2] - x3[0]
        I, Jr = np.arange(1, nx - 1), np.arange(1, ny - 1)
        ii2, jj2 = np.meshgrid(I, Jr, indexing="ij")
        fder = (w[ii2, jj2, 1] - w[ii2, jj2, 0]) / df1
        d3 = w[ii2, jj2, 0] * fder
        g1 = (w[ii2 - 1, jj2, 0] + w[ii2 + 1, jj2, 0] - 2 * w[ii2, jj2, 0]) / (self.dx * self.dx)
        g2 = (w[ii2, jj2 - 1, 0] + w[ii2, jj2 + 1, 0] - 2 * w[ii2, jj2, 0]) / (self.dy * self.dy)
        g3 = (2 * df1 * w[ii2, jj2, 2] - 2 * df2 * w[ii2, jj2, 1] + 2 * (df2 - df1) * w[ii2, jj2, 0]) / (df1 * df2 ** 2 - df2 * df1 ** 2)
        P[ii2, jj2, 0] = P[ii2, jj2, 1] - (-d3 + (g1 + g2 + g3) / re) * df1
        fder = (11.0 * w[ii2, jj2, nz - 1] - 18.0 * w[ii2, jj2, nz - 2] + 9.0 * w[ii2, jj2, nz - 3] - 2.0 * w[ii2, jj2, nz - 4]) / (6.0 * self.dxi)
        P[ii2, jj2, nz - 1] = fder * self.jinv[nz - 1] / re
        K = np.arange(1, nz - 1)
        jj3, kk3 = np.meshgrid(Jr, K, indexing="ij")
        P[nx - 1, jj3, kk3] = (3.0 * u[nx - 1, jj3, kk3] - 4.0 * u[nx - 2, jj3, kk3] + u[nx - 3, jj3, kk3]) / (2.0 * self.dx * re)
        u0 = u[0, jj3, kk3]
        d1 = u0 * ((u[1, jj3, kk3] - u0) / self.dx)
        d2 = v[0, jj3, kk3] * ((u[0, jj3 + 1, kk3] - u[0, jj3 - 1, kk3]) / (2.0 * self.dy))
        d3 = w[0, jj3, kk3] * ((u[0, jj3, kk3 + 1] - u[0, jj3, kk3 - 1]) / (2.0 * self.dxi))
        g1 = (u0 + u[2, jj3, kk3] - 2 * u[1, jj3, kk3]) / (self.dx * self.dx)
        g2 = (u[0, jj3 + 1, kk3] + u[0, jj3 - 1, kk3] - 2 * u0) / (self.dy * self.dy)
        fder = (u[0, jj3, kk3 + 1] - u[0, jj3, kk3 - 1]) / (2.0 * self.dxi)
        g3 = (-2 * u0 + u[0, jj3, kk3 + 1] + u[0, jj3, kk3 - 1]) / (self.dxi * self.dxi)
        lo = kk3 <= 1
        hi = kk3 >= nz - 2
        kp2 = np.minimum(kk3 + 2, nz - 1)
        km2 = np.maximum(kk3 - 2, 0)
        fder = np.where(lo, (u[0, jj3, kk3 + 1] - u0) / self.dxi, np.where(hi, (u0 - u[0, jj3, kk3 - 1]) / self.dxi, fder))
        g3 = np.where(lo, (u[0, jj3, kp2] - 2.0 * u[0, jj3, kk3 + 1] + u0) / (self.dxi * self.dxi),
                      np.where(hi, (u[0, jj3, km2] - 2.0 * u[0, jj3, kk3 - 1] + u0) / (self.dxi * self.dxi), g3))
        Jk = self.jinv[kk3]
        g3 = g3 * (Jk * Jk) - (self.m.jac2[kk3] * fder) * (Jk * Jk * Jk)
        fder2 = (u0 - uold1[jj3, kk3]) / dt
        P[0, jj3, kk3] = ((2 * self.dx * ((fder2 + d1 + d2 + d3 * Jk) - ((g1 + g2 + g3) / re))) - 0.0 - P[2, jj3, kk3] + 4 * P[1, jj3, kk3]) / 3.0
        for F in (u, v, w, P):
            F[:, 0, :] = F[:, ny - 2, :]
            F[:, ny - 1, :] = F[:, 1, :]

    # a9 (:1707-1722): the recycled plane refreshed on every slab
    def fluc(self, run_steps):
        ny, nz, ir = self.ny, self.nz, self.rp.irec - 1
        on = (run_steps > self.rp.recycle_after) if self.var == 2 else (self.nstep > self.rp.recycle_after)
        if on:
            for c, mn in enumerate((self.usum2, self.vsum2, self.wsum2)):
                self.fl_live[c][1:ny - 1, 1:nz - 1] = self.U[c][ir, 1:ny - 1, 1:nz - 1] - mn[ir, 1:nz - 1][None, :]

    # a9 (:1881-1993); dnssetbl unweighted / (ny-2) (dnssetbl.f90:936-983)
    def stats(self):
        nx, ny, nz, ir = self.nx, self.ny, self.nz, self.rp.irec - 1
        u, v, w = self.U
        self.cont += 1
        if self.nstep % self.rp.istat == 0:
            A = self.m.x2[ny - 1] - self.m.x2[1]
            dA = self.dy
            if self.var == 2:
                A, dA = float(ny - 2), 1.0
            jj = np.arange(1, ny - 1)
            su = 0.5 * (u[:, jj, :] + u[:, self.jp1[jj], :])
            sv = 0.5 * (v[:, jj, :] + v[:, self.jp1[jj], :])
            sw = 0.5 * (w[:, jj, :] + w[:, self.jp1[jj], :])
            for key, val in (("u", su), ("v", sv), ("w", sw), ("uu", su * su), ("vv", sv * sv), ("ww", sw * sw),
                             ("uv", su * sv), ("uw", su * sw), ("vw", sv * sw)):
                self.sums[key] += (val * dA).sum(axis=1) / A

    # a10 (:2084-2365)
    def rescale(self):
        from turbulentbl_gb300.synth import rescaling_state  # shared formulas, checked separately
        nx, ny, nz, ir, cum = self.nx, self.ny, self.nz, self.rp.irec - 1, float(self.rp.cum)
        self.usum2 = self.sums["u"] / cum
        self.vsum2 = self.sums["v"] / cum
        self.wsum2 = self.sums["w"] / cum
        x3, re, ue = self.m.x3, self.rp.re, self.rp.ue
        utau1 = np.sqrt(((self.usum2[0, 1] - self.usum2[0, 0]) / (x3[1] - x3[0])) / re)
        utau2 = np.sqrt(((self.usum2[ir, 1] - self.usum2[ir, 0]) / (x3[1] - x3[0])) / re)
        self.lamda = utau1 / utau2
        bl, wt, newk, ksep = rescaling_state(self.usum2, x3, ue, self.rp.irec, self.lamda, self.ksep, self.bltkns)
        self.bltkns, self.Wt, self.newk, self.ksep = bl, wt, newk, ksep
        k0, k1 = self.slabs[0] if self.var == 2 else (1, nz - 2)  # dnssetbl: rank 0's slab (dnssetbl.f90:1033)
        for c, mn in enumerate((self.usum2, self.vsum2, self.wsum2)):
            self.fl_live[c][1:ny - 1, k0:k1 + 1] = self.U[c][ir, 1:ny - 1, k0:k1 + 1] - mn[ir, k0:k1 + 1][None, :]
        for k in self.sums:
            self.sums[k][:] = 0.0

    def step(self, counts=None):
        self.nstep += 1
        uold1 = self.U[0][0].copy()
        if self.nstep > self.rp.recycle_after:
            self.inflow()
        self.conv_q()
        sweeps = self.gs(None if counts is None else counts[:3])
        self.div()
        kits = self.gmres(None if counts is None else counts[3:])
        self.project_bcs(uold1)
        if self.var == 2:  # statistics, rescaling on nstep, then the fluctuations (dnssetbl.f90:936, :986, :1223)
            self.stats()
            if self.nstep % self.rp.cum == 0:
                self.rescale()
            self.fluc(self.cont)
        else:
            self.fluc(self.cont + 1)
            self.stats()
            if self.cont % self.rp.cum == 0:
                self.rescale()
        self.cnt2 += 1
        return sweeps + [len(kits)] + kits
