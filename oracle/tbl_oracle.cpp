/*
 * tbl_oracle.cpp -- CPU restatement (FP64) of the turbulentBL time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU library is
 * checked against: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs may load it.  It is never part of the product path.
 *
 * It restates theparvezahmad/turbulentBL dnstbl2/dnstbl.f90, the body of the
 * time loop (:538-2375), with P virtual MPI ranks reproducing the
 * decomposition-dependent numerics of the MPI program:
 *   - slab partition in k (:469-485);
 *   - Gauss-Seidel halos exchanged after every sweep (block-Jacobi across
 *     slabs, :873-892): a slab reads its neighbours' boundary planes as they
 *     were after the previous sweep;
 *   - block-SSOR preconditioner per slab with zero halos and no periodic wrap
 *     (:1022-1042, :1115-1135; rhat outside the slab is never written);
 *   - reductions as per-rank partial sums in loop order combined in rank
 *     order (:824, :1048, :1145, :1155);
 *   - the recycled fluctuation plane Ufluc(irec,:,new(k),:) is "live" only
 *     when new(k) lies in the reading rank's own slab; otherwise a rank reads
 *     its copy from the restart file, which it never updates (:582-590 read,
 *     :1712-1722 and :2341-2349 write own slab only).
 * Floating-point expression order follows the Fortran source (left to right,
 * no contraction: build with -ffp-contract=off).
 *
 * tbl_config.variant switches to the differences of the reference's other
 * two programs of the method, originalTBL/fnldnstbl.f90 and
 * dnssetbl/dnssetbl.f90 (each cited where it is applied); everything else
 * follows dnstbl2.
 *
 * Parity status: UNPINNED against the reference binary.  No Fortran compiler
 * or MPI exists on either build machine, and the reference ships no tests,
 * golden vectors or input files.  The restatement is pinned instead by an
 * independent NumPy restatement (oracle/np_oracle.py), manufactured-solution
 * and known-answer tests (tests/).
 */
#include "../include/tbl_gpu.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>
#include <algorithm>

namespace {

struct Oracle {
    tbl_config c{};
    int nx = 0, ny = 0, nz = 0, P = 0;
    size_t N = 0;
    // mesh
    std::vector<double> x1, x2, x3, jac /* inverted on use range, :534-536 */, jac2, jac_raw;
    double dx = 0, dy = 0, dxi = 0, invdx = 0, invdy = 0, invdxi = 0, c12 = 1.0 / 12.0;
    double df1 = 0, df2 = 0;
    // slab partition
    std::vector<int> bn, en;
    // coefficients (An* == Av*, :498-528); constant in i, j
    double Aw = 0, As = 0;  // Anw = Ane = 1/dx^2, Ans = Ann = 1/dy^2
    std::vector<double> Ab, At, Ap, rAp;  // indexed by k (1-based)
    // state
    std::vector<double> U[3], P_, PC, Q[3], Q8, Uold1;
    std::vector<double> usum2, vsum2, wsum2, Wt, ume1, bltkns;
    std::vector<double> ufl_file[3], ufl_live[3];  // plane irec: (ny,nz)
    std::vector<double> ufl_full_file[3];          // full uploaded Ufluc (download)
    std::vector<double> usum2_last_fluc[3];        // usum2 used at last per-step Ufluc update (nx,nz)
    bool fluc_updated = false;
    std::vector<int> newk;
    double lamda = 1.0, lamda03 = 0, time = 0;
    int nstep = 0, cont = 0, ksep = 0, nstat = 0, cnt2 = 0;
    // statistics
    std::vector<double> usum, vsum, wsum, uusum, vvsum, wwsum, uvsum, uwsum, vwsum;
    std::vector<double> avg;  // 9 x (nx,nz): the sums / cum of the last rescaling (:2021-2049)
    std::vector<double> deltastar, theta, Ht, Reth, sumxz, tauw_window;
    double ubulk[5] = {0, 0, 0, 0, 0};
    // GMRES work
    std::vector<std::vector<double>> V;
    std::vector<double> r, rhat, h, g, cs, sn, y;
    // GS halo snapshots: plane en of each slab and bn of each slab, per component
    std::vector<double> snap_lo, snap_hi;
    // replay
    std::vector<int32_t> replay;
    size_t replay_pos = 0;
    std::vector<int32_t> last_counts;

    inline size_t id(int i, int j, int k) const {  // 1-based Fortran indices
        return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
    }
    inline size_t id2(int i, int k) const { return (size_t)(i - 1) + (size_t)nx * (size_t)(k - 1); }
    inline size_t idp(int j, int k) const { return (size_t)(j - 1) + (size_t)ny * (size_t)(k - 1); }
    inline int jm1(int j) const { return j == 2 ? ny - 1 : j - 1; }
    inline int jp1(int j) const { return j == ny - 1 ? 2 : j + 1; }
    inline int jm2(int j) const { int a = jm1(j) - 1; if (j == 3) a = ny - 1; return a; }
    inline int jp2(int j) const { int a = jp1(j) + 1; if (j == ny - 2) a = 2; return a; }
    int slab_of(int k) const {
        for (int r = 0; r < P; ++r) if (k >= bn[r] && k <= en[r]) return r;
        return -1;
    }
};

inline bool is_orig(const Oracle& o) { return o.c.variant == TBL_VARIANT_ORIGINAL; }
inline bool is_sete(const Oracle& o) { return o.c.variant == TBL_VARIANT_DNSSETBL; }

inline double fsign_ceil(double u) {
    // sgn = sign(1, ceiling(u)) (dnstbl2/dnstbl.f90:651): +1 when ceiling(u) >= 0
    return std::ceil(u) >= 0.0 ? 1.0 : -1.0;
}

int setup(Oracle& o, const tbl_config* cfg, const tbl_mesh* m) {
    o.c = *cfg;
    o.nx = cfg->nx; o.ny = cfg->ny; o.nz = cfg->nz; o.P = cfg->nproc;
    if (o.nx < 8 || o.ny < 6 || o.nz < 8 || o.P < 1) return TBL_ERR_BAD_ARG;
    if (cfg->irec < 2 || cfg->irec > o.nx - 1 || cfg->cum < 1 || cfg->istat < 1) return TBL_ERR_BAD_ARG;
    if (cfg->kmax < 1 || cfg->mmax < 1) return TBL_ERR_BAD_ARG;
    o.N = (size_t)o.nx * o.ny * o.nz;
    if (cfg->variant < TBL_VARIANT_DNSTBL2 || cfg->variant > TBL_VARIANT_DNSSETBL) return TBL_ERR_BAD_ARG;
    o.bn.resize(o.P); o.en.resize(o.P);
    if (cfg->variant == TBL_VARIANT_DNSSETBL) {
        // dnssetbl.f90:78-92: blocks of nz/P over k = 1..nz, one more point on
        // the last mod(nz,P) ranks; the first and last planes are boundaries
        int it1 = o.nz / o.P;
        const int it2 = o.P - o.nz % o.P;
        int b = 1;
        for (int r = 0; r < o.P; ++r) {
            if (r == it2) it1 = it1 + 1;
            o.bn[r] = b;
            o.en[r] = b + it1 - 1;
            b = o.en[r] + 1;
        }
        o.bn[0] = o.bn[0] + 1;
        o.en[o.P - 1] = o.en[o.P - 1] - 1;
        for (int r = 0; r < o.P; ++r)
            if (o.en[r] - o.bn[r] + 1 < 3) return TBL_ERR_BAD_ARG;
    } else {
        // partition (:469-475)
        int loc_n = (o.nz - 1) / o.P;
        if (loc_n < 3) return TBL_ERR_BAD_ARG;
        for (int r = 0; r < o.P; ++r) {
            o.bn[r] = 2 + r * loc_n;
            o.en[r] = o.bn[r] + loc_n - 1;
            if (r == o.P - 1) o.en[r] = o.nz - 1;
        }
    }
    o.x1.assign(m->x1, m->x1 + o.nx);
    o.x2.assign(m->x2, m->x2 + o.ny);
    o.x3.assign(m->x3, m->x3 + o.nz);
    o.jac_raw.assign(m->jac, m->jac + o.nz);
    o.jac2.assign(m->jac2, m->jac2 + o.nz);
    o.dx = cfg->dx; o.dy = cfg->dy; o.dxi = cfg->dxi;
    o.invdx = 1.0 / o.dx; o.invdy = 1.0 / o.dy; o.invdxi = 1.0 / o.dxi;
    o.df1 = o.x3[1] - o.x3[0];
    o.df2 = o.x3[2] - o.x3[0];
    // coefficients with the un-inverted Jacobian (:498-528); 1-based k
    o.Aw = 1.0 / (o.dx * o.dx);
    o.As = 1.0 / (o.dy * o.dy);
    o.Ab.assign(o.nz + 1, 0.0); o.At.assign(o.nz + 1, 0.0);
    o.Ap.assign(o.nz + 1, 0.0); o.rAp.assign(o.nz + 1, 0.0);
    for (int k = 2; k <= o.nz - 1; ++k) {
        double J = o.jac_raw[k - 1], J2 = o.jac2[k - 1];
        double a = 1.0 / (o.dxi * o.dxi * J * J);
        double b = J2 / (2.0 * o.dxi * J * J * J);
        o.Ab[k] = a + b;
        o.At[k] = a - b;
        o.Ap[k] = -2.0 * ((1.0 / (o.dx * o.dx)) + (1.0 / (o.dy * o.dy)) + (1.0 / (o.dxi * o.dxi * J * J)));
        o.rAp[k] = 1.0 / o.Ap[k];
    }
    // Jac <- 1/Jac on every rank's istart..iend, i.e. all k (:534-536)
    o.jac.resize(o.nz + 1);
    for (int k = 1; k <= o.nz; ++k) o.jac[k] = 1.0 / o.jac_raw[k - 1];
    for (int cc = 0; cc < 3; ++cc) {
        o.U[cc].assign(o.N, 0.0); o.Q[cc].assign(o.N, 0.0);
        o.ufl_file[cc].assign((size_t)o.ny * o.nz, 0.0);
        o.ufl_live[cc].assign((size_t)o.ny * o.nz, 0.0);
        o.ufl_full_file[cc].assign(o.N, 0.0);
        o.usum2_last_fluc[cc].assign((size_t)o.nx * o.nz, 0.0);
    }
    o.P_.assign(o.N, 0.0); o.PC.assign(o.N, 0.0); o.Q8.assign(o.N, 0.0);
    o.Uold1.assign((size_t)o.ny * o.nz, 0.0);
    size_t n2 = (size_t)o.nx * o.nz;
    for (auto* v : {&o.usum2, &o.vsum2, &o.wsum2, &o.Wt, &o.usum, &o.vsum, &o.wsum, &o.uusum,
                    &o.vvsum, &o.wwsum, &o.uvsum, &o.uwsum, &o.vwsum})
        v->assign(n2, 0.0);
    o.ume1.assign(o.nz, 0.0);
    o.avg.assign((size_t)9 * o.nx * o.nz, 0.0);
    o.newk.assign(o.nz, o.nz - 1);
    for (auto* v : {&o.bltkns, &o.deltastar, &o.theta, &o.Ht, &o.Reth, &o.sumxz, &o.tauw_window}) v->assign(o.nx, 0.0);
    o.V.assign(cfg->kmax + 1, std::vector<double>(o.N, 0.0));
    o.r.assign(o.N, 0.0); o.rhat.assign(o.N, 0.0);
    int K1 = cfg->kmax + 1;
    o.h.assign((size_t)K1 * K1, 0.0);
    o.g.assign(K1, 0.0); o.cs.assign(K1, 0.0); o.sn.assign(K1, 0.0); o.y.assign(K1, 0.0);
    o.snap_lo.assign((size_t)o.P * o.nx * o.ny, 0.0);
    o.snap_hi.assign((size_t)o.P * o.nx * o.ny, 0.0);
    return TBL_OK;
}

// ---------------------------------------------------------------- a1: inflow
// dnstbl2/dnstbl.f90:557-618.  originalTBL ramps the u mean from Ume1 to the
// recycled mean with eps = min(cnt2 * 5e-5, 1) (fnldnstbl.f90:561-587);
// dnssetbl ramps it with eps = min(nstep * 5e-5, 1), scales the v mean by
// lamda and blends with Wt(1,k) (dnssetbl.f90:259-300).
double inflow_eps(const Oracle& o) {
    double eps = (is_orig(o) ? (double)o.cnt2 : (double)o.nstep) * (5.0e-5);
    if (eps > 1.0) eps = 1.0;
    return eps;
}

void inflow(Oracle& o) {
    const int irec = o.c.irec, nx = o.nx, ny = o.ny;
    const bool ramp = is_orig(o) || is_sete(o);
    const double eps = inflow_eps(o);
    for (int rk = 0; rk < o.P; ++rk) {
        for (int k = o.bn[rk]; k <= o.en[rk]; ++k) {
            if (o.usum2[o.id2(irec, k)] < (0.99 * o.c.ue)) {
                int nk = o.newk[k - 1];
                double uin = ramp ? eps * (o.usum2[o.id2(irec, nk)]) + (1 - eps) * o.ume1[k - 1] : o.ume1[k - 1];
                double vin = is_sete(o) ? o.lamda * o.vsum2[o.id2(irec, nk)] : o.vsum2[o.id2(irec, nk)];
                double win = o.wsum2[o.id2(irec, nk)];
                bool live = (nk >= o.bn[rk] && nk <= o.en[rk]);
                // the redundant i loop leaves Wt(nX-1,k) in effect (:594-600);
                // dnssetbl uses Wt(1,k) (dnssetbl.f90:291-293)
                double wt = o.Wt[o.id2(is_sete(o) ? 1 : nx - 1, k)];
                for (int j = 2; j <= ny - 1; ++j) {
                    double f[3];
                    for (int cc = 0; cc < 3; ++cc) {
                        const std::vector<double>& src = live ? o.ufl_live[cc] : o.ufl_file[cc];
                        f[cc] = o.lamda * src[o.idp(j, nk)];
                    }
                    o.U[0][o.id(1, j, k)] = (uin + f[0]) * (1.0 - wt) + (uin + f[0]) * wt;
                    o.U[1][o.id(1, j, k)] = (vin + f[1]) * (1.0 - wt) + (vin + f[1]) * wt;
                    o.U[2][o.id(1, j, k)] = (win + f[2]) * (1.0 - wt) + (win + f[2]) * wt;
                }
            } else {
                for (int j = 2; j <= ny - 1; ++j) {
                    o.U[0][o.id(1, j, k)] = o.usum2[o.id2(irec, k)];
                    o.U[1][o.id(1, j, k)] = o.vsum2[o.id2(irec, k)];
                    o.U[2][o.id(1, j, k)] = o.wsum2[o.id2(irec, k)];
                }
            }
        }
    }
}

// ------------------------------------------------------- a2+a3: conv and Q
// dnstbl2/dnstbl.f90:621-768
// Peclet windows: dnstbl2 2 < Pe < 50 (x, y) and 2 < Pe < 5 (xi); originalTBL
// Pe > 2 (fnldnstbl.f90:665, :689, :711); dnssetbl |Re u h| > 2
// (dnssetbl.f90:311-345), which equals |Pe| > 2 for the signed Pe here.
inline bool pe_win(const Oracle& o, double Pe, double hi) {
    if (is_sete(o)) return std::fabs(Pe) > 2.0;
    if (is_orig(o)) return Pe > 2.0;
    return Pe > 2.0 && Pe < hi;
}

void conv_q(Oracle& o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    const double tf = o.c.re, dt = o.c.dt;
    const double c12 = o.c12;
    std::vector<double> conv(o.N * 3, 0.0);
    for (int jc = 0; jc < 3; ++jc) {
        const std::vector<double>& F = o.U[jc];
        const std::vector<double>& U1 = o.U[0];
        const std::vector<double>& U2 = o.U[1];
        const std::vector<double>& U3 = o.U[2];
#pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 1; ++i) {
                    int im1 = i - 1, im2 = im1 - 1, ip1 = i + 1, ip2 = ip1 + 1;
                    int jm1_ = o.jm1(j), jm2_ = o.jm2(j), jp1_ = o.jp1(j), jp2_ = o.jp2(j);
                    double d1, d2, d3, Pe, term1, term2;
                    double u = U1[o.id(i, j, k)];
                    Pe = fsign_ceil(u) * tf * u * o.dx;
                    if (i <= 2 || i >= nx - 1) {
                        d1 = u * (F[o.id(ip1, j, k)] - F[o.id(im1, j, k)]) / (2.0 * o.dx);
                    } else if (pe_win(o, Pe, 50.0)) {
                        term1 = (std::fabs(u)) *
                                (F[o.id(ip2, j, k)] - (4 * (F[o.id(ip1, j, k)])) + (6 * (F[o.id(i, j, k)])) -
                                 (4 * (F[o.id(im1, j, k)])) + F[o.id(im2, j, k)]) *
                                (0.25 * o.invdx);
                        term2 = (u) *
                                (-F[o.id(ip2, j, k)] + (8 * (F[o.id(ip1, j, k)])) - (8 * (F[o.id(im1, j, k)])) +
                                 F[o.id(im2, j, k)]) *
                                (c12 * o.invdx);
                        d1 = term1 + term2;
                    } else {
                        d1 = u * ((F[o.id(im2, j, k)] - 8 * F[o.id(im1, j, k)] + 8 * F[o.id(ip1, j, k)] -
                                   F[o.id(ip2, j, k)]) *
                                  (c12 * o.invdx));
                    }
                    double v = U2[o.id(i, j, k)];
                    Pe = fsign_ceil(v) * tf * v * o.dy;
                    if ((j == 2 || j == ny - 1) && is_sete(o)) {
                        // second-order central on the first/last rows (dnssetbl.f90:325-326)
                        d2 = v * (F[o.id(i, jp1_, k)] - F[o.id(i, jm1_, k)]) * 0.5 * o.invdy;
                    } else if (j == 2 || j == ny - 1) {
                        double a1 = std::max(v, 0.0), b = std::min(v, 0.0);
                        term1 = a1 * ((F[o.id(i, j, k)] - F[o.id(i, jm1_, k)]) * (o.invdy));
                        term2 = b * ((F[o.id(i, jp1_, k)] - F[o.id(i, j, k)]) * (o.invdy));
                        d2 = term1 + term2;
                    } else if (pe_win(o, Pe, 50.0)) {
                        term1 = (std::fabs(v)) *
                                (F[o.id(i, jp2_, k)] - (4 * (F[o.id(i, jp1_, k)])) + (6 * (F[o.id(i, j, k)])) -
                                 (4 * (F[o.id(i, jm1_, k)])) + F[o.id(i, jm2_, k)]) *
                                (0.25 * o.invdy);
                        term2 = (v) *
                                (-F[o.id(i, jp2_, k)] + (8 * (F[o.id(i, jp1_, k)])) - (8 * (F[o.id(i, jm1_, k)])) +
                                 F[o.id(i, jm2_, k)]) *
                                (c12 * o.invdy);
                        d2 = term1 + term2;
                    } else {
                        d2 = v * ((F[o.id(i, jm2_, k)] - 8 * F[o.id(i, jm1_, k)] + 8 * F[o.id(i, jp1_, k)] -
                                   F[o.id(i, jp2_, k)]) *
                                  (c12 * o.invdy));
                    }
                    double w = U3[o.id(i, j, k)];
                    Pe = (fsign_ceil(w) * tf * w * (o.x3[k] - o.x3[k - 1]));
                    if ((k <= 2) || (k >= nz - 1)) {
                        d3 = (w * (F[o.id(i, j, k + 1)] - F[o.id(i, j, k - 1)]) * (0.5 * o.invdxi));
                    } else if (pe_win(o, Pe, 5.0)) {
                        term1 = (std::fabs(w)) *
                                (F[o.id(i, j, k + 2)] - (4 * (F[o.id(i, j, k + 1)])) + (6 * (F[o.id(i, j, k)])) -
                                 (4 * (F[o.id(i, j, k - 1)])) + F[o.id(i, j, k - 2)]) *
                                (0.25 * o.invdxi);
                        term2 = (w) *
                                (-F[o.id(i, j, k + 2)] + (8 * (F[o.id(i, j, k + 1)])) - (8 * (F[o.id(i, j, k - 1)])) +
                                 F[o.id(i, j, k - 2)]) *
                                (c12 * o.invdxi);
                        d3 = (term1 + term2);
                    } else {
                        d3 = w * ((F[o.id(i, j, k - 2)] - 8 * F[o.id(i, j, k - 1)] + 8 * F[o.id(i, j, k + 1)] -
                                   F[o.id(i, j, k + 2)]) *
                                  (c12 * o.invdxi));
                    }
                    conv[o.id(i, j, k) * 3 + jc] = d1 + d2 + (d3 * o.jac[k]);
                }
    }
    // Q (:719-768); forc = 0, Ri = 0
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nz - 1; ++k)
        for (int j = 2; j <= ny - 1; ++j)
            for (int i = 2; i <= nx - 1; ++i) {
                size_t p = o.id(i, j, k);
                double g1 = 0.5 * (o.P_[o.id(i + 1, j, k)] - o.P_[o.id(i - 1, j, k)]) * (o.invdx);
                double g2 = 0.5 * (o.P_[o.id(i, o.jp1(j), k)] - o.P_[o.id(i, o.jm1(j), k)]) * (o.invdy);
                double g3 = 0.5 * (o.P_[o.id(i, j, k + 1)] - o.P_[o.id(i, j, k - 1)]) * (o.invdxi * o.jac[k]);
                double q5 = o.U[0][p] + (dt * (0.0 - conv[p * 3 + 0]));
                o.Q[0][p] = q5 - (dt * g1);
                double q6 = o.U[1][p] + (dt * (0.0 - conv[p * 3 + 1]));
                o.Q[1][p] = q6 - (dt * g2);
                double q7 = o.U[2][p] + (dt * (0.0 - conv[p * 3 + 2] + (0.0 * 0.0)));
                o.Q[2][p] = q7 - (dt * g3);
            }
}

// ------------------------------------------------------------ a4: GS solve
// dnstbl2/dnstbl.f90:771-896
void gs_solve(Oracle& o, int replay_sweeps[3], int out_sweeps[3], double out_resid[3]) {
    const int nx = o.nx, ny = o.ny;
    const double t = -o.c.dt / (o.c.re);
    const double cE = t * o.Aw, cW = t * o.Aw, cN = t * o.As, cS = t * o.As;
    const size_t plane = (size_t)nx * ny;
    for (int jc = 0; jc < 3; ++jc) {
        std::vector<double>& F = o.U[jc];
        const std::vector<double>& Qc = o.Q[jc];
        double sumnor = 0.0, sumav = 0.0;
        int sweeps = 0;
        const bool replay = replay_sweeps != nullptr;
        for (int it = 1; it <= o.c.mmax; ++it) {
            if (it % 2 == 1) {
                // residual with current halos (:781-828)
                double diver = 0.0;
                std::vector<double> part(o.P, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
                for (int rk = 0; rk < o.P; ++rk) {
                    double tmp = 0.0;
                    for (int k = o.bn[rk]; k <= o.en[rk]; ++k) {
                        double cT = t * o.At[k], cB = t * o.Ab[k], d = 1.0 + (t * o.Ap[k]);
                        for (int j = 2; j <= ny - 1; ++j)
                            for (int i = 2; i <= nx - 1; ++i) {
                                double res = Qc[o.id(i, j, k)] - d * F[o.id(i, j, k)] - cE * F[o.id(i + 1, j, k)] -
                                             cW * F[o.id(i - 1, j, k)] - cN * F[o.id(i, o.jp1(j), k)] -
                                             cS * F[o.id(i, o.jm1(j), k)] - cT * F[o.id(i, j, k + 1)] -
                                             cB * F[o.id(i, j, k - 1)];
                                tmp = tmp + std::fabs(res);
                            }
                    }
                    part[rk] = tmp;
                }
                for (int rk = 0; rk < o.P; ++rk) diver += part[rk];  // allreduce in rank order
                if (it == 1) sumnor = 1.0 / diver;
                sumav = diver * sumnor;
                // dnssetbl also stops on the absolute sum, res < 1e-12 with a
                // REAL(4) literal (dnssetbl.f90:392)
                bool stop = replay ? (sweeps >= replay_sweeps[jc])
                                   : (sumav < o.c.errorstop || (is_sete(o) && diver < (double)1e-12f));
                if (stop) break;
            }
            // snapshot the halo planes every rank receives after the previous sweep
            for (int rk = 0; rk < o.P; ++rk) {
                if (rk > 0) std::memcpy(&o.snap_lo[rk * plane], &F[o.id(1, 1, o.bn[rk] - 1)], plane * sizeof(double));
                if (rk < o.P - 1) std::memcpy(&o.snap_hi[rk * plane], &F[o.id(1, 1, o.en[rk] + 1)], plane * sizeof(double));
            }
            // lexicographic sweep per slab (:830-868), halos from the snapshot
#pragma omp parallel for schedule(dynamic, 1)
            for (int rk = 0; rk < o.P; ++rk) {
                const double* lo = &o.snap_lo[rk * plane];
                const double* hi = &o.snap_hi[rk * plane];
                for (int k = o.bn[rk]; k <= o.en[rk]; ++k) {
                    double cT = t * o.At[k], cB = t * o.Ab[k], d = 1.0 + (t * o.Ap[k]);
                    for (int j = 2; j <= ny - 1; ++j)
                        for (int i = 2; i <= nx - 1; ++i) {
                            size_t q = (size_t)(i - 1) + (size_t)nx * (j - 1);
                            double ukp = (k == o.en[rk] && rk < o.P - 1) ? hi[q] : F[o.id(i, j, k + 1)];
                            double ukm = (k == o.bn[rk] && rk > 0) ? lo[q] : F[o.id(i, j, k - 1)];
                            F[o.id(i, j, k)] = (Qc[o.id(i, j, k)] - cE * F[o.id(i + 1, j, k)] -
                                                cW * F[o.id(i - 1, j, k)] - cN * F[o.id(i, o.jp1(j), k)] -
                                                cS * F[o.id(i, o.jm1(j), k)] - cT * ukp - cB * ukm) /
                                               (d);
                        }
                }
            }
            ++sweeps;
        }
        out_sweeps[jc] = sweeps;
        out_resid[jc] = sumav;
    }
}

// ------------------------------------------------------ a5: Poisson RHS Q8
// dnstbl2/dnstbl.f90:905-935
void divergence(Oracle& o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nz - 1; ++k)
        for (int j = 2; j <= ny - 1; ++j)
            for (int i = 2; i <= nx - 1; ++i) {
                const std::vector<double>&U1 = o.U[0], &U2 = o.U[1], &U3 = o.U[2];
                double d1 = (((U1[o.id(i + 1, j, k)] + U1[o.id(i, j, k)]) * 0.5) -
                             (((U1[o.id(i, j, k)] + U1[o.id(i - 1, j, k)]) * 0.5))) * o.invdx;
                double d2 = (((U2[o.id(i, o.jp1(j), k)] + U2[o.id(i, j, k)]) * 0.5) -
                             (((U2[o.id(i, j, k)] + U2[o.id(i, o.jm1(j), k)]) * 0.5))) * o.invdy;
                double d3 = 2.0 * (((U3[o.id(i, j, k + 1)] + U3[o.id(i, j, k)]) * 0.5) -
                                   (((U3[o.id(i, j, k)] + U3[o.id(i, j, k - 1)]) * 0.5))) /
                            (o.x3[k] - o.x3[k - 2]);
                o.Q8[o.id(i, j, k)] = (d1 + d2 + d3) / o.c.dt;
            }
}

// ------------------------------------------------------------- a6: GMRES
inline double lap(const Oracle& o, const std::vector<double>& X, int i, int j, int k) {
    // L7 applied at an interior point, global halos (:1001-1006, :1098-1101)
    return o.Aw * X[o.id(i - 1, j, k)] + o.Aw * X[o.id(i + 1, j, k)] + o.As * X[o.id(i, o.jm1(j), k)] +
           o.As * X[o.id(i, o.jp1(j), k)] + o.Ab[k] * X[o.id(i, j, k - 1)] + o.At[k] * X[o.id(i, j, k + 1)] +
           o.Ap[k] * X[o.id(i, j, k)];
}

// block-SSOR per slab, zero halos (:1011-1042 / :1107-1137).  In: o.r holds the
// input on the interior; out: o.rhat.
void ssor(Oracle& o, const std::vector<double>& in) {
    const int nx = o.nx, ny = o.ny;
    const double w = o.c.omega;
    const double scale_w = (2 - w) / w;
    std::fill(o.rhat.begin(), o.rhat.end(), 0.0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int rk = 0; rk < o.P; ++rk) {
        auto R = [&](int i, int j, int k) -> double {
            if (i < 2 || i > nx - 1 || j < 2 || j > ny - 1 || k < o.bn[rk] || k > o.en[rk]) return 0.0;
            return o.rhat[o.id(i, j, k)];
        };
        for (int k = o.bn[rk]; k <= o.en[rk]; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 1; ++i)
                    o.rhat[o.id(i, j, k)] =
                        -w * (in[o.id(i, j, k)] + o.Aw * R(i - 1, j, k) + o.As * R(i, j - 1, k) + o.Ab[k] * R(i, j, k - 1)) *
                        o.rAp[k];
        for (int k = o.bn[rk]; k <= o.en[rk]; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 1; ++i) o.rhat[o.id(i, j, k)] = (scale_w * o.Ap[k]) * o.rhat[o.id(i, j, k)];
        for (int k = o.en[rk]; k >= o.bn[rk]; --k)
            for (int j = ny - 1; j >= 2; --j)
                for (int i = nx - 1; i >= 2; --i)
                    o.rhat[o.id(i, j, k)] =
                        -w * (o.rhat[o.id(i, j, k)] + o.Aw * R(i + 1, j, k) + o.As * R(i, j + 1, k) + o.At[k] * R(i, j, k + 1)) *
                        o.rAp[k];
    }
}

// sum over the interior of all slabs of a*b: per-rank partial, rank order
double dot(const Oracle& o, const std::vector<double>& a, const std::vector<double>& b) {
    double tot = 0.0;
    std::vector<double> part(o.P, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int rk = 0; rk < o.P; ++rk) {
        double s = 0.0;
        for (int k = o.bn[rk]; k <= o.en[rk]; ++k)
            for (int j = 2; j <= o.ny - 1; ++j)
                for (int i = 2; i <= o.nx - 1; ++i) s = s + a[o.id(i, j, k)] * b[o.id(i, j, k)];
        part[rk] = s;
    }
    for (int rk = 0; rk < o.P; ++rk) tot += part[rk];
    return tot;
}

int gmres(Oracle& o, const std::vector<int32_t>* rp, std::vector<int32_t>& counts, int& restarts, int& iters,
          double& resid) {
    const int nx = o.nx, ny = o.ny, nz = o.nz, kmax = o.c.kmax, K1 = kmax + 1;
    auto H = [&](int a, int b) -> double& { return o.h[(size_t)(a - 1) + (size_t)K1 * (b - 1)]; };
    // PCorr faces to zero (:940-950)
    for (int k = 1; k <= nz; ++k) {
        for (int j = 1; j <= ny; ++j) { o.PC[o.id(1, j, k)] = 0.0; o.PC[o.id(nx, j, k)] = 0.0; }
        for (int i = 1; i <= nx; ++i) { o.PC[o.id(i, 1, k)] = 0.0; o.PC[o.id(i, ny, k)] = 0.0; }
    }
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) { o.PC[o.id(i, j, 1)] = 0.0; o.PC[o.id(i, j, nz)] = 0.0; }
    double sumav = 1.0, sumnor = 0.0;
    int m = 0;
    restarts = 0; iters = 0;
    int nrest_replay = rp ? (*rp)[0] : 0;
    int status = TBL_OK;
    while (rp ? (m < nrest_replay) : ((sumav > o.c.errtol) && (m < o.c.mmax))) {
        m = m + 1;
        std::fill(o.h.begin(), o.h.end(), 0.0);
        for (auto& v : o.V) std::fill(v.begin(), v.end(), 0.0);
        std::fill(o.cs.begin(), o.cs.end(), 0.0); std::fill(o.sn.begin(), o.sn.end(), 0.0);
        std::fill(o.g.begin(), o.g.end(), 0.0); std::fill(o.y.begin(), o.y.end(), 0.0);
        // r = Q8 - L7 PCorr (:995-1008)
#pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 1; ++i)
                    o.r[o.id(i, j, k)] = o.Q8[o.id(i, j, k)] - (lap(o, o.PC, i, j, k));
        ssor(o, o.r);
#pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 1; ++i) o.r[o.id(i, j, k)] = o.rhat[o.id(i, j, k)];
        double rho = std::sqrt(dot(o, o.r, o.r));
        if (m == 1) {
            sumnor = rho;
            if (std::isnan(rho)) { status = TBL_ERR_NAN; resid = rho; break; }
            if (!(rho > 0.0)) { status = TBL_ERR_ZERO_RHS; resid = 0.0; break; }
        }
        sumav = rho / sumnor;
        o.g[0] = rho;
#pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 1; ++i) o.V[0][o.id(i, j, k)] = o.r[o.id(i, j, k)] / rho;
        int kit = 0;
        int kit_target = rp ? (*rp)[m] : 0;
        while (rp ? (kit < kit_target) : ((sumav > o.c.errtol) && (kit < kmax))) {
            kit = kit + 1;
            std::vector<double>& vk = o.V[kit - 1];
            std::vector<double>& vn = o.V[kit];
    #pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
                for (int j = 2; j <= ny - 1; ++j)
                    for (int i = 2; i <= nx - 1; ++i) vn[o.id(i, j, k)] = lap(o, vk, i, j, k);
            ssor(o, vn);
    #pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
                for (int j = 2; j <= ny - 1; ++j)
                    for (int i = 2; i <= nx - 1; ++i) vn[o.id(i, j, k)] = o.rhat[o.id(i, j, k)];
            // modified Gram-Schmidt (:1140-1150)
            for (int kk = 1; kk <= kit; ++kk) {
                H(kk, kit) = dot(o, o.V[kk - 1], vn);
                double hk = H(kk, kit);
                const std::vector<double>& vv = o.V[kk - 1];
        #pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
                    for (int j = 2; j <= ny - 1; ++j)
                        for (int i = 2; i <= nx - 1; ++i) vn[o.id(i, j, k)] = vn[o.id(i, j, k)] - hk * vv[o.id(i, j, k)];
            }
            H(kit + 1, kit) = std::sqrt(dot(o, vn, vn));
            if (H(kit + 1, kit) > 0.0 || H(kit + 1, kit) < 0.0) {
                double hh = H(kit + 1, kit);
        #pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
                    for (int j = 2; j <= ny - 1; ++j)
                        for (int i = 2; i <= nx - 1; ++i) vn[o.id(i, j, k)] = vn[o.id(i, j, k)] / hh;
            }
            // Givens (:1165-1189)
            if (kit > 1) {
                for (int i = 1; i <= kit - 1; ++i) {
                    double hik = o.cs[i - 1] * H(i, kit) - o.sn[i - 1] * H(i + 1, kit);
                    double hipk = o.sn[i - 1] * H(i, kit) + o.cs[i - 1] * H(i + 1, kit);
                    H(i, kit) = hik;
                    H(i + 1, kit) = hipk;
                }
            }
            double nu = std::sqrt(H(kit, kit) * H(kit, kit) + H(kit + 1, kit) * H(kit + 1, kit));
            if (nu > 0.0) {
                o.cs[kit - 1] = H(kit, kit) / nu;
                o.sn[kit - 1] = -H(kit + 1, kit) / nu;
                H(kit, kit) = o.cs[kit - 1] * H(kit, kit) - o.sn[kit - 1] * H(kit + 1, kit);
                H(kit + 1, kit) = 0;
                double gk = o.cs[kit - 1] * o.g[kit - 1] - o.sn[kit - 1] * o.g[kit];
                double gkp = o.sn[kit - 1] * o.g[kit - 1] + o.cs[kit - 1] * o.g[kit];
                o.g[kit - 1] = gk;
                o.g[kit] = gkp;
            }
            rho = std::fabs(o.g[kit]);
            sumav = rho / sumnor;
        }
        iters += kit;
        counts.push_back(kit);
        if (kit == 0) { resid = sumav; continue; }
        // back substitution (:1193-1200)
        o.y[kit - 1] = o.g[kit - 1] / H(kit, kit);
        for (int i = kit - 1; i >= 1; --i) {
            o.y[i - 1] = o.g[i - 1];
            for (int k = i + 1; k <= kit; ++k) o.y[i - 1] = o.y[i - 1] - H(i, k) * o.y[k - 1];
            o.y[i - 1] = o.y[i - 1] / H(i, i);
        }
        // PCorr += sum_i v_i y_i (:1202-1205)
        for (int i = 1; i <= kit; ++i) {
            const std::vector<double>& vv = o.V[i - 1];
            double yi = o.y[i - 1];
    #pragma omp parallel for schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
                for (int j = 2; j <= ny - 1; ++j)
                    for (int ii = 2; ii <= nx - 1; ++ii)
                        o.PC[o.id(ii, j, k)] = o.PC[o.id(ii, j, k)] + vv[o.id(ii, j, k)] * yi;
        }
        resid = sumav;
    }
    restarts = m;
    if (status == TBL_OK && !rp && sumav > o.c.errtol) status = TBL_ERR_NOT_CONVERGED;
    return status;
}

// ------------------------------------------------ a7+a8: projection and BCs
// dnstbl2/dnstbl.f90:1245-1469
void project_bcs(Oracle& o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    std::vector<double>& PC = o.PC;
    // p' boundary extrapolation (:1245-1262)
    for (int j = 2; j <= ny - 1; ++j)
        for (int i = 1; i <= nx; ++i)
            PC[o.id(i, j, 1)] = ((4.0 * PC[o.id(i, j, 2)]) - PC[o.id(i, j, 3)]) / 3.0;
    for (int j = 2; j <= ny - 1; ++j)
        for (int i = 1; i <= nx; ++i)
            PC[o.id(i, j, nz)] = (5.0 * PC[o.id(i, j, nz - 1)] + (-4.0 * PC[o.id(i, j, nz - 2)] + PC[o.id(i, j, nz - 3)])) / 2.0;
    for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
            PC[o.id(i, 1, k)] = PC[o.id(i, ny - 1, k)];
            PC[o.id(i, ny, k)] = PC[o.id(i, 2, k)];
        }
    for (int k = 1; k <= nz; ++k)
        for (int j = 2; j <= ny - 1; ++j)
            PC[o.id(1, j, k)] = (4.0 * PC[o.id(2, j, k)] - PC[o.id(3, j, k)]) / 3.0;
    for (int k = 1; k <= nz; ++k)
        for (int j = 2; j <= ny - 1; ++j)
            PC[o.id(nx, j, k)] = (5.0 * PC[o.id(nx - 1, j, k)] + (-4.0 * PC[o.id(nx - 2, j, k)] + PC[o.id(nx - 3, j, k)])) / 2.0;
    // P += p' (:1268), U -= dt grad p' (:1271-1314)
    const double dt = o.c.dt;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nz - 1; ++k)
        for (int j = 2; j <= ny - 1; ++j)
            for (int i = 2; i <= nx - 1; ++i) {
                size_t p = o.id(i, j, k);
                o.P_[p] = o.P_[p] + PC[p];
                double g1 = 0.5 * (PC[o.id(i + 1, j, k)] - PC[o.id(i - 1, j, k)]) * (o.invdx);
                double g2 = 0.5 * (PC[o.id(i, o.jp1(j), k)] - PC[o.id(i, o.jm1(j), k)]) * (o.invdy);
                double g3 = 0.5 * (PC[o.id(i, j, k + 1)] - PC[o.id(i, j, k - 1)]) * (o.invdxi * o.jac[k]);
                o.U[0][p] = o.U[0][p] - (dt * g1);
                o.U[1][p] = o.U[1][p] - (dt * g2);
                o.U[2][p] = o.U[2][p] - (dt * g3);
            }
    // velocity BCs (:1317-1342)
    for (int cc = 0; cc < 3; ++cc)
        for (int j = 2; j <= ny - 1; ++j)
            for (int i = 1; i <= nx; ++i) o.U[cc][o.id(i, j, 1)] = 0.0;
    for (int cc = 0; cc < 3; ++cc)
        for (int j = 2; j <= ny - 1; ++j)
            for (int i = 1; i <= nx; ++i)
                o.U[cc][o.id(i, j, nz)] = (4.0 * o.U[cc][o.id(i, j, nz - 1)] - o.U[cc][o.id(i, j, nz - 2)]) / 3.0;
    for (int cc = 0; cc < 3; ++cc)
        for (int k = 1; k <= nz; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                o.U[cc][o.id(nx, j, k)] = (4.0 * o.U[cc][o.id(nx - 1, j, k)] - o.U[cc][o.id(nx - 2, j, k)]) / 3.0;
    // pressure BCs: wall (:1352-1378)
    const std::vector<double>&U1 = o.U[0], &U2 = o.U[1], &U3 = o.U[2];
    const double df1 = o.df1, df2 = o.df2, re = o.c.re;
    for (int j = 2; j <= ny - 1; ++j)
        for (int i = 2; i <= nx - 1; ++i) {
            double fder = (U3[o.id(i, j, 2)] - U3[o.id(i, j, 1)]) / df1;
            double d3 = U3[o.id(i, j, 1)] * fder;
            double g1 = (U3[o.id(i - 1, j, 1)] + U3[o.id(i + 1, j, 1)] - 2 * U3[o.id(i, j, 1)]) / (o.dx * o.dx);
            double g2 = (U3[o.id(i, j - 1, 1)] + U3[o.id(i, j + 1, 1)] - 2 * U3[o.id(i, j, 1)]) / (o.dy * o.dy);
            double g3 = (2.0 * df1 * U3[o.id(i, j, 3)] - 2.0 * df2 * U3[o.id(i, j, 2)] + 2.0 * (df2 - df1) * U3[o.id(i, j, 1)]) /
                        (df1 * (df2 * df2) - (df2 * (df1 * df1)));
            double flux = -d3 + ((g1 + g2 + g3) / re);
            o.P_[o.id(i, j, 1)] = o.P_[o.id(i, j, 2)] - flux * df1;
        }
    // top (:1384-1408)
    for (int j = 2; j <= ny - 1; ++j)
        for (int i = 2; i <= nx - 1; ++i) {
            double fder = (11.0 * U3[o.id(i, j, nz)] - 18.0 * U3[o.id(i, j, nz - 1)] + 9.0 * U3[o.id(i, j, nz - 2)] -
                           2.0 * U3[o.id(i, j, nz - 3)]) /
                          (6.0 * o.dxi);
            double d3 = (fder * o.jac[nz]);
            o.P_[o.id(i, j, nz)] = (d3 / re);
        }
    // outflow (:1412-1431)
    for (int k = 2; k <= nz - 1; ++k)
        for (int j = 2; j <= ny - 1; ++j)
            o.P_[o.id(nx, j, k)] = ((3.0 * U1[o.id(nx, j, k)] - 4.0 * U1[o.id(nx - 1, j, k)] + U1[o.id(nx - 2, j, k)]) /
                                   (2.0 * o.dx * re));
    // inflow (:1433-1461)
    for (int k = 2; k <= nz - 1; ++k)
        for (int j = 2; j <= ny - 1; ++j) {
            double d1 = U1[o.id(1, j, k)] * ((U1[o.id(2, j, k)] - U1[o.id(1, j, k)]) / (o.dx));
            double d2 = U2[o.id(1, j, k)] * ((U1[o.id(1, j + 1, k)] - U1[o.id(1, j - 1, k)]) / (2.0 * o.dy));
            double d3 = U3[o.id(1, j, k)] * ((U1[o.id(1, j, k + 1)] - U1[o.id(1, j, k - 1)]) / (2.0 * o.dxi));
            double g1 = (U1[o.id(1, j, k)] + U1[o.id(3, j, k)] - 2 * U1[o.id(2, j, k)]) / (o.dx * o.dx);
            double g2 = (U1[o.id(1, j + 1, k)] + U1[o.id(1, j - 1, k)] - 2 * U1[o.id(1, j, k)]) / (o.dy * o.dy);
            double fder, g3;
            if (k <= 2) {
                fder = (U1[o.id(1, j, k + 1)] - U1[o.id(1, j, k)]) / o.dxi;
                g3 = (U1[o.id(1, j, k + 2)] - 2.0 * U1[o.id(1, j, k + 1)] + U1[o.id(1, j, k)]) / (o.dxi * o.dxi);
            } else if (k >= nz - 1) {
                fder = (U1[o.id(1, j, k)] - U1[o.id(1, j, k - 1)]) / o.dxi;
                g3 = (U1[o.id(1, j, k - 2)] - 2.0 * U1[o.id(1, j, k - 1)] + U1[o.id(1, j, k)]) / (o.dxi * o.dxi);
            } else {
                fder = (U1[o.id(1, j, k + 1)] - U1[o.id(1, j, k - 1)]) / (2.0 * o.dxi);
                g3 = (-2 * U1[o.id(1, j, k)] + U1[o.id(1, j, k + 1)] + U1[o.id(1, j, k - 1)]) / (o.dxi * o.dxi);
            }
            double J = o.jac[k];
            g3 = (g3 * (J * J)) - ((o.jac2[k - 1] * fder) * (J * J * J));
            double fder2 = (U1[o.id(1, j, k)] - o.Uold1[o.idp(j, k)]) / o.c.dt;
            o.P_[o.id(1, j, k)] =
                ((2 * o.dx * ((fder2 + d1 + d2 + d3 * J) - ((g1 + g2 + g3) / re))) - 0.0 - o.P_[o.id(3, j, k)] +
                 (4 * o.P_[o.id(2, j, k)])) /
                3.0;
        }
    // spanwise periodic copies (:1465-1469)
    for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
            for (int cc = 0; cc < 3; ++cc) {
                o.U[cc][o.id(i, 1, k)] = o.U[cc][o.id(i, ny - 1, k)];
                o.U[cc][o.id(i, ny, k)] = o.U[cc][o.id(i, 2, k)];
            }
            o.P_[o.id(i, 1, k)] = o.P_[o.id(i, ny - 1, k)];
            o.P_[o.id(i, ny, k)] = o.P_[o.id(i, 2, k)];
        }
}

// --------------------------------------------------- diagnostics (next row)
// divergence printout (:1526-1577)
double div_diag(const Oracle& o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    const std::vector<double>&U1 = o.U[0], &U2 = o.U[1], &U3 = o.U[2];
    double tot = 0.0;
    for (int rk = 0; rk < o.P; ++rk) {
        double tmp = 0.0;
        for (int k = o.bn[rk]; k <= o.en[rk]; ++k)
            for (int j = 2; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 1; ++i) {
                    double d1, d2, d3;
                    if (i == 2 || i == nx - 1) d1 = (U1[o.id(i + 1, j, k)] - U1[o.id(i - 1, j, k)]) * (0.5 * o.invdx);
                    else d1 = ((U1[o.id(i - 2, j, k)] - 8 * U1[o.id(i - 1, j, k)] + 8 * U1[o.id(i + 1, j, k)] - U1[o.id(i + 2, j, k)]) * (o.c12 * o.invdx));
                    if (j == 2 || j == ny - 1) d2 = (U2[o.id(i, o.jp1(j), k)] - U2[o.id(i, o.jm1(j), k)]) * (0.5 * o.invdy);
                    else d2 = ((U2[o.id(i, o.jm2(j), k)] - 8 * U2[o.id(i, o.jm1(j), k)] + 8 * U2[o.id(i, o.jp1(j), k)] - U2[o.id(i, o.jp2(j), k)]) * (o.c12 * o.invdy));
                    if (k <= 2 || k >= nz - 1) d3 = ((U3[o.id(i, j, k + 1)] - U3[o.id(i, j, k - 1)]) * (0.5 * o.invdxi));
                    else d3 = ((U3[o.id(i, j, k - 2)] - 8 * U3[o.id(i, j, k - 1)] + 8 * U3[o.id(i, j, k + 1)] - U3[o.id(i, j, k + 2)]) * (o.c12 * o.invdxi));
                    tmp = tmp + (d1 + d2 + (d3 * o.jac[k]));
                }
        tot += tmp;
    }
    const double q = std::fabs(tot) / ((double)(ny - 2) * (nx - 2) * (nz - 2));
    return is_orig(o) ? std::sqrt(q) : q;  // originalTBL prints the square root (fnldnstbl.f90:1586)
}

// Mass flux through five cross-stream planes (:1578-1594): per rank the cell
// sums over its k range (rank 0 also the first cell layer, the last rank not
// its top face), ranks summed in order, divided by the area Av (:448).
// Plane indices are the reference's literals (:95), clamped to nx-1.
// dnssetbl sums each slab's own planes only and divides by
// (x3(nz-1)-x3(2))(x2(ny-1)-x2(2)) (dnssetbl.f90:884-896).
void mass_flux(Oracle& o) {
    static const int plane[5] = {5, 20, 40, 60, 85};
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    const double Av = is_sete(o) ? (o.x3[nz - 2] - o.x3[1]) * (o.x2[ny - 2] - o.x2[1])
                                 : o.x3[nz - 1] * (o.x2[ny - 2] - o.x2[1]);
    for (int q = 0; q < 5; ++q) {
        const int ip = plane[q] < nx - 1 ? plane[q] : nx - 1;
        double tot = 0.0;
        for (int rk = 0; rk < o.P; ++rk) {
            const int k0 = (rk == 0 && !is_sete(o)) ? o.bn[rk] - 1 : o.bn[rk];
            double ub = 0.0;
            for (int k = k0; k <= o.en[rk]; ++k)
                for (int j = 2; j <= ny - 1; ++j) {
                    const int jp1 = j == ny - 1 ? 2 : j + 1;
                    const double dAv = o.dy * (o.x3[k] - o.x3[k - 1]);  // x3(k+1) - x3(k), 1-based
                    ub = ub + (0.25 * (o.U[0][o.id(ip, j, k)] + o.U[0][o.id(ip, jp1, k)] + o.U[0][o.id(ip, j, k + 1)] +
                                       o.U[0][o.id(ip, jp1, k + 1)]) * (dAv));
                }
            tot += ub;
        }
        o.ubulk[q] = tot / Av;
    }
}

// Wall shear (:1616-1681): span sum of (dw/dx + du/dz)/Re at the wall per
// column, accumulated every step in sumxz; every 500 steps the window mean is
// written (kept here as tauw_window) and the accumulator restarts.
void wall_shear(Oracle& o, double* tau_out = nullptr) {
    const int nx = o.nx, ny = o.ny;
    const double d1 = o.x3[1] - o.x3[0], d2 = o.x3[2] - o.x3[0];
    const std::vector<double>&U1 = o.U[0], &U3 = o.U[2];
    for (int i = 2; i <= nx - 1; ++i) {
        double tauxz = 0.0;
        for (int j = 2; j <= ny - 1; ++j) {
            double mfb1;
            if (i <= 3 || i >= nx - 2)
                mfb1 = (U3[o.id(i + 1, j, 1)] - U3[o.id(i - 1, j, 1)]) / (2.0 * o.dx);
            else
                mfb1 = (-U3[o.id(i - 3, j, 1)] + (9.0 * U3[o.id(i - 2, j, 1)]) - (45.0 * U3[o.id(i - 1, j, 1)]) +
                        (45.0 * U3[o.id(i + 1, j, 1)]) - (9.0 * U3[o.id(i + 2, j, 1)]) + U3[o.id(i + 3, j, 1)]) /
                       (60.0 * o.dx);
            const double fder = (((U1[o.id(i, j, 3)] - U1[o.id(i, j, 1)]) * (d1 * d1)) +
                                 ((U1[o.id(i, j, 1)] - U1[o.id(i, j, 2)]) * (d2 * d2))) /
                                ((d2 * (d1 * d1)) - ((d2 * d2) * d1));
            tauxz = tauxz + ((mfb1 + fder) / o.c.re);
        }
        if (tau_out) { tau_out[i - 1] = tauxz; continue; }
        o.sumxz[i - 1] = tauxz + o.sumxz[i - 1];
    }
    if (tau_out) return;
    const int win = is_orig(o) ? 1000 : 500;  // originalTBL: 1000 steps (fnldnstbl.f90:1679-1681)
    if (o.nstep % win == 0) {
        for (int i = 2; i <= nx - 1; ++i) o.tauw_window[i - 1] = o.sumxz[i - 1] / (double)win;
        for (double& v : o.sumxz) v = 0.0;
    }
}

// --------------------------------------------------- a9: statistics per step
// Ufluc per step (:1707-1722), KE (:1724-1741).  dnssetbl: when
// cnt > freqTimAvg, cnt counting this run's steps including the current one,
// over i = 2..nx-1 (dnssetbl.f90:1223-1254; its blow-up test also reads the
// never-refreshed columns i = 1 and nx, left out here).
// `run_steps` counts this run's steps including the current one.
void fluc_ke(Oracle& o, int run_steps, double& ke, int& blowup) {
    const int nx = o.nx, ny = o.ny, nz = o.nz, irec = o.c.irec;
    ke = 0.0; blowup = 0;
    const bool on = is_sete(o) ? (run_steps > o.c.recycle_after) : (o.nstep > o.c.recycle_after);
    const int i0 = is_sete(o) ? 2 : 1, i1 = is_sete(o) ? nx - 1 : nx;
    if (on) {
        double ke1tot = 0.0;
        for (int rk = 0; rk < o.P; ++rk) {
            double ke1 = 0.0;
            for (int k = o.bn[rk]; k <= o.en[rk]; ++k)
                for (int j = 2; j <= ny - 1; ++j)
                    for (int i = i0; i <= i1; ++i) {
                        double f1 = o.U[0][o.id(i, j, k)] - o.usum2[o.id2(i, k)];
                        double f2 = o.U[1][o.id(i, j, k)] - o.vsum2[o.id2(i, k)];
                        double f3 = o.U[2][o.id(i, j, k)] - o.wsum2[o.id2(i, k)];
                        ke1 = ke1 + f1 * f1 + f2 * f2 + f3 * f3;
                        if (f1 > 25.0 || f2 > 25.0 || f3 > 25.0) blowup = 1;
                        if (i == irec) {
                            o.ufl_live[0][o.idp(j, k)] = f1;
                            o.ufl_live[1][o.idp(j, k)] = f2;
                            o.ufl_live[2][o.idp(j, k)] = f3;
                        }
                    }
            ke1tot += ke1;
        }
        ke = ke1tot / ((double)nx * (ny - 2) * (nz - 2));
        for (int cc = 0; cc < 3; ++cc) {
            const std::vector<double>& s = cc == 0 ? o.usum2 : (cc == 1 ? o.vsum2 : o.wsum2);
            o.usum2_last_fluc[cc] = s;
        }
        o.fluc_updated = true;
    }
}

// Statistics (:1902-1993): span averages of the midpoint values weighted
// dA/A; dnssetbl sums them unweighted and divides by ny-2
// (dnssetbl.f90:936-983).
void accumulate_stats(Oracle& o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    o.cont = o.cont + 1;
    if (o.nstep % o.c.istat == 0) {
        o.nstat += 1;
        const bool unw = is_sete(o);
        const double dA = o.dy;
        const double A = unw ? (double)(ny - 2) : o.x2[ny - 1] - o.x2[1];
#pragma omp parallel for schedule(static)
        for (int i = 1; i <= nx; ++i)
            for (int k = 1; k <= nz; ++k) {
                double su_, sv_, sw_, tu = 0, tv = 0, tw = 0, tuu = 0, tvv = 0, tww = 0, tuv = 0, tuw = 0, tvw = 0;
                for (int j = 2; j <= ny - 1; ++j) {
                    int jp = o.jp1(j);
                    su_ = 0.50 * (o.U[0][o.id(i, j, k)] + o.U[0][o.id(i, jp, k)]);
                    sv_ = 0.50 * (o.U[1][o.id(i, j, k)] + o.U[1][o.id(i, jp, k)]);
                    sw_ = 0.50 * (o.U[2][o.id(i, j, k)] + o.U[2][o.id(i, jp, k)]);
                    if (unw) {
                        tu = tu + su_; tv = tv + sv_; tw = tw + sw_;
                        tuu = tuu + su_ * su_; tvv = tvv + sv_ * sv_; tww = tww + sw_ * sw_;
                        tuv = tuv + su_ * sv_; tuw = tuw + su_ * sw_; tvw = tvw + sv_ * sw_;
                        continue;
                    }
                    tu = tu + (su_ * dA); tv = tv + (sv_ * dA); tw = tw + (sw_ * dA);
                    tuu = tuu + (su_ * su_ * dA); tvv = tvv + (sv_ * sv_ * dA); tww = tww + (sw_ * sw_ * dA);
                    tuv = tuv + (su_ * sv_ * dA); tuw = tuw + (su_ * sw_ * dA); tvw = tvw + (sv_ * sw_ * dA);
                }
                size_t q = o.id2(i, k);
                o.usum[q] += (tu / A); o.vsum[q] += (tv / A); o.wsum[q] += (tw / A);
                o.uusum[q] += (tuu / A); o.vvsum[q] += (tvv / A); o.wwsum[q] += (tww / A);
                o.uvsum[q] += (tuv / A); o.uwsum[q] += (tuw / A); o.vwsum[q] += (tvw / A);
            }
    }
}

// ------------------------------------------- a10: rescaling bookkeeping
// Boundary-layer thickness: the first x3(k) where the time mean reaches
// 0.99 Ue (dnstbl2/dnstbl.f90:2150-2158).
static void bl_thickness(Oracle& o) {
    const int nx = o.nx, nz = o.nz;
    const double ue = o.c.ue;
    for (int i = 1; i <= nx; ++i)
        for (int k = 1; k <= nz; ++k)
            if (o.usum2[o.id2(i, k)] >= (0.99 * ue)) { o.bltkns[i - 1] = o.x3[k - 1]; break; }
}

// Displacement and momentum thickness, shape factor and Re_theta per i
// (dnstbl2/dnstbl.f90:2232-2256): left sums of (1 - u/Ue) and
// u/Ue (1 - u/Ue) over the cells [x3(k), x3(k+1)], the displacement sum
// stopping after the cell that starts at bltkns, the momentum sum after the
// first cell starting at or above it.  The reference accumulates into
// arrays that it zeroes only after the first use (:218-221, :2270-2271);
// these sums start at zero.
static void integral_thicknesses(Oracle& o) {
    const int nx = o.nx, nz = o.nz;
    const double ue = o.c.ue, re = o.c.re;
    for (int i = 1; i <= nx; ++i) {
        double ds = 0.0;
        for (int k = 1; k <= nz - 1; ++k) {
            ds = ds + ((1.0 - (o.usum2[o.id2(i, k)] / ue)) * (o.x3[k] - o.x3[k - 1]));
            if (o.x3[k - 1] == o.bltkns[i - 1]) break;
        }
        o.deltastar[i - 1] = ds;
        double th = 0.0;
        for (int k = 1; k <= nz - 1; ++k) {
            th = th + ((o.usum2[o.id2(i, k)] / ue) * (1.0 - (o.usum2[o.id2(i, k)] / ue)) * (o.x3[k] - o.x3[k - 1]));
            if (o.x3[k - 1] >= o.bltkns[i - 1]) break;
        }
        o.theta[i - 1] = th;
        o.Ht[i - 1] = ds / th;
        o.Reth[i - 1] = th * re * ue;
    }
}

// dnstbl2/dnstbl.f90:2084-2365
void rescale(Oracle& o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz, irec = o.c.irec;
    const double cum = (double)o.c.cum, ue = o.c.ue, re = o.c.re;
    {  // the averaged sums of the means/medians/taustress files (:2028-2048)
        const std::vector<double>* src[9] = {&o.usum, &o.vsum, &o.wsum, &o.uusum, &o.vvsum, &o.wwsum,
                                             &o.uvsum, &o.uwsum, &o.vwsum};
        const size_t n2 = (size_t)nx * nz;
        for (int m = 0; m < 9; ++m)
            for (size_t q = 0; q < n2; ++q) o.avg[m * n2 + q] = ((*src[m])[q] / cum);
    }
    for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
            size_t q = o.id2(i, k);
            o.usum2[q] = (o.usum[q] / cum);
            o.vsum2[q] = (o.vsum[q] / cum);
            o.wsum2[q] = (o.wsum[q] / cum);
        }
    double utau1 = std::sqrt(((o.usum2[o.id2(1, 2)] - o.usum2[o.id2(1, 1)]) / (o.x3[1] - o.x3[0])) / re);
    double utau2 = std::sqrt(((o.usum2[o.id2(irec, 2)] - o.usum2[o.id2(irec, 1)]) / (o.x3[1] - o.x3[0])) / re);
    o.lamda = (utau1) / (utau2);
    bl_thickness(o);
    o.lamda03 = o.bltkns[irec - 1] / o.bltkns[0];
    for (int i = 1; i <= nx; ++i)
        for (int k = 1; k <= nz; ++k) {
            double xb = o.x3[k - 1] / o.bltkns[i - 1];
            o.Wt[o.id2(i, k)] =
                0.5 * (1 + (std::tanh((4.0 * ((xb)-0.2)) / ((1 - 2.0 * 0.2) * (xb) + 0.2)) / std::tanh(4.0)));
        }
    std::vector<double> eta(nz + 1, 0.0), zrecy(nz + 1, 0.0);
    for (int k = 1; k <= nz; ++k) o.newk[k - 1] = nz - 1;
    for (int k = 1; k <= nz - 1; ++k) {
        if (o.Wt[o.id2(irec, k)] <= 0.99) { o.ksep = k; eta[k] = o.lamda; }
        else eta[k] = o.lamda03;
    }
    for (int k = 1; k <= nz - 1; ++k) zrecy[k] = eta[k] * o.x3[k - 1];
    int counter = 1;
    for (int k = 1; k <= nz - 1; ++k)
        if (counter <= o.ksep)
            if (o.x3[k - 1] >= zrecy[counter]) { o.newk[counter - 1] = k; counter = counter + 1; }
    counter = o.ksep + 1;
    for (int k = o.ksep + 1; k <= nz - 1; ++k)
        if (counter <= nz - 1)
            if (o.x3[k - 1] >= zrecy[counter]) { o.newk[counter - 1] = k; counter = counter + 1; }
    integral_thicknesses(o);
    // refresh Ufluc(irec,:,k,:) on every rank's own slab (:2341-2349);
    // dnssetbl refreshes rank 0's slab only (dnssetbl.f90:1016, :1033-1041)
    const int kr0 = is_sete(o) ? o.bn[0] : 2, kr1 = is_sete(o) ? o.en[0] : nz - 1;
    for (int k = kr0; k <= kr1; ++k)
        for (int j = 2; j <= ny - 1; ++j) {
            o.ufl_live[0][o.idp(j, k)] = o.U[0][o.id(irec, j, k)] - o.usum2[o.id2(irec, k)];
            o.ufl_live[1][o.idp(j, k)] = o.U[1][o.id(irec, j, k)] - o.vsum2[o.id2(irec, k)];
            o.ufl_live[2][o.idp(j, k)] = o.U[2][o.id(irec, j, k)] - o.wsum2[o.id2(irec, k)];
        }
    for (auto* v : {&o.usum, &o.vsum, &o.wsum, &o.uusum, &o.vvsum, &o.wwsum, &o.uvsum, &o.uwsum, &o.vwsum})
        std::fill(v->begin(), v->end(), 0.0);
}

int one_step(Oracle& o, tbl_step_stats* st) {
    tbl_step_stats s{};
    o.time = o.time + o.c.dt;
    o.nstep = o.nstep + 1;
    for (int k = 1; k <= o.nz; ++k)
        for (int j = 1; j <= o.ny; ++j) o.Uold1[o.idp(j, k)] = o.U[0][o.id(1, j, k)];
    if (o.nstep > o.c.recycle_after) inflow(o);
    conv_q(o);
    // replay record
    const bool replay = (o.c.flags & TBL_FLAG_REPLAY) != 0;
    int rs[3];
    std::vector<int32_t> rrec;
    if (replay) {
        if (o.replay_pos + 4 > o.replay.size()) return TBL_ERR_REPLAY;
        rs[0] = o.replay[o.replay_pos]; rs[1] = o.replay[o.replay_pos + 1]; rs[2] = o.replay[o.replay_pos + 2];
        int nr = o.replay[o.replay_pos + 3];
        if (o.replay_pos + 4 + nr > o.replay.size()) return TBL_ERR_REPLAY;
        rrec.push_back(nr);
        for (int q = 0; q < nr; ++q) rrec.push_back(o.replay[o.replay_pos + 4 + q]);
        o.replay_pos += 4 + nr;
    }
    gs_solve(o, replay ? rs : nullptr, s.gs_sweeps, s.gs_resid);
    divergence(o);
    std::vector<int32_t> kits;
    int status = gmres(o, replay ? &rrec : nullptr, kits, s.gmres_restarts, s.gmres_iters, s.gmres_resid);
    if (status == TBL_ERR_ZERO_RHS || status == TBL_ERR_NAN) return status;
    if (o.c.flags & TBL_FLAG_PPE_RESIDUAL) {
        double num = 0.0, den = 0.0;
        for (int k = 2; k <= o.nz - 1; ++k)
            for (int j = 2; j <= o.ny - 1; ++j)
                for (int i = 2; i <= o.nx - 1; ++i) {
                    double rr = lap(o, o.PC, i, j, k) - o.Q8[o.id(i, j, k)];
                    num += rr * rr;
                    den += o.Q8[o.id(i, j, k)] * o.Q8[o.id(i, j, k)];
                }
        s.ppe_rel_resid = den > 0 ? std::sqrt(num / den) : 0.0;
    }
    project_bcs(o);
    s.div_diag = div_diag(o);
    mass_flux(o);
    wall_shear(o);
    int blow = 0;
    s.cum_step = 0;
    if (is_sete(o)) {
        // dnssetbl: statistics, rescaling every freqTimAvg steps of nstep, then
        // the fluctuations and KE (dnssetbl.f90:936, :986, :1223)
        accumulate_stats(o);
        if (o.nstep % o.c.cum == 0) { rescale(o); s.cum_step = 1; }
        fluc_ke(o, o.cont, s.ke, blow);
    } else {
        fluc_ke(o, o.cont + 1, s.ke, blow);
        accumulate_stats(o);
        if (o.cont % o.c.cum == 0) { rescale(o); s.cum_step = 1; }
    }
    o.cnt2 = o.cnt2 + 1;  // end of the step (fnldnstbl.f90:2382, dnstbl.f90:2349)
    o.last_counts.clear();
    o.last_counts.push_back(s.gs_sweeps[0]); o.last_counts.push_back(s.gs_sweeps[1]); o.last_counts.push_back(s.gs_sweeps[2]);
    o.last_counts.push_back((int32_t)kits.size());
    for (int q : kits) o.last_counts.push_back(q);
    s.nstep = o.nstep; s.lamda = o.lamda; s.time = o.time;
    bool bad = false;
    for (int cc = 0; cc < 3 && !bad; ++cc)
        for (size_t q = 0; q < o.N; q += 1) if (!std::isfinite(o.U[cc][q])) { bad = true; break; }
    if (bad) status = TBL_ERR_NAN;
    else if (blow) status = TBL_ERR_BLOWUP;
    else if (status == TBL_OK)
        for (int cc = 0; cc < 3; ++cc) if (s.gs_sweeps[cc] >= o.c.mmax && !replay) status = TBL_ERR_NOT_CONVERGED;
    s.status = status;
    if (st) *st = s;
    return status;
}

}  // namespace

extern "C" {

struct orc_handle { Oracle o; };

int orc_create(const tbl_config* cfg, const tbl_mesh* mesh, orc_handle** out) {
    if (!cfg || !mesh || !out) return TBL_ERR_BAD_ARG;
    orc_handle* h = new (std::nothrow) orc_handle();
    if (!h) return TBL_ERR_BAD_ARG;
    int s = setup(h->o, cfg, mesh);
    if (s != TBL_OK) { delete h; return s; }
    *out = h;
    return TBL_OK;
}

int orc_upload_state(orc_handle* h, const tbl_state* st) {
    if (!h || !st || !st->u || !st->v || !st->w || !st->p) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    o.sumxz.assign(o.nx, 0.0);
    o.tauw_window.assign(o.nx, 0.0);
    for (double& b : o.ubulk) b = 0.0;
    std::memcpy(o.U[0].data(), st->u, o.N * 8);
    std::memcpy(o.U[1].data(), st->v, o.N * 8);
    std::memcpy(o.U[2].data(), st->w, o.N * 8);
    std::memcpy(o.P_.data(), st->p, o.N * 8);
    if (st->pcorr) std::memcpy(o.PC.data(), st->pcorr, o.N * 8); else std::fill(o.PC.begin(), o.PC.end(), 0.0);
    size_t n2 = (size_t)o.nx * o.nz;
    if (!st->usum2 || !st->vsum2 || !st->wsum2 || !st->wt || !st->newk || !st->ume1) return TBL_ERR_BAD_ARG;
    std::memcpy(o.usum2.data(), st->usum2, n2 * 8);
    std::memcpy(o.vsum2.data(), st->vsum2, n2 * 8);
    std::memcpy(o.wsum2.data(), st->wsum2, n2 * 8);
    std::memcpy(o.Wt.data(), st->wt, n2 * 8);
    std::memcpy(o.newk.data(), st->newk, (size_t)o.nz * 4);
    std::memcpy(o.ume1.data(), st->ume1, (size_t)o.nz * 8);
    for (int k = 0; k < o.nz; ++k) if (o.newk[k] < 1 || o.newk[k] > o.nz) return TBL_ERR_BAD_ARG;
    if (st->bltkns) std::memcpy(o.bltkns.data(), st->bltkns, (size_t)o.nx * 8);
    const double* uf[3] = {st->uf, st->vf, st->wf};
    for (int cc = 0; cc < 3; ++cc) {
        for (int k = 1; k <= o.nz; ++k)
            for (int j = 1; j <= o.ny; ++j) {
                double val = uf[cc] ? uf[cc][o.id(o.c.irec, j, k)]
                                    : (o.U[cc][o.id(o.c.irec, j, k)] -
                                       (cc == 0 ? o.usum2 : (cc == 1 ? o.vsum2 : o.wsum2))[o.id2(o.c.irec, k)]);
                o.ufl_file[cc][o.idp(j, k)] = val;
                o.ufl_live[cc][o.idp(j, k)] = val;
            }
        if (uf[cc]) std::memcpy(o.ufl_full_file[cc].data(), uf[cc], o.N * 8);
        else std::fill(o.ufl_full_file[cc].begin(), o.ufl_full_file[cc].end(), 0.0);
    }
    if (is_sete(o))  // dnssetbl computes the plane on each rank's own slab only: reads elsewhere see zeros
        for (int cc = 0; cc < 3; ++cc) std::fill(o.ufl_file[cc].begin(), o.ufl_file[cc].end(), 0.0);
    o.fluc_updated = false;
    o.lamda = st->lamda; o.time = st->time; o.nstep = st->nstep; o.cont = st->cont; o.ksep = st->ksep;
    o.cnt2 = st->cnt2;
    return TBL_OK;
}

int orc_step(orc_handle* h, int32_t nsteps, tbl_step_stats* stats) {
    if (!h || nsteps < 0) return TBL_ERR_BAD_ARG;
    int last = TBL_OK;
    for (int s = 0; s < nsteps; ++s) {
        last = one_step(h->o, stats ? &stats[s] : nullptr);
        if (last == TBL_ERR_NAN || last == TBL_ERR_BLOWUP || last == TBL_ERR_REPLAY || last == TBL_ERR_ZERO_RHS)
            return last;
    }
    return last;
}

int orc_download_state(orc_handle* h, tbl_state* st) {
    if (!h || !st) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    size_t n2 = (size_t)o.nx * o.nz;
    if (st->u) std::memcpy(st->u, o.U[0].data(), o.N * 8);
    if (st->v) std::memcpy(st->v, o.U[1].data(), o.N * 8);
    if (st->w) std::memcpy(st->w, o.U[2].data(), o.N * 8);
    if (st->p) std::memcpy(st->p, o.P_.data(), o.N * 8);
    if (st->pcorr) std::memcpy(st->pcorr, o.PC.data(), o.N * 8);
    if (st->usum2) std::memcpy(st->usum2, o.usum2.data(), n2 * 8);
    if (st->vsum2) std::memcpy(st->vsum2, o.vsum2.data(), n2 * 8);
    if (st->wsum2) std::memcpy(st->wsum2, o.wsum2.data(), n2 * 8);
    if (st->wt) std::memcpy(st->wt, o.Wt.data(), n2 * 8);
    if (st->newk) std::memcpy(st->newk, o.newk.data(), (size_t)o.nz * 4);
    if (st->ume1) std::memcpy(st->ume1, o.ume1.data(), (size_t)o.nz * 8);
    if (st->bltkns) std::memcpy(st->bltkns, o.bltkns.data(), (size_t)o.nx * 8);
    double* uf[3] = {st->uf, st->vf, st->wf};
    for (int cc = 0; cc < 3; ++cc) {
        if (!uf[cc]) continue;
        std::memcpy(uf[cc], o.ufl_full_file[cc].data(), o.N * 8);
        if (o.fluc_updated)
            for (int k = 2; k <= o.nz - 1; ++k)
                for (int j = 2; j <= o.ny - 1; ++j)
                    for (int i = 1; i <= o.nx; ++i)
                        uf[cc][o.id(i, j, k)] = o.U[cc][o.id(i, j, k)] - o.usum2_last_fluc[cc][o.id2(i, k)];
        for (int k = 1; k <= o.nz; ++k)
            for (int j = 2; j <= o.ny - 1; ++j)
                if (k >= 2 && k <= o.nz - 1) uf[cc][o.id(o.c.irec, j, k)] = o.ufl_live[cc][o.idp(j, k)];
    }
    st->lamda = o.lamda; st->time = o.time; st->nstep = o.nstep; st->cont = o.cont; st->ksep = o.ksep;
    st->cnt2 = o.cnt2;
    return TBL_OK;
}

// Test hook: the mass flux and the per-column span sums of the wall shear of
// the current state, without accumulating.
int orc_flux_shear(orc_handle* h, double* ub5, double* tau_nx) {
    if (!h || !ub5 || !tau_nx) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    double keep[5];
    std::memcpy(keep, o.ubulk, sizeof(keep));
    mass_flux(o);
    std::memcpy(ub5, o.ubulk, 5 * 8);
    std::memcpy(o.ubulk, keep, sizeof(keep));
    for (int i = 0; i < o.nx; ++i) tau_nx[i] = 0.0;
    wall_shear(o, tau_nx);
    return TBL_OK;
}

int orc_download_stats(orc_handle* h, tbl_stats_out* out) {
    if (!h || !out) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    size_t n2 = (size_t)o.nx * o.nz;
    double* dst[9] = {out->usum, out->vsum, out->wsum, out->uusum, out->vvsum, out->wwsum, out->uvsum, out->uwsum, out->vwsum};
    const std::vector<double>* src[9] = {&o.usum, &o.vsum, &o.wsum, &o.uusum, &o.vvsum, &o.wwsum, &o.uvsum, &o.uwsum, &o.vwsum};
    for (int q = 0; q < 9; ++q) if (dst[q]) std::memcpy(dst[q], src[q]->data(), n2 * 8);
    if (out->deltastar) std::memcpy(out->deltastar, o.deltastar.data(), o.nx * 8);
    if (out->theta) std::memcpy(out->theta, o.theta.data(), o.nx * 8);
    if (out->ht) std::memcpy(out->ht, o.Ht.data(), o.nx * 8);
    if (out->reth) std::memcpy(out->reth, o.Reth.data(), o.nx * 8);
    if (out->tauw_sum) std::memcpy(out->tauw_sum, o.sumxz.data(), o.nx * 8);
    if (out->ubulk) std::memcpy(out->ubulk, o.ubulk, 5 * 8);
    if (out->tauw_window) std::memcpy(out->tauw_window, o.tauw_window.data(), o.nx * 8);
    out->lamda03 = o.lamda03;
    out->nstat = o.nstat;
    return TBL_OK;
}

int orc_download_averages(orc_handle* h, double* avg) {
    if (!h || !avg) return TBL_ERR_BAD_ARG;
    std::memcpy(avg, h->o.avg.data(), h->o.avg.size() * 8);
    return TBL_OK;
}

int orc_set_replay(orc_handle* h, const int32_t* rec, int64_t len) {
    if (!h || (len > 0 && !rec) || len < 0) return TBL_ERR_BAD_ARG;
    h->o.replay.assign(rec, rec + len);
    h->o.replay_pos = 0;
    return TBL_OK;
}

int orc_last_counts(orc_handle* h, int32_t* buf, int32_t cap) {
    if (!h) return TBL_ERR_BAD_ARG;
    int n = (int)h->o.last_counts.size();
    for (int q = 0; q < n && q < cap; ++q) buf[q] = h->o.last_counts[q];
    return n;
}

void orc_destroy(orc_handle* h) { delete h; }

// Internal-operator access for tests (manufactured solutions, known answers).
// Applies L7 (global halos) to x on the interior; y zero elsewhere.
int orc_apply_lap(orc_handle* h, const double* x, double* y) {
    if (!h) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    std::vector<double> X(x, x + o.N);
    std::memset(y, 0, o.N * 8);
    for (int k = 2; k <= o.nz - 1; ++k)
        for (int j = 2; j <= o.ny - 1; ++j)
            for (int i = 2; i <= o.nx - 1; ++i) y[o.id(i, j, k)] = lap(o, X, i, j, k);
    return TBL_OK;
}

// Solves L7 x = rhs by the step's GMRES (block-SSOR preconditioned) from
// x = 0 with the configured kmax / errtol; returns the status and the
// number of Arnoldi steps.
int orc_solve_ppe(orc_handle* h, const double* rhs, double* x, int32_t* iters) {
    if (!h || !rhs || !x) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    std::memcpy(o.Q8.data(), rhs, o.N * 8);
    std::fill(o.PC.begin(), o.PC.end(), 0.0);
    std::vector<int32_t> kits;
    int restarts = 0, it = 0;
    double resid = 0.0;
    int s = gmres(o, nullptr, kits, restarts, it, resid);
    std::memcpy(x, o.PC.data(), o.N * 8);
    if (iters) *iters = it;
    return s;
}

// Applies the block-SSOR preconditioner to x (interior), result in y.
int orc_apply_ssor(orc_handle* h, const double* x, double* y) {
    if (!h) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    std::vector<double> X(x, x + o.N);
    ssor(o, X);
    std::memcpy(y, o.rhat.data(), o.N * 8);
    return TBL_OK;
}

// The thicknesses of the rescaling bookkeeping from a given time-mean
// streamwise velocity usum2 (nx x nz, column-major): bltkns, deltastar,
// theta, H and Re_theta (each nx), by the same code as the step.
int orc_thicknesses(orc_handle* h, const double* usum2, double* bltkns, double* deltastar, double* theta,
                    double* ht, double* reth) {
    if (!h || !usum2) return TBL_ERR_BAD_ARG;
    Oracle& o = h->o;
    std::memcpy(o.usum2.data(), usum2, (size_t)o.nx * o.nz * 8);
    bl_thickness(o);
    integral_thicknesses(o);
    const size_t b = (size_t)o.nx * 8;
    if (bltkns) std::memcpy(bltkns, o.bltkns.data(), b);
    if (deltastar) std::memcpy(deltastar, o.deltastar.data(), b);
    if (theta) std::memcpy(theta, o.theta.data(), b);
    if (ht) std::memcpy(ht, o.Ht.data(), b);
    if (reth) std::memcpy(reth, o.Reth.data(), b);
    return TBL_OK;
}

}  // extern "C"
