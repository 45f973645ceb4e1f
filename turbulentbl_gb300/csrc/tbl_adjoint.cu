// tbl_adjoint.cu -- wall-normal blowing control, the wall-shear objective and
// the discrete adjoint of a window of time steps.
//
// The map differentiated is one step of dnstbl2/dnstbl.f90:538-1469 with the
// implicit-diffusion and pressure-Poisson solves taken as converged (their
// adjoints are solves with the transposed operators) and with the branch
// decisions of the convection stencils (Peclet windows :655/:679/:701, the
// upwind side at the first/last span rows :670-677, |u|) frozen at the
// recorded trajectory.  Recycling means, Wt, new(k) and lamda are constants
// of a window (a window never contains a rescaling step).
//
// Stage by stage the adjoint step runs the forward stages in reverse:
//   periodic copies (:1465-1469)      k_adj_periodic
//   pressure BCs (:1352-1461)         k_adj_pbc_a (point terms, source weights)
//                                     k_adj_pbc_b (gather onto the wall and inflow planes)
//   outflow / wall+top velocity BCs   k_adj_vel_out, k_adj_vel_walltop (-> dL/dc)
//   projection + p' extrapolation     k_adj_pc_rhs  -> right-hand side of L7^T mu = .
//   Poisson solve (:940-1208)         the forward SSOR-GMRES with AbT/AtT
//   divergence (:905-935)             k_adj_div_gsrhs -> right-hand side of A^T nu = .
//   implicit diffusion (:771-896)     the forward wavefront Gauss-Seidel with AbT/AtT
//   convection + explicit RHS         k_adj_conv (gather form, no atomics)
//   recycling inflow (:557-618)       k_adj_inflow
// Every kernel writes each output point from exactly one thread, so the
// adjoint is deterministic run to run.
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>

#include "tbl_internal.cuh"
#include "tbl_kernels.cuh"
#include "tbl_reduce.cuh"

#define ATRY(x)                         \
    do {                                \
        int s_ = (x);                   \
        if (s_ != TBL_OK) return s_;    \
    } while (0)

namespace tbl {

struct Ckpt {
    double* U[3];
    double* P;
    double* PC;
    double* ufl;  // 3 x (ny, nz) live recycling plane
    int nstep, cont, nstat, cnt2;
    double time, lamda_host;
    bool fluc;
};

struct AdjTape {
    int W = 0, ck = 0, nseg = 0;
    size_t vol = 0;
    double* buf = nullptr;
    size_t buf_n = 0;
    std::vector<Ckpt> cks;
    std::vector<double*> segU1, segU3;  // ck entries of 3 x vol each
    Ckpt fin;
    double* fin_sums = nullptr;
    double* fin_diag = nullptr;  // sumxz, tauw window, mass flux at the end of the window
    double *lU[3] = {nullptr, nullptr, nullptr}, *lP = nullptr;
    double *lc = nullptr, *AW = nullptr, *LE = nullptr, *luold = nullptr;
    double *ocf = nullptr, *jacc = nullptr;
    std::vector<int> nstep_of;
    unsigned char* bits = nullptr;  // W x vol frozen-branch record (TBL_BRANCH_RECORD / _REPLAY)
    int branch_mode = TBL_BRANCH_FREE;
    bool bits_valid = false;        // a record of this window length exists
    bool valid = false;
    double forward_ms = 0.0;
};

namespace {

__device__ __forceinline__ long long ix(const Geom& g, int i, int j, int k) {
    return (long long)i + (long long)g.sx * ((long long)j + (long long)g.ny * k);
}
// row j (1..ny-2) moved by o on the periodic ring of unique rows
__device__ __forceinline__ int ring(const Geom& g, int j, int o) {
    const int J = g.ny - 2;
    int r = (j - 1 + o) % J;
    if (r < 0) r += J;
    return 1 + r;
}
__device__ __forceinline__ bool inner(const Geom& g, int i, int j, int k) {
    return i >= 1 && i <= g.nx - 2 && j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
}

struct AdjCoef {
    double dx, dy, dxi, dt, re, t;  // t = -dt/Re
    double df1, df2;                // x3(2)-x3(1), x3(3)-x3(1)
    double aw;                      // 1/dx^2
    double ue, lamda_unused;
};

// ------------------------------------------------------------ objective
// acc += sum over (i, j unique) of cf0 w(i,j,1) + cf1 u(i,j,1) + cf2 u(i,j,2) + cf3 u(i,j,3)
// (1-based k): the patch- and span-averaged wall shear as a linear form.
__global__ void __launch_bounds__(256) k_objective(Geom g, const double* __restrict__ cf,
                                                   const double* __restrict__ u, const double* __restrict__ w,
                                                   double* acc) {
    __shared__ double s_red[8];
    const int nx = g.nx;
    const long long n = (long long)nx * (g.ny - 2);
    double a = 0.0;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = (int)(t % nx), j = 1 + (int)(t / nx);
        a += cf[i] * w[ix(g, i, j, 0)] + cf[nx + i] * u[ix(g, i, j, 0)] + cf[2 * nx + i] * u[ix(g, i, j, 1)] +
             cf[3 * nx + i] * u[ix(g, i, j, 2)];
    }
    a = block_sum(a, s_red);
    if (threadIdx.x == 0) *acc += a;
}

__global__ void k_objective_adj(Geom g, const double* __restrict__ cf, double scale, double* __restrict__ lu,
                                double* __restrict__ lw) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx;
    if (t >= nx * (g.ny - 2)) return;
    const int i = t % nx, j = 1 + t / nx;
    lw[ix(g, i, j, 0)] += scale * cf[i];
    lu[ix(g, i, j, 0)] += scale * cf[nx + i];
    lu[ix(g, i, j, 1)] += scale * cf[2 * nx + i];
    lu[ix(g, i, j, 2)] += scale * cf[3 * nx + i];
}

// ------------------------------------------------------- periodic copies
// forward: F(:,1) = F(:,ny-2); F(:,ny-1) = F(:,1)  (0-based rows)
__global__ void k_adj_periodic(Geom g, double* l0, double* l1, double* l2, double* l3) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nx * g.nz) return;
    const int i = t % g.nx, k = t / g.nx;
    double* Ls[4] = {l0, l1, l2, l3};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        double* F = Ls[c];
        F[ix(g, i, 1, k)] += F[ix(g, i, g.ny - 1, k)];
        F[ix(g, i, g.ny - 1, k)] = 0.0;
        F[ix(g, i, g.ny - 2, k)] += F[ix(g, i, 0, k)];
        F[ix(g, i, 0, k)] = 0.0;
    }
}

// Velocities as the pressure BCs saw them: the step's output, except the
// spanwise ghost rows, which still held the step input's values (= U1's).
struct PreCopy {
    const double* u3;
    const double* u1;
    __device__ double operator()(const Geom& g, int i, int j, int k) const {
        return (j == 0 || j == g.ny - 1) ? u1[ix(g, i, j, k)] : u3[ix(g, i, j, k)];
    }
};

// -------------------------------------------------- pressure BCs, phase A
// One flat index space over wall (I x J), top (I x J), outflow (J x K) and
// inflow (J x K) sources, each writing only its own points; the weights that
// spread over neighbouring points go to AW (wall, nx x ny) and LE (inflow,
// ny x nz) for phase B.
__global__ void k_adj_pbc_a(Geom g, AdjCoef c, PreCopy U, PreCopy V, PreCopy Wv, const double* __restrict__ jacinv,
                            double* __restrict__ lu, double* __restrict__ lv, double* __restrict__ lw,
                            double* __restrict__ lP, double* __restrict__ AW, double* __restrict__ LE,
                            double* __restrict__ luold) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny, nz = g.nz, J = ny - 2, I = nx - 2, K = nz - 2;
    const long long nW = (long long)I * J, nO = (long long)J * K;
    if (t < nW) {  // wall: P0 = P1 - df1 (-w0 (w1-w0)/df1 + (g1+g2+g3)/Re)
        const int i = 1 + (int)(t % I), j = 1 + (int)(t / I);
        const double a = lP[ix(g, i, j, 0)];
        lP[ix(g, i, j, 0)] = 0.0;
        AW[i + (size_t)nx * j] = a;
        const double ld3 = c.df1 * a, lg = -c.df1 * a / c.re;
        const double w0 = Wv(g, i, j, 0);
        const double den = c.df1 * (c.df2 * c.df2) - c.df2 * (c.df1 * c.df1);
        lw[ix(g, i, j, 1)] += ld3 * w0 / c.df1 + lg * (-2.0 * c.df2) / den;
        lw[ix(g, i, j, 2)] += lg * 2.0 * c.df1 / den;
        return;
    }
    t -= nW;
    if (t < nW) {  // top: P = (11 w_n - 18 w_n-1 + 9 w_n-2 - 2 w_n-3)/(6 dxi) jinv / Re
        const int i = 1 + (int)(t % I), j = 1 + (int)(t / I);
        const double a = lP[ix(g, i, j, nz - 1)];
        lP[ix(g, i, j, nz - 1)] = 0.0;
        const double lf = a * jacinv[nz - 1] / c.re / (6.0 * c.dxi);
        lw[ix(g, i, j, nz - 1)] += 11.0 * lf;
        lw[ix(g, i, j, nz - 2)] += -18.0 * lf;
        lw[ix(g, i, j, nz - 3)] += 9.0 * lf;
        lw[ix(g, i, j, nz - 4)] += -2.0 * lf;
        return;
    }
    t -= nW;
    if (t < nO) {  // outflow: P = (3 u_n - 4 u_n-1 + u_n-2)/(2 dx Re)
        const int j = 1 + (int)(t % J), k = 1 + (int)(t / J);
        const double a = lP[ix(g, nx - 1, j, k)];
        lP[ix(g, nx - 1, j, k)] = 0.0;
        const double s = a / (2.0 * c.dx * c.re);
        lu[ix(g, nx - 1, j, k)] += 3.0 * s;
        lu[ix(g, nx - 2, j, k)] += -4.0 * s;
        lu[ix(g, nx - 3, j, k)] += s;
        return;
    }
    t -= nO;
    if (t < nO) {  // inflow: P0 = (2 dx E - P2 + 4 P1)/3
        const int j = 1 + (int)(t % J), k = 1 + (int)(t / J);
        const double a = lP[ix(g, 0, j, k)];
        lP[ix(g, 0, j, k)] = 0.0;
        lP[ix(g, 2, j, k)] += -a / 3.0;
        lP[ix(g, 1, j, k)] += 4.0 * a / 3.0;
        const double lE = 2.0 * c.dx * a / 3.0;
        LE[j + (size_t)ny * k] = lE;
        const double u0 = U(g, 0, j, k);
        const double Jk = jacinv[k];
        luold[j + (size_t)ny * k] += -lE / c.dt;
        lu[ix(g, 1, j, k)] += lE * u0 / c.dx - 2.0 * (-lE / c.re) / (c.dx * c.dx);
        lu[ix(g, 2, j, k)] += (-lE / c.re) / (c.dx * c.dx);
        lv[ix(g, 0, j, k)] += lE * (U(g, 0, j + 1, k) - U(g, 0, j - 1, k)) / (2.0 * c.dy);
        lw[ix(g, 0, j, k)] += lE * Jk * (U(g, 0, j, k + 1) - U(g, 0, j, k - 1)) / (2.0 * c.dxi);
    }
}

// Coefficient of u(0, j, k+off) in g3 of the inflow source at plane k
// (the one-sided forms at the first/last interior planes, :1444-1450).
__device__ __forceinline__ double g3_coef(const Geom& g, int k, int off, double lg3r, double lfd, double dxi) {
    const double d2 = dxi * dxi;
    if (k <= 1) {
        if (off == 0) return -lfd / dxi + lg3r / d2;
        if (off == 1) return lfd / dxi - 2.0 * lg3r / d2;
        if (off == 2) return lg3r / d2;
        return 0.0;
    }
    if (k >= g.nz - 2) {
        if (off == 0) return lfd / dxi + lg3r / d2;
        if (off == -1) return -lfd / dxi - 2.0 * lg3r / d2;
        if (off == -2) return lg3r / d2;
        return 0.0;
    }
    if (off == 0) return -2.0 * lg3r / d2;
    if (off == 1) return lfd / (2.0 * dxi) + lg3r / d2;
    if (off == -1) return -lfd / (2.0 * dxi) + lg3r / d2;
    return 0.0;
}

// -------------------------------------------------- pressure BCs, phase B
// Targets: w on the wall plane (nx x ny, ghost rows included) and u on the
// inflow plane (ny x nz, ghost rows included); each gathers every source
// that reads it.
__global__ void k_adj_pbc_b(Geom g, AdjCoef c, PreCopy U, PreCopy V, PreCopy Wv, const double* __restrict__ jacinv,
                            const double* __restrict__ jac2, const double* __restrict__ AW,
                            const double* __restrict__ LE, double* __restrict__ lu, double* __restrict__ lw,
                            double* __restrict__ lP) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const long long nWall = (long long)nx * ny, nIn = (long long)ny * nz;
    auto wall_src = [&](int i, int j) { return i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2; };
    if (t < nWall) {
        const int i = (int)(t % nx), j = (int)(t / nx);
        const double den = c.df1 * (c.df2 * c.df2) - c.df2 * (c.df1 * c.df1);
        const double dx2 = c.dx * c.dx, dy2 = c.dy * c.dy;
        double acc = 0.0;
        if (wall_src(i, j)) {
            const double a = AW[i + (size_t)nx * j];
            lP[ix(g, i, j, 1)] += a;
            const double ld3 = c.df1 * a, lg = -c.df1 * a / c.re;
            const double w0 = Wv(g, i, j, 0), w1 = Wv(g, i, j, 1);
            acc += ld3 * ((w1 - w0) / c.df1) - ld3 * w0 / c.df1;
            acc += -2.0 * lg / dx2 - 2.0 * lg / dy2 + lg * 2.0 * (c.df2 - c.df1) / den;
        }
        if (wall_src(i - 1, j)) acc += (-c.df1 * AW[(i - 1) + (size_t)nx * j] / c.re) / dx2;
        if (wall_src(i + 1, j)) acc += (-c.df1 * AW[(i + 1) + (size_t)nx * j] / c.re) / dx2;
        if (wall_src(i, j - 1)) acc += (-c.df1 * AW[i + (size_t)nx * (j - 1)] / c.re) / dy2;
        if (wall_src(i, j + 1)) acc += (-c.df1 * AW[i + (size_t)nx * (j + 1)] / c.re) / dy2;
        lw[ix(g, i, j, 0)] += acc;
        return;
    }
    t -= nWall;
    if (t < nIn) {
        const int j = (int)(t % ny), k = (int)(t / ny);
        auto in_src = [&](int jj, int kk) { return jj >= 1 && jj <= ny - 2 && kk >= 1 && kk <= nz - 2; };
        const double dx2 = c.dx * c.dx, dy2 = c.dy * c.dy;
        double acc = 0.0;
        if (in_src(j, k)) {
            const double lE = LE[j + (size_t)ny * k], lg = -lE / c.re;
            const double u0 = U(g, 0, j, k), u1 = U(g, 1, j, k);
            acc += lE / c.dt;                               // (u0 - uold)/dt
            acc += lE * ((u1 - u0) / c.dx - u0 / c.dx);     // u0 (u1 - u0)/dx
            acc += lg / dx2 - 2.0 * lg / dy2;               // g1, g2 centre
        }
        // spanwise neighbours: d2 = v0 (u(j+1) - u(j-1))/(2dy), g2
        if (in_src(j - 1, k)) {
            const double lE = LE[(j - 1) + (size_t)ny * k];
            acc += lE * V(g, 0, j - 1, k) / (2.0 * c.dy) + (-lE / c.re) / dy2;
        }
        if (in_src(j + 1, k)) {
            const double lE = LE[(j + 1) + (size_t)ny * k];
            acc += -lE * V(g, 0, j + 1, k) / (2.0 * c.dy) + (-lE / c.re) / dy2;
        }
        // wall-normal neighbours: d3 Jk = w0 (u(k+1) - u(k-1))/(2dxi) Jk
        if (in_src(j, k - 1)) {
            const double lE = LE[j + (size_t)ny * (k - 1)];
            acc += lE * jacinv[k - 1] * Wv(g, 0, j, k - 1) / (2.0 * c.dxi);
        }
        if (in_src(j, k + 1)) {
            const double lE = LE[j + (size_t)ny * (k + 1)];
            acc += -lE * jacinv[k + 1] * Wv(g, 0, j, k + 1) / (2.0 * c.dxi);
        }
        // g3 = g3r Jk^2 - jac2 fder Jk^3 of the sources at planes k-2..k+2
        if (j >= 1 && j <= ny - 2) {
            for (int ks = k - 2; ks <= k + 2; ++ks) {
                if (ks < 1 || ks > nz - 2) continue;
                const double lg = -LE[j + (size_t)ny * ks] / c.re;
                const double Jk = jacinv[ks];
                const double lg3r = lg * Jk * Jk, lfd = -lg * jac2[ks] * Jk * Jk * Jk;
                acc += g3_coef(g, ks, k - ks, lg3r, lfd, c.dxi);
            }
        }
        lu[ix(g, 0, j, k)] += acc;
    }
}

// ----------------------------------------------------- velocity BCs
// outflow (:1342): U(nx-1) = (4 U(nx-2) - U(nx-3))/3 for j unique, all k
__global__ void k_adj_vel_out(Geom g, double* l0, double* l1, double* l2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = g.ny - 2;
    if (t >= J * g.nz) return;
    const int j = 1 + t % J, k = t / J, nx = g.nx;
    double* Ls[3] = {l0, l1, l2};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double* F = Ls[c];
        const double a = F[ix(g, nx - 1, j, k)];
        F[ix(g, nx - 1, j, k)] = 0.0;
        F[ix(g, nx - 2, j, k)] += 4.0 * a / 3.0;
        F[ix(g, nx - 3, j, k)] += -a / 3.0;
    }
}

// wall (U = 0, w = c) and top (zero gradient) (:1317-1330), all i, j unique;
// the wall value of w is the control: dL/dc accumulates here.
__global__ void k_adj_vel_walltop(Geom g, double* l0, double* l1, double* l2, double* __restrict__ lc) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = g.ny - 2;
    if (t >= g.nx * J) return;
    const int i = t % g.nx, j = 1 + t / g.nx, nz = g.nz;
    double* Ls[3] = {l0, l1, l2};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double* F = Ls[c];
        const double a = F[ix(g, i, j, nz - 1)];
        F[ix(g, i, j, nz - 1)] = 0.0;
        F[ix(g, i, j, nz - 2)] += 4.0 * a / 3.0;
        F[ix(g, i, j, nz - 3)] += -a / 3.0;
    }
    lc[t] += l2[ix(g, i, j, 0)];
    l0[ix(g, i, j, 0)] = 0.0;
    l1[ix(g, i, j, 0)] = 0.0;
    l2[ix(g, i, j, 0)] = 0.0;
}

// ------------------------------------ projection + p' extrapolation
// Right-hand side of L7^T mu = r over the interior: r = dL/dP (the P += p'
// update) + grad^T(-dt dL/dU) + the transposed face extrapolations of p'
// (:1245-1262; faces with the other index interior; the periodic copy of p'
// is never read).
__global__ void __launch_bounds__(128) k_adj_pc_rhs(Geom g, double hx, double hy, double hz, double dt,
                                                    const double* __restrict__ jacinv,
                                                    const double* __restrict__ l0, const double* __restrict__ l1,
                                                    const double* __restrict__ l2, const double* __restrict__ lP,
                                                    double* __restrict__ R) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    const int nx = g.nx, nz = g.nz;
    if (i > nx - 2) return;
    auto A0 = [&](int ii, int jj, int kk) { return inner(g, ii, jj, kk) ? l0[ix(g, ii, jj, kk)] : 0.0; };
    auto A2 = [&](int ii, int jj, int kk) { return inner(g, ii, jj, kk) ? l2[ix(g, ii, jj, kk)] : 0.0; };
    double r = lP[ix(g, i, j, k)];
    r += -dt * (hx * (A0(i - 1, j, k) - A0(i + 1, j, k)) +
                hy * (l1[ix(g, i, ring(g, j, -1), k)] - l1[ix(g, i, ring(g, j, 1), k)]) +
                hz * (jacinv[k - 1] * A2(i, j, k - 1) - jacinv[k + 1] * A2(i, j, k + 1)));
    if (i == 1 || i == 2) {
        const double f = dt * hx * l0[ix(g, 1, j, k)];
        r += (i == 1 ? 4.0 / 3.0 : -1.0 / 3.0) * f;
    }
    if (i >= nx - 4 && i <= nx - 2) {
        const double f = -dt * hx * l0[ix(g, nx - 2, j, k)];
        r += (i == nx - 2 ? 2.5 : (i == nx - 3 ? -2.0 : 0.5)) * f;
    }
    if (k == 1 || k == 2) {
        const double f = dt * hz * jacinv[1] * l2[ix(g, i, j, 1)];
        r += (k == 1 ? 4.0 / 3.0 : -1.0 / 3.0) * f;
    }
    if (k >= nz - 4 && k <= nz - 2) {
        const double f = -dt * hz * jacinv[nz - 2] * l2[ix(g, i, j, nz - 2)];
        r += (k == nz - 2 ? 2.5 : (k == nz - 3 ? -2.0 : 0.5)) * f;
    }
    R[ix(g, i, j, k)] = r;
}

// ------------------------------------------------------ divergence^T
// dL/dU += div^T(mu)/dt over i, k all and j unique; the interior of the
// result is the right-hand side Qc of A^T nu = Qc (A = 1 - dt/Re L7).
__global__ void __launch_bounds__(128) k_adj_div_gsrhs(Geom g, double hx, double hy, double dt,
                                                       const double* __restrict__ x3, const double* __restrict__ mu,
                                                       double* __restrict__ l0, double* __restrict__ l1,
                                                       double* __restrict__ l2, double* __restrict__ q0,
                                                       double* __restrict__ q1, double* __restrict__ q2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y, k = blockIdx.z;
    if (i >= g.nx) return;
    auto M = [&](int ii, int jj, int kk) { return inner(g, ii, jj, kk) ? mu[ix(g, ii, jj, kk)] : 0.0; };
    const long long p = ix(g, i, j, k);
    const double idt = 1.0 / dt;
    const double a0 = l0[p] + idt * hx * (M(i - 1, j, k) - M(i + 1, j, k));
    const double a1 = l1[p] + idt * hy * (M(i, ring(g, j, -1), k) - M(i, ring(g, j, 1), k));
    double dz = 0.0;
    if (k - 1 >= 1 && k - 1 <= g.nz - 2) dz += M(i, j, k - 1) / (x3[k] - x3[k - 2]);
    if (k + 1 >= 1 && k + 1 <= g.nz - 2) dz -= M(i, j, k + 1) / (x3[k + 2] - x3[k]);
    const double a2 = l2[p] + idt * dz;
    l0[p] = a0;
    l1[p] = a1;
    l2[p] = a2;
    if (inner(g, i, j, k)) {
        q0[p] = a0;
        q1[p] = a1;
        q2[p] = a2;
    }
}

// ------------------------------------------------------ convection^T
struct ConvAdjCoef {
    double re, dx, dy, dt;
    double inv2x, q25x, c12x;
    double invdy, q25y, c12y;
    double inv2z, q25z, c12z;
};

// Stencil coefficients cf[o+2] (o = -2..2) of the convection term along one
// direction at a point with multiplier m (u, v or w there); dir 1 is the
// spanwise direction with its first-order upwind rows.
// b >= 0: frozen-branch record byte (bit 3+dir' sign of |m|; bits 4/5 the
// spanwise upwind sides), else the signs of m itself.
__device__ __forceinline__ void conv_stencil(int dir, double m, bool nearb, bool win, double inv2, double q25,
                                             double c12, double invdy, double cf[5], int b = -1) {
#pragma unroll
    for (int o = 0; o < 5; ++o) cf[o] = 0.0;
    if (nearb) {
        if (dir == 1) {
            const double ap = b >= 0 ? ((b & 16) ? m : 0.0) : fmax(m, 0.0);
            const double bn = b >= 0 ? ((b & 32) ? m : 0.0) : fmin(m, 0.0);
            cf[2] = (ap - bn) * invdy;
            cf[1] = -ap * invdy;
            cf[3] = bn * invdy;
        } else {
            cf[3] = m * inv2;
            cf[1] = -m * inv2;
        }
        return;
    }
    const int sbit = dir == 0 ? 8 : (dir == 1 ? 16 : 64);
    const double a = b >= 0 ? ((b & sbit) ? m : -m) : fabs(m);
    if (win) {
        cf[4] = a * q25 - m * c12;
        cf[3] = -4.0 * a * q25 + 8.0 * m * c12;
        cf[2] = 6.0 * a * q25;
        cf[1] = -4.0 * a * q25 - 8.0 * m * c12;
        cf[0] = a * q25 + m * c12;
    } else {
        cf[0] = m * c12;
        cf[1] = -8.0 * m * c12;
        cf[3] = 8.0 * m * c12;
        cf[4] = -m * c12;
    }
}

// Branch decision of the forward convection at interior point (i,j,k) along dir
// (sign(1, ceiling(m)) Peclet test as in the forward kernels), or from the
// frozen-branch record byte b (b >= 0; bits 0-2 the x/y/z windows).
__device__ __forceinline__ void conv_case(const Geom& g, const ConvAdjCoef& c, const double* __restrict__ x3,
                                          int dir, int i, int j, int k, double m, bool& nearb, bool& win,
                                          int b = -1) {
    if (b >= 0) {
        nearb = dir == 0 ? ((i <= 1) || (i >= g.nx - 2)) : (dir == 1 ? ((j == 1) || (j == g.ny - 2))
                                                                      : ((k <= 1) || (k >= g.nz - 2)));
        win = (b >> dir) & 1;
        return;
    }
    const double sgn = m > -1.0 ? 1.0 : -1.0;
    if (dir == 0) {
        nearb = (i <= 1) || (i >= g.nx - 2);
        const double Pe = sgn * c.re * m * c.dx;
        win = Pe > 2.0 && Pe < 50.0;
    } else if (dir == 1) {
        nearb = (j == 1) || (j == g.ny - 2);
        const double Pe = sgn * c.re * m * c.dy;
        win = Pe > 2.0 && Pe < 50.0;
    } else {
        nearb = (k <= 1) || (k >= g.nz - 2);
        const double dz = x3[k + 1] - x3[k];
        const double Pe = (sgn * c.re * m * dz);
        win = Pe > 2.0 && Pe < 5.0;
    }
}

// Adjoint of Q_c = U1_c - dt conv_c(U1) - dt grad_c P and of the GS solve's
// dependence on the boundary values of U1.  nu = A^-T (dL/dU2 interior).
// Each thread owns one point q (i, k all; j unique) and gathers from every
// interior p whose stencils read q.
__global__ void __launch_bounds__(128) k_adj_conv(Geom g, ConvAdjCoef c, double t_gs, double aw,
                                                  const double* __restrict__ Ab, const double* __restrict__ At,
                                                  const double* __restrict__ x3, const double* __restrict__ jacinv,
                                                  const double* __restrict__ u1, const double* __restrict__ v1,
                                                  const double* __restrict__ w1, const double* __restrict__ nu0,
                                                  const double* __restrict__ nu1, const double* __restrict__ nu2,
                                                  double* __restrict__ l0, double* __restrict__ l1,
                                                  double* __restrict__ l2, double* __restrict__ lP,
                                                  const unsigned char* __restrict__ bits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y, k = blockIdx.z;
    const int nx = g.nx, nz = g.nz;
    if (i >= nx) return;
    const double* Us[3] = {u1, v1, w1};
    const double* Ns[3] = {nu0, nu1, nu2};
    const long long q = ix(g, i, j, k);
    const bool qin = inner(g, i, j, k);
    double out[3];
    if (qin) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) out[cc] = Ns[cc][q];
    } else {
        double* Ls[3] = {l0, l1, l2};
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            double v = Ls[cc][q];
            const double* N = Ns[cc];
            const bool kin = k >= 1 && k <= nz - 2, iin = i >= 1 && i <= nx - 2;
            if (i == 0 && kin) v += -t_gs * aw * N[ix(g, 1, j, k)];
            if (i == nx - 1 && kin) v += -t_gs * aw * N[ix(g, nx - 2, j, k)];
            if (k == 0 && iin) v += -t_gs * Ab[1] * N[ix(g, i, j, 1)];
            if (k == nz - 1 && iin) v += -t_gs * At[nz - 2] * N[ix(g, i, j, nz - 2)];
            out[cc] = v;
        }
    }
    double lp = 0.0;
    // stencil part: sum over p = q - o e_d
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double inv2 = d == 0 ? c.inv2x : c.inv2z;
        const double q25 = d == 0 ? c.q25x : (d == 1 ? c.q25y : c.q25z);
        const double c12 = d == 0 ? c.c12x : (d == 1 ? c.c12y : c.c12z);
        for (int o = -2; o <= 2; ++o) {
            int pi = i, pj = j, pk = k;
            if (d == 0) pi = i - o;
            else if (d == 1) pj = ring(g, j, -o);
            else pk = k - o;
            if (!inner(g, pi, pj, pk)) continue;
            const long long p = ix(g, pi, pj, pk);
            const double m = Us[d][p];
            const int bp = bits ? (int)bits[p] : -1;
            bool nearb, win;
            conv_case(g, c, x3, d, pi, pj, pk, m, nearb, win, bp);
            double cf[5];
            conv_stencil(d, m, nearb, win, inv2, q25, c12, c.invdy, cf, bp);
            double w = cf[o + 2];
            if (d == 2) w *= jacinv[pk];
            if (w != 0.0) {
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) out[cc] += -c.dt * Ns[cc][p] * w;
            }
        }
    }
    // multiplier part at q itself: d conv / d(u, v, w)(q)
    if (qin) {
        const int ja = ring(g, j, -1), jb = ring(g, j, -2), jc = ring(g, j, 1), jd = ring(g, j, 2);
        const int bq = bits ? (int)bits[q] : -1;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double m = Us[d][q];
            bool nearb, win;
            conv_case(g, c, x3, d, i, j, k, m, nearb, win, bq);
            const double q25 = d == 0 ? c.q25x : (d == 1 ? c.q25y : c.q25z);
            const double c12 = d == 0 ? c.c12x : (d == 1 ? c.c12y : c.c12z);
            const int sbit = d == 0 ? 8 : (d == 1 ? 16 : 64);
            const double sg = bq >= 0 ? ((bq & sbit) ? 1.0 : -1.0) : ((m > 0.0) ? 1.0 : ((m < 0.0) ? -1.0 : 0.0));
            const bool vpos = bq >= 0 ? (bq & 16) != 0 : m >= 0.0;
            const bool vneg = bq >= 0 ? (bq & 32) != 0 : m <= 0.0;
            double acc = 0.0;
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                const double* F = Us[cc];
                double f[5];
                if (d == 0) {
                    f[1] = F[q - 1]; f[3] = F[q + 1];
                    f[0] = nearb ? 0.0 : F[q - 2];
                    f[4] = nearb ? 0.0 : F[q + 2];
                } else if (d == 1) {
                    f[0] = F[ix(g, i, jb, k)]; f[1] = F[ix(g, i, ja, k)];
                    f[3] = F[ix(g, i, jc, k)]; f[4] = F[ix(g, i, jd, k)];
                } else {
                    f[1] = F[q - g.ps]; f[3] = F[q + g.ps];
                    f[0] = nearb ? 0.0 : F[q - 2 * g.ps];
                    f[4] = nearb ? 0.0 : F[q + 2 * g.ps];
                }
                f[2] = F[q];
                double dm;
                if (nearb) {
                    if (d == 1)
                        dm = (vpos ? (f[2] - f[1]) * c.invdy : 0.0) + (vneg ? (f[3] - f[2]) * c.invdy : 0.0);
                    else
                        dm = (f[3] - f[1]) * (d == 0 ? c.inv2x : c.inv2z);
                } else if (win) {
                    dm = sg * q25 * (f[4] - 4.0 * f[3] + 6.0 * f[2] - 4.0 * f[1] + f[0]) +
                         c12 * (-f[4] + 8.0 * f[3] - 8.0 * f[1] + f[0]);
                } else {
                    dm = c12 * (f[0] - 8.0 * f[1] + 8.0 * f[3] - f[4]);
                }
                acc += -c.dt * Ns[cc][q] * dm;
            }
            if (d == 2) acc *= jacinv[k];
            out[d] += acc;
        }
    }
    // pressure gradient: g = 0.5 (P(+1) - P(-1)) / h  (z: times jinv of the row)
    {
        auto N0 = [&](int ii, int jj, int kk) { return inner(g, ii, jj, kk) ? nu0[ix(g, ii, jj, kk)] : 0.0; };
        auto N2 = [&](int ii, int jj, int kk) { return inner(g, ii, jj, kk) ? nu2[ix(g, ii, jj, kk)] : 0.0; };
        const double hx = 0.5 / c.dx, hy = 0.5 * c.invdy, hz = c.inv2z;
        lp += hx * (N0(i - 1, j, k) - N0(i + 1, j, k));
        if (k >= 1 && k <= nz - 2 && i >= 1 && i <= nx - 2)
            lp += hy * (nu1[ix(g, i, ring(g, j, -1), k)] - nu1[ix(g, i, ring(g, j, 1), k)]);
        double z = 0.0;
        if (k - 1 >= 1) z += jacinv[k - 1] * N2(i, j, k - 1);
        if (k + 1 <= nz - 2) z -= jacinv[k + 1] * N2(i, j, k + 1);
        lp += hz * z;
        lP[q] += -c.dt * lp;
    }
    l0[q] = out[0];
    l1[q] = out[1];
    l2[q] = out[2];
}

// ---------------------------------------------------- recycling inflow
// Inflow plane values are overwritten (:557-618); the live recycling plane
// U(irec, j, new(k)) carries lamda times their adjoint.  Then the saved
// Utold(1,:,:) (:549) adds its adjoint to the step input's u(1,:,:).
// One thread per unique span row j (the k loop is sequential, no conflicts:
// the sources are at i = 1, the targets at i = irec).
__global__ void k_adj_inflow(Geom g, int inflow_on, int irec0, double ue, const double* __restrict__ usum2,
                             const double* __restrict__ wt, const int* __restrict__ newk,
                             const int* __restrict__ slab_of_k, const SlabDesc* __restrict__ slabs,
                             const DevScalars* __restrict__ sc, const double* __restrict__ luold, double* l0,
                             double* l1, double* l2) {
    const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (j > g.ny - 2) return;
    const int nx = g.nx;
    double* Ls[3] = {l0, l1, l2};
    if (inflow_on) {
        const double lam = sc->lamda;
        for (int k = 1; k <= g.nz - 2; ++k) {
            const long long q = ix(g, 0, j, k);
            if (usum2[(size_t)irec0 + (size_t)nx * k] < (0.99 * ue)) {
                const int nk = newk[k] - 1;
                const SlabDesc s = slabs[slab_of_k[k]];
                const bool live = nk >= s.bn && nk < s.bn + s.K;
                const double w_ = wt[(size_t)(nx - 2) + (size_t)nx * k];
                const double f = lam * ((1.0 - w_) + w_);
                for (int c = 0; c < 3; ++c) {
                    const double a = Ls[c][q];
                    Ls[c][q] = 0.0;
                    if (live) Ls[c][ix(g, irec0, j, nk)] += f * a;
                }
            } else {
                for (int c = 0; c < 3; ++c) Ls[c][q] = 0.0;
            }
        }
    }
    for (int k = 0; k < g.nz; ++k) l0[ix(g, 0, j, k)] += luold[j + (size_t)g.ny * k];
}

inline dim3 inner_grid(const Geom& g) { return dim3((g.nx - 2 + 127) / 128, g.ny - 2, g.nz - 2); }
inline dim3 full_grid(const Geom& g) { return dim3((g.nx + 127) / 128, g.ny - 2, g.nz); }
inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// RAII swap of the wall-normal coefficients to the transposed operator
struct TransposeScope {
    tbl_handle* h;
    explicit TransposeScope(tbl_handle* h_) : h(h_) { swap(); }
    ~TransposeScope() { swap(); }
    void swap() {
        double* a = h->Ab; h->Ab = h->AbT; h->AbT = a;
        double* b = h->At; h->At = h->AtT; h->AtT = b;
    }
};

int dzero(tbl_handle* h, double* p, size_t n) {
    TBL_CUDA_TRY(cudaMemsetAsync(p, 0, n * sizeof(double), h->stream));
    return TBL_OK;
}
int dcopy(tbl_handle* h, double* dst, const double* src, size_t n) {
    TBL_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return TBL_OK;
}

AdjCoef adj_coef(const tbl_handle* h) {
    AdjCoef c;
    memset(&c, 0, sizeof(c));
    c.dx = h->cfg.dx; c.dy = h->cfg.dy; c.dxi = h->cfg.dxi; c.dt = h->cfg.dt; c.re = h->cfg.re;
    c.t = -h->cfg.dt / h->cfg.re;
    c.df1 = h->x3h[1] - h->x3h[0];
    c.df2 = h->x3h[2] - h->x3h[0];
    c.aw = 1.0 / (h->cfg.dx * h->cfg.dx);
    c.ue = h->cfg.ue;
    return c;
}

ConvAdjCoef conv_adj_coef(const tbl_handle* h) {
    ConvAdjCoef c;
    const double invdx = 1.0 / h->cfg.dx, invdy = 1.0 / h->cfg.dy, invdxi = 1.0 / h->cfg.dxi;
    const double c12 = 1.0 / 12.0;
    c.re = h->cfg.re; c.dx = h->cfg.dx; c.dy = h->cfg.dy; c.dt = h->cfg.dt;
    c.inv2x = 1.0 / (2.0 * h->cfg.dx); c.q25x = 0.25 * invdx; c.c12x = c12 * invdx;
    c.invdy = invdy; c.q25y = 0.25 * invdy; c.c12y = c12 * invdy;
    c.inv2z = 0.5 * invdxi; c.q25z = 0.25 * invdxi; c.c12z = c12 * invdxi;
    return c;
}

struct AdjCounters {
    int gs_sweeps = 0, gmres_iters = 0;
    double max_gs = 0.0, max_gmres = 0.0;
};

// Adjoint of one step.  u1: velocities after the step's inflow (3 x vol),
// u3: the step's output velocities.  T->lU / T->lP hold dL/d(output) on
// entry and dL/d(input) on return; dL/dc accumulates in T->lc.
int adj_step(tbl_handle* h, AdjTape* T, const double* u1, const double* u3, int nstep_of_step,
             const unsigned char* bits, AdjCounters& cnt) {
    const Geom& g = h->g;
    const size_t vol = (size_t)g.vol;
    const AdjCoef ac = adj_coef(h);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    double *l0 = T->lU[0], *l1 = T->lU[1], *l2 = T->lU[2], *lP = T->lP;
    const PreCopy Uu{u3, u1}, Uv{u3 + vol, u1 + vol}, Uw{u3 + 2 * vol, u1 + 2 * vol};
    const int t256 = 256;
    k_adj_periodic<<<nblk((long long)nx * nz, t256), t256, 0, h->stream>>>(g, l0, l1, l2, lP);
    ATRY(dzero(h, T->luold, (size_t)ny * nz));
    {
        const long long np = 2LL * (nx - 2) * (ny - 2) + 2LL * (ny - 2) * (nz - 2);
        k_adj_pbc_a<<<nblk(np, t256), t256, 0, h->stream>>>(g, ac, Uu, Uv, Uw, h->jacinv, l0, l1, l2, lP, T->AW,
                                                            T->LE, T->luold);
        const long long nb = (long long)nx * ny + (long long)ny * nz;
        k_adj_pbc_b<<<nblk(nb, t256), t256, 0, h->stream>>>(g, ac, Uu, Uv, Uw, h->jacinv, h->jac2, T->AW, T->LE, l0,
                                                            l2, lP);
    }
    k_adj_vel_out<<<nblk((long long)(ny - 2) * nz, t256), t256, 0, h->stream>>>(g, l0, l1, l2);
    k_adj_vel_walltop<<<nblk((long long)nx * (ny - 2), t256), t256, 0, h->stream>>>(g, l0, l1, l2, T->lc);
    // Poisson adjoint: L7^T mu = r
    ATRY(dzero(h, h->Q8, vol));
    k_adj_pc_rhs<<<inner_grid(g), 128, 0, h->stream>>>(g, 0.5 / h->cfg.dx, 0.5 / h->cfg.dy, 0.5 / h->cfg.dxi,
                                                       h->cfg.dt, h->jacinv, l0, l1, l2, lP, h->Q8);
    h->launches += 7;
    ATRY(dzero(h, h->PC, vol));
    {
        TransposeScope ts(h);
        std::vector<int32_t> kits;
        tbl_step_stats st;
        memset(&st, 0, sizeof(st));
        int s = gmres(h, nullptr, kits, st);
        if (s != TBL_OK && s != TBL_ERR_ZERO_RHS) return s;
        if (s == TBL_OK) {
            cnt.gmres_iters += st.gmres_iters;
            cnt.max_gmres = std::fmax(cnt.max_gmres, st.gmres_resid);
        }
    }
    // divergence^T, then A^T nu = . (same Gauss-Seidel, transposed coefficients)
    for (int c = 0; c < 3; ++c) ATRY(dzero(h, h->U[c], vol));
    k_adj_div_gsrhs<<<full_grid(g), 128, 0, h->stream>>>(g, 0.5 / h->cfg.dx, 0.5 / h->cfg.dy, h->cfg.dt, h->x3,
                                                         h->PC, l0, l1, l2, h->Q[0], h->Q[1], h->Q[2]);
    h->launches++;
    {
        TransposeScope ts(h);
        tbl_step_stats st;
        memset(&st, 0, sizeof(st));
        ATRY(gs_solve(h, nullptr, st, true));
        for (int c = 0; c < 3; ++c) {
            cnt.gs_sweeps += st.gs_sweeps[c];
            cnt.max_gs = std::fmax(cnt.max_gs, st.gs_resid[c]);
            if (st.gs_sweeps[c] >= h->cfg.mmax) return TBL_ERR_NOT_CONVERGED;
        }
    }
    k_adj_conv<<<full_grid(g), 128, 0, h->stream>>>(g, conv_adj_coef(h), ac.t, ac.aw, h->Ab, h->At, h->x3, h->jacinv,
                                                    u1, u1 + vol, u1 + 2 * vol, h->U[0], h->U[1], h->U[2], l0, l1,
                                                    l2, lP, bits);
    const int inflow_on = nstep_of_step > h->cfg.recycle_after ? 1 : 0;
    k_adj_inflow<<<nblk(ny - 2, 128), 128, 0, h->stream>>>(g, inflow_on, h->cfg.irec - 1, h->cfg.ue, h->usum2, h->wt,
                                                          h->newk, h->slab_of_k, h->slabs, h->sc, T->luold, l0, l1,
                                                          l2);
    h->launches += 2;
    TBL_CUDA_TRY(cudaGetLastError());
    return TBL_OK;
}

// ------------------------------------------------ checkpoints and tape
int save_ckpt(tbl_handle* h, Ckpt& c) {
    const size_t vol = (size_t)h->g.vol, pl = (size_t)h->g.ny * h->g.nz;
    for (int q = 0; q < 3; ++q) ATRY(dcopy(h, c.U[q], h->U[q], vol));
    ATRY(dcopy(h, c.P, h->Pr, vol));
    ATRY(dcopy(h, c.PC, h->PC, vol));
    ATRY(dcopy(h, c.ufl, h->ufl_live, 3 * pl));
    c.nstep = h->nstep; c.cont = h->cont; c.nstat = h->nstat; c.cnt2 = h->cnt2;
    c.time = h->time; c.lamda_host = h->lamda_host; c.fluc = h->fluc_updated;
    return TBL_OK;
}
int restore_ckpt(tbl_handle* h, const Ckpt& c) {
    const size_t vol = (size_t)h->g.vol, pl = (size_t)h->g.ny * h->g.nz;
    for (int q = 0; q < 3; ++q) ATRY(dcopy(h, h->U[q], c.U[q], vol));
    ATRY(dcopy(h, h->Pr, c.P, vol));
    ATRY(dcopy(h, h->PC, c.PC, vol));
    ATRY(dcopy(h, h->ufl_live, c.ufl, 3 * pl));
    h->nstep = c.nstep; h->cont = c.cont; h->nstat = c.nstat; h->cnt2 = c.cnt2;
    h->time = c.time; h->lamda_host = c.lamda_host; h->fluc_updated = c.fluc;
    return TBL_OK;
}

int tape_alloc(tbl_handle* h, int W, int ck) {
    AdjTape* T = h->adj;
    if (T && T->W == W && T->ck == ck) return TBL_OK;
    adj_free(h);
    T = new (std::nothrow) AdjTape();
    if (!T) return TBL_ERR_BAD_ARG;
    h->adj = T;
    const Geom& g = h->g;
    const size_t vol = (size_t)g.vol, pl = (size_t)g.ny * g.nz, n2 = (size_t)g.nx * g.nz;
    const int nseg = (W + ck - 1) / ck;
    const size_t ck_n = 5 * vol + 3 * pl;
    size_t n = (size_t)nseg * ck_n + (size_t)ck * 6 * vol + ck_n + 9 * n2 + 4 * vol;
    n += (size_t)g.nx * (g.ny - 2) + (size_t)g.nx * g.ny + 2 * pl + 4 * (size_t)g.nx + 8;
    n += 2 * (size_t)g.nx + 8;  // fin_diag
    TBL_CUDA_TRY(cudaMalloc((void**)&T->buf, n * sizeof(double)));
    TBL_CUDA_TRY(cudaMemset(T->buf, 0, n * sizeof(double)));
    T->buf_n = n;
    T->W = W; T->ck = ck; T->nseg = nseg; T->vol = vol;
    double* p = T->buf;
    auto take = [&](size_t m) { double* r = p; p += m; return r; };
    auto mk = [&](Ckpt& c) {
        for (int q = 0; q < 3; ++q) c.U[q] = take(vol);
        c.P = take(vol); c.PC = take(vol); c.ufl = take(3 * pl);
    };
    T->cks.resize(nseg);
    for (auto& c : T->cks) mk(c);
    T->segU1.resize(ck); T->segU3.resize(ck);
    for (int s = 0; s < ck; ++s) { T->segU1[s] = take(3 * vol); T->segU3[s] = take(3 * vol); }
    mk(T->fin);
    T->fin_sums = take(9 * n2);
    for (int q = 0; q < 3; ++q) T->lU[q] = take(vol);
    T->lP = take(vol);
    T->lc = take((size_t)g.nx * (g.ny - 2));
    T->AW = take((size_t)g.nx * g.ny);
    T->LE = take(pl);
    T->luold = take(pl);
    T->ocf = take(4 * (size_t)g.nx);
    T->jacc = take(8);
    T->fin_diag = take(2 * (size_t)g.nx + 8);
    T->nstep_of.assign(W, 0);
    return TBL_OK;
}

// Linear form of the patch wall shear (dnstbl2/dnstbl.f90:1636-1660) as
// per-column coefficients of w(i,j,k=1), u(i,j,k=1..3), averaged over the
// patch columns and the span, divided by Re.
int objective_coefs(const tbl_handle* h, double x_lo, double x_hi, std::vector<double>& cf) {
    const int nx = h->g.nx, ny = h->g.ny;
    std::vector<int> cols;
    for (int i = 1; i <= nx - 2; ++i)
        if (h->x1h[i] >= x_lo && h->x1h[i] <= x_hi) cols.push_back(i);
    if (cols.empty()) return TBL_ERR_BAD_ARG;
    cf.assign(4 * (size_t)nx, 0.0);
    const double s = 1.0 / ((double)cols.size() * (ny - 2) * h->cfg.re);
    const double dx = h->cfg.dx;
    const double df1 = h->x3h[1] - h->x3h[0], df2 = h->x3h[2] - h->x3h[0];
    const double den = df2 * df1 * df1 - df2 * df2 * df1;
    for (int i : cols) {
        if (i <= 2 || i >= nx - 3) {
            cf[i + 1] += s / (2.0 * dx);
            cf[i - 1] -= s / (2.0 * dx);
        } else {
            const double w6[7] = {-1.0, 9.0, -45.0, 0.0, 45.0, -9.0, 1.0};
            for (int o = -3; o <= 3; ++o) cf[i + o] += s * w6[o + 3] / (60.0 * dx);
        }
        cf[nx + i] += s * (-df1 * df1 + df2 * df2) / den;
        cf[2 * nx + i] += s * (-df2 * df2) / den;
        cf[3 * nx + i] += s * (df1 * df1) / den;
    }
    return TBL_OK;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

void adj_free(tbl_handle* h) {
    if (!h->adj) return;
    if (h->adj->buf) cudaFree(h->adj->buf);
    if (h->adj->bits) cudaFree(h->adj->bits);
    delete h->adj;
    h->adj = nullptr;
}

}  // namespace tbl

using namespace tbl;

extern "C" {

int tbl_set_wall_control(tbl_handle* h, const double* c) {
    if (!h) return TBL_ERR_BAD_ARG;
    const size_t n = (size_t)h->g.nx * (h->g.ny - 2);
    if (!c) {
        if (h->wallw) cudaFree(h->wallw);
        h->wallw = nullptr;
        return TBL_OK;
    }
    if (!h->wallw) TBL_CUDA_TRY(cudaMalloc((void**)&h->wallw, n * sizeof(double)));
    TBL_CUDA_TRY(cudaMemcpyAsync(h->wallw, c, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return TBL_OK;
}

int tbl_forward_window(tbl_handle* h, int32_t nsteps, const tbl_window_config* wc, double* objective,
                       tbl_step_stats* stats) {
    if (!h || !wc || nsteps < 1 || wc->ckpt_every < 1) return TBL_ERR_BAD_ARG;
    if (wc->branch_mode < TBL_BRANCH_FREE || wc->branch_mode > TBL_BRANCH_REPLAY) return TBL_ERR_BAD_ARG;
    const tbl_config& c = h->cfg;
    const int32_t not_adjoint = TBL_FLAG_REPLAY | TBL_FLAG_RB_ORDER | TBL_FLAG_RB_PRECOND |
                                TBL_FLAG_SSOR_SPAN_BLOCKS | TBL_FLAG_SSOR_STREAM_BLOCKS;
    if (c.precision != TBL_PREC_FP64 || (c.flags & not_adjoint) || c.variant != TBL_VARIANT_DNSTBL2)
        return TBL_ERR_BAD_ARG;
    for (int s = 1; s <= nsteps; ++s)
        if ((h->cont + s) % c.cum == 0) return TBL_ERR_BAD_ARG;  // a rescaling step inside the window
    std::vector<double> cf;
    ATRY(objective_coefs(h, wc->x_lo, wc->x_hi, cf));
    const int ck = wc->ckpt_every < nsteps ? wc->ckpt_every : nsteps;
    ATRY(tape_alloc(h, nsteps, ck));
    AdjTape* T = h->adj;
    T->valid = false;
    const Geom& g = h->g;
    const size_t vol = (size_t)g.vol;
    const int bm = wc->branch_mode;
    if (bm == TBL_BRANCH_REPLAY && !T->bits_valid) return TBL_ERR_BAD_ARG;  // no record of this window
    if (bm != TBL_BRANCH_FREE && !T->bits) {
        TBL_CUDA_TRY(cudaMalloc((void**)&T->bits, (size_t)nsteps * vol));
        TBL_CUDA_TRY(cudaMemset(T->bits, 0, (size_t)nsteps * vol));
    }
    if (bm == TBL_BRANCH_RECORD) T->bits_valid = false;
    T->branch_mode = bm;
    TBL_CUDA_TRY(cudaMemcpyAsync(T->ocf, cf.data(), cf.size() * 8, cudaMemcpyHostToDevice, h->stream));
    ATRY(dzero(h, T->jacc, 1));
    const auto t0 = std::chrono::steady_clock::now();
    const int last0 = (T->nseg - 1) * ck;
    for (int s = 0; s < nsteps; ++s) {
        if (s % ck == 0) ATRY(save_ckpt(h, T->cks[s / ck]));
        const bool rec = s >= last0;
        h->tape_u1 = rec ? T->segU1[s - last0] : nullptr;
        h->conv_bits_mode = bm;
        h->conv_bits = bm != TBL_BRANCH_FREE ? T->bits + (size_t)s * vol : nullptr;
        const int st = one_step(h, stats ? &stats[s] : nullptr);
        h->tape_u1 = nullptr;
        h->conv_bits_mode = TBL_BRANCH_FREE;
        h->conv_bits = nullptr;
        if (st != TBL_OK) return st;
        T->nstep_of[s] = h->nstep;
        if (rec)
            for (int q = 0; q < 3; ++q) ATRY(dcopy(h, T->segU3[s - last0] + q * vol, h->U[q], vol));
        k_objective<<<1, 256, 0, h->stream>>>(g, T->ocf, h->U[0], h->U[2], T->jacc);
        h->launches++;
    }
    TBL_CUDA_TRY(cudaGetLastError());
    ATRY(readback(h, T->jacc, sizeof(double)));
    const double J = h->hpin[0] / nsteps;
    ATRY(save_ckpt(h, T->fin));
    ATRY(dcopy(h, T->fin_sums, h->sums, 9 * (size_t)g.nx * g.nz));
    ATRY(dcopy(h, T->fin_diag, h->sumxz, (size_t)g.nx));
    ATRY(dcopy(h, T->fin_diag + g.nx, h->tauw_win, (size_t)g.nx));
    ATRY(dcopy(h, T->fin_diag + 2 * g.nx, h->ubulk, 5));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    T->forward_ms = ms_since(t0);
    if (bm == TBL_BRANCH_RECORD) T->bits_valid = true;
    T->valid = true;
    if (objective) *objective = J;
    return TBL_OK;
}

int tbl_backward_window(tbl_handle* h, double dL_dJ, const tbl_fields* dL_dfinal, double* dL_dc,
                        tbl_fields* dL_dinitial, tbl_adjoint_stats* out) {
    if (!h || !dL_dc || !h->adj || !h->adj->valid) return TBL_ERR_BAD_ARG;
    AdjTape* T = h->adj;
    const Geom& g = h->g;
    const size_t vol = (size_t)g.vol;
    const auto t0 = std::chrono::steady_clock::now();
    for (int q = 0; q < 3; ++q) ATRY(dzero(h, T->lU[q], vol));
    ATRY(dzero(h, T->lP, vol));
    ATRY(dzero(h, T->lc, (size_t)g.nx * (g.ny - 2)));
    if (dL_dfinal) {
        const double* src[4] = {dL_dfinal->u, dL_dfinal->v, dL_dfinal->w, dL_dfinal->p};
        double* dst[4] = {T->lU[0], T->lU[1], T->lU[2], T->lP};
        for (int q = 0; q < 4; ++q)
            if (src[q]) ATRY(put3(h, dst[q], src[q]));
    }
    AdjCounters cnt;
    int recomputed = 0;
    const int W = T->W, ck = T->ck;
    int status = TBL_OK;
    for (int seg = T->nseg - 1; seg >= 0 && status == TBL_OK; --seg) {
        const int s0 = seg * ck, s1 = (s0 + ck < W) ? s0 + ck : W;
        if (seg != T->nseg - 1) {  // recompute the segment from its checkpoint
            ATRY(restore_ckpt(h, T->cks[seg]));
            for (int s = s0; s < s1; ++s) {
                h->tape_u1 = T->segU1[s - s0];
                if (T->branch_mode != TBL_BRANCH_FREE) {  // the recorded decisions reproduce the window exactly
                    h->conv_bits_mode = TBL_BRANCH_REPLAY;
                    h->conv_bits = T->bits + (size_t)s * vol;
                }
                status = one_step(h, nullptr);
                h->tape_u1 = nullptr;
                h->conv_bits_mode = TBL_BRANCH_FREE;
                h->conv_bits = nullptr;
                if (status != TBL_OK) break;
                for (int q = 0; q < 3; ++q) ATRY(dcopy(h, T->segU3[s - s0] + q * vol, h->U[q], vol));
                recomputed++;
            }
            if (status != TBL_OK) break;
        }
        for (int s = s1 - 1; s >= s0; --s) {
            k_objective_adj<<<nblk((long long)g.nx * (g.ny - 2), 256), 256, 0, h->stream>>>(
                g, T->ocf, dL_dJ / W, T->lU[0], T->lU[2]);
            h->launches++;
            status = adj_step(h, T, T->segU1[s - s0], T->segU3[s - s0], T->nstep_of[s],
                              T->branch_mode != TBL_BRANCH_FREE ? T->bits + (size_t)s * vol : nullptr, cnt);
            if (status != TBL_OK) break;
        }
    }
    if (status == TBL_OK) {
        TBL_CUDA_TRY(cudaMemcpyAsync(dL_dc, T->lc, (size_t)g.nx * (g.ny - 2) * 8, cudaMemcpyDeviceToHost,
                                     h->stream));
        if (dL_dinitial) {
            double* dst[4] = {dL_dinitial->u, dL_dinitial->v, dL_dinitial->w, dL_dinitial->p};
            const double* src[4] = {T->lU[0], T->lU[1], T->lU[2], T->lP};
            for (int q = 0; q < 4; ++q)
                if (dst[q]) ATRY(get3(h, dst[q], src[q]));
        }
    }
    // the handle returns to the state at the end of the window
    ATRY(restore_ckpt(h, T->fin));
    ATRY(dcopy(h, h->sums, T->fin_sums, 9 * (size_t)g.nx * g.nz));
    ATRY(dcopy(h, h->sumxz, T->fin_diag, (size_t)g.nx));
    ATRY(dcopy(h, h->tauw_win, T->fin_diag + g.nx, (size_t)g.nx));
    ATRY(dcopy(h, h->ubulk, T->fin_diag + 2 * g.nx, 5));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (out) {
        memset(out, 0, sizeof(*out));
        out->steps = W;
        out->recomputed_steps = recomputed;
        out->adj_gs_sweeps = cnt.gs_sweeps;
        out->adj_gmres_iters = cnt.gmres_iters;
        out->status = status;
        out->max_gs_resid = cnt.max_gs;
        out->max_gmres_resid = cnt.max_gmres;
        out->forward_ms = T->forward_ms;
        out->backward_ms = ms_since(t0);
    }
    return status;
}

}  // extern "C"
