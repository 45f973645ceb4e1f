// tbl_stencil.cu -- point-parallel FP64 kernels of the time step: inflow
// recycling, convection + explicit RHS, GS residual, divergence, projection,
// boundary conditions, statistics and the rescaling bookkeeping.
//
// Each kernel cites the reference loop nest it replaces
// (theparvezahmad/turbulentBL dnstbl2/dnstbl.f90).  Expression order follows
// the reference; the compiler may contract a*b+c into FMA (well inside the
// 1e-12 parity tolerance).
#include "tbl_internal.cuh"
#include "tbl_reduce.cuh"
#include "tbl_kernels.cuh"

namespace tbl {

__device__ __forceinline__ long long idx(const Geom& g, int i, int j, int k) {
    return (long long)i + (long long)g.sx * ((long long)j + (long long)g.ny * k);
}
// 0-based periodic neighbours over the unique rows 1..ny-2
__device__ __forceinline__ int jm1(const Geom& g, int j) { return j == 1 ? g.ny - 2 : j - 1; }
__device__ __forceinline__ int jp1(const Geom& g, int j) { return j == g.ny - 2 ? 1 : j + 1; }
__device__ __forceinline__ int jm2(const Geom& g, int j) { return j == 2 ? g.ny - 2 : jm1(g, j) - 1; }
__device__ __forceinline__ int jp2(const Geom& g, int j) { return j == g.ny - 3 ? 1 : jp1(g, j) + 1; }

// ------------------------------------------------------------------ inflow
// Utold(1,:,:,1) = Ut(1,:,:,1) (dnstbl2/dnstbl.f90:549; only this plane is read later)
template <typename T>
__global__ void k_save_uold(Geom g, const T* __restrict__ u1, double* __restrict__ uold1) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.ny * g.nz) return;
    int j = t % g.ny, k = t / g.ny;
    uold1[t] = u1[idx(g, 0, j, k)];
}

// Recycling inflow (dnstbl2/dnstbl.f90:557-618).  One thread per (j,k).
// ramp: the u mean is eps usum2(irec,new(k)) + (1-eps) Ume1(k) (originalTBL
// fnldnstbl.f90:577, dnssetbl dnssetbl.f90:268); vlam: the v mean is scaled
// by lamda (dnssetbl.f90:271); wcol: the Wt column of the blend, nx-2 for the
// redundant i loop (:594-600), 0 for dnssetbl's Wt(1,k) (dnssetbl.f90:291).
template <typename T>
__global__ void k_inflow(Geom g, T* __restrict__ u1, T* __restrict__ u2, T* __restrict__ u3,
                         const double* __restrict__ usum2, const double* __restrict__ vsum2,
                         const double* __restrict__ wsum2, const double* __restrict__ wt,
                         const double* __restrict__ ume1, const int* __restrict__ newk,
                         const double* __restrict__ ufl_file, const double* __restrict__ ufl_live,
                         const int* __restrict__ slab_of_k, const SlabDesc* __restrict__ slabs,
                         const DevScalars* __restrict__ sc, int irec0, double ue, int ramp, double eps, int vlam,
                         int wcol) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int J = g.ny - 2;
    if (t >= J * (g.nz - 2)) return;
    int j = 1 + t % J, k = 1 + t / J;
    const int nx = g.nx;
    const long long q = idx(g, 0, j, k);
    const size_t ir = (size_t)irec0 + (size_t)nx * k;
    if (usum2[ir] < (0.99 * ue)) {
        int nk = newk[k] - 1;  // 0-based source plane
        double uin = ramp ? eps * (usum2[(size_t)irec0 + (size_t)nx * nk]) + (1 - eps) * ume1[k] : ume1[k];
        double vin = vsum2[(size_t)irec0 + (size_t)nx * nk];
        if (vlam) vin = sc->lamda * vin;
        double win = wsum2[(size_t)irec0 + (size_t)nx * nk];
        const SlabDesc s = slabs[slab_of_k[k]];
        bool live = nk >= s.bn && nk < s.bn + s.K;
        const double* src = live ? ufl_live : ufl_file;
        size_t pl = (size_t)g.ny * g.nz;
        size_t pj = (size_t)j + (size_t)g.ny * nk;
        double lam = sc->lamda;
        double f1 = lam * src[pj], f2 = lam * src[pl + pj], f3 = lam * src[2 * pl + pj];
        double w_ = wt[(size_t)wcol + (size_t)nx * k];
        u1[q] = (T)((uin + f1) * (1.0 - w_) + (uin + f1) * w_);
        u2[q] = (T)((vin + f2) * (1.0 - w_) + (vin + f2) * w_);
        u3[q] = (T)((win + f3) * (1.0 - w_) + (win + f3) * w_);
    } else {
        u1[q] = (T)usum2[ir];
        u2[q] = (T)vsum2[ir];
        u3[q] = (T)wsum2[ir];
    }
}

// ------------------------------------------------------- convection + RHS
template <typename R>
struct ConvCoef {
    R tf, dx, dy, invdx, invdy, invdxi;
    R inv2dx;    // 1/(2 dx)
    R c12x, c12y, c12z;  // onetwelfth*inv
    R q25x, q25y, q25z;  // 0.25*inv
    R h05z;      // 0.5*invdxi
    R h05y;      // 0.5*invdy
    R dt;
    int pe_mode; // Peclet window: 0 dnstbl2 2 < Pe < 50 (5 in xi); 1 originalTBL Pe > 2; 2 dnssetbl |Pe| > 2
    int ycen;    // 1: central differences on the first/last span rows (dnssetbl.f90:325-326)
};

// The dissipative window of one direction (hi = 50 in x and y, 5 in xi):
// dnstbl2 2 < Pe < hi (:655, :679, :701); originalTBL Pe > 2
// (fnldnstbl.f90:665, :689, :711); dnssetbl |Re u h| > 2 (dnssetbl.f90:311,
// :323, :335), which is |Pe| > 2 for the signed Pe.
template <typename R>
__device__ __forceinline__ bool pe_window(R Pe, R hi, int mode) {
    if (mode == 2) return abs(Pe) > R(2);
    if (mode == 1) return Pe > R(2);
    return Pe > R(2) && Pe < hi;
}

// Convection of F along x (dnstbl2/dnstbl.f90:651-664)
template <typename R>
__device__ __forceinline__ R conv_x(R u, bool nearb, R fm2, R fm1, R f0, R fp1, R fp2,
                                    const ConvCoef<R>& c) {
    R sgn = u > R(-1) ? R(1) : R(-1);  // sign(1, ceiling(u))
    R Pe = sgn * c.tf * u * c.dx;
    if (nearb) return u * (fp1 - fm1) * c.inv2dx;
    if (pe_window(Pe, R(50), c.pe_mode)) {
        R t1 = abs(u) * (fp2 - R(4) * fp1 + R(6) * f0 - R(4) * fm1 + fm2) * c.q25x;
        R t2 = u * (-fp2 + R(8) * fp1 - R(8) * fm1 + fm2) * c.c12x;
        return t1 + t2;
    }
    return u * ((fm2 - R(8) * fm1 + R(8) * fp1 - fp2) * c.c12x);
}

// y: first-order upwind at the first/last unique rows (:670-677)
template <typename R>
__device__ __forceinline__ R conv_y(R v, bool nearb, R fm2, R fm1, R f0, R fp1, R fp2,
                                    const ConvCoef<R>& c) {
    R sgn = v > R(-1) ? R(1) : R(-1);
    R Pe = sgn * c.tf * v * c.dy;
    if (nearb) {
        if (c.ycen) return v * (fp1 - fm1) * c.h05y;
        R a1 = max(v, R(0)), b = min(v, R(0));
        return a1 * ((f0 - fm1) * c.invdy) + b * ((fp1 - f0) * c.invdy);
    }
    if (pe_window(Pe, R(50), c.pe_mode)) {
        R t1 = abs(v) * (fp2 - R(4) * fp1 + R(6) * f0 - R(4) * fm1 + fm2) * c.q25y;
        R t2 = v * (-fp2 + R(8) * fp1 - R(8) * fm1 + fm2) * c.c12y;
        return t1 + t2;
    }
    return v * ((fm2 - R(8) * fm1 + R(8) * fp1 - fp2) * c.c12y);
}

// xi: Pe from the physical spacing, window 2 < Pe < 5 (:690-713)
template <typename R>
__device__ __forceinline__ R conv_z(R w, R dz, bool nearb, R fm2, R fm1, R f0, R fp1, R fp2,
                                    const ConvCoef<R>& c) {
    R sgn = w > R(-1) ? R(1) : R(-1);
    R Pe = (sgn * c.tf * w * dz);
    if (nearb) return (w * (fp1 - fm1) * c.h05z);
    if (pe_window(Pe, R(5), c.pe_mode)) {
        R t1 = abs(w) * (fp2 - R(4) * fp1 + R(6) * f0 - R(4) * fm1 + fm2) * c.q25z;
        R t2 = w * (-fp2 + R(8) * fp1 - R(8) * fm1 + fm2) * c.c12z;
        return t1 + t2;
    }
    return w * ((fm2 - R(8) * fm1 + R(8) * fp1 - fp2) * c.c12z);
}

// conv(i,j,k,1..3) and Q(i,j,k,1..3) (dnstbl2/dnstbl.f90:621-768), fused:
// conv is never stored.  One thread per interior point.
template <typename T>
__global__ void __launch_bounds__(128) k_conv_q(Geom g, ConvCoef<T> c, const T* __restrict__ U1,
                                                const T* __restrict__ U2, const T* __restrict__ U3,
                                                const T* __restrict__ Pr, const double* __restrict__ x3,
                                                const double* __restrict__ jacinv, T* __restrict__ Q1,
                                                T* __restrict__ Q2, T* __restrict__ Q3) {
    int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    const long long p = idx(g, i, j, k);
    const long long sy = g.sx, sz = g.ps;
    const int ja = jm1(g, j), jb = jm2(g, j), jc = jp1(g, j), jd = jp2(g, j);
    const long long pjm1 = idx(g, i, ja, k), pjm2 = idx(g, i, jb, k), pjp1 = idx(g, i, jc, k),
                    pjp2 = idx(g, i, jd, k);
    const bool nbx = (i <= 1) || (i >= g.nx - 2);
    const bool nby = (j == 1) || (j == g.ny - 2);
    const bool nbz = (k <= 1) || (k >= g.nz - 2);
    const T u = U1[p], v = U2[p], w = U3[p];
    const T dz = (T)(x3[k + 1] - x3[k]);
    const T jk = (T)jacinv[k];
    const T* Fs[3] = {U1, U2, U3};
    T conv[3];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
        const T* F = Fs[cc];
        T f0 = F[p];
        T d1 = conv_x<T>(u, nbx, nbx ? T(0) : F[p - 2], F[p - 1], f0, F[p + 1], nbx ? T(0) : F[p + 2], c);
        T d2 = conv_y<T>(v, nby, F[pjm2], F[pjm1], f0, F[pjp1], F[pjp2], c);
        T d3 = conv_z<T>(w, dz, nbz, nbz ? T(0) : F[p - 2 * sz], F[p - sz], f0, F[p + sz],
                           nbz ? T(0) : F[p + 2 * sz], c);
        conv[cc] = d1 + d2 + (d3 * jk);
    }
    (void)sy;
    T g1 = T(0.5) * (Pr[p + 1] - Pr[p - 1]) * c.invdx;
    T g2 = T(0.5) * (Pr[pjp1] - Pr[pjm1]) * c.invdy;
    T g3 = T(0.5) * (Pr[p + sz] - Pr[p - sz]) * (c.invdxi * jk);
    T q5 = u + (c.dt * (T(0) - conv[0]));
    Q1[p] = q5 - (c.dt * g1);
    T q6 = v + (c.dt * (T(0) - conv[1]));
    Q2[p] = q6 - (c.dt * g2);
    T q7 = w + (c.dt * (T(0) - conv[2]));
    Q3[p] = q7 - (c.dt * g3);
}

// ------------------------------------------ frozen-branch convection (FP64)
// The same convection + explicit RHS with its data-dependent decisions
// either recorded (BM = 1) or taken from a record (BM = 2) instead of from the
// current field: used by adjoint windows to make finite differences follow
// the branch decisions the adjoint differentiates.  One byte per point:
// bits 0-2 the x/y/z Peclet windows, bit 3 u >= 0, bit 4 v >= 0, bit 5 v <= 0,
// bit 6 w >= 0.  With BM = 1 every value is bitwise that of k_conv_q.
__device__ __forceinline__ unsigned conv_decide(double u, double v, double w, double dz, const ConvCoef<double>& c) {
    unsigned b = 0;
    double s = u > -1.0 ? 1.0 : -1.0;
    double Pe = s * c.tf * u * c.dx;
    if (Pe > 2.0 && Pe < 50.0) b |= 1u;
    s = v > -1.0 ? 1.0 : -1.0;
    Pe = s * c.tf * v * c.dy;
    if (Pe > 2.0 && Pe < 50.0) b |= 2u;
    s = w > -1.0 ? 1.0 : -1.0;
    Pe = (s * c.tf * w * dz);
    if (Pe > 2.0 && Pe < 5.0) b |= 4u;
    if (u >= 0.0) b |= 8u;
    if (v >= 0.0) b |= 16u;
    if (v <= 0.0) b |= 32u;
    if (w >= 0.0) b |= 64u;
    return b;
}

// x and xi: central (near the ends), windowed dissipative, or 4th-order central
__device__ __forceinline__ double conv_fxz(double m, bool nearb, bool win, bool pos, double fm2, double fm1, double f0,
                                          double fp1, double fp2, double near_c, double q25, double c12) {
    if (nearb) return m * (fp1 - fm1) * near_c;
    if (win) {
        const double a = pos ? m : -m;
        double t1 = a * (fp2 - 4.0 * fp1 + 6.0 * f0 - 4.0 * fm1 + fm2) * q25;
        double t2 = m * (-fp2 + 8.0 * fp1 - 8.0 * fm1 + fm2) * c12;
        return t1 + t2;
    }
    return m * ((fm2 - 8.0 * fm1 + 8.0 * fp1 - fp2) * c12);
}

__device__ __forceinline__ double conv_fy(double v, bool nearb, bool win, bool vp, bool vn, double fm2, double fm1,
                                         double f0, double fp1, double fp2, const ConvCoef<double>& c) {
    if (nearb) {
        const double a1 = vp ? v : 0.0, b = vn ? v : 0.0;
        return a1 * ((f0 - fm1) * c.invdy) + b * ((fp1 - f0) * c.invdy);
    }
    if (win) {
        const double a = vp ? v : -v;
        double t1 = a * (fp2 - 4.0 * fp1 + 6.0 * f0 - 4.0 * fm1 + fm2) * c.q25y;
        double t2 = v * (-fp2 + 8.0 * fp1 - 8.0 * fm1 + fm2) * c.c12y;
        return t1 + t2;
    }
    return v * ((fm2 - 8.0 * fm1 + 8.0 * fp1 - fp2) * c.c12y);
}

template <int BM>
__global__ void __launch_bounds__(128) k_conv_q_br(Geom g, ConvCoef<double> c, const double* __restrict__ U1,
                                                   const double* __restrict__ U2, const double* __restrict__ U3,
                                                   const double* __restrict__ Pr, const double* __restrict__ x3,
                                                   const double* __restrict__ jacinv, double* __restrict__ Q1,
                                                   double* __restrict__ Q2, double* __restrict__ Q3,
                                                   unsigned char* __restrict__ bits) {
    int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    const long long p = idx(g, i, j, k);
    const long long sz = g.ps;
    const int ja = jm1(g, j), jb = jm2(g, j), jc = jp1(g, j), jd = jp2(g, j);
    const long long pjm1 = idx(g, i, ja, k), pjm2 = idx(g, i, jb, k), pjp1 = idx(g, i, jc, k),
                    pjp2 = idx(g, i, jd, k);
    const bool nbx = (i <= 1) || (i >= g.nx - 2);
    const bool nby = (j == 1) || (j == g.ny - 2);
    const bool nbz = (k <= 1) || (k >= g.nz - 2);
    const double u = U1[p], v = U2[p], w = U3[p];
    const double dz = (x3[k + 1] - x3[k]);
    const double jk = jacinv[k];
    unsigned b;
    if (BM == 2) {
        b = bits[p];
    } else {
        b = conv_decide(u, v, w, dz, c);
        bits[p] = (unsigned char)b;
    }
    const bool wx = b & 1u, wy = b & 2u, wz = b & 4u, up = b & 8u, vp = b & 16u, vn = b & 32u, wp = b & 64u;
    const double* Fs[3] = {U1, U2, U3};
    double conv[3];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
        const double* F = Fs[cc];
        double f0 = F[p];
        double d1 = conv_fxz(u, nbx, wx, up, nbx ? 0.0 : F[p - 2], F[p - 1], f0, F[p + 1], nbx ? 0.0 : F[p + 2],
                             c.inv2dx, c.q25x, c.c12x);
        double d2 = conv_fy(v, nby, wy, vp, vn, F[pjm2], F[pjm1], f0, F[pjp1], F[pjp2], c);
        double d3 = conv_fxz(w, nbz, wz, wp, nbz ? 0.0 : F[p - 2 * sz], F[p - sz], f0, F[p + sz],
                             nbz ? 0.0 : F[p + 2 * sz], c.h05z, c.q25z, c.c12z);
        conv[cc] = d1 + d2 + (d3 * jk);
    }
    double g1 = 0.5 * (Pr[p + 1] - Pr[p - 1]) * c.invdx;
    double g2 = 0.5 * (Pr[pjp1] - Pr[pjm1]) * c.invdy;
    double g3 = 0.5 * (Pr[p + sz] - Pr[p - sz]) * (c.invdxi * jk);
    double q5 = u + (c.dt * (0.0 - conv[0]));
    Q1[p] = q5 - (c.dt * g1);
    double q6 = v + (c.dt * (0.0 - conv[1]));
    Q2[p] = q6 - (c.dt * g2);
    double q7 = w + (c.dt * (0.0 - conv[2]));
    Q3[p] = q7 - (c.dt * g3);
}

// ---------------------------------------------------------- GS residual
// L1 norm of the residual of (1 - dt/Re L7) U = Q over all slabs' interiors,
// with current (global) halos (dnstbl2/dnstbl.f90:781-828).  blockIdx.y picks
// the component from `comps`; result -> sc->red[comp].
struct GsCoef {
    double cE, cW, cN, cS;  // t*Av{e,w,n,s}, t = -dt/Re
};

// One block per (plane, row) at a time; the per-plane coefficients come from
// the table k_gs_coef fills at the start of every GS solve ([d|cT|cB] at
// 4nz..7nz, the same values as 1 + t Ap(k), t At(k), t Ab(k)).  A row's |res|
// is summed in T, the rows in FP64.
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_gs_resid(Geom g, GsCoef gc, const double* __restrict__ pc,
                                                          const T* __restrict__ U0, const T* __restrict__ U1,
                                                          const T* __restrict__ U2, const T* __restrict__ Q0,
                                                          const T* __restrict__ Q1, const T* __restrict__ Q2,
                                                          int3 comps, int ncomp, RedWork rw, DevScalars* sc) {
    __shared__ double s_red[RED_THREADS / 32];
    const int cid = blockIdx.y;
    const int comp = cid == 0 ? comps.x : (cid == 1 ? comps.y : comps.z);
    const T* F = comp == 0 ? U0 : (comp == 1 ? U1 : U2);
    const T* Qc = comp == 0 ? Q0 : (comp == 1 ? Q1 : Q2);
    const int J = g.ny - 2, nk = g.nz - 2, nz = g.nz;
    const int rows = J * nk;
    const T cE = (T)gc.cE, cW = (T)gc.cW, cN = (T)gc.cN, cS = (T)gc.cS;
    double acc = 0.0;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int j = 1 + r % J, k = 1 + r / J;
        const T d = (T)pc[4 * nz + k], cT = (T)pc[5 * nz + k], cB = (T)pc[6 * nz + k];
        const long long row = idx(g, 0, j, k);
        const long long rjp = idx(g, 0, jp1(g, j), k), rjm = idx(g, 0, jm1(g, j), k);
        T racc = T(0);
        for (int i = 1 + threadIdx.x; i <= g.nx - 2; i += blockDim.x) {
            const long long p = row + i;
            T res = Qc[p] - d * F[p] - cE * F[p + 1] - cW * F[p - 1] - cN * F[rjp + i] - cS * F[rjm + i] -
                    cT * F[p + g.ps] - cB * F[p - g.ps];
            racc += abs(res);
        }
        acc += (double)racc;
    }
    double bt = block_sum(acc, s_red);
    grid_finish(bt, rw, comp, gridDim.x, blockIdx.x, &sc->red[comp], 0);
}

// ------------------------------------------------------------ divergence
// Q8 = div(U*)/dt (dnstbl2/dnstbl.f90:905-935)
template <typename T>
__global__ void __launch_bounds__(128) k_div(Geom g, double invdx, double invdy, double dt,
                                             const T* __restrict__ U1, const T* __restrict__ U2,
                                             const T* __restrict__ U3, const double* __restrict__ x3,
                                             double* __restrict__ Q8) {
    int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    long long p = idx(g, i, j, k);
    const double u0 = U1[p], v0 = U2[p], w0 = U3[p];
    double d1 = ((((double)U1[p + 1] + u0) * 0.5) - (((u0 + (double)U1[p - 1]) * 0.5))) * invdx;
    double d2 = ((((double)U2[idx(g, i, jp1(g, j), k)] + v0) * 0.5) -
                 (((v0 + (double)U2[idx(g, i, jm1(g, j), k)]) * 0.5))) * invdy;
    double d3 = 2.0 * ((((double)U3[p + g.ps] + w0) * 0.5) - (((w0 + (double)U3[p - g.ps]) * 0.5))) /
                (x3[k + 1] - x3[k - 1]);
    Q8[p] = (d1 + d2 + d3) / dt;
}

// -------------------------------------------------- PCorr faces (:940-950)
__global__ void k_pc_zero_faces(Geom g, double* __restrict__ PC) {
    // faces i = 0, nx-1 (all j,k); j = 0, ny-1 (all i,k); k = 0, nz-1 (all i,j)
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nA = (long long)g.ny * g.nz, nB = (long long)g.nx * g.nz, nC = (long long)g.nx * g.ny;
    if (t < nA) {
        int j = (int)(t % g.ny), k = (int)(t / g.ny);
        PC[idx(g, 0, j, k)] = 0.0; PC[idx(g, g.nx - 1, j, k)] = 0.0;
        return;
    }
    t -= nA;
    if (t < nB) {
        int i = (int)(t % g.nx), k = (int)(t / g.nx);
        PC[idx(g, i, 0, k)] = 0.0; PC[idx(g, i, g.ny - 1, k)] = 0.0;
        return;
    }
    t -= nB;
    if (t < nC) {
        int i = (int)(t % g.nx), j = (int)(t / g.nx);
        PC[idx(g, i, j, 0)] = 0.0; PC[idx(g, i, j, g.nz - 1)] = 0.0;
    }
}

// p' extrapolation, wall and top (:1245-1255).  One thread per (i, j unique).
__global__ void k_pc_bc_walltop(Geom g, double* __restrict__ PC) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int J = g.ny - 2;
    if (t >= g.nx * J) return;
    int i = t % g.nx, j = 1 + t / g.nx;
    int nz = g.nz;
    PC[idx(g, i, j, 0)] = ((4.0 * PC[idx(g, i, j, 1)]) - PC[idx(g, i, j, 2)]) / 3.0;
    PC[idx(g, i, j, nz - 1)] =
        (5.0 * PC[idx(g, i, j, nz - 2)] + (-4.0 * PC[idx(g, i, j, nz - 3)] + PC[idx(g, i, j, nz - 4)])) / 2.0;
}

// spanwise periodic copy of p' (:1257-1258), one thread per (i,k)
__global__ void k_pc_periodic(Geom g, double* __restrict__ PC) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nx * g.nz) return;
    int i = t % g.nx, k = t / g.nx;
    PC[idx(g, i, 0, k)] = PC[idx(g, i, g.ny - 2, k)];
    PC[idx(g, i, g.ny - 1, k)] = PC[idx(g, i, 1, k)];
}

// p' inflow/outflow extrapolation (:1260-1262), one thread per (j unique, k)
__global__ void k_pc_bc_inout(Geom g, double* __restrict__ PC) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int J = g.ny - 2;
    if (t >= J * g.nz) return;
    int j = 1 + t % J, k = t / J;
    int nx = g.nx;
    PC[idx(g, 0, j, k)] = (4.0 * PC[idx(g, 1, j, k)] - PC[idx(g, 2, j, k)]) / 3.0;
    PC[idx(g, nx - 1, j, k)] =
        (5.0 * PC[idx(g, nx - 2, j, k)] + (-4.0 * PC[idx(g, nx - 3, j, k)] + PC[idx(g, nx - 4, j, k)])) / 2.0;
}

// P += p', U -= dt grad p' (dnstbl2/dnstbl.f90:1268-1314)
template <typename T>
__global__ void __launch_bounds__(128) k_project(Geom g, double invdx, double invdy, double invdxi, double dt,
                                                 const double* __restrict__ jacinv, const double* __restrict__ PC,
                                                 T* __restrict__ Pr, T* __restrict__ U1,
                                                 T* __restrict__ U2, T* __restrict__ U3) {
    int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    long long p = idx(g, i, j, k);
    Pr[p] = (T)((double)Pr[p] + PC[p]);
    double g1 = 0.5 * (PC[p + 1] - PC[p - 1]) * (invdx);
    double g2 = 0.5 * (PC[idx(g, i, jp1(g, j), k)] - PC[idx(g, i, jm1(g, j), k)]) * (invdy);
    double g3 = 0.5 * (PC[p + g.ps] - PC[p - g.ps]) * (invdxi * jacinv[k]);
    U1[p] = (T)((double)U1[p] - (dt * g1));
    U2[p] = (T)((double)U2[p] - (dt * g2));
    U3[p] = (T)((double)U3[p] - (dt * g3));
}

// velocity BCs, wall and top (:1317-1330), one thread per (i, j unique).
// wallw (nx*(ny-2), or null for the reference's w = 0) is the wall-normal
// blowing/suction velocity set by tbl_set_wall_control.
template <typename T>
__global__ void k_vel_bc_walltop(Geom g, T* __restrict__ U1, T* __restrict__ U2, T* __restrict__ U3,
                                 const double* __restrict__ wallw) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int J = g.ny - 2;
    if (t >= g.nx * J) return;
    int i = t % g.nx, j = 1 + t / g.nx;
    int nz = g.nz;
    T* Us[3] = {U1, U2, U3};
    Us[0][idx(g, i, j, 0)] = T(0);
    Us[1][idx(g, i, j, 0)] = T(0);
    Us[2][idx(g, i, j, 0)] = wallw ? (T)wallw[t] : T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c)
        Us[c][idx(g, i, j, nz - 1)] =
            (T)((4.0 * (double)Us[c][idx(g, i, j, nz - 2)] - (double)Us[c][idx(g, i, j, nz - 3)]) / 3.0);
}

// outflow (:1342), one thread per (j unique, k all)
template <typename T>
__global__ void k_vel_bc_out(Geom g, T* __restrict__ U1, T* __restrict__ U2, T* __restrict__ U3) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int J = g.ny - 2;
    if (t >= J * g.nz) return;
    int j = 1 + t % J, k = t / J;
    int nx = g.nx;
    T* Us[3] = {U1, U2, U3};
#pragma unroll
    for (int c = 0; c < 3; ++c)
        Us[c][idx(g, nx - 1, j, k)] =
            (T)((4.0 * (double)Us[c][idx(g, nx - 2, j, k)] - (double)Us[c][idx(g, nx - 3, j, k)]) / 3.0);
}

struct PbcCoef {
    double dx, dy, dxi, re, dt, df1, df2;
};

// pressure BCs (:1352-1461): wall, top, outflow, inflow -- independent of
// each other, one flat index space.
template <typename T>
__global__ void k_press_bc(Geom g, PbcCoef c, const T* __restrict__ U1p, const T* __restrict__ U2p,
                           const T* __restrict__ U3p, const double* __restrict__ uold1,
                           const double* __restrict__ jacinv, const double* __restrict__ jac2,
                           T* __restrict__ Prp) {
    struct Rd {
        const T* p;
        __device__ double operator[](long long q) const { return (double)p[q]; }
    };
    struct Wr {
        T* p;
        struct Ref {
            T* a;
            __device__ void operator=(double v) { *a = (T)v; }
            __device__ operator double() const { return (double)*a; }
        };
        __device__ Ref operator[](long long q) const { return Ref{p + q}; }
    };
    const Rd U1{U1p}, U2{U2p}, U3{U3p};
    const Wr Pr{Prp};
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny, nz = g.nz, J = ny - 2, I = nx - 2, K = nz - 2;
    const long long nW = (long long)I * J, nO = (long long)J * K;
    if (t < nW) {  // wall (k=0)
        int i = 1 + (int)(t % I), j = 1 + (int)(t / I);
        double fder = (U3[idx(g, i, j, 1)] - U3[idx(g, i, j, 0)]) / c.df1;
        double d3 = U3[idx(g, i, j, 0)] * fder;
        double g1 = (U3[idx(g, i - 1, j, 0)] + U3[idx(g, i + 1, j, 0)] - 2.0 * U3[idx(g, i, j, 0)]) / (c.dx * c.dx);
        double g2 = (U3[idx(g, i, j - 1, 0)] + U3[idx(g, i, j + 1, 0)] - 2.0 * U3[idx(g, i, j, 0)]) / (c.dy * c.dy);
        double g3 = (2.0 * c.df1 * U3[idx(g, i, j, 2)] - 2.0 * c.df2 * U3[idx(g, i, j, 1)] +
                     2.0 * (c.df2 - c.df1) * U3[idx(g, i, j, 0)]) /
                    (c.df1 * (c.df2 * c.df2) - (c.df2 * (c.df1 * c.df1)));
        double flux = -d3 + ((g1 + g2 + g3) / c.re);
        Pr[idx(g, i, j, 0)] = Pr[idx(g, i, j, 1)] - flux * c.df1;
        return;
    }
    t -= nW;
    if (t < nW) {  // top (k=nz-1)
        int i = 1 + (int)(t % I), j = 1 + (int)(t / I);
        double fder = (11.0 * U3[idx(g, i, j, nz - 1)] - 18.0 * U3[idx(g, i, j, nz - 2)] +
                       9.0 * U3[idx(g, i, j, nz - 3)] - 2.0 * U3[idx(g, i, j, nz - 4)]) /
                      (6.0 * c.dxi);
        double d3 = (fder * jacinv[nz - 1]);
        Pr[idx(g, i, j, nz - 1)] = (d3 / c.re);
        return;
    }
    t -= nW;
    if (t < nO) {  // outflow
        int j = 1 + (int)(t % J), k = 1 + (int)(t / J);
        Pr[idx(g, nx - 1, j, k)] = ((3.0 * U1[idx(g, nx - 1, j, k)] - 4.0 * U1[idx(g, nx - 2, j, k)] +
                                     U1[idx(g, nx - 3, j, k)]) /
                                    (2.0 * c.dx * c.re));
        return;
    }
    t -= nO;
    if (t < nO) {  // inflow
        int j = 1 + (int)(t % J), k = 1 + (int)(t / J);
        double u0 = U1[idx(g, 0, j, k)];
        double d1 = u0 * ((U1[idx(g, 1, j, k)] - u0) / (c.dx));
        double d2 = U2[idx(g, 0, j, k)] * ((U1[idx(g, 0, j + 1, k)] - U1[idx(g, 0, j - 1, k)]) / (2.0 * c.dy));
        double d3 = U3[idx(g, 0, j, k)] * ((U1[idx(g, 0, j, k + 1)] - U1[idx(g, 0, j, k - 1)]) / (2.0 * c.dxi));
        double g1 = (u0 + U1[idx(g, 2, j, k)] - 2.0 * U1[idx(g, 1, j, k)]) / (c.dx * c.dx);
        double g2 = (U1[idx(g, 0, j + 1, k)] + U1[idx(g, 0, j - 1, k)] - 2.0 * u0) / (c.dy * c.dy);
        double fder, g3;
        if (k <= 1) {
            fder = (U1[idx(g, 0, j, k + 1)] - u0) / c.dxi;
            g3 = (U1[idx(g, 0, j, k + 2)] - 2.0 * U1[idx(g, 0, j, k + 1)] + u0) / (c.dxi * c.dxi);
        } else if (k >= nz - 2) {
            fder = (u0 - U1[idx(g, 0, j, k - 1)]) / c.dxi;
            g3 = (U1[idx(g, 0, j, k - 2)] - 2.0 * U1[idx(g, 0, j, k - 1)] + u0) / (c.dxi * c.dxi);
        } else {
            fder = (U1[idx(g, 0, j, k + 1)] - U1[idx(g, 0, j, k - 1)]) / (2.0 * c.dxi);
            g3 = (-2.0 * u0 + U1[idx(g, 0, j, k + 1)] + U1[idx(g, 0, j, k - 1)]) / (c.dxi * c.dxi);
        }
        double Jk = jacinv[k];
        g3 = (g3 * (Jk * Jk)) - ((jac2[k] * fder) * (Jk * Jk * Jk));
        double fder2 = (u0 - uold1[(size_t)j + (size_t)ny * k]) / c.dt;
        Pr[idx(g, 0, j, k)] = ((2.0 * c.dx * ((fder2 + d1 + d2 + d3 * Jk) - ((g1 + g2 + g3) / c.re))) - 0.0 -
                               Pr[idx(g, 2, j, k)] + (4.0 * Pr[idx(g, 1, j, k)])) /
                              3.0;
    }
}

// spanwise periodic copies of U and P (:1465-1469), one thread per (i,k)
template <typename T>
__global__ void k_periodic(Geom g, T* __restrict__ U1, T* __restrict__ U2, T* __restrict__ U3,
                           T* __restrict__ Pr) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nx * g.nz) return;
    int i = t % g.nx, k = t / g.nx;
    long long a0 = idx(g, i, 0, k), a1 = idx(g, i, g.ny - 2, k), b0 = idx(g, i, g.ny - 1, k), b1 = idx(g, i, 1, k);
    U1[a0] = U1[a1]; U1[b0] = U1[b1];
    U2[a0] = U2[a1]; U2[b0] = U2[b1];
    U3[a0] = U3[a1]; U3[b0] = U3[b1];
    Pr[a0] = Pr[a1]; Pr[b0] = Pr[b1];
}

// -------------------------------------------- diagnostics: divergence print
// (dnstbl2/dnstbl.f90:1526-1577): sum of the 4th-order divergence -> red[3]
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_div_diag(Geom g, double invdx, double invdy, double invdxi,
                                                          const T* __restrict__ U1, const T* __restrict__ U2,
                                                          const T* __restrict__ U3,
                                                          const double* __restrict__ jacinv, RedWork rw,
                                                          DevScalars* sc, int slot) {
    __shared__ double s_red[RED_THREADS / 32];
    const int ni = g.nx - 2, J = g.ny - 2, nk = g.nz - 2;
    const long long n = (long long)ni * J * nk;
    const double c12 = 1.0 / 12.0;
    double acc = 0.0;
    for (long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; t0 < n;
         t0 += (long long)gridDim.x * blockDim.x) {
        int i = 1 + (int)(t0 % ni);
        long long r = t0 / ni;
        int j = 1 + (int)(r % J);
        int k = 1 + (int)(r / J);
        long long p = idx(g, i, j, k);
        double d1, d2, d3;
        if (i == 1 || i == g.nx - 2) d1 = ((double)U1[p + 1] - (double)U1[p - 1]) * (0.5 * invdx);
        else d1 = (((double)U1[p - 2] - 8.0 * (double)U1[p - 1] + 8.0 * (double)U1[p + 1] - (double)U1[p + 2]) * (c12 * invdx));
        if (j == 1 || j == g.ny - 2)
            d2 = ((double)U2[idx(g, i, jp1(g, j), k)] - (double)U2[idx(g, i, jm1(g, j), k)]) * (0.5 * invdy);
        else
            d2 = (((double)U2[idx(g, i, jm2(g, j), k)] - 8.0 * (double)U2[idx(g, i, jm1(g, j), k)] +
                   8.0 * (double)U2[idx(g, i, jp1(g, j), k)] - (double)U2[idx(g, i, jp2(g, j), k)]) *
                  (c12 * invdy));
        if (k <= 1 || k >= g.nz - 2) d3 = (((double)U3[p + g.ps] - (double)U3[p - g.ps]) * (0.5 * invdxi));
        else d3 = (((double)U3[p - 2 * g.ps] - 8.0 * (double)U3[p - g.ps] + 8.0 * (double)U3[p + g.ps] -
                    (double)U3[p + 2 * g.ps]) * (c12 * invdxi));
        acc += (d1 + d2 + (d3 * jacinv[k]));
    }
    double bt = block_sum(acc, s_red);
    grid_finish(bt, rw, slot, gridDim.x, blockIdx.x, &sc->red[slot], 0);
}

// -------------------------- per-step fluctuations, KE, blowup (:1707-1775)
// Ufluc = U - means on every slab's planes; only the recycling plane irec is
// kept (ufl_live); KE sum -> red[slot]; max fluctuation -> red[slot+1].
// Columns i_lo..i_hi (0-based): all, or 1..nx-2 for dnssetbl
// (dnssetbl.f90:1228-1236).
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_fluc_ke(Geom g, const T* __restrict__ U1,
                                                         const T* __restrict__ U2, const T* __restrict__ U3,
                                                         const double* __restrict__ usum2,
                                                         const double* __restrict__ vsum2,
                                                         const double* __restrict__ wsum2, double* __restrict__ ufl_live,
                                                         int irec0, RedWork rw, DevScalars* sc, int slot, int i_lo,
                                                         int i_hi) {
    __shared__ double s_red[RED_THREADS / 32];
    const int nx = g.nx, J = g.ny - 2, nk = g.nz - 2;
    const long long n = (long long)nx * J * nk;
    double acc = 0.0, mx = -1e300;
    const size_t pl = (size_t)g.ny * g.nz;
    for (long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; t0 < n;
         t0 += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t0 % nx);
        if (i < i_lo || i > i_hi) continue;
        long long r = t0 / nx;
        int j = 1 + (int)(r % J);
        int k = 1 + (int)(r / J);
        long long p = idx(g, i, j, k);
        size_t q = (size_t)i + (size_t)nx * k;
        double f1 = (double)U1[p] - usum2[q], f2 = (double)U2[p] - vsum2[q], f3 = (double)U3[p] - wsum2[q];
        acc += f1 * f1 + f2 * f2 + f3 * f3;
        mx = fmax(mx, fmax(f1, fmax(f2, f3)));
        if (i == irec0) {
            size_t pj = (size_t)j + (size_t)g.ny * k;
            ufl_live[pj] = f1; ufl_live[pl + pj] = f2; ufl_live[2 * pl + pj] = f3;
        }
    }
    double bt = block_sum(acc, s_red);
    // max via a second pass of the same machinery: store -max as a "sum" would be wrong; use atomic on bits
    mx = warp_max(mx);
    if ((threadIdx.x & 31) == 0) {
        unsigned long long* mp = reinterpret_cast<unsigned long long*>(&sc->red[slot + 1]);
        // non-negative doubles order like their bit patterns; clamp below at 0
        double m0 = fmax(mx, 0.0);
        atomicMax(mp, __double_as_longlong(m0));
    }
    grid_finish(bt, rw, slot, gridDim.x, blockIdx.x, &sc->red[slot], 0);
}

// ------------------------------------------- statistics (:1902-1993)
// one thread per (i,k), k over all planes 0..nz-1, spanwise sums in row order
template <typename T>
__global__ void k_stats(Geom g, double dA, double A, const T* __restrict__ U1, const T* __restrict__ U2,
                        const T* __restrict__ U3, double* __restrict__ sums) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nx * g.nz) return;
    int i = t % g.nx, k = t / g.nx;
    double tu = 0, tv = 0, tw = 0, tuu = 0, tvv = 0, tww = 0, tuv = 0, tuw = 0, tvw = 0;
    for (int j = 1; j <= g.ny - 2; ++j) {
        long long p = idx(g, i, j, k), pp = idx(g, i, jp1(g, j), k);
        double su = 0.50 * ((double)U1[p] + (double)U1[pp]);
        double sv = 0.50 * ((double)U2[p] + (double)U2[pp]);
        double sw = 0.50 * ((double)U3[p] + (double)U3[pp]);
        tu = tu + (su * dA); tv = tv + (sv * dA); tw = tw + (sw * dA);
        tuu = tuu + (su * su * dA); tvv = tvv + (sv * sv * dA); tww = tww + (sw * sw * dA);
        tuv = tuv + (su * sv * dA); tuw = tuw + (su * sw * dA); tvw = tvw + (sv * sw * dA);
    }
    size_t n2 = (size_t)g.nx * g.nz, q = (size_t)t;
    sums[q] += tu / A; sums[n2 + q] += tv / A; sums[2 * n2 + q] += tw / A;
    sums[3 * n2 + q] += tuu / A; sums[4 * n2 + q] += tvv / A; sums[5 * n2 + q] += tww / A;
    sums[6 * n2 + q] += tuv / A; sums[7 * n2 + q] += tuw / A; sums[8 * n2 + q] += tvw / A;
}

// The averaged statistics of a rescaling, kept for the monitor files: every
// running sum divided by cum (:2021-2049, :2063-2078), before the reset.
__global__ void k_averages(long long n9, double cum, const double* __restrict__ sums, double* __restrict__ avg) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n9) avg[q] = sums[q] / cum;
}

// ------------------------------- rescaling bookkeeping (:2084-2277), 1 block
__global__ void k_rescale(Geom g, int irec0, double cum, double ue, double re, const double* __restrict__ x3,
                          double* __restrict__ sums, double* __restrict__ usum2, double* __restrict__ vsum2,
                          double* __restrict__ wsum2, double* __restrict__ wt, double* __restrict__ bltkns,
                          int* __restrict__ newk, double* __restrict__ bl_out, DevScalars* sc) {
    const int nx = g.nx, nz = g.nz;
    const size_t n2 = (size_t)nx * nz;
    for (size_t q = threadIdx.x; q < n2; q += blockDim.x) {
        usum2[q] = (sums[q] / cum);
        vsum2[q] = (sums[n2 + q] / cum);
        wsum2[q] = (sums[2 * n2 + q] / cum);
    }
    __syncthreads();
    // bltkns: first k with usum2 >= 0.99 Ue (keeps its previous value if none)
    for (int i = threadIdx.x; i < nx; i += blockDim.x)
        for (int k = 0; k < nz; ++k)
            if (usum2[(size_t)i + (size_t)nx * k] >= (0.99 * ue)) { bltkns[i] = x3[k]; break; }
    __syncthreads();
    for (size_t q = threadIdx.x; q < n2; q += blockDim.x) {
        int i = (int)(q % nx), k = (int)(q / nx);
        double xb = x3[k] / bltkns[i];
        wt[q] = 0.5 * (1.0 + (tanh((4.0 * ((xb)-0.2)) / ((1.0 - 2.0 * 0.2) * (xb) + 0.2)) / tanh(4.0)));
    }
    // deltastar, theta, H, Re_theta per i (:2255-2277)
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        double ds = 0.0, th = 0.0;
        for (int k = 0; k < nz - 1; ++k) {
            ds = ds + ((1.0 - (usum2[(size_t)i + (size_t)nx * k] / ue)) * (x3[k + 1] - x3[k]));
            if (x3[k] == bltkns[i]) break;
        }
        for (int k = 0; k < nz - 1; ++k) {
            double a = usum2[(size_t)i + (size_t)nx * k] / ue;
            th = th + ((a) * (1.0 - (a)) * (x3[k + 1] - x3[k]));
            if (x3[k] >= bltkns[i]) break;
        }
        bl_out[i] = ds; bl_out[nx + i] = th; bl_out[2 * nx + i] = ds / th; bl_out[3 * nx + i] = th * re * ue;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double utau1 = sqrt(((usum2[(size_t)nx * 1] - usum2[0]) / (x3[1] - x3[0])) / re);
        double utau2 = sqrt(((usum2[(size_t)irec0 + (size_t)nx * 1] - usum2[irec0]) / (x3[1] - x3[0])) / re);
        double lamda = (utau1) / (utau2);
        double lamda03 = bltkns[irec0] / bltkns[0];
        sc->lamda = lamda;
        sc->lamda03 = lamda03;
        int ksep = sc->ksep;
        // eta, zrecy and the monotone index map new(k) (:2209-2252); 1-based k
        for (int k = 1; k <= nz - 1; ++k)
            if (wt[(size_t)irec0 + (size_t)nx * (k - 1)] <= 0.99) ksep = k;
        for (int k = 1; k <= nz; ++k) newk[k - 1] = nz - 1;
        int counter = 1;
        for (int k = 1; k <= nz - 1; ++k) {
            if (counter <= ksep) {
                double eta = wt[(size_t)irec0 + (size_t)nx * (counter - 1)] <= 0.99 ? lamda : lamda03;
                double zr = eta * x3[counter - 1];
                if (x3[k - 1] >= zr) { newk[counter - 1] = k; counter = counter + 1; }
            }
        }
        counter = ksep + 1;
        for (int k = ksep + 1; k <= nz - 1; ++k) {
            if (counter <= nz - 1) {
                double eta = wt[(size_t)irec0 + (size_t)nx * (counter - 1)] <= 0.99 ? lamda : lamda03;
                double zr = eta * x3[counter - 1];
                if (x3[k - 1] >= zr) { newk[counter - 1] = k; counter = counter + 1; }
            }
        }
        sc->ksep = ksep;
    }
}

// refresh Ufluc(irec,:,k,:) with the new means on planes k_lo..k_hi
// (0-based; every slab's, :2341-2349, or rank 0's for dnssetbl,
// dnssetbl.f90:1033-1041) and zero the sums (:2351-2365)
template <typename T>
__global__ void k_rescale_tail(Geom g, int irec0, const T* __restrict__ U1, const T* __restrict__ U2,
                               const T* __restrict__ U3, const double* __restrict__ usum2,
                               const double* __restrict__ vsum2, const double* __restrict__ wsum2,
                               double* __restrict__ ufl_live, double* __restrict__ sums, int k_lo, int k_hi) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = g.ny - 2;
    const size_t n2 = (size_t)g.nx * g.nz;
    if (t < J * (g.nz - 2) && 1 + t / J >= k_lo && 1 + t / J <= k_hi) {
        int j = 1 + t % J, k = 1 + t / J;
        long long p = idx(g, irec0, j, k);
        size_t q = (size_t)irec0 + (size_t)g.nx * k, pl = (size_t)g.ny * g.nz, pj = (size_t)j + (size_t)g.ny * k;
        ufl_live[pj] = (double)U1[p] - usum2[q];
        ufl_live[pl + pj] = (double)U2[p] - vsum2[q];
        ufl_live[2 * pl + pj] = (double)U3[p] - wsum2[q];
    }
    for (size_t q = t; q < 9 * n2; q += (size_t)gridDim.x * blockDim.x) sums[q] = 0.0;
}

// ------------------------------------------------------------- host glue
#define LAUNCH_COUNT(h) (h)->launches++

static inline dim3 interior_grid(const Geom& g) {
    return dim3((g.nx - 2 + 127) / 128, g.ny - 2, g.nz - 2);
}
static inline bool mixed(const tbl_handle* h) { return h->cfg.precision == TBL_PREC_MIXED; }

int launch_save_uold(tbl_handle* h) {
    const Geom& g = h->g;
    int n = g.ny * g.nz;
    if (mixed(h)) k_save_uold<float><<<(n + 255) / 256, 256, 0, h->stream>>>(g, h->Uf[0], h->uold1);
    else k_save_uold<double><<<(n + 255) / 256, 256, 0, h->stream>>>(g, h->U[0], h->uold1);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

int launch_inflow(tbl_handle* h) {
    const Geom& g = h->g;
    int n = (g.ny - 2) * (g.nz - 2);
    const int var = h->cfg.variant;
    // eps = min(cnt2 * 5e-5, 1) (fnldnstbl.f90:561-565), min(nstep * 5e-5, 1) (dnssetbl.f90:259-262)
    double eps = (var == TBL_VARIANT_ORIGINAL ? (double)h->cnt2 : (double)h->nstep) * (5.0e-5);
    if (eps > 1.0) eps = 1.0;
    const int ramp = var != TBL_VARIANT_DNSTBL2, vlam = var == TBL_VARIANT_DNSSETBL;
    const int wcol = var == TBL_VARIANT_DNSSETBL ? 0 : g.nx - 2;
    if (mixed(h))
        k_inflow<float><<<(n + 127) / 128, 128, 0, h->stream>>>(g, h->Uf[0], h->Uf[1], h->Uf[2], h->usum2, h->vsum2,
                                                                 h->wsum2, h->wt, h->ume1, h->newk, h->ufl_file,
                                                                 h->ufl_live, h->slab_of_k, h->slabs, h->sc,
                                                                 h->cfg.irec - 1, h->cfg.ue, ramp, eps, vlam, wcol);
    else
        k_inflow<double><<<(n + 127) / 128, 128, 0, h->stream>>>(g, h->U[0], h->U[1], h->U[2], h->usum2, h->vsum2,
                                                                  h->wsum2, h->wt, h->ume1, h->newk, h->ufl_file,
                                                                  h->ufl_live, h->slab_of_k, h->slabs, h->sc,
                                                                  h->cfg.irec - 1, h->cfg.ue, ramp, eps, vlam, wcol);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

template <typename R>
static ConvCoef<R> conv_coef(const tbl_config& c) {
    ConvCoef<R> cc;
    const double invdx = 1.0 / c.dx, invdy = 1.0 / c.dy, invdxi = 1.0 / c.dxi, c12 = 1.0 / 12.0;
    cc.tf = (R)c.re; cc.dx = (R)c.dx; cc.dy = (R)c.dy;
    cc.invdx = (R)invdx; cc.invdy = (R)invdy; cc.invdxi = (R)invdxi;
    cc.inv2dx = (R)(1.0 / (2.0 * c.dx));
    cc.c12x = (R)(c12 * invdx); cc.c12y = (R)(c12 * invdy); cc.c12z = (R)(c12 * invdxi);
    cc.q25x = (R)(0.25 * invdx); cc.q25y = (R)(0.25 * invdy); cc.q25z = (R)(0.25 * invdxi);
    cc.h05z = (R)(0.5 * invdxi);
    cc.h05y = (R)(0.5 * invdy);
    cc.dt = (R)c.dt;
    cc.pe_mode = c.variant == TBL_VARIANT_DNSSETBL ? 2 : (c.variant == TBL_VARIANT_ORIGINAL ? 1 : 0);
    cc.ycen = c.variant == TBL_VARIANT_DNSSETBL ? 1 : 0;
    return cc;
}

int launch_conv_q(tbl_handle* h) {
    const Geom& g = h->g;
    if (mixed(h))
        k_conv_q<float><<<interior_grid(g), 128, 0, h->stream>>>(g, conv_coef<float>(h->cfg), h->Uf[0], h->Uf[1],
                                                                 h->Uf[2], h->Pf, h->x3, h->jacinv, h->Qf[0],
                                                                 h->Qf[1], h->Qf[2]);
    else if (h->conv_bits_mode == TBL_BRANCH_RECORD && h->conv_bits)
        k_conv_q_br<1><<<interior_grid(g), 128, 0, h->stream>>>(g, conv_coef<double>(h->cfg), h->U[0], h->U[1],
                                                                 h->U[2], h->Pr, h->x3, h->jacinv, h->Q[0], h->Q[1],
                                                                 h->Q[2], h->conv_bits);
    else if (h->conv_bits_mode == TBL_BRANCH_REPLAY && h->conv_bits)
        k_conv_q_br<2><<<interior_grid(g), 128, 0, h->stream>>>(g, conv_coef<double>(h->cfg), h->U[0], h->U[1],
                                                                 h->U[2], h->Pr, h->x3, h->jacinv, h->Q[0], h->Q[1],
                                                                 h->Q[2], h->conv_bits);
    else
        k_conv_q<double><<<interior_grid(g), 128, 0, h->stream>>>(g, conv_coef<double>(h->cfg), h->U[0], h->U[1],
                                                                  h->U[2], h->Pr, h->x3, h->jacinv, h->Q[0], h->Q[1],
                                                                  h->Q[2]);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

// GS residual of the listed components.  In mixed precision the iteration is
// on the increment D (delta form) with right-hand side r0 stored in Qf.
int launch_gs_resid(tbl_handle* h, const int* comps, int ncomp, int nblocks) {
    const Geom& g = h->g;
    const double t = -h->cfg.dt / (h->cfg.re);
    const double aw = 1.0 / (h->cfg.dx * h->cfg.dx), as = 1.0 / (h->cfg.dy * h->cfg.dy);
    GsCoef gc{t * aw, t * aw, t * as, t * as};
    int3 cs = make_int3(comps[0], ncomp > 1 ? comps[1] : 0, ncomp > 2 ? comps[2] : 0);
    if (mixed(h))
        k_gs_resid<float><<<dim3(nblocks, ncomp), RED_THREADS, 0, h->stream>>>(
            g, gc, h->gs_coef, h->Df[0], h->Df[1], h->Df[2], h->Qf[0], h->Qf[1], h->Qf[2], cs, ncomp, h->red, h->sc);
    else
        k_gs_resid<double><<<dim3(nblocks, ncomp), RED_THREADS, 0, h->stream>>>(
            g, gc, h->gs_coef, h->U[0], h->U[1], h->U[2], h->Q[0], h->Q[1], h->Q[2], cs, ncomp, h->red, h->sc);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

// Mixed precision, delta form of the Gauss-Seidel solve of (I + t L7) U = Q:
// the FP32 sweeps iterate on an increment D with right-hand side r = Q - A U.
// In exact arithmetic U + D are the reference's iterates (a sweep is affine),
// at every restart of the increment too.  The residuals are formed in FP64
// from the FP32 data and rounded once, so r carries no FP32 cancellation.
//
// Start: r0 = Q - A U in place of Q, D = 0.
__global__ void __launch_bounds__(128) k_gs_delta_init(Geom g, double t, double aw, double as,
                                                       const double* __restrict__ Ab, const double* __restrict__ At,
                                                       const double* __restrict__ Ap, const float* __restrict__ U,
                                                       float* __restrict__ Q, float* __restrict__ D) {
    int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    long long p = idx(g, i, j, k);
    const double d = 1.0 + t * Ap[k], cE = t * aw, cN = t * as, cT = t * At[k], cB = t * Ab[k];
    const double r = (double)Q[p] - d * (double)U[p] - cE * (double)U[p + 1] - cE * (double)U[p - 1] -
                     cN * (double)U[idx(g, i, jp1(g, j), k)] - cN * (double)U[idx(g, i, jm1(g, j), k)] -
                     cT * (double)U[p + g.ps] - cB * (double)U[p - g.ps];
    Q[p] = (float)r;
    D[p] = 0.0f;
}

// Restart of the increment, first half: r -= A D (the residual of U + D).
__global__ void __launch_bounds__(128) k_gs_delta_rhs(Geom g, double t, double aw, double as,
                                                      const double* __restrict__ Ab, const double* __restrict__ At,
                                                      const double* __restrict__ Ap, const float* __restrict__ D,
                                                      float* __restrict__ Q) {
    int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    long long p = idx(g, i, j, k);
    const double d = 1.0 + t * Ap[k], cE = t * aw, cN = t * as, cT = t * At[k], cB = t * Ab[k];
    const double r = (double)Q[p] - d * (double)D[p] - cE * (double)D[p + 1] - cE * (double)D[p - 1] -
                     cN * (double)D[idx(g, i, jp1(g, j), k)] - cN * (double)D[idx(g, i, jm1(g, j), k)] -
                     cT * (double)D[p + g.ps] - cB * (double)D[p - g.ps];
    Q[p] = (float)r;
}

// U += D on the interior (end of the delta-form GS); with zero_d the increment
// restarts from 0 (second half of a restart).
__global__ void __launch_bounds__(128) k_gs_delta_apply(Geom g, float* __restrict__ D, float* __restrict__ U,
                                                        int zero_d) {
    int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    long long p = idx(g, i, j, k);
    U[p] = U[p] + D[p];
    if (zero_d) D[p] = 0.0f;
}

int launch_gs_delta_init(tbl_handle* h, int comp) {
    const Geom& g = h->g;
    const double t = -h->cfg.dt / (h->cfg.re);
    k_gs_delta_init<<<interior_grid(g), 128, 0, h->stream>>>(g, t, 1.0 / (h->cfg.dx * h->cfg.dx),
                                                            1.0 / (h->cfg.dy * h->cfg.dy), h->Ab, h->At, h->Ap,
                                                            h->Uf[comp], h->Qf[comp], h->Df[comp]);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

int launch_gs_delta_apply(tbl_handle* h, int comp) {
    k_gs_delta_apply<<<interior_grid(h->g), 128, 0, h->stream>>>(h->g, h->Df[comp], h->Uf[comp], 0);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

// Restart of the increment of one component: r -= A D, U += D, D = 0.
int launch_gs_delta_restart(tbl_handle* h, int comp) {
    const Geom& g = h->g;
    const double t = -h->cfg.dt / (h->cfg.re);
    k_gs_delta_rhs<<<interior_grid(g), 128, 0, h->stream>>>(g, t, 1.0 / (h->cfg.dx * h->cfg.dx),
                                                           1.0 / (h->cfg.dy * h->cfg.dy), h->Ab, h->At, h->Ap,
                                                           h->Df[comp], h->Qf[comp]);
    k_gs_delta_apply<<<interior_grid(g), 128, 0, h->stream>>>(g, h->Df[comp], h->Uf[comp], 1);
    h->launches += 2;
    return TBL_OK;
}

int launch_div(tbl_handle* h) {
    const Geom& g = h->g;
    if (mixed(h))
        k_div<float><<<interior_grid(g), 128, 0, h->stream>>>(g, 1.0 / h->cfg.dx, 1.0 / h->cfg.dy, h->cfg.dt,
                                                              h->Uf[0], h->Uf[1], h->Uf[2], h->x3, h->Q8);
    else
        k_div<double><<<interior_grid(g), 128, 0, h->stream>>>(g, 1.0 / h->cfg.dx, 1.0 / h->cfg.dy, h->cfg.dt,
                                                               h->U[0], h->U[1], h->U[2], h->x3, h->Q8);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

int launch_pc_zero_faces(tbl_handle* h) {
    const Geom& g = h->g;
    long long n = (long long)g.ny * g.nz + (long long)g.nx * g.nz + (long long)g.nx * g.ny;
    k_pc_zero_faces<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(g, h->PC);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

template <typename T>
static void project_bcs_t(tbl_handle* h, T* U0, T* U1, T* U2, T* Pr) {
    const Geom& g = h->g;
    const tbl_config& c = h->cfg;
    int n1 = g.nx * (g.ny - 2), n2 = g.nx * g.nz, n3 = (g.ny - 2) * g.nz;
    k_pc_bc_walltop<<<(n1 + 255) / 256, 256, 0, h->stream>>>(g, h->PC);
    k_pc_periodic<<<(n2 + 255) / 256, 256, 0, h->stream>>>(g, h->PC);
    k_pc_bc_inout<<<(n3 + 255) / 256, 256, 0, h->stream>>>(g, h->PC);
    k_project<T><<<interior_grid(g), 128, 0, h->stream>>>(g, 1.0 / c.dx, 1.0 / c.dy, 1.0 / c.dxi, c.dt, h->jacinv,
                                                          h->PC, Pr, U0, U1, U2);
    k_vel_bc_walltop<T><<<(n1 + 255) / 256, 256, 0, h->stream>>>(g, U0, U1, U2, h->wallw);
    k_vel_bc_out<T><<<(n3 + 255) / 256, 256, 0, h->stream>>>(g, U0, U1, U2);
    PbcCoef pc;
    pc.dx = c.dx; pc.dy = c.dy; pc.dxi = c.dxi; pc.re = c.re; pc.dt = c.dt;
    pc.df1 = h->x3h[1] - h->x3h[0];
    pc.df2 = h->x3h[2] - h->x3h[0];
    long long np = 2LL * (g.nx - 2) * (g.ny - 2) + 2LL * (g.ny - 2) * (g.nz - 2);
    k_press_bc<T><<<(unsigned)((np + 255) / 256), 256, 0, h->stream>>>(g, pc, U0, U1, U2, h->uold1, h->jacinv,
                                                                       h->jac2, Pr);
    k_periodic<T><<<(n2 + 255) / 256, 256, 0, h->stream>>>(g, U0, U1, U2, Pr);
    h->launches += 8;
}

int launch_project_bcs(tbl_handle* h) {
    if (mixed(h)) project_bcs_t<float>(h, h->Uf[0], h->Uf[1], h->Uf[2], h->Pf);
    else project_bcs_t<double>(h, h->U[0], h->U[1], h->U[2], h->Pr);
    return TBL_OK;
}

// ------------------------------------ diagnostics: mass flux, wall shear
// Mass flux through the five cross-stream planes i = 5, 20, 40, 60, 85
// (1-based, :95; clamped to nx-1) (:1578-1594): cell averages of u times the
// cell area dy (x3(k+1) - x3(k)) over the span and the whole height, divided
// by the area Av.  One block per plane.  k_lo = 1 starts at the second cell
// layer: dnssetbl sums each slab's own planes, so the wall layer drops out
// (dnssetbl.f90:887-893).
template <typename T>
__global__ void __launch_bounds__(256) k_mass_flux(Geom g, double dy, double Av, const double* __restrict__ x3,
                                                   const T* __restrict__ U1, double* __restrict__ ub, int k_lo) {
    __shared__ double s_red[256 / 32];
    const int planes[5] = {5, 20, 40, 60, 85};
    const int q = blockIdx.x;
    const int ip = (planes[q] < g.nx - 1 ? planes[q] : g.nx - 1) - 1;  // 0-based
    const int J = g.ny - 2;
    const int ncell = J * (g.nz - 1 - k_lo);
    double acc = 0.0;
    for (int t = threadIdx.x; t < ncell; t += blockDim.x) {
        const int j = 1 + t % J, k = k_lo + t / J;
        const int jp = j == g.ny - 2 ? 1 : j + 1;
        const double dAv = dy * (x3[k + 1] - x3[k]);
        acc += (0.25 * ((double)U1[idx(g, ip, j, k)] + (double)U1[idx(g, ip, jp, k)] +
                        (double)U1[idx(g, ip, j, k + 1)] + (double)U1[idx(g, ip, jp, k + 1)]) *
                (dAv));
    }
    acc = block_sum(acc, s_red);
    if (threadIdx.x == 0) ub[q] = acc / Av;
}

// Wall shear (:1616-1681): for every interior column the span sum of
// (dw/dx + du/dz)/Re at the wall -- dw/dx 6th-order central, 2nd order within
// three points of the ends; du/dz one-sided 2nd order on the stretched grid --
// added to the accumulator sumxz; at a window end (every `win` steps: 500,
// originalTBL 1000, fnldnstbl.f90:1679-1681) the window mean sumxz/win is
// kept and the accumulator restarts.  One block per column.
template <typename T>
__global__ void __launch_bounds__(128) k_wall_shear(Geom g, double dx, double re, double d1, double d2,
                                                    const T* __restrict__ U1, const T* __restrict__ U3,
                                                    double* __restrict__ sumxz, double* __restrict__ window,
                                                    int close_window, double win) {
    __shared__ double s_red[128 / 32];
    const int i = 1 + blockIdx.x;  // 0-based interior column
    const int nx = g.nx;
    double acc = 0.0;
    for (int j = 1 + threadIdx.x; j <= g.ny - 2; j += blockDim.x) {
        auto w0 = [&](int ii) { return (double)U3[idx(g, ii, j, 0)]; };
        double mfb1;
        if (i <= 2 || i >= nx - 3)
            mfb1 = (w0(i + 1) - w0(i - 1)) / (2.0 * dx);
        else
            mfb1 = (-w0(i - 3) + (9.0 * w0(i - 2)) - (45.0 * w0(i - 1)) + (45.0 * w0(i + 1)) - (9.0 * w0(i + 2)) +
                    w0(i + 3)) /
                   (60.0 * dx);
        const double u0 = U1[idx(g, i, j, 0)], u1 = U1[idx(g, i, j, 1)], u2 = U1[idx(g, i, j, 2)];
        const double fder = (((u2 - u0) * (d1 * d1)) + ((u0 - u1) * (d2 * d2))) / ((d2 * (d1 * d1)) - ((d2 * d2) * d1));
        acc += ((mfb1 + fder) / re);
    }
    acc = block_sum(acc, s_red);
    if (threadIdx.x == 0) {
        const double s = acc + sumxz[i];
        if (close_window) {
            window[i] = s / win;
            sumxz[i] = 0.0;
        } else {
            sumxz[i] = s;
        }
    }
}

int launch_flux_shear(tbl_handle* h) {
    const Geom& g = h->g;
    const double d1 = h->x3h[1] - h->x3h[0], d2 = h->x3h[2] - h->x3h[0];
    const int win = h->cfg.variant == TBL_VARIANT_ORIGINAL ? 1000 : 500;
    const int close = (h->nstep % win == 0) ? 1 : 0;
    const int k_lo = h->cfg.variant == TBL_VARIANT_DNSSETBL ? 1 : 0;
    if (close) TBL_CUDA_TRY(cudaMemsetAsync(h->tauw_win, 0, (size_t)g.nx * 8, h->stream));
    if (mixed(h)) {
        k_mass_flux<float><<<5, 256, 0, h->stream>>>(g, h->cfg.dy, h->area_mf, h->x3, h->Uf[0], h->ubulk, k_lo);
        k_wall_shear<float><<<g.nx - 2, 128, 0, h->stream>>>(g, h->cfg.dx, h->cfg.re, d1, d2, h->Uf[0], h->Uf[2],
                                                             h->sumxz, h->tauw_win, close, (double)win);
    } else {
        k_mass_flux<double><<<5, 256, 0, h->stream>>>(g, h->cfg.dy, h->area_mf, h->x3, h->U[0], h->ubulk, k_lo);
        k_wall_shear<double><<<g.nx - 2, 128, 0, h->stream>>>(g, h->cfg.dx, h->cfg.re, d1, d2, h->U[0], h->U[2],
                                                              h->sumxz, h->tauw_win, close, (double)win);
    }
    h->launches += 2;
    return TBL_OK;
}

int launch_div_diag(tbl_handle* h, int nblocks, int slot) {
    const Geom& g = h->g;
    if (mixed(h))
        k_div_diag<float><<<nblocks, RED_THREADS, 0, h->stream>>>(g, 1.0 / h->cfg.dx, 1.0 / h->cfg.dy,
                                                                  1.0 / h->cfg.dxi, h->Uf[0], h->Uf[1], h->Uf[2],
                                                                  h->jacinv, h->red, h->sc, slot);
    else
        k_div_diag<double><<<nblocks, RED_THREADS, 0, h->stream>>>(g, 1.0 / h->cfg.dx, 1.0 / h->cfg.dy,
                                                                   1.0 / h->cfg.dxi, h->U[0], h->U[1], h->U[2],
                                                                   h->jacinv, h->red, h->sc, slot);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

int launch_fluc_ke(tbl_handle* h, int nblocks, int slot) {
    const Geom& g = h->g;
    const bool sete = h->cfg.variant == TBL_VARIANT_DNSSETBL;
    const int i_lo = sete ? 1 : 0, i_hi = sete ? g.nx - 2 : g.nx - 1;
    TBL_CUDA_TRY(cudaMemsetAsync(&h->sc->red[slot + 1], 0, sizeof(double), h->stream));
    if (mixed(h))
        k_fluc_ke<float><<<nblocks, RED_THREADS, 0, h->stream>>>(g, h->Uf[0], h->Uf[1], h->Uf[2], h->usum2,
                                                                 h->vsum2, h->wsum2, h->ufl_live, h->cfg.irec - 1,
                                                                 h->red, h->sc, slot, i_lo, i_hi);
    else
        k_fluc_ke<double><<<nblocks, RED_THREADS, 0, h->stream>>>(g, h->U[0], h->U[1], h->U[2], h->usum2, h->vsum2,
                                                                  h->wsum2, h->ufl_live, h->cfg.irec - 1, h->red,
                                                                  h->sc, slot, i_lo, i_hi);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

int launch_stats(tbl_handle* h) {
    const Geom& g = h->g;
    int n = g.nx * g.nz;
    if (mixed(h))
        k_stats<float><<<(n + 127) / 128, 128, 0, h->stream>>>(g, h->stats_dA, h->stats_A, h->Uf[0], h->Uf[1],
                                                               h->Uf[2], h->sums);
    else
        k_stats<double><<<(n + 127) / 128, 128, 0, h->stream>>>(g, h->stats_dA, h->stats_A, h->U[0], h->U[1], h->U[2],
                                                                h->sums);
    LAUNCH_COUNT(h);
    return TBL_OK;
}

int launch_rescale(tbl_handle* h) {
    const Geom& g = h->g;
    const long long n9 = 9LL * g.nx * g.nz;
    k_averages<<<(int)((n9 + 255) / 256), 256, 0, h->stream>>>(n9, (double)h->cfg.cum, h->sums, h->avg);
    k_rescale<<<1, 256, 0, h->stream>>>(g, h->cfg.irec - 1, (double)h->cfg.cum, h->cfg.ue, h->cfg.re, h->x3, h->sums,
                                        h->usum2, h->vsum2, h->wsum2, h->wt, h->bltkns, h->newk, h->bl_out, h->sc);
    int n = (g.ny - 2) * (g.nz - 2);
    int nb = (n + 255) / 256;
    if (nb < 64) nb = 64;
    const bool sete = h->cfg.variant == TBL_VARIANT_DNSSETBL;
    const int k_lo = sete ? h->bn[0] : 1, k_hi = sete ? h->en[0] : g.nz - 2;
    if (mixed(h))
        k_rescale_tail<float><<<nb, 256, 0, h->stream>>>(g, h->cfg.irec - 1, h->Uf[0], h->Uf[1], h->Uf[2], h->usum2,
                                                         h->vsum2, h->wsum2, h->ufl_live, h->sums, k_lo, k_hi);
    else
        k_rescale_tail<double><<<nb, 256, 0, h->stream>>>(g, h->cfg.irec - 1, h->U[0], h->U[1], h->U[2], h->usum2,
                                                          h->vsum2, h->wsum2, h->ufl_live, h->sums, k_lo, k_hi);
    h->launches += 3;
    return TBL_OK;
}

}  // namespace tbl
