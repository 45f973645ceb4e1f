// tbl_api.cu -- the C ABI (include/tbl_gpu.h): handle lifecycle, state
// transfer and the per-step driver that sequences the kernels in the order
// of the reference time loop (dnstbl2/dnstbl.f90:538-2375).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "tbl_internal.cuh"
#include "tbl_kernels.cuh"

namespace tbl {

static thread_local char g_last_error[512] = {0};

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
}

static int take_event(tbl_handle* h) {
    if (h->prof_used == h->prof_ev.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return -1;
        h->prof_ev.push_back(e);
    }
    return (int)h->prof_used++;
}

ProfScope::ProfScope(tbl_handle* h_, int g_, double b_) : h(h_), group(g_), bytes(b_), e0(-1), l0(h_->launches) {
    if (!h->prof_on) return;
    e0 = take_event(h);
    if (e0 >= 0) cudaEventRecord(h->prof_ev[e0], h->stream);
}

ProfScope::~ProfScope() {
    if (!h->prof_on || e0 < 0) return;
    int e1 = take_event(h);
    if (e1 < 0) return;
    cudaEventRecord(h->prof_ev[e1], h->stream);
    h->prof_marks.push_back({group, e0, e1, bytes, h->launches - l0});
}

// Accumulates the recorded event pairs (the stream must be idle).
int prof_drain(tbl_handle* h) {
    for (const auto& m : h->prof_marks) {
        float ms = 0.f;
        TBL_CUDA_TRY(cudaEventElapsedTime(&ms, h->prof_ev[m.e0], h->prof_ev[m.e1]));
        h->prof_ms[m.group] += ms;
        h->prof_bytes[m.group] += m.bytes;
        h->prof_n[m.group] += m.launches;
    }
    h->prof_marks.clear();
    h->prof_used = 0;
    return TBL_OK;
}

int readback(tbl_handle* h, const void* dev, size_t bytes) {
    TBL_CUDA_TRY(cudaMemcpyAsync(h->hpin, dev, bytes, cudaMemcpyDeviceToHost, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return TBL_OK;
}

// 3-D host (nx,ny,nz) <-> device (sx,ny,nz)
int put3(tbl_handle* h, double* dst, const double* src) {
    const Geom& g = h->g;
    TBL_CUDA_TRY(cudaMemcpy2DAsync(dst, (size_t)g.sx * 8, src, (size_t)g.nx * 8, (size_t)g.nx * 8,
                                   (size_t)g.ny * g.nz, cudaMemcpyHostToDevice, h->stream));
    return TBL_OK;
}
int get3(tbl_handle* h, double* dst, const double* src) {
    const Geom& g = h->g;
    TBL_CUDA_TRY(cudaMemcpy2DAsync(dst, (size_t)g.nx * 8, src, (size_t)g.sx * 8, (size_t)g.nx * 8,
                                   (size_t)g.ny * g.nz, cudaMemcpyDeviceToHost, h->stream));
    return TBL_OK;
}

// FP32 fields: converted on the host through a staging buffer
static int put3f(tbl_handle* h, float* dst, const double* src) {
    const Geom& g = h->g;
    const size_t n = (size_t)g.nx * g.ny * g.nz;
    std::vector<float> tmp(n);
    for (size_t q = 0; q < n; ++q) tmp[q] = (float)src[q];
    TBL_CUDA_TRY(cudaMemcpy2DAsync(dst, (size_t)g.sx * 4, tmp.data(), (size_t)g.nx * 4, (size_t)g.nx * 4,
                                   (size_t)g.ny * g.nz, cudaMemcpyHostToDevice, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return TBL_OK;
}
static int get3f(tbl_handle* h, double* dst, const float* src) {
    const Geom& g = h->g;
    const size_t n = (size_t)g.nx * g.ny * g.nz;
    std::vector<float> tmp(n);
    TBL_CUDA_TRY(cudaMemcpy2DAsync(tmp.data(), (size_t)g.nx * 4, src, (size_t)g.sx * 4, (size_t)g.nx * 4,
                                   (size_t)g.ny * g.nz, cudaMemcpyDeviceToHost, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (size_t q = 0; q < n; ++q) dst[q] = (double)tmp[q];
    return TBL_OK;
}

template <typename T>
static int dalloc(T** p, size_t n) {
    TBL_CUDA_TRY(cudaMalloc((void**)p, n * sizeof(T)));
    TBL_CUDA_TRY(cudaMemset(*p, 0, n * sizeof(T)));
    return TBL_OK;
}

#define TRY(x)                          \
    do {                                \
        int s_ = (x);                   \
        if (s_ != TBL_OK) return s_;    \
    } while (0)

static void free_all(tbl_handle* h) {
    void* mptrs[] = {h->Uf[0], h->Uf[1], h->Uf[2], h->Pf, h->Qf[0], h->Qf[1], h->Qf[2], h->Df[0], h->Df[1],
                     h->Df[2], h->Vf, h->RHf, h->R64, h->PREf, h->PRE, h->lsg_partial, h->lsg_L, h->lsg_d, h->lsg_g};
    for (void* p : mptrs)
        if (p) cudaFree(p);
    void* ptrs[] = {h->U[0], h->U[1], h->U[2], h->Pr, h->PC, h->Q[0], h->Q[1], h->Q[2], h->Q8, h->RH, h->V,
                    h->uold1, h->x3, h->jacinv, h->jac2, h->Ab, h->At, h->Ap, h->rAp, h->gs_coef, h->gs_coef_f, h->lap_scale, h->coef_f, h->usum2, h->vsum2,
                    h->wsum2, h->wt, h->ume1, h->bltkns, h->newk, h->ufl_file, h->ufl_live, h->ufl_full,
                    h->usum2_fl, h->sums, h->avg, h->bl_out, h->ubulk, h->sumxz, h->tauw_win, h->slab_of_k, h->sc, h->h, h->gg, h->gc, h->gs, h->gy,
                    h->red.partial, h->red.count, h->halo, h->flags, h->ctas, h->slabs, h->err};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    adj_free(h);
    if (h->wallw) cudaFree(h->wallw);
    if (h->AbT) cudaFree(h->AbT);
    if (h->AtT) cudaFree(h->AtT);
    if (h->hpin) cudaFreeHost(h->hpin);
    for (cudaEvent_t e : h->ahead_ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : h->prof_ev) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
}

// 0-based slabs [bn, en] of the P virtual ranks: dnstbl2 loc_n = (nz-1)/P
// planes each from k = 2, the remainder on the last rank (:469-475); dnssetbl
// nz/P from k = 1 with one more on the last mod(nz, P) ranks, the wall and
// top planes left out (dnssetbl.f90:78-92).  False when a slab has fewer than
// 3 planes.
bool slab_partition(const tbl_config& c, std::vector<int>& bn, std::vector<int>& en) {
    const int P = c.nproc, nz = c.nz;
    if (P < 1) return false;
    bn.assign(P, 0);
    en.assign(P, 0);
    if (c.variant == TBL_VARIANT_DNSSETBL) {
        int it1 = nz / P, b = 0;
        const int it2 = P - nz % P;
        for (int r = 0; r < P; ++r) {
            if (r == it2) it1 = it1 + 1;
            bn[r] = b;
            en[r] = b + it1 - 1;
            b = en[r] + 1;
        }
        bn[0] += 1;
        en[P - 1] -= 1;
    } else {
        const int loc_n = (nz - 1) / P;
        for (int r = 0; r < P; ++r) {
            bn[r] = 1 + r * loc_n;
            en[r] = bn[r] + loc_n - 1;
            if (r == P - 1) en[r] = nz - 2;
        }
    }
    for (int r = 0; r < P; ++r)
        if (en[r] - bn[r] + 1 < 3) return false;
    return true;
}

static int create_impl(const tbl_config* cfg, const tbl_mesh* mesh, tbl_handle* h) {
    h->cfg = *cfg;
    const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
    Geom& g = h->g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.sx = ((nx + 7) + 7) / 8 * 8;  // a 32-byte chunk starting at i <= nx-2 stays inside the row
    g.ps = (long long)g.sx * ny;
    g.vol = g.ps * nz;
    g.J = ny - 2;
    h->npts = (double)nx * ny * nz;
    h->P = cfg->nproc;
    if (!slab_partition(*cfg, h->bn, h->en)) return TBL_ERR_BAD_ARG;
    TBL_CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    {
        int dev = 0;
        TBL_CUDA_TRY(cudaGetDevice(&dev));
        TBL_CUDA_TRY(cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, dev));
    }
    TBL_CUDA_TRY(cudaMallocHost(&h->hpin, 4096));
    for (cudaEvent_t& e : h->ahead_ev) TBL_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const size_t vol = (size_t)g.vol, n2 = (size_t)nx * nz, pl = (size_t)ny * nz;
    TRY(dalloc(&h->PC, vol));
    TRY(dalloc(&h->Q8, vol));
    if (cfg->precision == TBL_PREC_MIXED) {
        for (int c = 0; c < 3; ++c) {
            TRY(dalloc(&h->Uf[c], vol));
            TRY(dalloc(&h->Qf[c], vol));
            TRY(dalloc(&h->Df[c], vol));
        }
        TRY(dalloc(&h->Pf, vol));
        TRY(dalloc(&h->RHf, vol));
        TRY(dalloc(&h->PREf, 3 * vol));
        // the basis v_0 .. v_kmax, then the Arnoldi vector w before its normalisation
        TRY(dalloc(&h->Vf, vol * (size_t)(cfg->mixed_kmax + 2)));
        const int K1m = cfg->mixed_kmax + 1, ngr = (K1m + 7) / 8;
        TRY(dalloc(&h->lsg_partial, (size_t)2 * 8 * ngr * 2048));
        TRY(dalloc(&h->lsg_L, (size_t)K1m * K1m));
        TRY(dalloc(&h->lsg_d, (size_t)K1m));
        TRY(dalloc(&h->lsg_g, (size_t)K1m));
    } else {
        for (int c = 0; c < 3; ++c) { TRY(dalloc(&h->U[c], vol)); TRY(dalloc(&h->Q[c], vol)); }
        TRY(dalloc(&h->Pr, vol)); TRY(dalloc(&h->RH, vol)); TRY(dalloc(&h->PRE, 3 * vol));
        TRY(dalloc(&h->V, vol * (size_t)(cfg->kmax + 1)));
    }
    TRY(dalloc(&h->uold1, pl));
    TRY(dalloc(&h->x3, (size_t)nz)); TRY(dalloc(&h->jacinv, (size_t)nz)); TRY(dalloc(&h->jac2, (size_t)nz));
    TRY(dalloc(&h->Ab, (size_t)nz)); TRY(dalloc(&h->At, (size_t)nz)); TRY(dalloc(&h->Ap, (size_t)nz));
    TRY(dalloc(&h->rAp, (size_t)nz));
    TRY(dalloc(&h->gs_coef, 8 * (size_t)nz));
    TRY(dalloc(&h->gs_coef_f, 5 * (size_t)nz));
    TRY(dalloc(&h->lap_scale, (size_t)nz));
    TRY(dalloc(&h->coef_f, 4 * (size_t)nz));
    TRY(dalloc(&h->usum2, n2)); TRY(dalloc(&h->vsum2, n2)); TRY(dalloc(&h->wsum2, n2)); TRY(dalloc(&h->wt, n2));
    TRY(dalloc(&h->ume1, (size_t)nz)); TRY(dalloc(&h->bltkns, (size_t)nx)); TRY(dalloc(&h->newk, (size_t)nz));
    TRY(dalloc(&h->ufl_file, 3 * pl)); TRY(dalloc(&h->ufl_live, 3 * pl));
    TRY(dalloc(&h->ufl_full, 3 * vol)); TRY(dalloc(&h->usum2_fl, 3 * n2));
    TRY(dalloc(&h->sums, 9 * n2)); TRY(dalloc(&h->avg, 9 * n2)); TRY(dalloc(&h->bl_out, 4 * (size_t)nx));
    TRY(dalloc(&h->ubulk, 5)); TRY(dalloc(&h->sumxz, (size_t)nx)); TRY(dalloc(&h->tauw_win, (size_t)nx));
    TRY(dalloc(&h->slab_of_k, (size_t)nz));
    TRY(dalloc(&h->sc, 1));
    const int K1 = (cfg->precision == TBL_PREC_MIXED ? cfg->mixed_kmax : cfg->kmax) + 1;
    TRY(dalloc(&h->h, (size_t)K1 * K1)); TRY(dalloc(&h->gg, (size_t)K1)); TRY(dalloc(&h->gc, (size_t)K1));
    TRY(dalloc(&h->gs, (size_t)K1)); TRY(dalloc(&h->gy, (size_t)K1));
    h->red.max_blocks = 2048;
    TRY(dalloc(&h->red.partial, (size_t)16 * h->red.max_blocks));
    TRY(dalloc(&h->red.count, (size_t)16));
    TRY(dalloc(&h->halo, (size_t)2 * 3 * 2 * h->P * g.ps));
    TRY(dalloc(&h->err, 1));
    // mesh and per-k coefficients (:487-536); An* == Av*
    std::vector<double> x3(mesh->x3, mesh->x3 + nz), jinv(nz), j2(mesh->jac2, mesh->jac2 + nz);
    std::vector<double> Ab(nz, 0.0), At(nz, 0.0), Ap(nz, 0.0), rAp(nz, 0.0);
    const double dx = cfg->dx, dy = cfg->dy, dxi = cfg->dxi;
    for (int k = 1; k <= nz - 2; ++k) {
        double J = mesh->jac[k], J2 = mesh->jac2[k];
        double a = 1.0 / (dxi * dxi * J * J);
        double b = J2 / (2.0 * dxi * J * J * J);
        Ab[k] = a + b;
        At[k] = a - b;
        Ap[k] = -2.0 * ((1.0 / (dx * dx)) + (1.0 / (dy * dy)) + (1.0 / (dxi * dxi * J * J)));
        rAp[k] = 1.0 / Ap[k];
    }
    for (int k = 0; k < nz; ++k) jinv[k] = 1.0 / mesh->jac[k];
    h->x3h = x3;
    const bool sete = cfg->variant == TBL_VARIANT_DNSSETBL;
    h->stats_dA = sete ? 1.0 : cfg->dy;  // dnssetbl: unweighted span sums over ny-2 (dnssetbl.f90:951-981)
    h->stats_A = sete ? (double)(ny - 2) : mesh->x2[ny - 1] - mesh->x2[1];
    h->area_mf = sete ? (x3[nz - 2] - x3[1]) * (mesh->x2[ny - 2] - mesh->x2[1])  // dnssetbl.f90:896
                      : x3[nz - 1] * (mesh->x2[ny - 2] - mesh->x2[1]);          // Av (:448)
    TBL_CUDA_TRY(cudaMemcpy(h->x3, x3.data(), nz * 8, cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemcpy(h->jacinv, jinv.data(), nz * 8, cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemcpy(h->jac2, j2.data(), nz * 8, cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemcpy(h->Ab, Ab.data(), nz * 8, cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemcpy(h->At, At.data(), nz * 8, cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemcpy(h->Ap, Ap.data(), nz * 8, cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemcpy(h->rAp, rAp.data(), nz * 8, cudaMemcpyHostToDevice));
    {   // the forward sweep's -w/Ap(k) in FP64, and the FP32 matvec's coefficients (casts of the FP64 values)
        std::vector<double> sc(nz, 0.0);
        std::vector<float> cf(4 * (size_t)nz, 0.0f);
        for (int k = 0; k < nz; ++k) {
            sc[k] = -cfg->omega * rAp[k];
            cf[k] = (float)Ab[k]; cf[nz + k] = (float)At[k]; cf[2 * nz + k] = (float)Ap[k];
            cf[3 * nz + k] = (float)sc[k];
        }
        TBL_CUDA_TRY(cudaMemcpy(h->lap_scale, sc.data(), nz * 8, cudaMemcpyHostToDevice));
        TBL_CUDA_TRY(cudaMemcpy(h->coef_f, cf.data(), 4 * (size_t)nz * 4, cudaMemcpyHostToDevice));
    }
    std::vector<double> AbT(nz, 0.0), AtT(nz, 0.0);  // L7^T: row k couples k-1 by At[k-1], k+1 by Ab[k+1]
    for (int k = 1; k <= nz - 2; ++k) { AbT[k] = At[k - 1]; AtT[k] = Ab[k + 1]; }
    TRY(dalloc(&h->AbT, (size_t)nz)); TRY(dalloc(&h->AtT, (size_t)nz));
    TBL_CUDA_TRY(cudaMemcpy(h->AbT, AbT.data(), nz * 8, cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemcpy(h->AtT, AtT.data(), nz * 8, cudaMemcpyHostToDevice));
    h->x1h.assign(mesh->x1, mesh->x1 + nx);
    std::vector<int> sok(nz, 0);
    for (int r = 0; r < h->P; ++r)
        for (int k = h->bn[r]; k <= h->en[r]; ++k) sok[k] = r;
    TBL_CUDA_TRY(cudaMemcpy(h->slab_of_k, sok.data(), nz * 4, cudaMemcpyHostToDevice));
    DevScalars s0;
    memset(&s0, 0, sizeof(s0));
    s0.lamda = 1.0;
    TBL_CUDA_TRY(cudaMemcpy(h->sc, &s0, sizeof(s0), cudaMemcpyHostToDevice));
    TRY(build_sweep_ctas(h));
    TRY(check_cooperative(h));
    h->nstep = 0; h->cont = 0; h->nstat = 0; h->cnt2 = 0; h->time = 0.0;
    h->fluc_updated = false;
    h->replay_pos = 0;
    h->lamda_host = 1.0;
    return TBL_OK;
}

// ------------------------------------------------------------ GS solve
int gs_solve(tbl_handle* h, const int* target, tbl_step_stats& st, bool zero_ok) {
    const int mmax = h->cfg.mmax;
    bool active[3] = {true, true, true};
    int sweeps[3] = {0, 0, 0};
    double sumnor[3] = {0, 0, 0}, sumav[3] = {0, 0, 0};
    int parity = 0;
    const bool mixed = h->cfg.precision == TBL_PREC_MIXED;
    // Mixed precision: the increment D of the delta form restarts from zero
    // (r -= A D in FP64, U += D) each time the residual has fallen 100-fold
    // since its last start, so that D stays within two orders of magnitude of
    // the residual it corrects and FP32 rounding of D does not floor the
    // residual ratio above errorstop (it did at 1024 x 258 x 192).
    constexpr double kRestartDrop = 1e-2;
    double restart_at[3] = {1.0, 1.0, 1.0};
    if (mixed)
        for (int c = 0; c < 3; ++c) TRY(launch_gs_delta_init(h, c));
    TRY(launch_halo_init(h, parity));
    const int nb = red_blocks(h);
    for (int it = 1; it <= mmax; ++it) {
        int comps[3], n = 0;
        for (int c = 0; c < 3; ++c)
            if (active[c]) comps[n++] = c;
        if (it % 2 == 1) {  // residual check every other sweep (:781-828)
            {
                ProfScope ps(h, TBL_PROF_GS_RESID, 2.0 * 8.0 * h->npts * n);
                TRY(launch_gs_resid(h, comps, n, nb > 512 ? 512 : nb));
            }
            TRY(readback(h, &h->sc->red[0], 3 * sizeof(double)));
            const double* red = h->hpin;
            int m = 0;
            bool restarted = false;
            for (int q = 0; q < n; ++q) {
                int c = comps[q];
                double diver = red[c];
                if (it == 1 && zero_ok && diver == 0.0) {  // zero right-hand side: the zero guess is exact
                    active[c] = false;
                    sumav[c] = 0.0;
                    continue;
                }
                if (it == 1) sumnor[c] = 1.0 / diver;
                sumav[c] = diver * sumnor[c];
                // dnssetbl also stops on the absolute sum, res < 1e-12 with a
                // REAL(4) literal (dnssetbl.f90:392)
                bool stop = target ? (sweeps[c] >= target[c])
                                   : (sumav[c] < h->cfg.errorstop ||
                                      (h->cfg.variant == TBL_VARIANT_DNSSETBL && diver < (double)1e-12f));
                if (stop) {
                    active[c] = false;
                    continue;
                }
                comps[m++] = c;
                if (mixed && sumav[c] <= kRestartDrop * restart_at[c]) {
                    TRY(launch_gs_delta_restart(h, c));
                    restart_at[c] = sumav[c];
                    restarted = true;
                }
            }
            n = m;
            if (n == 0) break;
            if (restarted) TRY(launch_halo_init(h, parity));  // the restarted increments' halo planes are 0
        }
        {
            ProfScope ps(h, TBL_PROF_GS_SWEEP, 3.0 * 8.0 * h->npts * n);
            TRY(launch_gs_sweep(h, comps, n, parity));
        }
        parity ^= 1;
        for (int q = 0; q < n; ++q) sweeps[comps[q]]++;
    }
    for (int c = 0; c < 3; ++c) { st.gs_sweeps[c] = sweeps[c]; st.gs_resid[c] = sumav[c]; }
    if (mixed)
        for (int c = 0; c < 3; ++c) TRY(launch_gs_delta_apply(h, c));
    return TBL_OK;
}

// ------------------------------------- Arnoldi steps enqueued one step ahead
// The host enqueues Arnoldi step k+1 before it waits for step k's residual
// estimate (an asynchronous copy and an event per step), so the device never
// idles while the host decides whether the cycle goes on.  Step k's Givens
// kernel sets sc->stop when the estimate reaches stop_at -- the host's own
// test, on the same double -- and every kernel of step k+1 then returns at
// once.  The iteration counts are those of the step-by-step loop
// (:1187-1188).  Returns the last step taken in kit and its estimate in
// sumav; the bytes of a step that did nothing are removed from the profile.
template <typename Step>
static int arnoldi_ahead(tbl_handle* h, int kmax, double stop_at, Step& step, int& kit, double& sumav) {
    const int* skip = &h->sc->stop;
    auto post = [&](int k) -> int {
        TBL_CUDA_TRY(cudaMemcpyAsync(h->hpin + 64 + (k & 1), &h->sc->sumav, sizeof(double), cudaMemcpyDeviceToHost,
                                     h->stream));
        TBL_CUDA_TRY(cudaEventRecord(h->ahead_ev[k & 1], h->stream));
        return TBL_OK;
    };
    TRY(step(1, skip));
    TRY(post(1));
    for (int k = 1;; ++k) {
        const size_t mark0 = h->prof_marks.size();
        const bool more = k < kmax;
        if (more) {
            TRY(step(k + 1, skip));
            TRY(post(k + 1));
        }
        TBL_CUDA_TRY(cudaEventSynchronize(h->ahead_ev[k & 1]));
        sumav = h->hpin[64 + (k & 1)];
        if (!(sumav > stop_at) || !more) {
            kit = k;
            if (more)
                for (size_t q = mark0; q < h->prof_marks.size(); ++q) h->prof_marks[q].bytes = 0.0;
            return TBL_OK;
        }
    }
}

// ---------------------------------------------- mixed-precision Poisson solve
// FP64 iterative refinement around FP32 GMRES(mixed_kmax): every outer pass
// forms r = Q8 - L7 p' in FP64, runs one FP32 Arnoldi cycle with the FP32
// block-SSOR preconditioner (FP64 Gram-Schmidt sums, Hessenberg and Givens),
// and adds the correction to the FP64 p'.  Stops when the preconditioned
// residual relative to the first pass is <= mixed_outer_tol; an inner cycle
// stops at mixed_kmax, at mixed_inner_tol relative to its own start, or at the
// outer tolerance.
static int gmres_mixed(tbl_handle* h, std::vector<int32_t>& kits, tbl_step_stats& st) {
    const int kmax = h->cfg.mixed_kmax, K1 = kmax + 1;
    const size_t vol = (size_t)h->g.vol;
    const double outer_tol = h->cfg.mixed_outer_tol, inner_tol = h->cfg.mixed_inner_tol;
    const double true_tol = h->cfg.mixed_true_tol;
    double sumav = 1.0, sumnor = 0.0, true_rel = 0.0;
    int m = 0, iters = 0;
    int status = TBL_OK;
    bool done = false, true_fresh = false;
    const double wN = 4.0 * h->npts;
    while (!done && m < h->cfg.mixed_max_outer) {
        m = m + 1;
        float* V0 = h->Vf;
        if (true_tol > 0.0 && !true_fresh) {  // true relative residual of the current p' (FP64)
            {
                ProfScope ps(h, TBL_PROF_VEC, 2.0 * 8.0 * h->npts);
                TRY(launch_ppe_resid(h));
            }
            TRY(readback(h, &h->sc->red[9], 2 * sizeof(double)));
            true_rel = h->hpin[1] > 0 ? std::sqrt(h->hpin[0] / h->hpin[1]) : 0.0;
        }
        {
            ProfScope ps(h, TBL_PROF_SSOR_FWD, 2.0 * wN + 2.0 * 8.0 * h->npts);
            TRY(launch_ssor_fwd_f(h, nullptr, h->PC, h->Q8));
        }
        {
            ProfScope ps(h, TBL_PROF_SSOR_BWD, 2.0 * wN);
            TRY(launch_ssor_bwd_f(h, V0));
        }
        {
            ProfScope ps(h, TBL_PROF_MGS, 1.0 * wN);
            TRY(launch_dot_f(h, V0, V0, &h->sc->rho, 1));
        }
        TRY(launch_restart_init_k(h, m == 1, K1));
        TRY(readback(h, &h->sc->rho, 4 * sizeof(double)));
        const double rho_m = h->hpin[0];
        if (m == 1) {
            if (std::isnan(rho_m)) { status = TBL_ERR_NAN; break; }
            if (!(rho_m > 0.0)) { status = TBL_ERR_ZERO_RHS; break; }
            sumnor = rho_m;
        }
        sumav = h->hpin[2];
        const bool true_ok = true_tol <= 0.0 || true_rel <= true_tol;
        if (sumav <= outer_tol && true_ok) { kits.push_back(0); done = true; break; }
        // this pass's target for the preconditioned residual: the outer
        // tolerance, tightened in proportion when the true residual is short
        double target = outer_tol;
        if (!true_ok) target = std::fmin(outer_tol, 0.5 * sumav * (true_tol / true_rel));
        {
            ProfScope ps(h, TBL_PROF_VEC, 2.0 * wN);
            TRY(launch_scale_by_inv_f(h, V0, &h->sc->rho));
        }
        int kit = 0;
        // the cycle stops when the estimate reaches the pass's target or its
        // inner tolerance relative to the cycle's start (sumav <= thr)
        const double thr = std::fmax(target, inner_tol * rho_m / sumnor);
        // w_k is formed in the slot after the basis; step k+1's matvec divides
        // it by H(k+1,k) as it reads it and writes v_k into the basis (the
        // separate scaling pass folded into the TMA matvec, same values)
        float* W = h->Vf + (size_t)K1 * vol;
        auto arnoldi_step = [&](int k, const int* skip) -> int {
            {
                ProfScope ps(h, TBL_PROF_SSOR_FWD, (k > 1 ? 3.0 : 2.0) * wN);
                if (k == 1)
                    TRY(launch_ssor_fwd_f(h, V0, nullptr, nullptr, skip));
                else
                    TRY(launch_ssor_fwd_f(h, W, nullptr, nullptr, skip, &h->sc->red[8], h->Vf + (size_t)(k - 1) * vol));
            }
            {
                ProfScope ps(h, TBL_PROF_SSOR_BWD, 2.0 * wN);
                TRY(launch_ssor_bwd_f(h, W, skip));
            }
            double* hcol = h->h + (size_t)K1 * (k - 1);
            {
                // low-synch MGS: one dot pass over the basis (+1 vector per extra group), one update pass
                const int ngr = (k + 7) / 8;
                ProfScope ps(h, TBL_PROF_MGS, ((k + 2.0 * ngr) + (k + 2.0)) * wN);
                TRY(launch_lsg_f(h, W, k, hcol, skip));
            }
            {
                ProfScope ps(h, TBL_PROF_SMALL, 0.0);
                TRY(launch_givens_k(h, k, K1, skip, thr));
            }
            return TBL_OK;
        };
        if (h->cfg.flags & TBL_FLAG_RB_PRECOND) {  // one step at a time, read back after each
            while (kit < kmax && sumav > thr) {
                kit = kit + 1;
                TRY(arnoldi_step(kit, nullptr));
                TRY(readback(h, &h->sc->sumav, sizeof(double)));
                sumav = h->hpin[0];
            }
        } else if (kmax > 0 && sumav > thr) {
            TRY(arnoldi_ahead(h, kmax, thr, arnoldi_step, kit, sumav));
        }
        iters += kit;
        kits.push_back(kit);
        if (kit > 0) {
            ProfScope ps(h, TBL_PROF_VEC, (kit * 4.0 + 16.0) * h->npts);
            TRY(launch_backsub_update_f(h, kit));
        }
        // the cycle's residual estimate reached its target: accept, after
        // checking the true residual when that criterion is on
        true_fresh = false;
        if (sumav <= target) {
            if (true_tol > 0.0) {
                {
                    ProfScope ps(h, TBL_PROF_VEC, 2.0 * 8.0 * h->npts);
                    TRY(launch_ppe_resid(h));
                }
                TRY(readback(h, &h->sc->red[9], 2 * sizeof(double)));
                true_rel = h->hpin[1] > 0 ? std::sqrt(h->hpin[0] / h->hpin[1]) : 0.0;
                true_fresh = true;
                done = sumav <= outer_tol && true_rel <= true_tol;
            } else {
                done = sumav <= outer_tol;
            }
        }
    }
    st.gmres_restarts = m;
    st.outer_iters = m;
    st.gmres_iters = iters;
    st.gmres_resid = sumav;
    if (status == TBL_OK && !done) status = TBL_ERR_NOT_CONVERGED;
    return status;
}

// ------------------------------------------------------------ GMRES
int gmres(tbl_handle* h, const int32_t* rec, std::vector<int32_t>& kits, tbl_step_stats& st) {
    const int kmax = h->cfg.kmax, K1 = kmax + 1;
    const size_t vol = (size_t)h->g.vol;
    double sumav = 1.0;
    int m = 0, iters = 0;
    const int nr = rec ? rec[0] : 0;
    int status = TBL_OK;
    while (rec ? (m < nr) : ((sumav > h->cfg.errtol) && (m < h->cfg.mmax))) {
        m = m + 1;
        double* V0 = h->V;
        const double wN = 8.0 * h->npts;
        {
            ProfScope ps(h, TBL_PROF_SSOR_FWD, 3.0 * wN);
            TRY(launch_ssor_fwd(h, h->PC, h->Q8));  // r = Q8 - L7 p', then SSOR (:995-1042)
        }
        {
            ProfScope ps(h, TBL_PROF_SSOR_BWD, 2.0 * wN);
            TRY(launch_ssor_bwd(h, V0));
        }
        {
            ProfScope ps(h, TBL_PROF_MGS, 1.0 * wN);
            TRY(launch_dot(h, V0, V0, &h->sc->rho, 1));
        }
        TRY(launch_restart_init(h, m == 1));
        TRY(readback(h, &h->sc->rho, 4 * sizeof(double)));  // rho, sumnor, sumav
        double rho = h->hpin[0];
        if (m == 1 && std::isnan(rho)) { status = TBL_ERR_NAN; break; }
        if (m == 1 && !(rho > 0.0)) { status = TBL_ERR_ZERO_RHS; break; }
        sumav = h->hpin[2];
        {
            ProfScope ps(h, TBL_PROF_VEC, 2.0 * wN);
            TRY(launch_scale_by_inv(h, V0, &h->sc->rho));
        }
        int kit = 0;
        const int target = rec ? rec[m] : 0;
        // One Arnoldi step (:1059-1191): preconditioned matvec, MGS, Givens,
        // normalisation.  With skip, every kernel returns at once when an
        // earlier step's Givens stopped the cycle.
        auto arnoldi_step = [&](int k, const int* skip) -> int {
            double* W = h->V + (size_t)k * vol;
            {
                ProfScope ps(h, TBL_PROF_SSOR_FWD, 2.0 * wN);
                TRY(launch_ssor_fwd(h, h->V + (size_t)(k - 1) * vol, nullptr, skip));
            }
            {
                ProfScope ps(h, TBL_PROF_SSOR_BWD, 2.0 * wN);
                TRY(launch_ssor_bwd(h, W, skip));
            }
            double* hcol = h->h + (size_t)K1 * (k - 1);
            {
                // passes: <v1,w>; (k-1) x {w -= h v_k; <v_k+1,w>}; w -= h v_k, ||w||
                ProfScope ps(h, TBL_PROF_MGS, (2.0 + 4.0 * (k - 1) + 3.0) * wN);
                TRY(launch_mgs(h, W, nullptr, nullptr, V0, &hcol[0], 0, skip));
                for (int kk = 1; kk <= k - 1; ++kk)
                    TRY(launch_mgs(h, W, h->V + (size_t)(kk - 1) * vol, &hcol[kk - 1], h->V + (size_t)kk * vol,
                                   &hcol[kk], 0, skip));
                TRY(launch_mgs(h, W, h->V + (size_t)(k - 1) * vol, &hcol[k - 1], nullptr, &hcol[k], 1, skip));
            }
            {
                ProfScope ps(h, TBL_PROF_SMALL, 0.0);
                TRY(launch_givens(h, k, skip, h->cfg.errtol));
            }
            {
                ProfScope ps(h, TBL_PROF_VEC, 2.0 * wN);
                TRY(launch_scale_by_inv(h, W, &h->sc->red[8], skip));
            }
            return TBL_OK;
        };
        if (rec || (h->cfg.flags & TBL_FLAG_RB_PRECOND)) {  // one step at a time, read back after each
            while (rec ? (kit < target) : ((sumav > h->cfg.errtol) && (kit < kmax))) {
                kit = kit + 1;
                TRY(arnoldi_step(kit, nullptr));
                TRY(readback(h, &h->sc->sumav, sizeof(double)));
                sumav = h->hpin[0];
            }
        } else if (sumav > h->cfg.errtol && kmax > 0) {
            TRY(arnoldi_ahead(h, kmax, h->cfg.errtol, arnoldi_step, kit, sumav));
        }
        iters += kit;
        kits.push_back(kit);
        if (kit > 0) {
            ProfScope ps(h, TBL_PROF_VEC, (kit + 2.0) * wN);
            TRY(launch_backsub_update(h, kit));
        }
    }
    st.gmres_restarts = m;
    st.gmres_iters = iters;
    st.gmres_resid = sumav;
    if (status == TBL_OK && !rec && sumav > h->cfg.errtol) status = TBL_ERR_NOT_CONVERGED;
    return status;
}

int one_step(tbl_handle* h, tbl_step_stats* out) {
    tbl_step_stats st;
    memset(&st, 0, sizeof(st));
    const tbl_config& c = h->cfg;
    h->time = h->time + c.dt;
    h->nstep = h->nstep + 1;
    // replay record for this step
    const bool replay = (c.flags & TBL_FLAG_REPLAY) != 0;
    const int32_t* rec = nullptr;
    int gs_target[3];
    if (replay) {
        if (h->replay_pos + 4 > h->replay.size()) return TBL_ERR_REPLAY;
        const int32_t* r = h->replay.data() + h->replay_pos;
        for (int q = 0; q < 3; ++q) gs_target[q] = r[q];
        if (h->replay_pos + 4 + (size_t)r[3] > h->replay.size()) return TBL_ERR_REPLAY;
        rec = r + 3;
        h->replay_pos += 4 + r[3];
    }
    const double wN = 8.0 * h->npts;
    {
        ProfScope ps(h, TBL_PROF_BC, 0.0);
        TRY(launch_save_uold(h));
        if (h->nstep > c.recycle_after) TRY(launch_inflow(h));
        if (h->tape_u1)  // adjoint window: the velocities the convection sees
            for (int q = 0; q < 3; ++q)
                TBL_CUDA_TRY(cudaMemcpyAsync(h->tape_u1 + (size_t)q * h->g.vol, h->U[q], (size_t)h->g.vol * 8,
                                             cudaMemcpyDeviceToDevice, h->stream));
    }
    {
        ProfScope ps(h, TBL_PROF_CONV, 7.0 * wN);
        TRY(launch_conv_q(h));
    }
    TRY(gs_solve(h, replay ? gs_target : nullptr, st, false));
    {
        ProfScope ps(h, TBL_PROF_BC, 4.0 * wN);
        TRY(launch_div(h));
        TRY(launch_pc_zero_faces(h));
    }
    std::vector<int32_t> kits;
    int status = c.precision == TBL_PREC_MIXED ? gmres_mixed(h, kits, st) : gmres(h, rec, kits, st);
    if (status == TBL_ERR_ZERO_RHS || status < 0 && status != TBL_ERR_NOT_CONVERGED) return status;
    if (c.flags & TBL_FLAG_PPE_RESIDUAL) {
        TRY(launch_ppe_resid(h));
        TRY(readback(h, &h->sc->red[9], 2 * sizeof(double)));
        st.ppe_rel_resid = h->hpin[1] > 0 ? std::sqrt(h->hpin[0] / h->hpin[1]) : 0.0;
    }
    {
        ProfScope ps(h, TBL_PROF_BC, 9.0 * wN);
        TRY(launch_project_bcs(h));
    }
    const int nb = red_blocks(h);
    // dnssetbl: statistics, then the rescaling every cum steps of nstep, then
    // the fluctuations and KE when this run's step count cnt > recycle_after
    // (dnssetbl.f90:936, :986, :1223); dnstbl2: fluctuations when
    // nstep > recycle_after, statistics, rescaling every cum steps of cont
    // (:1686, :1881, :1974).
    const bool sete = c.variant == TBL_VARIANT_DNSSETBL;
    const bool fluc = sete ? (h->cont + 1 > c.recycle_after) : (h->nstep > c.recycle_after);
    {
        ProfScope ps_stats(h, TBL_PROF_STATS, (fluc ? 9.0 : 6.0) * wN);
        TRY(launch_div_diag(h, nb > 512 ? 512 : nb, 3));
        TRY(launch_flux_shear(h));
        auto fluc_ke = [&]() -> int {
            TRY(launch_fluc_ke(h, nb > 512 ? 512 : nb, 4));
            const size_t n2 = (size_t)c.nx * c.nz;
            TBL_CUDA_TRY(cudaMemcpyAsync(h->usum2_fl, h->usum2, n2 * 8, cudaMemcpyDeviceToDevice, h->stream));
            TBL_CUDA_TRY(cudaMemcpyAsync(h->usum2_fl + n2, h->vsum2, n2 * 8, cudaMemcpyDeviceToDevice, h->stream));
            TBL_CUDA_TRY(cudaMemcpyAsync(h->usum2_fl + 2 * n2, h->wsum2, n2 * 8, cudaMemcpyDeviceToDevice, h->stream));
            h->fluc_updated = true;
            return TBL_OK;
        };
        if (fluc && !sete) TRY(fluc_ke());
        h->cont = h->cont + 1;
        if (h->nstep % c.istat == 0) {
            TRY(launch_stats(h));
            h->nstat++;
        }
        st.cum_step = 0;
        if ((sete ? h->nstep : h->cont) % c.cum == 0) {
            TRY(launch_rescale(h));
            st.cum_step = 1;
        }
        if (fluc && sete) TRY(fluc_ke());
    }
    h->cnt2 = h->cnt2 + 1;  // end of the step (fnldnstbl.f90:2382, dnstbl.f90:2349)
    // scalars back: red[3] div, red[4] KE, red[5] max fluct, lamda, err
    TRY(readback(h, h->sc, sizeof(DevScalars)));
    if (h->prof_on) TRY(prof_drain(h));
    DevScalars sc;
    memcpy(&sc, h->hpin, sizeof(sc));
    int err = 0;
    TBL_CUDA_TRY(cudaMemcpy(&err, h->err, sizeof(int), cudaMemcpyDeviceToHost));
    st.div_diag = std::fabs(sc.red[3]) / ((double)(c.ny - 2) * (c.nx - 2) * (c.nz - 2));
    if (c.variant == TBL_VARIANT_ORIGINAL) st.div_diag = std::sqrt(st.div_diag);  // fnldnstbl.f90:1586
    st.ke = fluc ? sc.red[4] / ((double)c.nx * (c.ny - 2) * (c.nz - 2)) : 0.0;
    st.lamda = sc.lamda;
    h->lamda_host = sc.lamda;
    st.nstep = h->nstep;
    st.time = h->time;
    h->last_counts.clear();
    for (int q = 0; q < 3; ++q) h->last_counts.push_back(st.gs_sweeps[q]);
    h->last_counts.push_back((int32_t)kits.size());
    for (int q : kits) h->last_counts.push_back(q);
    if (err != 0) status = err;
    else if (!std::isfinite(sc.red[3]) || (fluc && !std::isfinite(sc.red[4]))) status = TBL_ERR_NAN;
    else if (fluc && sc.red[5] > 25.0) status = TBL_ERR_BLOWUP;
    else if (status == TBL_OK && !replay)
        for (int q = 0; q < 3; ++q)
            if (st.gs_sweeps[q] >= c.mmax) status = TBL_ERR_NOT_CONVERGED;
    st.status = status;
    if (out) *out = st;
    return status;
}

}  // namespace tbl

using namespace tbl;

extern "C" {

int tbl_create(const tbl_config* cfg, const tbl_mesh* mesh, tbl_handle** out) {
    if (!cfg || !mesh || !out || !mesh->x1 || !mesh->x2 || !mesh->x3 || !mesh->jac || !mesh->jac2)
        return TBL_ERR_BAD_ARG;
    if (cfg->nx < 8 || cfg->ny < 6 || cfg->nz < 8 || cfg->nproc < 1) return TBL_ERR_BAD_ARG;
    if (cfg->variant < TBL_VARIANT_DNSTBL2 || cfg->variant > TBL_VARIANT_DNSSETBL) return TBL_ERR_BAD_ARG;
    {
        std::vector<int> b, e;
        if (!tbl::slab_partition(*cfg, b, e)) return TBL_ERR_BAD_ARG;
    }
    if (cfg->irec < 2 || cfg->irec > cfg->nx - 1 || cfg->cum < 1 || cfg->istat < 1) return TBL_ERR_BAD_ARG;
    if (cfg->kmax < 1 || cfg->mmax < 1 || !(cfg->dt > 0) || !(cfg->re > 0)) return TBL_ERR_BAD_ARG;
    if (cfg->precision != TBL_PREC_FP64 && cfg->precision != TBL_PREC_MIXED) return TBL_ERR_BAD_ARG;
    if (cfg->precision == TBL_PREC_MIXED &&
        (cfg->mixed_kmax < 1 || cfg->mixed_kmax > 63 || cfg->mixed_max_outer < 1 || !(cfg->mixed_true_tol >= 0) || !(cfg->mixed_outer_tol > 0) || !(cfg->mixed_inner_tol > 0)))
        return TBL_ERR_BAD_ARG;
    if (cfg->precision == TBL_PREC_MIXED && (cfg->flags & TBL_FLAG_REPLAY)) return TBL_ERR_BAD_ARG;
    if ((cfg->flags & TBL_FLAG_RB_ORDER) && ((cfg->ny - 2) % 2 != 0)) return TBL_ERR_BAD_ARG;  // colouring vs wrap
    if ((cfg->flags & TBL_FLAG_RB_PRECOND) && !(cfg->flags & TBL_FLAG_RB_ORDER)) return TBL_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return TBL_ERR_NO_DEVICE;
    tbl_handle* h = new (std::nothrow) tbl_handle();
    if (!h) return TBL_ERR_BAD_ARG;
    memset((void*)&h->cfg, 0, sizeof(h->cfg));
    h->U[0] = h->U[1] = h->U[2] = nullptr;
    int s = create_impl(cfg, mesh, h);
    if (s != TBL_OK) {
        free_all(h);
        delete h;
        return s;
    }
    *out = h;
    return TBL_OK;
}

int tbl_upload_state(tbl_handle* h, const tbl_state* st) {
    if (!h || !st || !st->u || !st->v || !st->w || !st->p || !st->usum2 || !st->vsum2 || !st->wsum2 || !st->wt ||
        !st->newk || !st->ume1)
        return TBL_ERR_BAD_ARG;
    const tbl_config& c = h->cfg;
    for (int k = 0; k < c.nz; ++k)
        if (st->newk[k] < 1 || st->newk[k] > c.nz) return TBL_ERR_BAD_ARG;
    const size_t n2 = (size_t)c.nx * c.nz, pl = (size_t)c.ny * c.nz;
    if (c.precision == TBL_PREC_MIXED) {
        TRY(put3f(h, h->Uf[0], st->u));
        TRY(put3f(h, h->Uf[1], st->v));
        TRY(put3f(h, h->Uf[2], st->w));
        TRY(put3f(h, h->Pf, st->p));
    } else {
        TRY(put3(h, h->U[0], st->u));
        TRY(put3(h, h->U[1], st->v));
        TRY(put3(h, h->U[2], st->w));
        TRY(put3(h, h->Pr, st->p));
    }
    if (st->pcorr) TRY(put3(h, h->PC, st->pcorr));
    else TBL_CUDA_TRY(cudaMemsetAsync(h->PC, 0, (size_t)h->g.vol * 8, h->stream));
    TBL_CUDA_TRY(cudaMemcpyAsync(h->usum2, st->usum2, n2 * 8, cudaMemcpyHostToDevice, h->stream));
    TBL_CUDA_TRY(cudaMemcpyAsync(h->vsum2, st->vsum2, n2 * 8, cudaMemcpyHostToDevice, h->stream));
    TBL_CUDA_TRY(cudaMemcpyAsync(h->wsum2, st->wsum2, n2 * 8, cudaMemcpyHostToDevice, h->stream));
    TBL_CUDA_TRY(cudaMemcpyAsync(h->wt, st->wt, n2 * 8, cudaMemcpyHostToDevice, h->stream));
    TBL_CUDA_TRY(cudaMemcpyAsync(h->newk, st->newk, (size_t)c.nz * 4, cudaMemcpyHostToDevice, h->stream));
    TBL_CUDA_TRY(cudaMemcpyAsync(h->ume1, st->ume1, (size_t)c.nz * 8, cudaMemcpyHostToDevice, h->stream));
    if (st->bltkns)
        TBL_CUDA_TRY(cudaMemcpyAsync(h->bltkns, st->bltkns, (size_t)c.nx * 8, cudaMemcpyHostToDevice, h->stream));
    // Ufluc: full copy for the restart output and the recycling plane (file and live copies)
    std::vector<double> plane(3 * pl, 0.0);
    const double* uf[3] = {st->uf, st->vf, st->wf};
    const double* us[3] = {st->usum2, st->vsum2, st->wsum2};
    const double* U[3] = {st->u, st->v, st->w};
    const int ir = c.irec - 1;
    for (int cc = 0; cc < 3; ++cc) {
        for (int k = 0; k < c.nz; ++k)
            for (int j = 0; j < c.ny; ++j) {
                size_t p = (size_t)ir + (size_t)c.nx * ((size_t)j + (size_t)c.ny * k);
                plane[cc * pl + (size_t)j + (size_t)c.ny * k] =
                    uf[cc] ? uf[cc][p] : (U[cc][p] - us[cc][(size_t)ir + (size_t)c.nx * k]);
            }
        if (uf[cc]) TRY(put3(h, h->ufl_full + (size_t)cc * h->g.vol, uf[cc]));
        else TBL_CUDA_TRY(cudaMemsetAsync(h->ufl_full + (size_t)cc * h->g.vol, 0, (size_t)h->g.vol * 8, h->stream));
    }
    TBL_CUDA_TRY(cudaMemcpyAsync(h->ufl_live, plane.data(), 3 * pl * 8, cudaMemcpyHostToDevice, h->stream));
    if (c.variant == TBL_VARIANT_DNSSETBL)  // computed on each rank's own slab only: reads elsewhere see zeros
        std::fill(plane.begin(), plane.end(), 0.0);  // (dnssetbl.f90:141-149)
    TBL_CUDA_TRY(cudaMemcpyAsync(h->ufl_file, plane.data(), 3 * pl * 8, cudaMemcpyHostToDevice, h->stream));
    // scalars
    DevScalars s0;
    TBL_CUDA_TRY(cudaMemcpyAsync(&s0, h->sc, sizeof(s0), cudaMemcpyDeviceToHost, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    s0.lamda = st->lamda;
    s0.ksep = st->ksep;
    TBL_CUDA_TRY(cudaMemcpy(h->sc, &s0, sizeof(s0), cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMemsetAsync(h->sums, 0, 9 * n2 * 8, h->stream));
    TBL_CUDA_TRY(cudaMemsetAsync(h->ubulk, 0, 5 * 8, h->stream));
    TBL_CUDA_TRY(cudaMemsetAsync(h->sumxz, 0, (size_t)c.nx * 8, h->stream));
    TBL_CUDA_TRY(cudaMemsetAsync(h->tauw_win, 0, (size_t)c.nx * 8, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->nstep = st->nstep;
    h->cont = st->cont;
    h->cnt2 = st->cnt2;
    h->time = st->time;
    h->fluc_updated = false;
    h->lamda_host = st->lamda;
    return TBL_OK;
}

int tbl_upload_fields(tbl_handle* h, const double* u, const double* v, const double* w, const double* p,
                      const double* pcorr) {
    if (!h || !u || !v || !w || !p) return TBL_ERR_BAD_ARG;
    if (h->cfg.precision == TBL_PREC_MIXED) {
        TRY(put3f(h, h->Uf[0], u));
        TRY(put3f(h, h->Uf[1], v));
        TRY(put3f(h, h->Uf[2], w));
        TRY(put3f(h, h->Pf, p));
    } else {
        TRY(put3(h, h->U[0], u));
        TRY(put3(h, h->U[1], v));
        TRY(put3(h, h->U[2], w));
        TRY(put3(h, h->Pr, p));
    }
    if (pcorr) TRY(put3(h, h->PC, pcorr));
    return TBL_OK;
}

int tbl_profile(tbl_handle* h, int enable) {
    if (!h) return TBL_ERR_BAD_ARG;
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->prof_marks.clear();
    h->prof_used = 0;
    for (int q = 0; q < TBL_PROF_NGROUPS; ++q) { h->prof_ms[q] = 0; h->prof_bytes[q] = 0; h->prof_n[q] = 0; }
    h->prof_on = enable != 0;
    return TBL_OK;
}

int tbl_profile_read(tbl_handle* h, double* ms, double* bytes, int64_t* launches, int ngroups) {
    if (!h || ngroups < 0) return TBL_ERR_BAD_ARG;
    for (int q = 0; q < ngroups && q < TBL_PROF_NGROUPS; ++q) {
        if (ms) ms[q] = h->prof_ms[q];
        if (bytes) bytes[q] = h->prof_bytes[q];
        if (launches) launches[q] = h->prof_n[q];
    }
    return TBL_OK;
}

static int step_loop(tbl_handle* h, int32_t nsteps, tbl_step_stats* stats) {
    int last = TBL_OK;
    for (int s = 0; s < nsteps; ++s) {
        last = one_step(h, stats ? &stats[s] : nullptr);
        if (last == TBL_ERR_NAN || last == TBL_ERR_BLOWUP || last == TBL_ERR_REPLAY || last == TBL_ERR_ZERO_RHS ||
            last == TBL_ERR_CUDA || last == TBL_ERR_TIMEOUT)
            return last;
    }
    return last;
}

int tbl_step(tbl_handle* h, int32_t nsteps, tbl_step_stats* stats) {
    if (!h || nsteps < 0) return TBL_ERR_BAD_ARG;
    if (!h->prof_on) return step_loop(h, nsteps, stats);
    cudaEvent_t a, b;
    TBL_CUDA_TRY(cudaEventCreate(&a));
    TBL_CUDA_TRY(cudaEventCreate(&b));
    const int64_t l0 = h->launches;
    TBL_CUDA_TRY(cudaEventRecord(a, h->stream));
    int last = step_loop(h, nsteps, stats);
    TBL_CUDA_TRY(cudaEventRecord(b, h->stream));
    TBL_CUDA_TRY(cudaEventSynchronize(b));
    float ms = 0.f;
    TBL_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
    h->prof_ms[TBL_PROF_TOTAL] += ms;
    h->prof_n[TBL_PROF_TOTAL] += h->launches - l0;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return last;
}

int tbl_download_state(tbl_handle* h, tbl_state* st) {
    if (!h || !st) return TBL_ERR_BAD_ARG;
    const tbl_config& c = h->cfg;
    const size_t n2 = (size_t)c.nx * c.nz, pl = (size_t)c.ny * c.nz, N = (size_t)c.nx * c.ny * c.nz;
    const bool mx = c.precision == TBL_PREC_MIXED;
    if (st->u) TRY(mx ? get3f(h, st->u, h->Uf[0]) : get3(h, st->u, h->U[0]));
    if (st->v) TRY(mx ? get3f(h, st->v, h->Uf[1]) : get3(h, st->v, h->U[1]));
    if (st->w) TRY(mx ? get3f(h, st->w, h->Uf[2]) : get3(h, st->w, h->U[2]));
    if (st->p) TRY(mx ? get3f(h, st->p, h->Pf) : get3(h, st->p, h->Pr));
    if (st->pcorr) TRY(get3(h, st->pcorr, h->PC));
    if (st->usum2) TBL_CUDA_TRY(cudaMemcpyAsync(st->usum2, h->usum2, n2 * 8, cudaMemcpyDeviceToHost, h->stream));
    if (st->vsum2) TBL_CUDA_TRY(cudaMemcpyAsync(st->vsum2, h->vsum2, n2 * 8, cudaMemcpyDeviceToHost, h->stream));
    if (st->wsum2) TBL_CUDA_TRY(cudaMemcpyAsync(st->wsum2, h->wsum2, n2 * 8, cudaMemcpyDeviceToHost, h->stream));
    if (st->wt) TBL_CUDA_TRY(cudaMemcpyAsync(st->wt, h->wt, n2 * 8, cudaMemcpyDeviceToHost, h->stream));
    if (st->newk) TBL_CUDA_TRY(cudaMemcpyAsync(st->newk, h->newk, (size_t)c.nz * 4, cudaMemcpyDeviceToHost, h->stream));
    if (st->ume1) TBL_CUDA_TRY(cudaMemcpyAsync(st->ume1, h->ume1, (size_t)c.nz * 8, cudaMemcpyDeviceToHost, h->stream));
    if (st->bltkns)
        TBL_CUDA_TRY(cudaMemcpyAsync(st->bltkns, h->bltkns, (size_t)c.nx * 8, cudaMemcpyDeviceToHost, h->stream));
    double* uf[3] = {st->uf, st->vf, st->wf};
    bool any_uf = uf[0] || uf[1] || uf[2];
    if (any_uf) {
        // Ufluc as the reference holds it: uploaded columns, overwritten on the
        // slabs' planes by the last per-step update U - means (:1712-1722), and
        // the recycling plane by its live copy (:2341-2349).
        std::vector<double> U(N), live(3 * pl), means(3 * n2);
        TBL_CUDA_TRY(cudaMemcpyAsync(live.data(), h->ufl_live, 3 * pl * 8, cudaMemcpyDeviceToHost, h->stream));
        TBL_CUDA_TRY(cudaMemcpyAsync(means.data(), h->usum2_fl, 3 * n2 * 8, cudaMemcpyDeviceToHost, h->stream));
        for (int cc = 0; cc < 3; ++cc) {
            if (!uf[cc]) continue;
            TRY(get3(h, uf[cc], h->ufl_full + (size_t)cc * h->g.vol));
            TRY(mx ? get3f(h, U.data(), h->Uf[cc]) : get3(h, U.data(), h->U[cc]));
            TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
            if (h->fluc_updated)
                for (int k = 1; k <= c.nz - 2; ++k)
                    for (int j = 1; j <= c.ny - 2; ++j)
                        for (int i = 0; i < c.nx; ++i) {
                            size_t p = (size_t)i + (size_t)c.nx * ((size_t)j + (size_t)c.ny * k);
                            uf[cc][p] = U[p] - means[cc * n2 + (size_t)i + (size_t)c.nx * k];
                        }
            const int ir = c.irec - 1;
            for (int k = 1; k <= c.nz - 2; ++k)
                for (int j = 1; j <= c.ny - 2; ++j)
                    uf[cc][(size_t)ir + (size_t)c.nx * ((size_t)j + (size_t)c.ny * k)] =
                        live[cc * pl + (size_t)j + (size_t)c.ny * k];
        }
    }
    DevScalars sc;
    TBL_CUDA_TRY(cudaMemcpyAsync(&sc, h->sc, sizeof(sc), cudaMemcpyDeviceToHost, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    st->lamda = sc.lamda;
    st->ksep = sc.ksep;
    st->time = h->time;
    st->nstep = h->nstep;
    st->cont = h->cont;
    st->cnt2 = h->cnt2;
    return TBL_OK;
}

int tbl_download_stats(tbl_handle* h, tbl_stats_out* out) {
    if (!h || !out) return TBL_ERR_BAD_ARG;
    const tbl_config& c = h->cfg;
    const size_t n2 = (size_t)c.nx * c.nz;
    double* dst[9] = {out->usum, out->vsum, out->wsum, out->uusum, out->vvsum, out->wwsum, out->uvsum, out->uwsum, out->vwsum};
    for (int q = 0; q < 9; ++q)
        if (dst[q]) TBL_CUDA_TRY(cudaMemcpyAsync(dst[q], h->sums + q * n2, n2 * 8, cudaMemcpyDeviceToHost, h->stream));
    double* bl[4] = {out->deltastar, out->theta, out->ht, out->reth};
    for (int q = 0; q < 4; ++q)
        if (bl[q]) TBL_CUDA_TRY(cudaMemcpyAsync(bl[q], h->bl_out + (size_t)q * c.nx, (size_t)c.nx * 8,
                                                cudaMemcpyDeviceToHost, h->stream));
    if (out->tauw_sum)
        TBL_CUDA_TRY(cudaMemcpyAsync(out->tauw_sum, h->sumxz, (size_t)c.nx * 8, cudaMemcpyDeviceToHost, h->stream));
    if (out->ubulk) TBL_CUDA_TRY(cudaMemcpyAsync(out->ubulk, h->ubulk, 5 * 8, cudaMemcpyDeviceToHost, h->stream));
    if (out->tauw_window)
        TBL_CUDA_TRY(cudaMemcpyAsync(out->tauw_window, h->tauw_win, (size_t)c.nx * 8, cudaMemcpyDeviceToHost,
                                     h->stream));
    DevScalars sc;
    TBL_CUDA_TRY(cudaMemcpyAsync(&sc, h->sc, sizeof(sc), cudaMemcpyDeviceToHost, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    out->lamda03 = sc.lamda03;
    out->nstat = h->nstat;
    return TBL_OK;
}

int tbl_download_averages(tbl_handle* h, double* avg) {
    if (!h || !avg) return TBL_ERR_BAD_ARG;
    const size_t n2 = (size_t)h->cfg.nx * h->cfg.nz;
    TBL_CUDA_TRY(cudaMemcpyAsync(avg, h->avg, 9 * n2 * 8, cudaMemcpyDeviceToHost, h->stream));
    TBL_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return TBL_OK;
}

int tbl_set_replay(tbl_handle* h, const int32_t* rec, int64_t len) {
    if (!h || len < 0 || (len > 0 && !rec)) return TBL_ERR_BAD_ARG;
    h->replay.assign(rec, rec + len);
    h->replay_pos = 0;
    return TBL_OK;
}

int tbl_last_counts(tbl_handle* h, int32_t* buf, int32_t cap) {
    if (!h || (cap > 0 && !buf)) return TBL_ERR_BAD_ARG;
    int n = (int)h->last_counts.size();
    for (int q = 0; q < n && q < cap; ++q) buf[q] = h->last_counts[q];
    return n;
}

void tbl_destroy(tbl_handle* h) {
    if (!h) return;
    cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
}

const char* tbl_status_string(int status) {
    switch (status) {
        case TBL_OK: return "ok";
        case TBL_ERR_CUDA: return g_last_error[0] ? g_last_error : "CUDA runtime error";
        case TBL_ERR_BAD_ARG: return "invalid argument";
        case TBL_ERR_NOT_CONVERGED: return "GS or GMRES reached mmax";
        case TBL_ERR_NAN: return "non-finite value in the state";
        case TBL_ERR_BLOWUP: return "fluctuation above 25 (reference blow-up stop)";
        case TBL_ERR_TIMEOUT: return "bounded device wait gave up";
        case TBL_ERR_NO_DEVICE: return "no CUDA device";
        case TBL_ERR_REPLAY: return "replay counts exhausted";
        case TBL_ERR_ZERO_RHS: return "zero PPE residual at the first restart";
        case TBL_ERR_TOO_LARGE: return "grid larger than the fixed scratch of the allocation-free entry point";
        case TBL_ERR_IO: return "restart or counter file could not be opened, read, parsed or written";
        default: return "unknown status";
    }
}

int64_t tbl_launch_count(tbl_handle* h) { return h ? h->launches : -1; }

int tbl_selftest_bounded_wait(int32_t* observed, double* seconds) {
    if (!observed) return TBL_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return TBL_ERR_NO_DEVICE;
    int v = 0;
    const int st = tbl::selftest_bounded_wait(&v, seconds);
    *observed = v;
    return st;
}

}  // extern "C"
