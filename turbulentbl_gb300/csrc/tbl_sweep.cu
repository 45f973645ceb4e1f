// tbl_sweep.cu -- pipelined wavefront sweeps (FP64): lexicographic
// Gauss-Seidel for the implicit diffusion and the forward/backward block-SSOR
// preconditioner of GMRES.
//
// The reference sweeps each MPI slab in lexicographic order (i fastest, then
// j, then k; dnstbl2/dnstbl.f90:830-868, :1022-1042, :1115-1135).  A point
// reads new values at (i-1), (j-1), (k-1) and old values at (i+1), (j+1),
// (k+1), so any schedule that respects that partial order performs exactly
// the same arithmetic per point.  The schedule used here:
//
//   * every (j,k) line of a slab is owned by one lane; a lane walks its line
//     in chunks of CHUNK=4 consecutive i (one 32-byte sector);
//   * line (j,k) processes chunk c at logical step T = c + j + k, so its
//     (j-1) and (k-1) predecessors finished chunk c at step T-1;
//   * a warp holds 32 consecutive rows of one plane (the j-1 value comes from
//     the neighbouring lane by shuffle); a CTA holds KG planes;
//   * every warp waits only for the warps producing its inputs: the warp of
//     the row block above (global progress flag, acquire/release) and the
//     warp of the plane below (shared-memory progress inside the CTA, a
//     global flag across CTAs); waits are bounded spins, a timeout sets an
//     error word and the warp returns;
//   * slabs are independent (block-Jacobi GS halos come from a snapshot of the
//     previous sweep, SSOR halos are zero), so all slabs and, for GS, all three
//     velocity components run concurrently in one cooperative launch.
//
// The backward SSOR sweep is the same schedule on mirrored indices.
#include <cooperative_groups.h>

#include "tbl_internal.cuh"
#include "tbl_kernels.cuh"

namespace tbl {

enum SweepMode { SW_GS = 0, SW_FWD = 1, SW_BWD = 2 };

struct SweepArgs {
    Geom g;
    const SweepCta* ctas;
    const SlabDesc* slabs;
    int n_cta, P, C;           // CTAs per component, slab count, chunks per line
    unsigned long long* flags;  // [comp][n_cta]
    unsigned long long epoch;
    int* err;
    const double *Ab, *At, *Ap, *rAp;  // per-k coefficients
    double aw, as;              // 1/dx^2, 1/dy^2
    // GS
    double t;                   // -dt/Re
    double* F[3];
    const double* Q[3];
    int comp[3];
    const double* halo_in;      // [comp][side][slab] planes
    double* halo_out;
    // SSOR
    double omega, sw;           // w, (2-w)/w
    const double* X;            // matvec input (FWD) / PCorr (FWD residual mode)
    const double* Q8;           // residual mode when non-null
    double* RH;                 // FWD output (unscaled) / BWD input
    double* OUT;                // BWD output
};

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

constexpr long long SPIN_LIMIT = 1LL << 24;  // ~1 s of polling, then the wait gives up

// Poll a global progress flag until it reports step >= target (returns the
// step seen, or -2 on timeout).  Flags hold (epoch << 20) + step + 1.
__device__ __forceinline__ long long wait_global(const unsigned long long* f, unsigned long long tag, long long target) {
    long long spins = 0;
    for (;;) {
        unsigned long long v = ld_acquire(f);
        long long seen = v >= tag + 1 ? (long long)(v - tag) - 1 : -1;
        if (seen >= target) return seen;
        if (++spins > SPIN_LIMIT) return -2;
        if (spins > 64) __nanosleep(64);
    }
}

// Same for a warp of this CTA through shared memory.
__device__ __forceinline__ bool wait_shared(volatile int* p, int target) {
    long long spins = 0;
    while (*p < target) {
        if (++spins > SPIN_LIMIT) return false;
        if (spins > 256) __nanosleep(32);
    }
    __threadfence_block();
    return true;
}

// Every warp is an independent unit of the dataflow: it waits only for the
// warps that produce its (j-1) and (k-1) inputs and publishes its own
// progress after each step (shared memory for the next plane in the CTA,
// a global flag for the CTAs downstream).  No CTA-wide barrier in the loop.
template <int MODE>
__global__ void __launch_bounds__(KG * 32) k_sweep(SweepArgs a) {
    const Geom& g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const SweepCta cta = a.ctas[blockIdx.x];
    const SlabDesc sl = a.slabs[cta.slab];
    const int J = g.ny - 2, K = sl.K, C = a.C;
    const int compi = blockIdx.y;
    const int comp = MODE == SW_GS ? a.comp[compi] : 0;
    unsigned long long* flags = a.flags + (size_t)compi * a.n_cta * KG;
    __shared__ volatile int s_prog[KG];
    if (lane == 0) s_prog[wid] = -1;
    __syncthreads();

    // logical line coordinates
    const int jl = 32 * cta.jb + lane;  // logical row
    const int kl = KG * cta.kg + wid;   // logical plane
    if (kl >= K) return;                // no lines: nobody waits for this warp
    const bool line_ok = jl < J;
    // physical coordinates (mirrored for the backward sweep)
    const int jidx = MODE == SW_BWD ? J - 1 - jl : jl;
    const int kidx = MODE == SW_BWD ? K - 1 - kl : kl;
    const int j = 1 + jidx, k = sl.bn + kidx;
    const int jm = (j == 1) ? g.ny - 2 : j - 1;
    const int jp = (j == g.ny - 2) ? 1 : j + 1;
    const long long line = (long long)g.sx * ((long long)j + (long long)g.ny * k);

    // this warp's step range and its upstream warps
    const int jl_last = min(32 * cta.jb + 31, J - 1);
    const int T0 = 32 * cta.jb + kl;
    const int T1 = jl_last + kl + C - 1;
    const int tend_k = jl_last + kl - 1 + C - 1;  // last step of the (k-1) upstream warp
    const unsigned long long* fj = cta.up_j >= 0 ? &flags[(size_t)cta.up_j * KG + wid] : nullptr;
    const unsigned long long* fk = (wid == 0 && cta.up_k >= 0) ? &flags[(size_t)cta.up_k * KG + KG - 1] : nullptr;
    unsigned long long* fme = &flags[(size_t)blockIdx.x * KG + wid];
    const unsigned long long tag = a.epoch << 20;

    // per-plane coefficients
    double cW = 0, cE = 0, cS = 0, cN = 0, cB = 0, cT = 0, rd = 0, wr = 0, sk = 0, ab = 0, at = 0, ap = 0;
    if (MODE == SW_GS) {
        cE = a.t * a.aw; cW = cE; cN = a.t * a.as; cS = cN;
        cT = a.t * a.At[k]; cB = a.t * a.Ab[k];
        rd = 1.0 / (1.0 + (a.t * a.Ap[k]));
    } else {
        wr = -a.omega * a.rAp[k];  // -w * rAnp
        sk = a.sw * a.Ap[k];       // ((2-w)/w) * Anp
        ab = a.Ab[k]; at = a.At[k]; ap = a.Ap[k];
    }
    double* F = MODE == SW_GS ? a.F[comp] : nullptr;
    const double* Qc = MODE == SW_GS ? a.Q[comp] : nullptr;
    const size_t hplane = (size_t)g.ps;
    const double* halo_lo = nullptr;
    const double* halo_hi = nullptr;
    if (MODE == SW_GS) {
        const size_t base = (size_t)comp * 2 * a.P;
        halo_lo = a.halo_in + (base + 0 * a.P + cta.slab) * hplane;
        halo_hi = a.halo_in + (base + 1 * a.P + cta.slab) * hplane;
    }

    double last[CHUNK];  // values this lane produced at the previous step
    double carry = 0.0;  // logical previous point on the own line
#pragma unroll
    for (int e = 0; e < CHUNK; ++e) last[e] = 0.0;
    long long seen_j = -1, seen_k = -1;  // upstream progress known to lane 0

    for (int T = T0; T <= T1; ++T) {
        const int cl = T - jl - kl;  // logical chunk of this lane
        const bool act = line_ok && cl >= 0 && cl < C;
        const int c = MODE == SW_BWD ? C - 1 - cl : cl;  // physical chunk
        const int i0 = 4 * c;
        // ---- operands that do not depend on this step's predecessors
        double rhs[CHUNK], oi[CHUNK], ojp[CHUNK], okp[CHUNK];
        double nxt = 0.0;
        if (act) {
            if (MODE == SW_GS) {
                const double* Fl = F + line + i0;
                const double* Ql = Qc + line + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) { oi[e] = Fl[e]; rhs[e] = Ql[e]; }
                if (i0 + 3 <= g.nx - 2) nxt = Fl[4];
                if (jp != 1) {  // the wrapped row holds new values: read after the wait
                    const double* Fj = F + (long long)g.sx * ((long long)jp + (long long)g.ny * k) + i0;
#pragma unroll
                    for (int e = 0; e < CHUNK; ++e) ojp[e] = __ldcg(Fj + e);
                }
                const double* Fk = (kidx == K - 1 && cta.slab < a.P - 1) ? halo_hi + (long long)g.sx * j + i0
                                                                         : F + line + g.ps + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) okp[e] = __ldcg(Fk + e);
            } else if (MODE == SW_FWD) {
                // r = L7 X (matvec) or Q8 - L7 X (restart residual), global halos
                const double* Xl = a.X + line + i0;
                const double* Xjm = a.X + (long long)g.sx * ((long long)jm + (long long)g.ny * k) + i0;
                const double* Xjp = a.X + (long long)g.sx * ((long long)jp + (long long)g.ny * k) + i0;
                const double* Xkm = Xl - g.ps;
                const double* Xkp = Xl + g.ps;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) {
                    const int i = i0 + e;
                    rhs[e] = 0.0;
                    if (i >= 1 && i <= g.nx - 2) {
                        double lap = a.aw * Xl[e - 1] + a.aw * Xl[e + 1] + a.as * Xjm[e] + a.as * Xjp[e] +
                                     ab * Xkm[e] + at * Xkp[e] + ap * Xl[e];
                        rhs[e] = a.Q8 ? (a.Q8[line + i0 + e] - (lap)) : lap;
                    }
                }
            } else {
                const double* Rl = a.RH + line + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) rhs[e] = sk * Rl[e];
            }
        }
        // ---- wait for the producers of step T-1 (lane 0 polls for the warp)
        const int cl0 = T - 32 * cta.jb - kl;           // lane 0's chunk
        const bool lane0_act = cl0 >= 0 && cl0 < C;
        const bool any_act = cl0 >= 0 && (T - jl_last - kl) < C;
        int abort = 0;
        if (lane == 0 && any_act) {
            if (fj && lane0_act && seen_j < T - 1) {
                seen_j = wait_global(fj, tag, T - 1);
                if (seen_j < 0) abort = 1;
            }
            if (!abort && kl > 0) {
                const int target = min(T - 1, tend_k);
                if (wid > 0) {
                    if (!wait_shared(&s_prog[wid - 1], target)) abort = 1;
                } else if (fk && seen_k < target) {
                    seen_k = wait_global(fk, tag, target);
                    if (seen_k < 0) abort = 1;
                }
            }
            if (abort) atomicExch(a.err, TBL_ERR_TIMEOUT);
        }
        abort = __shfl_sync(0xffffffffu, abort, 0);
        if (abort) return;
        __syncwarp();
        // ---- predecessor values: (j-1) by shuffle or global, (k-1) through memory
        double pj[CHUNK], pk[CHUNK];
#pragma unroll
        for (int e = 0; e < CHUNK; ++e) pj[e] = __shfl_up_sync(0xffffffffu, last[e], 1);
        if (act) {
            if (MODE == SW_GS && jp == 1) {
                const double* Fj = F + (long long)g.sx * ((long long)jp + (long long)g.ny * k) + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) ojp[e] = __ldcg(Fj + e);
            }
            if (lane == 0) {
                if (MODE == SW_GS) {  // row j-1 (wrapped: old value of the last row for j=1)
                    const double* s = F + (long long)g.sx * ((long long)jm + (long long)g.ny * k) + i0;
#pragma unroll
                    for (int e = 0; e < CHUNK; ++e) pj[e] = __ldcg(s + e);
                } else {
                    const bool edge = MODE == SW_FWD ? (jidx == 0) : (jidx == J - 1);
                    const double* base = MODE == SW_FWD ? a.RH : a.OUT;
                    const int jn = MODE == SW_FWD ? j - 1 : j + 1;
                    const double* s = base + (long long)g.sx * ((long long)jn + (long long)g.ny * k) + i0;
#pragma unroll
                    for (int e = 0; e < CHUNK; ++e) pj[e] = edge ? 0.0 : __ldcg(s + e);
                }
            }
            if (MODE == SW_GS) {
                const double* s = (kidx == 0 && cta.slab > 0) ? halo_lo + (long long)g.sx * j + i0
                                                              : F + line - g.ps + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) pk[e] = __ldcg(s + e);
            } else {
                const bool edge = MODE == SW_FWD ? (kidx == 0) : (kidx == K - 1);
                const double* base = MODE == SW_FWD ? a.RH : a.OUT;
                const double* s = base + line + (MODE == SW_FWD ? -g.ps : g.ps) + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) pk[e] = edge ? 0.0 : __ldcg(s + e);
            }
            // ---- the chunk, sequential along the line
            double nv[CHUNK];
            if (MODE == SW_GS) {
                double prev = (c == 0) ? oi[0] : carry;  // i=0 is the inflow boundary value
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) {
                    const int i = i0 + e;
                    if (i >= 1 && i <= g.nx - 2) {
                        double oip = e < CHUNK - 1 ? oi[e + 1] : nxt;
                        double x = rhs[e] - cE * oip - cW * prev - cN * ojp[e] - cS * pj[e] - cT * okp[e] - cB * pk[e];
                        x = x * rd;
                        nv[e] = x;
                        prev = x;
                    } else {
                        nv[e] = oi[e];
                        prev = oi[e];
                    }
                }
                carry = prev;
                double* Fl = F + line + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) {
                    const int i = i0 + e;
                    if (i >= 1 && i <= g.nx - 2) Fl[e] = nv[e];
                }
                // next sweep's halo planes of the neighbouring slabs
                if (kidx == 0 && cta.slab > 0) {
                    double* hd = a.halo_out + ((size_t)comp * 2 * a.P + 1 * a.P + (cta.slab - 1)) * hplane +
                                 (long long)g.sx * j + i0;
#pragma unroll
                    for (int e = 0; e < CHUNK; ++e)
                        if (i0 + e >= 1 && i0 + e <= g.nx - 2) hd[e] = nv[e];
                }
                if (kidx == K - 1 && cta.slab < a.P - 1) {
                    double* hd = a.halo_out + ((size_t)comp * 2 * a.P + 0 * a.P + (cta.slab + 1)) * hplane +
                                 (long long)g.sx * j + i0;
#pragma unroll
                    for (int e = 0; e < CHUNK; ++e)
                        if (i0 + e >= 1 && i0 + e <= g.nx - 2) hd[e] = nv[e];
                }
            } else if (MODE == SW_FWD) {
                double prev = (c == 0) ? 0.0 : carry;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) {
                    const int i = i0 + e;
                    if (i >= 1 && i <= g.nx - 2) {
                        double x = (rhs[e] + a.aw * prev + a.as * pj[e] + ab * pk[e]) * wr;
                        nv[e] = x;
                        prev = x;
                    } else {
                        nv[e] = 0.0;
                        prev = 0.0;
                    }
                }
                carry = prev;
                double* Rl = a.RH + line + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) Rl[e] = nv[e];
            } else {  // SW_BWD: descending i inside the chunk
                double prev = (c == C - 1) ? 0.0 : carry;
#pragma unroll
                for (int e = CHUNK - 1; e >= 0; --e) {
                    const int i = i0 + e;
                    if (i >= 1 && i <= g.nx - 2) {
                        double y = (rhs[e] + a.aw * prev + a.as * pj[e] + at * pk[e]) * wr;
                        nv[e] = y;
                        prev = y;
                    } else {
                        nv[e] = 0.0;
                        prev = 0.0;
                    }
                }
                carry = prev;
                double* Ol = a.OUT + line + i0;
#pragma unroll
                for (int e = 0; e < CHUNK; ++e) Ol[e] = nv[e];
            }
#pragma unroll
            for (int e = 0; e < CHUNK; ++e) last[e] = nv[e];
        }
        // ---- publish step T: the next plane of this CTA, then the CTAs downstream
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            s_prog[wid] = T;
            st_release(fme, tag + (unsigned long long)(T + 1));
        }
    }
}

// ------------------------------------------------------------- host glue

// Build the CTA table for the slab partition (called once at create).
int build_sweep_ctas(tbl_handle* h) {
    const int J = h->g.ny - 2;
    const int njb = (J + 31) / 32;
    std::vector<SweepCta> ctas;
    std::vector<SlabDesc> slabs(h->P);
    for (int r = 0; r < h->P; ++r) {
        slabs[r].bn = h->bn[r];
        slabs[r].K = h->en[r] - h->bn[r] + 1;
        const int nkg = (slabs[r].K + KG - 1) / KG;
        const int base = (int)ctas.size();
        for (int kg = 0; kg < nkg; ++kg)
            for (int jb = 0; jb < njb; ++jb) {
                SweepCta c;
                c.slab = r; c.jb = jb; c.kg = kg;
                c.up_j = jb > 0 ? base + kg * njb + (jb - 1) : -1;
                c.up_k = kg > 0 ? base + (kg - 1) * njb + jb : -1;
                ctas.push_back(c);
            }
    }
    h->n_cta = (int)ctas.size();
    TBL_CUDA_TRY(cudaMalloc(&h->ctas, ctas.size() * sizeof(SweepCta)));
    TBL_CUDA_TRY(cudaMemcpy(h->ctas, ctas.data(), ctas.size() * sizeof(SweepCta), cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMalloc(&h->slabs, slabs.size() * sizeof(SlabDesc)));
    TBL_CUDA_TRY(cudaMemcpy(h->slabs, slabs.data(), slabs.size() * sizeof(SlabDesc), cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMalloc(&h->flags, (size_t)3 * h->n_cta * KG * sizeof(unsigned long long)));
    TBL_CUDA_TRY(cudaMemset(h->flags, 0, (size_t)3 * h->n_cta * KG * sizeof(unsigned long long)));
    h->epoch = 1;
    return TBL_OK;
}

static SweepArgs base_args(tbl_handle* h) {
    SweepArgs a;
    memset(&a, 0, sizeof(a));
    a.g = h->g;
    a.ctas = h->ctas;
    a.slabs = h->slabs;
    a.n_cta = h->n_cta;
    a.P = h->P;
    a.C = (h->g.nx - 2) / CHUNK + 1;
    a.flags = h->flags;
    a.epoch = h->epoch++;
    a.err = h->err;
    a.Ab = h->Ab; a.At = h->At; a.Ap = h->Ap; a.rAp = h->rAp;
    a.aw = 1.0 / (h->cfg.dx * h->cfg.dx);
    a.as = 1.0 / (h->cfg.dy * h->cfg.dy);
    a.omega = h->cfg.omega;
    a.sw = (2 - h->cfg.omega) / h->cfg.omega;
    a.t = -h->cfg.dt / (h->cfg.re);
    return a;
}

template <int MODE>
static int launch_sweep(tbl_handle* h, SweepArgs& a, int ncomp) {
    void* args[] = {&a};
    dim3 grid(h->n_cta, ncomp), block(KG * 32);
    TBL_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_sweep<MODE>, grid, block, args, 0, h->stream));
    h->launches++;
    return TBL_OK;
}

// GS sweep for the listed components; halo buffers ping-pong by `parity`.
int launch_gs_sweep(tbl_handle* h, const int* comps, int ncomp, int parity) {
    SweepArgs a = base_args(h);
    for (int c = 0; c < 3; ++c) { a.F[c] = h->U[c]; a.Q[c] = h->Q[c]; }
    for (int c = 0; c < ncomp; ++c) a.comp[c] = comps[c];
    const size_t hsz = (size_t)3 * 2 * h->P * h->g.ps;
    a.halo_in = h->halo + (size_t)(parity & 1) * hsz;
    a.halo_out = h->halo + (size_t)((parity + 1) & 1) * hsz;
    return launch_sweep<SW_GS>(h, a, ncomp);
}

// Forward SSOR sweep of r = L7 X (Q8 == nullptr) or r = Q8 - L7 X.
int launch_ssor_fwd(tbl_handle* h, const double* X, const double* Q8) {
    SweepArgs a = base_args(h);
    a.X = X;
    a.Q8 = Q8;
    a.RH = h->RH;
    return launch_sweep<SW_FWD>(h, a, 1);
}

int launch_ssor_bwd(tbl_handle* h, double* out) {
    SweepArgs a = base_args(h);
    a.RH = h->RH;
    a.OUT = out;
    return launch_sweep<SW_BWD>(h, a, 1);
}

// Snapshot of the planes every slab reads from its neighbours before the
// first sweep (the end-of-step halo of the previous step).
__global__ void k_halo_init(Geom g, const SlabDesc* __restrict__ slabs, int P, const double* __restrict__ U0,
                            const double* __restrict__ U1, const double* __restrict__ U2, double* __restrict__ halo) {
    // blockIdx.y = comp*2P + side*P + slab
    const int comp = blockIdx.y / (2 * P), rem = blockIdx.y % (2 * P), side = rem / P, r = rem % P;
    const SlabDesc s = slabs[r];
    if (side == 0 && r == 0) return;
    if (side == 1 && r == P - 1) return;
    const int kk = side == 0 ? s.bn - 1 : s.bn + s.K;
    const double* F = comp == 0 ? U0 : (comp == 1 ? U1 : U2);
    double* dst = halo + (size_t)blockIdx.y * g.ps;
    const double* src = F + (long long)kk * g.ps;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < g.ps; q += (long long)gridDim.x * blockDim.x)
        dst[q] = src[q];
}

int launch_halo_init(tbl_handle* h, int parity) {
    const size_t hsz = (size_t)3 * 2 * h->P * h->g.ps;
    k_halo_init<<<dim3(32, 3 * 2 * h->P), 256, 0, h->stream>>>(h->g, h->slabs, h->P, h->U[0], h->U[1], h->U[2],
                                                               h->halo + (size_t)(parity & 1) * hsz);
    h->launches++;
    return TBL_OK;
}

int check_cooperative(tbl_handle* h) {
    int dev = 0, sms = 0, coop = 0;
    TBL_CUDA_TRY(cudaGetDevice(&dev));
    TBL_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    TBL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int per_sm = 0;
    TBL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_sweep<SW_GS>, KG * 32, 0));
    h->coop_ok = coop && (long long)per_sm * sms >= 3LL * h->n_cta;
    return h->coop_ok ? TBL_OK : TBL_ERR_BAD_ARG;
}

}  // namespace tbl
