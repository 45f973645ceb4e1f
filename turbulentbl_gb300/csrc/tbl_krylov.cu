// tbl_krylov.cu -- GMRES(kmax) building blocks in FP64
// (dnstbl2/dnstbl.f90:952-1208): modified Gram-Schmidt passes with fused
// grid reductions, normalisation, Givens rotations and back substitution in
// one device thread, and the solution update p' += V y.
//
// Vector kernels stream the whole padded volume: Krylov vectors are zero
// outside the interior, so boundary and padding entries add nothing to the dot
// products and stay zero under the updates.
#include "tbl_internal.cuh"
#include "tbl_reduce.cuh"
#include "tbl_kernels.cuh"

namespace tbl {

// Grid of the streaming reductions: one resident wave (8 blocks of 256 threads
// per SM), so no partial second wave idles part of the GPU at the tail.
int red_blocks(tbl_handle* h) {
    long long n2 = h->g.vol / 2;
    long long b = (n2 + RED_THREADS * 4 - 1) / (RED_THREADS * 4);
    const long long wave = 8LL * (h->n_sm > 0 ? h->n_sm : 148);
    if (b > wave) b = wave;
    if (b > h->red.max_blocks) b = h->red.max_blocks;
    if (b < 1) b = 1;
    return (int)b;
}

// sum(a*b) over the volume -> *out (op 1: sqrt)
__global__ void __launch_bounds__(RED_THREADS, 8) k_dot(long long n2, const double2* __restrict__ a,
                                                     const double2* __restrict__ b, RedWork rw, int slot,
                                                     double* out, int op) {
    __shared__ double s_red[RED_THREADS / 32];
    double acc = 0.0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n2; q += (long long)gridDim.x * blockDim.x) {
        double2 x = a[q], y = b[q];
        acc += x.x * y.x;
        acc += x.y * y.y;
    }
    double bt = block_sum(acc, s_red);
    grid_finish(bt, rw, slot, gridDim.x, blockIdx.x, out, op);
}

// L2 eviction-priority policy for data that should stay in L2 across
// kernels (evict-last), and 16-byte loads and stores under it.
__device__ __forceinline__ unsigned long long l2_keep_policy() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ double2 ld_keep(const double2* a, unsigned long long pol) {
    double2 v;
    asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_keep(double2* a, double2 v, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(a), "d"(v.x), "d"(v.y), "l"(pol)
                 : "memory");
}

// One modified Gram-Schmidt pass (:1140-1150):
//   w -= (*hk) * vk          (skipped when vk == nullptr)
//   *out = sum(vn * w)       (vn == nullptr: sum(w*w), op 1 takes the sqrt)
// Two elements per thread per iteration on a grid of MGS_BLOCKS_PER_SM
// blocks per SM.  The basis vectors stream through with evict-first loads;
// w, read and written by every pass of an Arnoldi step (69 MB at
// 512x130x128, inside the 129 MB L2), is loaded and stored evict-last so
// that it stays in L2 from pass to pass.  With everything evict-first a
// pass ran at 1.01 of the measured copy bandwidth in a stand-alone copy
// (0.78 with one element, default caching and 8 blocks per SM).
constexpr int MGS_BLOCKS_PER_SM = 4;
__global__ void __launch_bounds__(RED_THREADS) k_mgs(long long n2, double2* __restrict__ w,
                                                  const double2* __restrict__ vk, const double* __restrict__ hk,
                                                  const double2* __restrict__ vn, RedWork rw, int slot, double* out,
                                                  int op, const int* __restrict__ skip) {
    if (skip && *skip) return;  // an Arnoldi step enqueued ahead of a converged one
    __shared__ double s_red[RED_THREADS / 32];
    const double hv = vk ? *hk : 0.0;
    const unsigned long long keep = l2_keep_policy();
    double acc = 0.0;
    const long long st = (long long)gridDim.x * blockDim.x;
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; q + st < n2; q += 2 * st) {
        double2 x0 = ld_keep(w + q, keep), x1 = ld_keep(w + q + st, keep);
        if (vk) {
            const double2 v0 = __ldcs(vk + q), v1 = __ldcs(vk + q + st);
            x0.x = x0.x - hv * v0.x;
            x0.y = x0.y - hv * v0.y;
            x1.x = x1.x - hv * v1.x;
            x1.y = x1.y - hv * v1.y;
            st_keep(w + q, x0, keep);
            st_keep(w + q + st, x1, keep);
        }
        const double2 y0 = vn ? __ldcs(vn + q) : x0, y1 = vn ? __ldcs(vn + q + st) : x1;
        acc += y0.x * x0.x;
        acc += y0.y * x0.y;
        acc += y1.x * x1.x;
        acc += y1.y * x1.y;
    }
    if (q < n2) {
        double2 x = ld_keep(w + q, keep);
        if (vk) {
            const double2 v = __ldcs(vk + q);
            x.x = x.x - hv * v.x;
            x.y = x.y - hv * v.y;
            st_keep(w + q, x, keep);
        }
        const double2 y = vn ? __ldcs(vn + q) : x;
        acc += y.x * x.x;
        acc += y.y * x.y;
    }
    double bt = block_sum(acc, s_red);
    grid_finish(bt, rw, slot, gridDim.x, blockIdx.x, out, op);
}

// w /= *denom when *denom != 0 (:1158-1161); multiplies by the reciprocal
__global__ void k_scale_inv(long long n2, double2* __restrict__ w, const double* __restrict__ denom,
                            const int* __restrict__ skip) {
    if (skip && *skip) return;
    const double d = *denom;
    if (!(d > 0.0 || d < 0.0)) return;
    const double r = 1.0 / d;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n2; q += (long long)gridDim.x * blockDim.x) {
        double2 x = w[q];
        x.x *= r;
        x.y *= r;
        w[q] = x;
    }
}

// Start of a restart (:958-963, :1048-1056): zero h, c, s, g, y; g(1) = rho;
// sumnor at the first restart; sumav = rho/sumnor.
__global__ void k_restart_init(int K1, double* h, double* gg, double* gc, double* gs, double* gy, DevScalars* sc,
                               int first) {
    for (int q = threadIdx.x; q < K1 * K1; q += blockDim.x) h[q] = 0.0;
    for (int q = threadIdx.x; q < K1; q += blockDim.x) { gg[q] = 0.0; gc[q] = 0.0; gs[q] = 0.0; gy[q] = 0.0; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double rho = sc->rho;
        sc->stop = 0;
        if (first) sc->sumnor = rho;
        sc->sumav = rho / sc->sumnor;
        gg[0] = rho;
    }
}

// Givens rotations for column kit (1-based) (:1165-1189).  h(kit+1,kit) holds
// the norm of the orthogonalised vector; it is saved for the normalisation.
// With skip (Arnoldi steps enqueued ahead): returns at once when a previous
// step stopped the cycle, and stops it itself when the estimate sumav reaches
// stop_at (the host's loop test, evaluated on the same double).
__global__ void k_givens(int K1, int kit, double* h, double* gg, double* gc, double* gs, DevScalars* sc,
                         const int* skip, double stop_at) {
    if (threadIdx.x != 0) return;
    if (skip && *skip) return;
    auto H = [&](int a, int b) -> double& { return h[(a - 1) + K1 * (b - 1)]; };
    sc->red[8] = H(kit + 1, kit);
    if (kit > 1) {
        for (int i = 1; i <= kit - 1; ++i) {
            double hik = gc[i - 1] * H(i, kit) - gs[i - 1] * H(i + 1, kit);
            double hipk = gs[i - 1] * H(i, kit) + gc[i - 1] * H(i + 1, kit);
            H(i, kit) = hik;
            H(i + 1, kit) = hipk;
        }
    }
    double nu = sqrt(H(kit, kit) * H(kit, kit) + H(kit + 1, kit) * H(kit + 1, kit));
    if (nu > 0.0) {
        gc[kit - 1] = H(kit, kit) / nu;
        gs[kit - 1] = -H(kit + 1, kit) / nu;
        H(kit, kit) = gc[kit - 1] * H(kit, kit) - gs[kit - 1] * H(kit + 1, kit);
        H(kit + 1, kit) = 0.0;
        double gk = gc[kit - 1] * gg[kit - 1] - gs[kit - 1] * gg[kit];
        double gkp = gs[kit - 1] * gg[kit - 1] + gc[kit - 1] * gg[kit];
        gg[kit - 1] = gk;
        gg[kit] = gkp;
    }
    double rho = fabs(gg[kit]);
    sc->rho = rho;
    sc->sumav = rho / sc->sumnor;
    if (skip && !(sc->sumav > stop_at)) sc->stop = 1;
}

// y from the triangular h (:1193-1200), one thread
__global__ void k_backsub(int K1, int kit, const double* h, const double* gg, double* gy) {
    if (threadIdx.x != 0) return;
    auto H = [&](int a, int b) -> double { return h[(a - 1) + K1 * (b - 1)]; };
    gy[kit - 1] = gg[kit - 1] / H(kit, kit);
    for (int i = kit - 1; i >= 1; --i) {
        double yi = gg[i - 1];
        for (int k = i + 1; k <= kit; ++k) yi = yi - H(i, k) * gy[k - 1];
        gy[i - 1] = yi / H(i, i);
    }
}

// p' += sum_i v_i y_i, accumulated in the reference's order (:1202-1205)
__global__ void k_update(long long n2, double2* __restrict__ pc, const double2* __restrict__ V, long long vstride2,
                         const double* __restrict__ gy, int kit) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n2; q += (long long)gridDim.x * blockDim.x) {
        double2 x = pc[q];
        for (int i = 0; i < kit; ++i) {
            double2 v = V[(long long)i * vstride2 + q];
            double y = gy[i];
            x.x = x.x + v.x * y;
            x.y = x.y + v.y * y;
        }
        pc[q] = x;
    }
}

// ||L7 p' - Q8||^2 and ||Q8||^2 over the interior -> red[9], red[10]
__global__ void __launch_bounds__(RED_THREADS) k_ppe_resid(Geom g, double aw, double as, const double* __restrict__ Ab,
                                                           const double* __restrict__ At, const double* __restrict__ Ap,
                                                           const double* __restrict__ PC, const double* __restrict__ Q8,
                                                           RedWork rw, DevScalars* sc) {
    __shared__ double s_red[RED_THREADS / 32];
    const int ni = g.nx - 2, J = g.ny - 2, nk = g.nz - 2;
    const long long n = (long long)ni * J * nk;
    double num = 0.0, den = 0.0;
    for (long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; t0 < n; t0 += (long long)gridDim.x * blockDim.x) {
        int i = 1 + (int)(t0 % ni);
        long long r = t0 / ni;
        int j = 1 + (int)(r % J);
        int k = 1 + (int)(r / J);
        long long p = (long long)i + (long long)g.sx * ((long long)j + (long long)g.ny * k);
        int jm = j == 1 ? g.ny - 2 : j - 1, jp = j == g.ny - 2 ? 1 : j + 1;
        long long pjm = (long long)i + (long long)g.sx * ((long long)jm + (long long)g.ny * k);
        long long pjp = (long long)i + (long long)g.sx * ((long long)jp + (long long)g.ny * k);
        double lap = aw * PC[p - 1] + aw * PC[p + 1] + as * PC[pjm] + as * PC[pjp] + Ab[k] * PC[p - g.ps] +
                     At[k] * PC[p + g.ps] + Ap[k] * PC[p];
        double rr = lap - Q8[p];
        num += rr * rr;
        den += Q8[p] * Q8[p];
    }
    double b1 = block_sum(num, s_red);
    __syncthreads();
    double b2 = block_sum(den, s_red);
    grid_finish(b1, rw, 9, gridDim.x, blockIdx.x, &sc->red[9], 0);
    __syncthreads();
    grid_finish(b2, rw, 10, gridDim.x, blockIdx.x, &sc->red[10], 0);
}

// ------------------------------------------------ mixed precision (FP32)
// Inner GMRES vectors are FP32; dot products accumulate in FP64 (the FP32
// products of 4 consecutive elements are summed in FP32, then added in FP64),
// and h, g, c, s, y stay FP64 (k_restart_init / k_givens / k_backsub above).

__device__ __forceinline__ double dot4(float4 a, float4 b) {
    return (double)fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)));
}

__global__ void __launch_bounds__(RED_THREADS, 8) k_dot_f(long long n4, const float4* __restrict__ a,
                                                       const float4* __restrict__ b, RedWork rw, int slot,
                                                       double* out, int op) {
    __shared__ double s_red[RED_THREADS / 32];
    double acc = 0.0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x)
        acc += dot4(a[q], b[q]);
    double bt = block_sum(acc, s_red);
    grid_finish(bt, rw, slot, gridDim.x, blockIdx.x, out, op);
}


__global__ void k_scale_inv_f(long long n4, float4* __restrict__ w, const double* __restrict__ denom,
                              const int* __restrict__ skip) {
    if (skip && *skip) return;
    const double d = *denom;
    if (!(d > 0.0 || d < 0.0)) return;
    const float r = (float)(1.0 / d);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
        float4 x = w[q];
        x.x *= r; x.y *= r; x.z *= r; x.w *= r;
        w[q] = x;
    }
}

// p' (FP64) += sum_i y_i v_i: the FP32 correction of one inner cycle, added in FP64
__global__ void k_update_f(long long n4, double* __restrict__ pc, const float4* __restrict__ V, long long vstride4,
                           const double* __restrict__ gy, int kit) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
        float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
        for (int i = 0; i < kit; ++i) {
            const float4 v = V[(long long)i * vstride4 + q];
            const float y = (float)gy[i];
            c.x = fmaf(y, v.x, c.x); c.y = fmaf(y, v.y, c.y); c.z = fmaf(y, v.z, c.z); c.w = fmaf(y, v.w, c.w);
        }
        double2* p2 = reinterpret_cast<double2*>(pc) + 2 * q;
        double2 x0 = p2[0], x1 = p2[1];
        x0.x += (double)c.x; x0.y += (double)c.y; x1.x += (double)c.z; x1.y += (double)c.w;
        p2[0] = x0;
        p2[1] = x1;
    }
}

// ------------------------------------------------------------- host glue
int launch_dot(tbl_handle* h, const double* a, const double* b, double* out, int op) {
    int nb = red_blocks(h);
    k_dot<<<nb, RED_THREADS, 0, h->stream>>>(h->g.vol / 2, (const double2*)a, (const double2*)b, h->red, 7, out, op);
    h->launches++;
    return TBL_OK;
}

int launch_mgs(tbl_handle* h, double* w, const double* vk, const double* hk, const double* vn, double* out, int op,
               const int* skip) {
    int nb = MGS_BLOCKS_PER_SM * (h->n_sm > 0 ? h->n_sm : 148);
    if (nb > red_blocks(h)) nb = red_blocks(h);
    k_mgs<<<nb, RED_THREADS, 0, h->stream>>>(h->g.vol / 2, (double2*)w, (const double2*)vk, hk, (const double2*)vn,
                                             h->red, 7, out, op, skip);
    h->launches++;
    return TBL_OK;
}

int launch_scale_by_inv(tbl_handle* h, double* w, const double* denom, const int* skip) {
    int nb = red_blocks(h);
    k_scale_inv<<<nb, RED_THREADS, 0, h->stream>>>(h->g.vol / 2, (double2*)w, denom, skip);
    h->launches++;
    return TBL_OK;
}

int launch_restart_init(tbl_handle* h, int first) {
    const int K1 = h->cfg.kmax + 1;
    k_restart_init<<<1, 256, 0, h->stream>>>(K1, h->h, h->gg, h->gc, h->gs, h->gy, h->sc, first);
    h->launches++;
    return TBL_OK;
}

int launch_givens(tbl_handle* h, int kit, const int* skip, double stop_at) {
    const int K1 = h->cfg.kmax + 1;
    k_givens<<<1, 32, 0, h->stream>>>(K1, kit, h->h, h->gg, h->gc, h->gs, h->sc, skip, stop_at);
    h->launches++;
    return TBL_OK;
}

int launch_backsub_update(tbl_handle* h, int kit) {
    const int K1 = h->cfg.kmax + 1;
    k_backsub<<<1, 32, 0, h->stream>>>(K1, kit, h->h, h->gg, h->gy);
    int nb = red_blocks(h);
    k_update<<<nb, RED_THREADS, 0, h->stream>>>(h->g.vol / 2, (double2*)h->PC, (const double2*)h->V, h->g.vol / 2,
                                                h->gy, kit);
    h->launches += 2;
    return TBL_OK;
}

// ------------------------- low-synchronisation Gram-Schmidt (FP32 inner GMRES)
// Modified Gram-Schmidt in its inverse compact-WY form: for a basis
// Q = [v_0 .. v_{n-1}] with L the strictly lower triangle of Q^T Q, the product
// of the n MGS projections is I - Q (I + L)^-1 Q^T (exactly, also when Q has
// lost orthogonality).  One pass forms Q^T w and the new row of L
// (Q^T v_{n-1}); a forward substitution gives the Hessenberg column t; a
// second pass applies w -= Q t and forms ||w||.  2n+3 vector passes per
// Arnoldi step instead of MGS's 4n+1; the FP64 outer refinement of the mixed
// solve makes the different rounding irrelevant to the final accuracy.
constexpr int LSG_G = 8;  // basis vectors per group (grid.y) of the dot pass

__device__ __forceinline__ float dot4f(float4 a, float4 b) {
    return fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)));
}

// Warp sum of 16 FP64 values per lane, as a reduce-scatter: at each of the
// offsets 16, 8, 4, 2 a lane keeps half of its values, sends the other half to
// lane ^ offset and adds what it receives; a last exchange with lane ^ 1
// completes the sums.  Lane l then holds the warp total of value l >> 1: 16
// FP64 additions per lane instead of the 80 of 16 shuffle trees (FP64 runs at
// 1/64 of the FP32 rate on this GPU).  Fixed order: deterministic.
__device__ __forceinline__ double warp_reduce_scatter16(double (&a)[16]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int half = 8; half >= 1; half >>= 1) {
        const bool up = (lane & (2 * half)) != 0;  // keeps the upper half of the current values
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const double keep = up ? a[i + half] : a[i];
            const double send = up ? a[i] : a[i + half];
            a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 2 * half);
        }
    }
    return a[0] + __shfl_xor_sync(0xffffffffu, a[0], 1);
}

// d[i] = <v_i, w>, g[i] = <v_i, v_{nv-1}> for the G basis vectors of group
// blockIdx.y (first vector g0 + G*blockIdx.y).  The products are FP32 (the
// vectors are); each thread sums its share (about 16 float4 loads, 64
// products) in FP32, and from these per-thread partials on every sum is FP64:
// the warp's, the block's and k_lsg_reduce's (each value's block partials,
// fixed order).  An FP64 sum per float4 instead cost the mixed step 14 ms at
// 512 x 130 x 128 (22% of its Gram-Schmidt time).  (Finishing in
// the last block -- a fence, an atomic, then the 2G sums -- cost as much as
// the pass's loads, hence the separate reduction.)
template <int G>
__global__ void __launch_bounds__(RED_THREADS) k_lsg_dots_f(long long n4, const float4* __restrict__ w,
                                                            const float4* __restrict__ V, long long vstride4, int nv,
                                                            int g0, double* __restrict__ partial, int max_blocks,
                                                            const int* __restrict__ skip) {
    static_assert(2 * G <= 16, "the warp reduce-scatter takes 16 values");
    if (skip && *skip) return;
    constexpr int NW = RED_THREADS / 32;
    __shared__ double s_red[16 * NW];
    const int grp = g0 / LSG_G + blockIdx.y;  // slot index of this group
    const int i0 = g0 + blockIdx.y * G;
    const float4* vl = V + (long long)(nv - 1) * vstride4;
    float fd[G], fg[G];
#pragma unroll
    for (int e = 0; e < G; ++e) { fd[e] = 0.f; fg[e] = 0.f; }
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
        const float4 x = w[q], l = vl[q];
#pragma unroll
        for (int e = 0; e < G; ++e) {
            const float4 v = __ldcs(V + (long long)(i0 + e) * vstride4 + q);  // read once: evict first
            fd[e] += dot4f(v, x);
            fg[e] += dot4f(v, l);
        }
    }
    double acc[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[e] = e < 2 * G ? (double)(e % 2 == 0 ? fd[e / 2] : fg[e / 2]) : 0.0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const double tot = warp_reduce_scatter16(acc);  // value lane >> 1
    if ((lane & 1) == 0) s_red[(lane >> 1) * NW + wid] = tot;
    __syncthreads();
    if (threadIdx.x < 2 * G) {
        double a = 0.0;
        for (int k = 0; k < NW; ++k) a += s_red[threadIdx.x * NW + k];
        partial[((size_t)grp * 2 * LSG_G + threadIdx.x) * max_blocks + blockIdx.x] = a;
    }
}

// The 2 nv values of the dot pass: one warp per value sums its nb block
// partials (lanes strided over the blocks, four loads in flight per lane,
// then the shuffle tree); d[i] for even slots, g[i] (i < nv-1) for odd.
__global__ void __launch_bounds__(256) k_lsg_reduce(const double* __restrict__ partial, int max_blocks, int nb,
                                                    int nv, double* __restrict__ dout, double* __restrict__ gout,
                                                    const int* __restrict__ skip) {
    if (skip && *skip) return;
    const int lane = threadIdx.x & 31;
    const int v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);  // value 0 .. 2 nv - 1
    if (v >= 2 * nv) return;
    const int grp = v / (2 * LSG_G), within = v % (2 * LSG_G);
    const double* p = partial + ((size_t)grp * 2 * LSG_G + within) * max_blocks;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int b = lane;
    for (; b + 96 < nb; b += 128) {
        a0 += p[b];
        a1 += p[b + 32];
        a2 += p[b + 64];
        a3 += p[b + 96];
    }
    for (; b < nb; b += 32) a0 += p[b];
    const double acc = warp_sum((a0 + a1) + (a2 + a3));
    if (lane == 0) {
        const int i = grp * LSG_G + within / 2;
        if (within % 2 == 0) dout[i] = acc;
        else if (i < nv - 1) gout[i] = acc;
    }
}

// New row of L (row nv-1: <v_{nv-1}, v_j>, j < nv-1), then (I + L) t = d by
// column-oriented forward substitution in shared memory, one warp (nv <= 64:
// each lane owns rows lane and lane+32).  Rows of older vectors were written
// when each was the newest.
__global__ void __launch_bounds__(32) k_lsg_solve(int K1, int nv, double* __restrict__ Lm,
                                                  const double* __restrict__ d, const double* __restrict__ gnew,
                                                  double* __restrict__ hcol, const int* __restrict__ skip) {
    if (skip && *skip) return;
    __shared__ double sL[64][65];
    __shared__ double st[64];
    const int lane = threadIdx.x, r = nv - 1;
    for (int j = lane; j < r; j += 32) Lm[(size_t)r * K1 + j] = gnew[j];
    __syncwarp();
    for (int i = 0; i < nv; ++i)
        for (int j = lane; j < i; j += 32) sL[i][j] = i == r ? gnew[j] : Lm[(size_t)i * K1 + j];
    for (int i = lane; i < nv; i += 32) st[i] = d[i];
    __syncwarp();
    for (int j = 0; j < nv; ++j) {
        const double tj = st[j];  // final: every earlier column has been applied
        for (int i = j + 1 + lane; i < nv; i += 32) st[i] -= sL[i][j] * tj;
        __syncwarp();
    }
    for (int i = lane; i < nv; i += 32) hcol[i] = st[i];
}

// w -= sum_i t_i v_i (FP32), then ||w|| -> *out (sqrt of the deterministic sum)
__global__ void __launch_bounds__(RED_THREADS, 6) k_lsg_update_f(long long n4, float4* __restrict__ w,
                                                              const float4* __restrict__ V, long long vstride4, int nv,
                                                              const double* __restrict__ t, RedWork rw, int slot,
                                                              double* out, const int* __restrict__ skip) {
    if (skip && *skip) return;
    __shared__ double s_red[RED_THREADS / 32];
    __shared__ float s_t[64];
    for (int i = threadIdx.x; i < nv && i < 64; i += blockDim.x) s_t[i] = (float)t[i];
    __syncthreads();
    double acc = 0.0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
        float4 x = w[q];
#pragma unroll 4
        for (int i = 0; i < nv; ++i) {
            const float4 v = __ldcs(V + (long long)i * vstride4 + q);  // read once: evict first
            const float ti = s_t[i];
            x.x = fmaf(-ti, v.x, x.x);
            x.y = fmaf(-ti, v.y, x.y);
            x.z = fmaf(-ti, v.z, x.z);
            x.w = fmaf(-ti, v.w, x.w);
        }
        w[q] = x;
        acc += (double)dot4f(x, x);
    }
    const double bt = block_sum(acc, s_red);
    grid_finish(bt, rw, slot, gridDim.x, blockIdx.x, out, 1);
}

int launch_lsg_f(tbl_handle* h, float* W, int kit, double* hcol, const int* skip) {
    const int K1 = h->cfg.mixed_kmax + 1;
    if (kit > 64 || kit > K1) return TBL_ERR_BAD_ARG;
    const int nb = red_blocks(h);
    const long long n4 = h->g.vol / 4;
    // dot pass: full groups of 8 vectors, then the remainder group; about 16
    // float4 per thread
    int nbd = (int)((n4 + RED_THREADS * 16 - 1) / (RED_THREADS * 16));
    if (nbd < 1) nbd = 1;
    if (nbd > nb) nbd = nb;
    const int nfull = kit / LSG_G, rem = kit % LSG_G;
    const float4* Wc = (const float4*)W;
    const float4* Vc = (const float4*)h->Vf;
    if (nfull > 0)
        k_lsg_dots_f<LSG_G><<<dim3(nbd, nfull), RED_THREADS, 0, h->stream>>>(n4, Wc, Vc, n4, kit, 0,
                                                                             h->lsg_partial, h->red.max_blocks, skip);
    if (rem > 0) {
        const int g0 = nfull * LSG_G;
        switch (rem) {
#define TBL_LSG_REM(R)                                                                                              \
    case R:                                                                                                         \
        k_lsg_dots_f<R><<<dim3(nbd, 1), RED_THREADS, 0, h->stream>>>(n4, Wc, Vc, n4, kit, g0, h->lsg_partial,       \
                                                                    h->red.max_blocks, skip);                      \
        break;
            TBL_LSG_REM(1) TBL_LSG_REM(2) TBL_LSG_REM(3) TBL_LSG_REM(4) TBL_LSG_REM(5) TBL_LSG_REM(6)
            TBL_LSG_REM(7)
#undef TBL_LSG_REM
        }
    }
    k_lsg_reduce<<<(2 * kit + 7) / 8, 256, 0, h->stream>>>(h->lsg_partial, h->red.max_blocks, nbd, kit, h->lsg_d,
                                                            h->lsg_g, skip);
    k_lsg_solve<<<1, 32, 0, h->stream>>>(K1, kit, h->lsg_L, h->lsg_d, h->lsg_g, hcol, skip);  // kit <= 63
    int nbu = 6 * (h->n_sm > 0 ? h->n_sm : 148);  // one resident wave at 6 blocks per SM
    if (nbu > nb) nbu = nb;
    k_lsg_update_f<<<nbu, RED_THREADS, 0, h->stream>>>(n4, (float4*)W, (const float4*)h->Vf, n4, kit, hcol, h->red, 7,
                                                      &hcol[kit], skip);
    h->launches += 3 + (nfull > 0) + (rem > 0);
    return TBL_OK;
}

int launch_dot_f(tbl_handle* h, const float* a, const float* b, double* out, int op) {
    int nb = red_blocks(h);
    k_dot_f<<<nb, RED_THREADS, 0, h->stream>>>(h->g.vol / 4, (const float4*)a, (const float4*)b, h->red, 7, out, op);
    h->launches++;
    return TBL_OK;
}

int launch_scale_by_inv_f(tbl_handle* h, float* w, const double* denom, const int* skip) {
    int nb = red_blocks(h);
    k_scale_inv_f<<<nb, RED_THREADS, 0, h->stream>>>(h->g.vol / 4, (float4*)w, denom, skip);
    h->launches++;
    return TBL_OK;
}

int launch_backsub_update_f(tbl_handle* h, int kit) {
    const int K1 = h->cfg.mixed_kmax + 1;
    k_backsub<<<1, 32, 0, h->stream>>>(K1, kit, h->h, h->gg, h->gy);
    int nb = red_blocks(h);
    k_update_f<<<nb, RED_THREADS, 0, h->stream>>>(h->g.vol / 4, h->PC, (const float4*)h->Vf, h->g.vol / 4, h->gy,
                                                  kit);
    h->launches += 2;
    return TBL_OK;
}

int launch_restart_init_k(tbl_handle* h, int first, int K1) {
    k_restart_init<<<1, 256, 0, h->stream>>>(K1, h->h, h->gg, h->gc, h->gs, h->gy, h->sc, first);
    h->launches++;
    return TBL_OK;
}

int launch_givens_k(tbl_handle* h, int kit, int K1, const int* skip, double stop_at) {
    k_givens<<<1, 32, 0, h->stream>>>(K1, kit, h->h, h->gg, h->gc, h->gs, h->sc, skip, stop_at);
    h->launches++;
    return TBL_OK;
}

int launch_ppe_resid(tbl_handle* h) {
    int nb = red_blocks(h);
    k_ppe_resid<<<nb, RED_THREADS, 0, h->stream>>>(h->g, 1.0 / (h->cfg.dx * h->cfg.dx), 1.0 / (h->cfg.dy * h->cfg.dy),
                                                   h->Ab, h->At, h->Ap, h->PC, h->Q8, h->red, h->sc);
    h->launches++;
    return TBL_OK;
}

}  // namespace tbl
