// tbl_lap.cu -- the Arnoldi matvec R = s(k) * L7 X of the preconditioned
// GMRES (dnstbl2/dnstbl.f90:1086-1101; the forward SSOR sweep's -w/Ap(k)
// scale folded in), with TMA halo tiles along the wall-normal direction.
//
// A CTA owns a tile of 128 streamwise points x 8 span rows and marches up a
// range of wall-normal planes.  Each plane of the tile, with its halo (one
// point either side in i, the span rows j-1 and j+1 with the periodic wrap),
// arrives in shared memory by three `cp.async.bulk.tensor` loads (the tile's
// rows, and each halo row as its own one-row box, so that the wrap rows
// need no special case); a four-stage plane ring, one mbarrier per stage,
// keeps planes k-1, k, k+1 resident while plane k+2 is in flight.  Every input
// value comes from HBM once per tile (halo rows and the two extra planes of a
// range come from L2 mostly), and the result is written with coalesced
// stores.  The point arithmetic is k_lap's, term for term, so the results
// are bit-identical to it.  Measured at 512 x 130 x 128 (ncu): 32-33 us per
// launch, DRAM reads 34.2 MB (the input once) and the result left in L2 --
// the same time as k_lap's one thread per point; the march is latency-bound
// (16-row tiles with an eight-stage ring at 2 CTAs per SM took 37 us).
//
// In the mixed solver's Arnoldi loop the kernel also finishes the previous
// step: its input is that step's vector before the division by H(k+1,k),
// which the kernel applies to each plane tile as it lands, writing the
// normalised basis vector as it goes (one pass and one launch fewer per
// Arnoldi step than a separate scaling pass; results bit-identical).
//
// Waits are bounded: thread 0 polls the stage's mbarrier at most LT_SPIN
// times, then sets TBL_ERR_TIMEOUT in the error word, waits (bounded again)
// for the CTA's other loads in flight and the CTA returns.
#include <cuda.h>

#include "tbl_internal.cuh"
#include "tbl_kernels.cuh"

namespace tbl {

namespace {

constexpr int LT_I = 128;       // interior points per tile along i
constexpr int LT_J = 8;         // span rows per tile
constexpr int LT_NS = 4;        // plane stages (planes k-1 .. k+2 resident or in flight)
constexpr int LT_THREADS = 256;
constexpr long long LT_SPIN = 1LL << 24;

// Row width of a plane tile in elements: i from 128 bx (the point before the
// tile's first) to 128 bx + 129, rounded up to a 16-byte multiple (a TMA box's
// inner extent), and the byte offsets of the three pieces of a stage, each
// 128-byte aligned.
template <typename T> constexpr int lt_bx() { return sizeof(T) == 4 ? 132 : 130; }
template <typename T> constexpr int lt_row_bytes() { return ((lt_bx<T>() * (int)sizeof(T)) + 127) / 128 * 128; }
template <typename T> constexpr int lt_main_bytes() { return ((lt_bx<T>() * LT_J * (int)sizeof(T)) + 127) / 128 * 128; }
template <typename T> constexpr int lt_stage_bytes() { return 2 * lt_row_bytes<T>() + lt_main_bytes<T>(); }
// Bytes one stage receives: the three boxes (out-of-range elements count too).
template <typename T> constexpr unsigned lt_tx_bytes() { return (unsigned)(lt_bx<T>() * (LT_J + 2) * sizeof(T)); }

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void lt_mb_init(uint64_t* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void lt_expect(uint64_t* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool lt_try_wait(uint64_t* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool lt_wait(uint64_t* b, unsigned parity) {
    for (long long s = 0; s < LT_SPIN; ++s)
        if (lt_try_wait(b, parity)) return true;
    return false;
}
// One box of the 3-D tensor (x = i, y = j, z = k) into shared memory.
__device__ __forceinline__ void lt_load(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <typename T>
__global__ void __launch_bounds__(LT_THREADS) k_lap_tma(const __grid_constant__ CUtensorMap map_rows,
                                                        const __grid_constant__ CUtensorMap map_row, Geom g, T aw,
                                                        T as, const T* __restrict__ Ab, const T* __restrict__ At,
                                                        const T* __restrict__ Ap, const T* __restrict__ scale,
                                                        T* __restrict__ R, int kc, const int* __restrict__ skip,
                                                        int* err, const double* __restrict__ denom,
                                                        T* __restrict__ vout) {
    if (skip && *skip) return;  // an Arnoldi step enqueued ahead of a converged one
    constexpr int BX = lt_bx<T>(), RB = lt_row_bytes<T>(), MB = lt_main_bytes<T>(), SB = lt_stage_bytes<T>();
    extern __shared__ __align__(128) unsigned char lt_smem[];
    __shared__ __align__(8) uint64_t full[LT_NS];
    __shared__ int s_abort;
    const int tid = threadIdx.x;
    const int ib = LT_I * blockIdx.x;                  // element 0 of a tile row is i = ib
    const int j0 = 1 + LT_J * blockIdx.y;              // first span row of the tile
    const int nr = min(LT_J, g.ny - 2 - (j0 - 1));     // rows of the tile (the last tile may be short)
    const int k_lo = 1 + kc * blockIdx.z, k_hi = min(g.nz - 2, k_lo + kc - 1);
    if (k_lo > k_hi) return;
    const int jm = j0 == 1 ? g.ny - 2 : j0 - 1;               // halo row before the tile (periodic)
    const int jl = j0 + nr - 1;
    const int jp = jl == g.ny - 2 ? 1 : jl + 1;               // halo row after the tile (periodic)
    auto stage = [&](int s) { return lt_smem + (size_t)s * SB; };
    // row r of a stage: 0 = the row before, 1..LT_J = the tile's rows, LT_J+1 = the row after
    auto row = [&](int s, int r) -> const T* {
        unsigned char* b = stage(s);
        if (r == 0) return reinterpret_cast<const T*>(b);
        if (r == LT_J + 1) return reinterpret_cast<const T*>(b + RB + MB);
        return reinterpret_cast<const T*>(b + RB) + (size_t)(r - 1) * BX;
    };
    auto issue = [&](int kk) {  // thread 0: plane kk into stage kk % LT_NS
        const int s = kk & (LT_NS - 1);
        unsigned char* b = stage(s);
        lt_expect(&full[s], lt_tx_bytes<T>());
        lt_load(b, &map_row, ib, jm, kk, &full[s]);
        lt_load(b + RB, &map_rows, ib, j0, kk, &full[s]);
        lt_load(b + RB + MB, &map_row, ib, jp, kk, &full[s]);
    };
    auto parity = [&](int kk) { return (unsigned)(((kk - (k_lo - 1)) / LT_NS) & 1); };
    // Normalisation folded in (denom non-null): the input is the Arnoldi
    // vector before its division by H(k+1,k) = *denom; every value of a
    // stage is multiplied by the same reciprocal the separate pass used,
    // (T)(1 / d) (none when d is 0), before the stencil reads it, and the
    // tile's own points of the result go to vout, the basis slot.
    T rs = T(1);
    if (denom) {
        const double d = *denom;
        if (d > 0.0 || d < 0.0) rs = (T)(1.0 / d);
    }
    auto scale_stage = [&](int s) {  // all threads: the three pieces of a stage
        unsigned char* b = stage(s);
        T* r0 = reinterpret_cast<T*>(b);
        T* rm = reinterpret_cast<T*>(b + RB);
        T* r1 = reinterpret_cast<T*>(b + RB + MB);
        for (int e = tid; e < BX; e += LT_THREADS) {
            r0[e] = r0[e] * rs;
            r1[e] = r1[e] * rs;
        }
        for (int e = tid; e < BX * LT_J; e += LT_THREADS) rm[e] = rm[e] * rs;
        // the stage is refilled by TMA later: order these generic writes before it
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    };
    if (tid == 0) {
        for (int s = 0; s < LT_NS; ++s) lt_mb_init(&full[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    __syncthreads();
    const int kpre = min(k_lo + LT_NS - 2, k_hi + 1);
    if (tid == 0)
        for (int kk = k_lo - 1; kk <= kpre; ++kk) issue(kk);
    int issued = kpre;  // last plane issued (thread 0's view)
    const int il = tid % LT_I;  // point i = ib + 1 + il, element il + 1 of a row
    const int i = ib + 1 + il;
    const bool i_ok = i <= g.nx - 2;
    for (int k = k_lo; k <= k_hi; ++k) {
        if (tid == 0) {
            bool ok = true;
            if (k == k_lo) ok = lt_wait(&full[(k - 1) & (LT_NS - 1)], parity(k - 1)) &&
                                lt_wait(&full[k & (LT_NS - 1)], parity(k));
            ok = ok && lt_wait(&full[(k + 1) & (LT_NS - 1)], parity(k + 1));
            if (!ok) s_abort = 1;
        }
        __syncthreads();
        if (s_abort) break;
        const int sp = (k - 1) & (LT_NS - 1), sc = k & (LT_NS - 1), sn = (k + 1) & (LT_NS - 1);
        if (denom) {  // planes k-1 and k were scaled as the next plane of earlier iterations
            if (k == k_lo) {
                scale_stage(sp);
                scale_stage(sc);
            }
            scale_stage(sn);
            __syncthreads();
        }
        const T ab = Ab[k], at = At[k], ap = Ap[k], sk = scale ? scale[k] : T(1);
        for (int r = 1 + tid / LT_I; r <= nr; r += LT_THREADS / LT_I) {
            if (!i_ok) continue;
            const T* c = row(sc, r);
            const int rjm = r - 1, rjp = r == nr ? LT_J + 1 : r + 1;
            const T xjm = row(sc, rjm)[il + 1];
            const T xjp = row(sc, rjp)[il + 1];
            // k_lap's arithmetic, term for term
            const T lap = aw * c[il] + aw * c[il + 2] + as * xjm + as * xjp + ab * row(sp, r)[il + 1] +
                          at * row(sn, r)[il + 1] + ap * c[il + 1];
            const long long p = (long long)i + (long long)g.sx * ((long long)(j0 + r - 1) + (long long)g.ny * k);
            R[p] = scale ? sk * lap : lap;
            if (denom) vout[p] = c[il + 1];
        }
        __syncthreads();  // stage sp is no longer read
        if (tid == 0 && k + LT_NS - 1 <= k_hi + 1) {  // into the stage plane k-1 used
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(k + LT_NS - 1);
            issued = k + LT_NS - 1;
        }
    }
    if (tid == 0 && s_abort) {
        atomicExch(err, TBL_ERR_TIMEOUT);
        // bounded waits for this CTA's loads still in flight before its shared memory is released
        for (int kk = k_lo - 1; kk <= issued; ++kk) lt_wait(&full[kk & (LT_NS - 1)], parity(kk));
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// The field X (padded layout, sx x ny x nz) as a 3-D tensor with a box of
// `rows` span rows of one plane.
template <typename T>
bool encode(CUtensorMap* m, const T* X, const Geom& g, int rows) {
    EncodeTiled fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.sx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.sx * sizeof(T), (cuuint64_t)g.ps * sizeof(T)};
    const cuuint32_t box[3] = {(cuuint32_t)lt_bx<T>(), (cuuint32_t)rows, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return fn(m, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
              const_cast<T*>(X), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// R = scale(k) * L7 X on the interior, in one wave of CTAs.  Used for the
// FP32 matvec of the mixed solver's inner GMRES; the FP64 matvec keeps
// k_lap (one thread per point), which is bound by the FP64 issue rate and
// stays balanced over the SMs: this kernel, at 2-3 CTAs per SM in FP64, was
// 7.6 ms a step slower there.  Returns TBL_ERR_CUDA when a tensor map cannot
// be made.
template <typename T>
int launch_lap_tma(tbl_handle* h, const T* X, T* R, T aw, T as, const T* Ab, const T* At, const T* Ap,
                   const T* scale, const int* skip, const double* denom, T* vout) {
    if ((denom == nullptr) != (vout == nullptr) || (vout && (const T*)vout == X)) return TBL_ERR_BAD_ARG;
    const Geom& g = h->g;
    CUtensorMap rows, row;
    if (!encode<T>(&rows, X, g, LT_J) || !encode<T>(&row, X, g, 1)) {
        set_last_cuda_error(cudaErrorInvalidValue, "cuTensorMapEncodeTiled", __FILE__, __LINE__);
        return TBL_ERR_CUDA;
    }
    const int gx = (g.nx - 2 + LT_I - 1) / LT_I, gy = (g.ny - 2 + LT_J - 1) / LT_J;
    const int planes = g.nz - 2;
    const size_t smem = (size_t)LT_NS * lt_stage_bytes<T>();
    static int per_sm[2] = {0, 0};
    if (per_sm[sizeof(T) == 8] == 0) {
        TBL_CUDA_TRY(cudaFuncSetAttribute((const void*)k_lap_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        int n = 0;
        TBL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lap_tma<T>, LT_THREADS, smem));
        per_sm[sizeof(T) == 8] = n > 0 ? n : 1;
    }
    // one resident wave: as many plane ranges per tile as fill the SMs'
    // slots (a second, partial wave would leave most SMs idle at its end)
    const int slots = per_sm[sizeof(T) == 8] * (h->n_sm > 0 ? h->n_sm : 148);
    int nkc = slots / (gx * gy);
    if (nkc > planes) nkc = planes;
    if (nkc < 1) nkc = 1;
    const int kc = (planes + nkc - 1) / nkc;
    nkc = (planes + kc - 1) / kc;
    k_lap_tma<T><<<dim3(gx, gy, nkc), LT_THREADS, smem, h->stream>>>(rows, row, g, aw, as, Ab, At, Ap, scale, R, kc,
                                                                     skip, h->err, denom, vout);
    TBL_CUDA_TRY(cudaGetLastError());
    h->launches++;
    return TBL_OK;
}

template int launch_lap_tma<float>(tbl_handle*, const float*, float*, float, float, const float*, const float*,
                                   const float*, const float*, const int*, const double*, float*);

}  // namespace tbl
