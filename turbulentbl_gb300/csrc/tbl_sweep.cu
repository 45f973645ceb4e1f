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
//   * every (j,k) line of a slab is owned by one lane; a lane updates
//     CH consecutive points of its line per step (4 in FP64, 8 in FP32);
//   * a warp holds 32 consecutive rows of one plane, a CTA holds KG planes;
//     point i of row j is updated one position after point i of row j-1 (the
//     value comes from the neighbouring lane by shuffle, within the step or
//     from the step before) and one step after point i of plane k-1 (through
//     shared memory), so a sweep takes about nx/4 + K + 9 (ny-2)/32 steps
//     instead of the nx/4 + K + (ny-2) of a chunk-per-row lag;
//   * every warp waits only for the warps producing its inputs: the warp of
//     the row block above (global progress flag, acquire/release) and the
//     warp of the plane below (shared-memory progress inside the CTA; across
//     CTAs, a ring in distributed shared memory when the CTAs of a slab
//     column form a thread-block cluster, else a global flag); waits are
//     bounded spins, a timeout sets an error word and the warp returns;
//   * slabs are independent (block-Jacobi GS halos come from a snapshot of the
//     previous sweep, SSOR halos are zero), so all slabs and, for GS, all three
//     velocity components run concurrently in one launch whose CTAs are all
//     resident (clusters of a slab column's CTAs, or a cooperative launch).
//
// The backward SSOR sweep is the same schedule on mirrored indices.
#include <cooperative_groups.h>
#include <algorithm>
#include <type_traits>

#include "tbl_internal.cuh"
#include "tbl_kernels.cuh"

namespace tbl {

enum SweepMode { SW_GS = 0, SW_FWD = 1, SW_BWD = 2 };

template <typename T>
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
    T* F[3];
    const T* Q[3];
    const T* PRE[3];            // per-point terms of old values (k_gs_pre)
    int comp[3];
    const T* halo_in;           // [comp][side][slab] planes
    T* halo_out;
    // SSOR
    double omega, sw;           // w, (2-w)/w
    int jb_rows;                // SSOR: rows per span block (a multiple of 32; 0 = one block per slab)
    int nib;                    // SSOR: streamwise blocks (grid.y), 1 = one block per line
    int plag;                   // positions a row lags the row above: 1, or CH (see base_args)
    const T* X;                 // matvec input (FWD) / PCorr (FWD residual mode)
    const double* Q8;           // residual mode when non-null
    T* RH;                      // FWD input r, overwritten with the (unscaled) forward result; BWD input
    T* OUT;                     // BWD output
    const int* skip;            // non-null in Arnoldi steps enqueued ahead: return at once when set
    int xk;                     // plane-CTA hand-off through distributed shared memory (CTAs of a slab
                                // column form one cluster along k), 0 = global flags
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

constexpr int RING = 4;  // plane-to-plane exchange slots per warp (shared memory)
constexpr int XR_SLOTS = 8;  // slots of the ring a CTA receives its plane-below values in (cluster hand-off)
// Points per lane per step: 4 in FP64 (one 32-byte sector), 8 in FP32.  An
// FP64 step is bound by its chain of dependent FP64 FMAs (GB300 issues FP64
// at 1/64 of the FP32 rate), an FP32 step by its fixed synchronisation cost,
// which 8 points amortise over twice the work (measured at 512 x 130 x 128:
// FP32 sweeps 185 -> 159 ms a step; 8-point FP64 sweeps and 16-point FP32
// sweeps were slower).  Each lane's operand buffer holds 4 CH positions:
// position q of the line at element q % (4 CH); chunks are copied two steps
// ahead, so the live positions span 3 CH - 1 < 4 CH.
template <typename Val> constexpr int sweep_ch() { return sizeof(Val) == 4 ? 8 : 4; }
// Dynamic shared memory of a sweep CTA: the plane-to-plane ring and the operand buffers.
template <typename Val> constexpr size_t sweep_smem() {
    return sizeof(Val) * KG * (RING * 32 * sweep_ch<Val>() + 32 * 4 * sweep_ch<Val>()) +
           sizeof(Val) * XR_SLOTS * 32 * sweep_ch<Val>();
}

// 16-byte asynchronous global -> shared copy (cp.async, L2 only), its group
// commit and the wait for all but the most recent N groups.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
constexpr int PUB = 4;   // global progress is published every PUB steps (and at the end)

// ---- plane hand-off across the CTAs of a cluster (distributed shared memory)
// The CTAs of a slab column (same slab and row block, plane groups
// kg = 0..nkc-1) form one thread-block cluster.  The last warp of a CTA
// pushes each step's CH values per lane into a ring of XR slots in the
// shared memory of the CTA above with st.async, whose bytes complete a
// transaction on that slot's "full" mbarrier there; the consumer (warp 0 of
// that CTA) waits for the slot's phase, reads it, re-arms it and frees it
// with a remote arrive on the producer's "empty" mbarrier.  No fence and no
// global flag: the mbarrier phases order the data (the pattern of a TMA
// pipeline: default CTA-scope semantics on the wait and the remote arrive;
// cluster-scope release on the arrive measured 10-12% slower sweeps, as it
// waits for the warp's earlier global stores).  Lifetimes: every remote
// access targets a warp that waits for it (the consumer waits for every
// step it is sent, the producer for every slot release it is sent), and two
// end words keep a warp alive while its partner may still reach its shared
// memory after a timeout: the producer reports its end (1) or abort (2) to
// the consumer, and after an abort waits for the consumer's acknowledgement.
constexpr int XR = XR_SLOTS;
constexpr long long XLINGER = 1LL << 27;  // bounded wait for the partner at the end

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned mapa_rank(unsigned addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive_remote(unsigned raddr) {
    asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(raddr) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the completion of the phase of the given parity.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity) {
    long long spins = 0;
    while (!mbar_try_wait(b, parity)) {
        if (++spins > SPIN_LIMIT) return false;
    }
    return true;
}
// One lane's CH values of a step into the consumer's ring slot.
template <int CH>
__device__ __forceinline__ void xpush(unsigned rd, unsigned rb, const double (&v)[CH]) {
#pragma unroll
    for (int b = 0; b < CH / 2; ++b)
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];" ::"r"(
                         rd + 16u * b),
                     "d"(v[2 * b]), "d"(v[2 * b + 1]), "r"(rb)
                     : "memory");
}
template <int CH>
__device__ __forceinline__ void xpush(unsigned rd, unsigned rb, const float (&v)[CH]) {
#pragma unroll
    for (int b = 0; b < CH / 4; ++b)
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                         rd + 16u * b),
                     "f"(v[4 * b]), "f"(v[4 * b + 1]), "f"(v[4 * b + 2]), "f"(v[4 * b + 3]), "r"(rb)
                     : "memory");
}
__device__ __forceinline__ void st_remote_s32(unsigned raddr, int v) {
    asm volatile("st.relaxed.cluster.shared::cluster.s32 [%0], %1;" ::"r"(raddr), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_cluster(const int* p) {
    int v;
    asm volatile("ld.relaxed.cluster.shared::cta.s32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}
// Bounded wait until a word of this CTA (written by the partner CTA) is non-zero.
__device__ __forceinline__ int wait_word(const int* p) {
    for (long long spins = 0; spins < XLINGER; ++spins) {
        const int v = ld_relaxed_cluster(p);
        if (v) return v;
        if (spins > 64) __nanosleep(64);
    }
    return 0;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ int ld_acquire_cta(const int* p) {
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"((unsigned)__cvta_generic_to_shared(p)) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cta(int* p, int v) {
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "r"(v) : "memory");
}

// Wait until the shared progress word reaches target (false on timeout).
__device__ __forceinline__ bool wait_cta(const int* p, int target) {
    long long spins = 0;
    while (ld_acquire_cta(p) < target) {
        if (++spins > SPIN_LIMIT) return false;
        if (spins > 1024) __nanosleep(32);
    }
    return true;
}

// Every warp is an independent unit of the dataflow: it waits only for the
// warps that produce its (j-1) and (k-1) inputs and publishes its own
// progress (shared memory every step for the next plane in the CTA, a global
// flag every PUB steps for the CTAs downstream, or, in a cluster, each step's
// values pushed into the next CTA's ring).  No CTA-wide barrier.
//
// Per step a lane updates CH points of its line.  The point update is
// reassociated so that only one FMA depends on the previous point:
//   GS : x = rd*Q - rd*cE*U(i+1) - rd*cN*U(j+1) - rd*cT*U(k+1)       (k_gs_pre)
//            - rd*cS*x(j-1) - rd*cB*x(k-1)                            (after wait)
//            - rd*cW*x(i-1)                                           (chain)
//   FWD: x = w'*r + w'*As*x(j-1) + w'*Ab*x(k-1) + w'*Aw*x(i-1),   w' = -w/Ap
//   BWD: y = w'*s*rhat + w'*As*y(j+1) + w'*At*y(k+1) + w'*Aw*y(i+1)
// which changes only the rounding of the reference's left-to-right sums.
// Operands of step T that do not depend on other lines arrive in shared
// memory two steps ahead (cp.async) and are read before the warp waits for
// its producers; the (k-1) values of the plane below come through a shared
// memory ring (RING steps deep, with back-pressure; XR steps deep and filled
// by st.async from the CTA below for warp 0 of a cluster's upper CTAs), the
// (j-1) values of the row above by shuffle within the step or, for lane 0,
// from global memory.
// Both precisions keep 4 CTAs per SM (at most 128 registers; 40 KB of shared
// memory in FP64 and 24 KB in FP32), so that the Gauss-Seidel sweeps of the
// three velocity components stay co-resident at 512 x 130 x 128.
template <int MODE, typename Val>
__global__ void __launch_bounds__(KG * 32, 4) k_sweep(SweepArgs<Val> a) {
    if (a.skip && *a.skip) return;  // every CTA reads the same word, written by an earlier launch
    constexpr int CH = sweep_ch<Val>();
    constexpr int OPB = 4 * CH;
    constexpr int LG = CH == 8 ? 3 : 2;  // log2(CH)
    static_assert(CH == (1 << LG), "positions map to chunks by shifts");
    const Geom& g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const SweepCta cta = a.ctas[blockIdx.x];
    const SlabDesc sl = a.slabs[cta.slab];
    const int J = g.ny - 2, K = sl.K;
    const int C = (g.nx - 2) / CH + 1;     // chunks per line
    const int compi = blockIdx.y;
    // SSOR with streamwise blocks: grid.y picks the block of chunks
    // [c_lo, c_hi] this CTA sweeps (zero halo at its start, as across slabs);
    // each block has its own progress flags (the per-component flag sets)
    const int nib = MODE != SW_GS ? a.nib : 1;
    const int CB = (C + nib - 1) / nib;
    const int c_lo = MODE != SW_GS ? (int)blockIdx.y * CB : 0;
    const int c_hi = min(C, c_lo + CB) - 1;
    const int Cl = c_hi - c_lo + 1;        // chunks of this block
    const int comp = MODE == SW_GS ? a.comp[compi] : 0;
    unsigned long long* flags = a.flags + (size_t)compi * a.n_cta * KG;
    __shared__ int s_prog[KG];
    extern __shared__ __align__(16) unsigned char s_dyn[];
    Val (*s_ring)[RING][32][CH] = reinterpret_cast<Val (*)[RING][32][CH]>(s_dyn);
    Val (*s_op)[32][OPB] = reinterpret_cast<Val (*)[32][OPB]>(s_dyn + sizeof(Val) * KG * RING * 32 * CH);
    Val (*s_xring)[32][CH] =
        reinterpret_cast<Val (*)[32][CH]>(s_dyn + sizeof(Val) * KG * (RING * 32 * CH + 32 * OPB));
    __shared__ __align__(8) unsigned long long s_full[XR], s_empty[XR];
    __shared__ int s_xend, s_xack;  // written by the partner CTA: producer finished (1) / aborted (2); abort seen
    constexpr unsigned XBYTES = 32 * CH * sizeof(Val);  // one step of a warp
    if (lane == 0) s_prog[wid] = -1;
    const bool xk = a.xk > 1;
    if (xk && threadIdx.x == 0) {
        for (int q = 0; q < XR; ++q) {
            mbar_init(&s_full[q], 1);
            mbar_init(&s_empty[q], 1);
        }
        s_xend = 0;
        s_xack = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // the consumer arms every slot for its first phase before any producer
    // can write (a transaction may also complete before it is armed)
    if (xk && threadIdx.x == 0 && cta.up_k >= 0)
        for (int q = 0; q < XR; ++q) mbar_arrive_expect_tx(&s_full[q], XBYTES);
    if (xk) cluster_sync_all();  // barriers initialised in every CTA of the cluster
    const unsigned xrank = xk ? cluster_rank() : 0u;

    const int jl = 32 * cta.jb + lane;  // logical row
    // SSOR with span blocks: rows restart the schedule at every block of
    // jb_rows rows (the row before a block reads zero, as across slabs)
    const int jblk0 = (MODE != SW_GS && a.jb_rows > 0) ? (32 * cta.jb / a.jb_rows) * a.jb_rows : 0;
    const int jr = jl - jblk0;          // row within its span block
    const int bj = (32 * cta.jb - jblk0) >> 5;  // 32-row block of this warp within the span block
    const int kl = KG * cta.kg + wid;   // logical plane
    if (kl >= K) return;                // no lines: nobody waits for this warp
    const bool line_ok = jl < J;
    const int jidx = MODE == SW_BWD ? J - 1 - jl : jl;
    const int kidx = MODE == SW_BWD ? K - 1 - kl : kl;
    const int j = 1 + max(0, min(jidx, J - 1)), k = sl.bn + kidx;
    const int jm = (j == 1) ? g.ny - 2 : j - 1;
    const int jp = (j == g.ny - 2) ? 1 : j + 1;
    const long long line = (long long)g.sx * ((long long)j + (long long)g.ny * k);
    const long long sy = g.sx;

    // Schedule.  The block's positions along a line are q = 0 .. Q-1 in sweep
    // order (i = CH*c_lo + q, or CH*c_hi + CH-1 - q backwards).  Lane l of
    // this warp updates positions q = CH*(T - T0) - plag*l + e, e = 0..CH-1,
    // at step T: a row lags the row above by plag positions (its (j-1) input
    // at the same q is the neighbour lane's point e - plag of this step, or of
    // the step before), the plane above lags by one step (its (k-1) input is
    // the same lane's point e of the plane below one step earlier), and a
    // 32-row block lags the block above by blag steps, the least that puts
    // its row-above inputs in the block above's completed steps.
    const int plag = a.plag;
    const int blag = (31 * plag + 2 * CH - 1) / CH;
    const int lane_last = min(32 * cta.jb + 31, J - 1) - 32 * cta.jb;  // last row of the warp
    const int Q = CH * Cl;
    const int T0 = kl + blag * bj;                              // lane 0's first step
    const int T1 = T0 + (Q - 1 + plag * lane_last) / CH;        // the last row's last step
    const int tend_k = T1 - 1;          // last step of the (k-1) upstream warp
    const int dl = plag * lane;         // this lane's lag in positions
    const bool has_down = wid < KG - 1 && kl + 1 < K;
    const unsigned long long* fj =
        (cta.up_j >= 0 && 32 * cta.jb != jblk0) ? &flags[(size_t)cta.up_j * KG + wid] : nullptr;
    const unsigned long long* fk =
        (wid == 0 && cta.up_k >= 0 && !xk) ? &flags[(size_t)cta.up_k * KG + KG - 1] : nullptr;
    const bool xprod = xk && wid == KG - 1 && cta.dn_k;  // pushes its plane to the CTA above in the cluster
    const bool xcons = xk && wid == 0 && cta.up_k >= 0;   // receives the plane below from the CTA below
    unsigned long long* fme = &flags[(size_t)blockIdx.x * KG + wid];
    // the device-scope progress flag (a fence of ~1100 cycles every PUB
    // steps) is published only by warps that another CTA waits for: the
    // block below in j (unless span blocks restart there) and, for the last
    // warp, the CTA above in k
    const bool j_reader = cta.dn_j && !(MODE != SW_GS && a.jb_rows > 0 && (32 * (cta.jb + 1)) % a.jb_rows == 0);
    const bool publish = j_reader || (wid == KG - 1 && cta.dn_k && !xk);
    const unsigned long long tag = a.epoch << 20;
    // physical i of position q
    const int ibase = MODE == SW_BWD ? CH * c_hi + CH - 1 : CH * c_lo;
    const int idir = MODE == SW_BWD ? -1 : 1;

    // coefficients of this plane, pre-scaled for the reassociated update (FP64)
    double c0 = 0, c1 = 0, c2 = 0, c3 = 0, cjd = 0, ckd = 0, cid = 0;
    if (MODE == SW_GS) {
        const double rd = 1.0 / (1.0 + (a.t * a.Ap[k]));
        c0 = rd;                       // * Q
        c1 = -(a.t * a.aw) * rd;       // * U(i+1)
        c2 = -(a.t * a.as) * rd;       // * U(j+1)
        c3 = -(a.t * a.At[k]) * rd;    // * U(k+1)
        cjd = -(a.t * a.as) * rd;      // * x(j-1)
        ckd = -(a.t * a.Ab[k]) * rd;   // * x(k-1)
        cid = -(a.t * a.aw) * rd;      // * x(i-1)
    } else {
        const double wr = -a.omega * a.rAp[k];  // -w * rAnp
        c0 = MODE == SW_FWD ? wr : wr * (a.sw * a.Ap[k]);
        cjd = wr * a.as;
        ckd = wr * (MODE == SW_FWD ? a.Ab[k] : a.At[k]);
        cid = wr * a.aw;
    }
    const Val p0 = (Val)c0, p2 = (Val)c2, cj = (Val)cjd, ck = (Val)ckd, ci = (Val)cid;
    (void)c1;
    (void)c3;

    // line pointers (physical chunk c at element CH*c)
    Val* F = MODE == SW_GS ? a.F[comp] + line : nullptr;
    const Val* Fjp = MODE == SW_GS ? a.F[comp] + sy * ((long long)jp + (long long)g.ny * k) : nullptr;
    const Val* kin = nullptr;  // plane below (global): warp 0 across CTAs, slab edge
    const Val* jin = nullptr;  // row above (global): lane 0
    bool kin_zero = false, jin_zero = false;
    Val* hout = nullptr;  // GS: next sweep's halo copy of this plane
    if (MODE == SW_GS) {
        const size_t hp = (size_t)g.ps, base = (size_t)comp * 2 * a.P;
        kin = (kidx == 0 && cta.slab > 0) ? a.halo_in + (base + 0 * a.P + cta.slab) * hp + sy * j
                                          : a.F[comp] + line - g.ps;
        jin = a.F[comp] + sy * ((long long)jm + (long long)g.ny * k);
        if (kidx == 0 && cta.slab > 0) hout = a.halo_out + (base + 1 * a.P + (cta.slab - 1)) * hp + sy * j;
        if (kidx == K - 1 && cta.slab < a.P - 1) hout = a.halo_out + (base + 0 * a.P + (cta.slab + 1)) * hp + sy * j;
    } else {
        Val* io = MODE == SW_FWD ? a.RH : a.OUT;
        kin_zero = MODE == SW_FWD ? (kidx == 0) : (kidx == K - 1);
        kin = io + line + (MODE == SW_FWD ? -g.ps : g.ps);
        jin_zero = jr == 0;  // the first row of the slab (FWD: j = 1; BWD: j = J) or of a span block
        jin = io + sy * ((long long)(jin_zero ? j : (MODE == SW_FWD ? j - 1 : j + 1)) + (long long)g.ny * k);
    }
    Val* outp = MODE == SW_GS ? F : (MODE == SW_FWD ? a.RH : a.OUT) + line;
    const Val* inp = MODE == SW_GS ? a.PRE[comp] + line : a.RH + line;
    const bool wrap = MODE == SW_GS && jp == 1;  // the row after j holds new values (periodic GS)

    Val last[CH];  // this lane's outputs of the previous step
#pragma unroll
    for (int e = 0; e < CH; ++e) last[e] = Val(0);
    Val carry = Val(0);
    long long seen_j = -1, seen_k = -1;

    // raw operands.  The lane's window of step ts ends in chunk
    // a(ts) = (CH*(ts - T0) - dl + CH-1) / CH of the block (floor); each lane
    // copies that chunk (32 bytes FP64, 16 bytes FP32) with cp.async two steps
    // ahead into its operand buffer, position q of the block at element
    // q % OPB (one commit group per step, empty when the chunk is outside the
    // block or the lane has no line), and waits for the group at the top of
    // step ts.  The backward sweep's chunk holds its positions in reverse
    // memory order, so position q sits at element (q ^ 3) % OPB.
    // GS: the old-value terms come precomputed (k_gs_pre); FWD: r comes
    // pre-scaled by -w/Ap (k_lap); BWD: scaled here.
    Val* const opb = &s_op[wid][lane][0];
    auto chunk_of = [&](int ts) { return (CH * (ts - T0) - dl + CH - 1) >> LG; };
    auto issue_raw = [&](int ts) {
        const int ac = chunk_of(ts);
        if (line_ok && ts <= T1 && ac >= 0 && ac < Cl) {
            const int i0 = CH * (MODE == SW_BWD ? c_hi - ac : c_lo + ac);
            Val* dst = opb + ((CH * ac) & (OPB - 1));
#pragma unroll
            for (int b = 0; b < (int)(CH * sizeof(Val)) / 16; ++b)
                cp_async16(dst + b * (16 / sizeof(Val)), inp + i0 + b * (16 / sizeof(Val)));
        }
        cp_async_commit();
    };
    const Val bnd = MODE == SW_GS ? F[0] : Val(0);  // GS: U(0), the inflow boundary value of the line
    issue_raw(T0);
    issue_raw(T0 + 1);
    Val pj_pf[CH], pk_pf[CH];
    bool pj_ok = false, pk_ok = false;

    // Positions a step may take without any point being a boundary or
    // outside the block: i in 1..nx-2 and q in 1..Q-1.  A step whose 32
    // lanes all have lines and all lie there (most steps of a long line)
    // runs the body specialised for it: no per-point predicates.
    const int qlo = max(1, MODE == SW_BWD ? ibase - (g.nx - 2) : 1 - ibase);
    const int qhi = min(Q - 1, MODE == SW_BWD ? ibase - 1 : g.nx - 2 - ibase);
    const bool full_warp = plag == 1 && 32 * cta.jb + 31 < J;

    // One wavefront step; false when a wait timed out (the error word is set).
    auto step = [&](const int T, auto fast_tag) -> bool {
        constexpr bool FAST = decltype(fast_tag)::value;
        const int qb = CH * (T - T0) - dl;  // position of point 0
        int ix[CH];
        bool act[CH], inr[CH];
#pragma unroll
        for (int e = 0; e < CH; ++e) {
            const int q = qb + e;
            act[e] = FAST || (line_ok && q >= 0 && q < Q);
            ix[e] = ibase + idir * q;
            inr[e] = FAST || (ix[e] >= 1 && ix[e] <= g.nx - 2);
        }
        // this step's operands, read from the operand buffer and scaled
        // before the warp waits for its producers.  A register prefetch a
        // step ahead was slower (loads still in flight at the end-of-step
        // release have to complete first); cp.async copies are not ordered
        // by that release, so they run two steps ahead.
        cp_async_wait<1>();  // all but the group of step T + 1
        Val cur[CH];
#pragma unroll
        for (int e = 0; e < CH; ++e) {
            cur[e] = Val(0);
            if (act[e]) {
                const int q = qb + e;
                const Val r = opb[(MODE == SW_BWD ? (q ^ (CH - 1)) : q) & (OPB - 1)];
                cur[e] = MODE == SW_BWD ? p0 * r : r;
            }
        }
        // ---- wait for the producers of step T-1 (lane 0 for the warp)
        int abort = 0;
        if (lane == 0) {
            if (fj && T - T0 < Cl && !pj_ok && seen_j < T - 1) {
                seen_j = wait_global(fj, tag, T - 1);
                if (seen_j < 0) abort = 1;
            }
            if (kl > 0) {
                const int target = min(T - 1, tend_k);
                if (wid > 0) {
                    if (!wait_cta(&s_prog[wid - 1], target)) abort = 1;
                } else if (fk && !pk_ok && seen_k < target) {
                    seen_k = wait_global(fk, tag, target);
                    if (seen_k < 0) abort = 1;
                }
            }
        }
        // the plane below from the CTA below in the cluster: its step T-1 is
        // the (T - T0)-th it pushes, in ring slot (T - T0) % XR
        const int xu = T - T0;
        if (xcons && !mbar_wait(&s_full[xu % XR], (unsigned)(xu / XR) & 1u)) abort = 1;
        if (__any_sync(0xffffffffu, abort)) return false;
        // ---- inputs of the plane below (same positions, one step earlier)
        // and of the row above for lane 0 (chunk-aligned: lane 0 lags by 0)
        Val pk[CH], pj0[CH];
        if (wid > 0) {
            const Val* rs = &s_ring[wid - 1][(T - 1) & (RING - 1)][lane][0];
#pragma unroll
            for (int e = 0; e < CH; ++e) pk[e] = act[e] ? rs[e] : Val(0);
        } else {
#pragma unroll
            for (int e = 0; e < CH; ++e)
                pk[e] = !act[e] ? Val(0)
                                : (xcons ? s_xring[xu % XR][lane][e]
                                         : (pk_ok ? pk_pf[e] : (kin_zero ? Val(0) : __ldcg(kin + ix[e]))));
        }
#pragma unroll
        for (int e = 0; e < CH; ++e)
            pj0[e] = (lane != 0 || !act[e]) ? Val(0) : (pj_ok ? pj_pf[e] : (jin_zero ? Val(0) : __ldcg(jin + ix[e])));
        if (xcons) {  // slot read by every lane: re-arm it and hand it back when it is written again
            __syncwarp();
            if (lane == 0 && xu + XR <= T1 - T0) {
                mbar_arrive_expect_tx(&s_full[xu % XR], XBYTES);
                if (ld_relaxed_cluster(&s_xend) != 2) mbar_arrive_remote(mapa_rank(smem_u32(&s_empty[xu % XR]), xrank - 1));
            }
        }
        if (wrap) {
#pragma unroll
            for (int e = 0; e < CH; ++e)
                if (act[e]) cur[e] = fma(p2, __ldcg(Fjp + ix[e]), cur[e]);
        }
#pragma unroll
        for (int e = 0; e < CH; ++e) cur[e] = fma(ck, pk[e], cur[e]);
        // ---- the points in sweep order: the (j-1) input of point e is the
        // neighbour lane's point e - plag (this step) or e - plag + CH (the
        // step before), by shuffle; lane 0 has it from the row above
        const int pl = FAST ? 1 : plag;
        Val out[CH];
#pragma unroll
        for (int e = 0; e < CH; ++e) {
            const Val src = pl == 1 ? (e == 0 ? last[CH - 1] : out[e > 0 ? e - 1 : 0]) : last[e];
            Val pj = __shfl_up_sync(0xffffffffu, src, 1);
            if (lane == 0) pj = pj0[e];
            const Val nv = fma(cj, pj, cur[e]);
            if (FAST) {
                carry = fma(ci, carry, nv);
                out[e] = carry;
            } else {
                out[e] = Val(0);
                if (act[e]) {
                    if (qb + e == 0) carry = Val(0);  // first position of the block: nothing before it
                    if (inr[e]) {
                        carry = fma(ci, carry, nv);
                        out[e] = carry;
                    } else {  // outside 1..nx-2: the GS inflow boundary value, or zero
                        out[e] = (MODE == SW_GS && ix[e] == 0) ? bnd : Val(0);
                        carry = out[e];
                    }
                }
            }
        }
#pragma unroll
        for (int e = 0; e < CH; ++e) last[e] = out[e];
        // ---- hand the points to the next plane (ring slot T % RING), publish
        if (has_down) {
            if (lane == 0 && T - RING + 1 >= T0 + 1)
                if (!wait_cta(&s_prog[wid + 1], min(T - RING + 1, T1 + 1))) abort = 1;
            if (__shfl_sync(0xffffffffu, abort, 0)) return false;
            Val* ws = &s_ring[wid][T & (RING - 1)][lane][0];
#pragma unroll
            for (int e = 0; e < CH; ++e) ws[e] = out[e];
        }
        if (xprod) {  // push to the CTA above: wait until the consumer has released the slot's last use
            if (xu >= XR && !mbar_wait(&s_empty[xu % XR], (unsigned)(xu / XR - 1) & 1u)) abort = 1;
            if (__any_sync(0xffffffffu, abort)) return false;
            xpush<CH>(mapa_rank(smem_u32(&s_xring[xu % XR][lane][0]), xrank + 1),
                      mapa_rank(smem_u32(&s_full[xu % XR]), xrank + 1), out);
        }
        __syncwarp();
        if (lane == 0) st_release_cta(&s_prog[wid], T);
        // the results go to global memory after the hand-off to the next
        // plane, which reads the ring only, so that release does not wait for
        // these stores; the device-scope progress flag (for the CTAs that
        // read the rows and planes from global memory) is released after them.
        // GS writes the interior points only (i = 0 holds the boundary value).
#pragma unroll
        for (int e = 0; e < CH; ++e) {
            if (act[e] && (MODE != SW_GS || inr[e])) {
                outp[ix[e]] = out[e];
                if (MODE == SW_GS && hout) hout[ix[e]] = out[e];
            }
        }
        if (publish && ((T - T0) % PUB == PUB - 1 || T == T1)) {
            __syncwarp();
            if (lane == 0) st_release(fme, tag + (unsigned long long)(T + 1));
        }
        // ---- cross-CTA inputs of step T+1 when their producer is known to be ahead
        pj_ok = false;
        pk_ok = false;
        if (T < T1) {
            if (lane == 0 && fj && seen_j >= T) {
#pragma unroll
                for (int e = 0; e < CH; ++e) {
                    const int qn = qb + CH + e;
                    pj_pf[e] = (jin_zero || !line_ok || qn < 0 || qn >= Q) ? Val(0) : __ldcg(jin + ix[e] + idir * CH);
                }
                pj_ok = true;
            }
            if (wid == 0 && fk) {
                const int pf = __shfl_sync(0xffffffffu, (lane == 0 && seen_k >= min(T, tend_k)) ? 1 : 0, 0);
                if (pf) {
#pragma unroll
                    for (int e = 0; e < CH; ++e) {
                        const int qn = qb + CH + e;
                        pk_pf[e] = (kin_zero || !line_ok || qn < 0 || qn >= Q) ? Val(0) : __ldcg(kin + ix[e] + idir * CH);
                    }
                }
                pk_ok = pf != 0;
            }
        }
        issue_raw(T + 2);
        return true;
    };

    for (int T = T0; T <= T1; ++T) {
        const int q0 = CH * (T - T0);  // lane 0's first position; lane 31's is q0 - 31
        const bool ok = (full_warp && q0 - 31 >= qlo && q0 + CH - 1 <= qhi) ? step(T, std::true_type{})
                                                                             : step(T, std::false_type{});
        if (!ok) {
            if (lane == 0) atomicExch(a.err, TBL_ERR_TIMEOUT);
            cp_async_wait<0>();  // no copy into this CTA's shared memory outlives the warp
            if (lane == 0) {
                // stay until the partner can no longer reach this CTA's shared memory
                if (xprod) {
                    st_remote_s32(mapa_rank(smem_u32(&s_xend), xrank + 1), 2);
                    wait_word(&s_xack);
                }
                if (xcons && wait_word(&s_xend) == 2) st_remote_s32(mapa_rank(smem_u32(&s_xack), xrank - 1), 1);
            }
            __syncwarp();
            return;
        }
    }
    cp_async_wait<0>();
    if (lane == 0) {
        if (xprod) st_remote_s32(mapa_rank(smem_u32(&s_xend), xrank + 1), 1);
        if (xcons && wait_word(&s_xend) == 2) st_remote_s32(mapa_rank(smem_u32(&s_xack), xrank - 1), 1);
    }
    __syncwarp();
}

// The part of a Gauss-Seidel point update that reads only values the sweep
// has not yet replaced (Q, U(i+1), U(j+1) except on the periodic wrap row,
// U(k+1) or the slab's halo snapshot), in the sweep's reassociated form and
// FMA order: PRE = fma(p3, U(k+1), fma(p2, U(j+1), fma(p1, U(i+1), p0 Q))).
// Fully parallel, so the wavefront sweep keeps only the three FMAs that
// depend on new values.  blockIdx.z runs over (component, plane).
constexpr int ROWS_PER_BLOCK = 4;  // span rows per block of the fully parallel per-point passes

template <typename T>
struct Ptr3 {
    const T* p[3];
};

// Per-plane coefficients of the reassociated GS update (the values the sweep
// computes per warp), [p0 | p1 | p2 | p3] x nz, and of the GS residual
// (1 + t Ap, t At, t Ab), [d | cT | cB] x nz.
__global__ void k_gs_coef(int nz, double t, double aw_, double as_, const double* __restrict__ Ap,
                          const double* __restrict__ At, const double* __restrict__ Ab, double* __restrict__ pc,
                          float* __restrict__ pcf) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    const double rd = 1.0 / (1.0 + (t * Ap[k]));
    pc[k] = rd;
    pc[nz + k] = -(t * aw_) * rd;
    pc[2 * nz + k] = -(t * as_) * rd;
    pc[3 * nz + k] = -(t * At[k]) * rd;
    pc[4 * nz + k] = 1.0 + (t * Ap[k]);
    pc[5 * nz + k] = t * At[k];
    pc[6 * nz + k] = t * Ab[k];
    pc[7 * nz + k] = -(t * Ab[k]) * rd;  // red-black GS: coefficient of U(k-1)
    for (int q = 0; q < 4; ++q) pcf[q * nz + k] = (float)pc[q * nz + k];  // the FP32 sweep's (float) casts
    pcf[4 * nz + k] = (float)pc[7 * nz + k];
}

template <typename T>
__global__ void __launch_bounds__(256) k_gs_pre(Geom g, const T* __restrict__ pc,
                                                const int* __restrict__ slab_of_k,
                                                const SlabDesc* __restrict__ slabs, int P, int c0_, int c1_, int c2_,
                                                Ptr3<T> Fs, Ptr3<T> Qs, Ptr3<T> PREs,
                                                const T* __restrict__ halo_in) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int K = g.nz - 2;
    const int ci = blockIdx.z / K, k = 1 + blockIdx.z % K;
    if (i > g.nx - 2) return;
    const int comp = ci == 0 ? c0_ : (ci == 1 ? c1_ : c2_);
    const T* F = Fs.p[comp];
    const int nz = g.nz;
    const T p0 = pc[k], p1 = pc[nz + k], p2 = pc[2 * nz + k], p3 = pc[3 * nz + k];
    const int r = slab_of_k[k];
    const SlabDesc sl = slabs[r];
    const bool halo = k == sl.bn + sl.K - 1 && r < P - 1;
    for (int jr = 0; jr < ROWS_PER_BLOCK; ++jr) {  // a few rows per block: fewer, longer blocks
        const int j = 1 + blockIdx.y * ROWS_PER_BLOCK + jr;
        if (j > g.ny - 2) break;
        const long long line = (long long)g.sx * ((long long)j + (long long)g.ny * k);
        const int jp = (j == g.ny - 2) ? 1 : j + 1;
        const T* Fkp = halo ? halo_in + ((size_t)comp * 2 * P + 1 * P + r) * (size_t)g.ps + (size_t)g.sx * j
                            : F + line + g.ps;
        T x = fma(p1, F[line + i + 1], p0 * Qs.p[comp][line + i]);
        if (jp != 1) x = fma(p2, F[(long long)g.sx * ((long long)jp + (long long)g.ny * k) + i], x);
        const_cast<T*>(PREs.p[comp])[line + i] = fma(p3, Fkp[i], x);
    }
}

// ------------------------------ red-black ordering (TBL_FLAG_RB_ORDER)
// Throughput mode, not the reference's arithmetic.  Points are coloured by
// the parity of i+j+k (the number of unique span rows is even, so the
// periodic wrap keeps the colouring); every neighbour of a point has the other
// colour, so a colour pass updates all its points at once.  Threads map onto
// the points of the pass's colour only (i = rb_i0 + 2t along a row), so no
// lane of a warp idles: the FP64 passes are bound by FP64 issue, which a warp
// pays in full however many of its lanes are active.

// First interior i of colour `color` on row (j, k): i + j + k has the
// colour's parity.
__device__ __forceinline__ int rb_i0(int color, int j, int k) { return 2 - ((color + j + k) & 1); }

// Gauss-Seidel half sweep of the listed components over one colour, the whole
// domain as one block (no slab halos), periodic in j:
//   U = p0 Q + p1 (U(i+1) + U(i-1)) + p2 (U(j+1) + U(j-1)) + p3 U(k+1) + pb U(k-1)
// with the per-plane coefficients of the GS update (k_gs_coef).
template <typename T>
__global__ void __launch_bounds__(256) k_rb_gs(Geom g, const T* __restrict__ pc, const T* __restrict__ pbv,
                                               Ptr3<T> Fs, Ptr3<T> Qs, int c0_, int c1_, int c2_, int color) {
    const int K = g.nz - 2;
    const int ci = blockIdx.z / K, k = 1 + blockIdx.z % K;
    const int comp = ci == 0 ? c0_ : (ci == 1 ? c1_ : c2_);
    T* F = const_cast<T*>(Fs.p[comp]);
    const T* Q = Qs.p[comp];
    const int nz = g.nz;
    const T p0 = pc[k], p1 = pc[nz + k], p2 = pc[2 * nz + k], p3 = pc[3 * nz + k], pb = pbv[k];
    for (int jr = 0; jr < ROWS_PER_BLOCK; ++jr) {  // a few rows per block: fewer, longer blocks
        const int j = 1 + blockIdx.y * ROWS_PER_BLOCK + jr;
        if (j > g.ny - 2) break;
        const int i = rb_i0(color, j, k) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
        if (i > g.nx - 2) continue;
        const int jm = j == 1 ? g.ny - 2 : j - 1, jp = j == g.ny - 2 ? 1 : j + 1;
        const long long p = (long long)i + (long long)g.sx * ((long long)j + (long long)g.ny * k);
        const long long pjm = (long long)i + (long long)g.sx * ((long long)jm + (long long)g.ny * k);
        const long long pjp = (long long)i + (long long)g.sx * ((long long)jp + (long long)g.ny * k);
        F[p] = p0 * Q[p] + p1 * (F[p + 1] + F[p - 1]) + p2 * (F[pjp] + F[pjm]) + p3 * F[p + g.ps] +
               pb * F[p - g.ps];
    }
}

// Red-black SSOR preconditioner (one global block, periodic in j), the same
// splitting and sign convention as the lexicographic one: with RH = -w r/Ap
// from the matvec and c = -w (2-w)/w,
//   pass 1, black (odd) points: OUT = c (RH + s_k N(RH))
//   pass 2, red (even) points:  OUT = c RH + s_k N(OUT)
// where N(X) = Aw (X(i+1)+X(i-1)) + As (X(j+1)+X(j-1)) + Ab X(k-1) + At X(k+1)
// and s_k = -w/Ap(k).  Faces of RH and OUT are zero.
template <typename T>
__global__ void __launch_bounds__(256) k_rb_ssor(Geom g, T aw, T as, const T* __restrict__ Ab,
                                                 const T* __restrict__ At, const T* __restrict__ sk, T cfac,
                                                 const T* __restrict__ RH, T* __restrict__ OUT, int pass) {
    const int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    const int color = pass == 1 ? 1 : 0;
    const int i = rb_i0(color, j, k) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i > g.nx - 2) return;
    const int jm = j == 1 ? g.ny - 2 : j - 1, jp = j == g.ny - 2 ? 1 : j + 1;
    const long long p = (long long)i + (long long)g.sx * ((long long)j + (long long)g.ny * k);
    const long long pjm = (long long)i + (long long)g.sx * ((long long)jm + (long long)g.ny * k);
    const long long pjp = (long long)i + (long long)g.sx * ((long long)jp + (long long)g.ny * k);
    const T* X = pass == 1 ? RH : OUT;
    const T nb = aw * (X[p + 1] + X[p - 1]) + as * (X[pjp] + X[pjm]) + Ab[k] * X[p - g.ps] + At[k] * X[p + g.ps];
    OUT[p] = pass == 1 ? cfac * (RH[p] + sk[k] * nb) : cfac * RH[p] + sk[k] * nb;
}

// r = L7 X (Q8 == nullptr) or r = Q8 - L7 X on the interior, written to R
// (:1001-1006 restart residual, :1098-1101 Arnoldi matvec), global halos.
// With rAp non-null the result is multiplied by the forward sweep's
// coefficient -w/Ap(k) (rounded to the sweep's type first, as the sweep did).
template <typename TI, typename TO, typename TC>
// Coefficient tables come in the arithmetic type TC (and the scale in the
// output type TO), so an FP32 matvec does no double-to-float conversion per
// point (those run at the FP64 rate).
__global__ void __launch_bounds__(256) k_lap(Geom g, TC aw, TC as, const TC* __restrict__ Ab,
                                             const TC* __restrict__ At, const TC* __restrict__ Ap,
                                             const TI* __restrict__ X, const double* __restrict__ Q8,
                                             TO* __restrict__ R, const TO* __restrict__ scale,
                                             const int* __restrict__ skip) {
    if (skip && *skip) return;
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > g.nx - 2) return;
    const long long p = (long long)i + (long long)g.sx * ((long long)j + (long long)g.ny * k);
    const int jm = j == 1 ? g.ny - 2 : j - 1, jp = j == g.ny - 2 ? 1 : j + 1;
    const TC xjm = (TC)X[(long long)i + (long long)g.sx * ((long long)jm + (long long)g.ny * k)];
    const TC xjp = (TC)X[(long long)i + (long long)g.sx * ((long long)jp + (long long)g.ny * k)];
    TC lap = aw * (TC)X[p - 1] + aw * (TC)X[p + 1] + as * xjm + as * xjp + Ab[k] * (TC)X[p - g.ps] +
             At[k] * (TC)X[p + g.ps] + Ap[k] * (TC)X[p];
    const TO r = (TO)(Q8 ? ((TC)Q8[p] - (lap)) : lap);
    R[p] = scale ? scale[k] * r : r;
}

// ------------------------------------------------------ bounded-wait self-test
// One thread waits, with the sweeps' own bounded wait, on a progress flag that
// nothing sets; the wait gives up after SPIN_LIMIT polls and reports
// TBL_ERR_TIMEOUT through the error word, as a stalled sweep warp does.
__global__ void k_wait_selftest(const unsigned long long* flag, int* err) {
    if (threadIdx.x != 0) return;
    if (wait_global(flag, 1ull << 20, 0) < 0) atomicExch(err, TBL_ERR_TIMEOUT);
}

int selftest_bounded_wait(int* observed, double* seconds) {
    unsigned long long* flag = nullptr;
    int* err = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = TBL_OK;
    auto fail = [&](cudaError_t e) { if (e != cudaSuccess && st == TBL_OK) st = TBL_ERR_CUDA; };
    fail(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    fail(cudaMalloc(&flag, sizeof(unsigned long long)));
    fail(cudaMalloc(&err, sizeof(int)));
    fail(cudaEventCreate(&e0));
    fail(cudaEventCreate(&e1));
    if (st == TBL_OK) {
        fail(cudaMemsetAsync(flag, 0, sizeof(unsigned long long), s));
        fail(cudaMemsetAsync(err, 0, sizeof(int), s));
        fail(cudaEventRecord(e0, s));
        k_wait_selftest<<<1, 32, 0, s>>>(flag, err);
        fail(cudaGetLastError());
        fail(cudaEventRecord(e1, s));
        fail(cudaStreamSynchronize(s));
        int v = 0;
        fail(cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost));
        float ms = 0.f;
        fail(cudaEventElapsedTime(&ms, e0, e1));
        if (observed) *observed = v;
        if (seconds) *seconds = ms * 1e-3;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (flag) cudaFree(flag);
    if (err) cudaFree(err);
    if (s) cudaStreamDestroy(s);
    return st;
}

// ------------------------------------------------------------- host glue

// Build the CTA table for the slab partition (called once at create).
int build_sweep_ctas(tbl_handle* h) {
    const int J = h->g.ny - 2;
    const int njb = (J + 31) / 32;
    std::vector<SweepCta> ctas;
    std::vector<SlabDesc> slabs(h->P);
    // The CTAs of a slab column (same slab and row block, kg = 0..nkc-1) are
    // consecutive, so that they can form one thread-block cluster; slabs
    // with fewer plane groups get idle CTAs at the top of their columns.
    int nkc = 1;
    for (int r = 0; r < h->P; ++r) nkc = std::max(nkc, (h->en[r] - h->bn[r] + 1 + KG - 1) / KG);
    for (int r = 0; r < h->P; ++r) {
        slabs[r].bn = h->bn[r];
        slabs[r].K = h->en[r] - h->bn[r] + 1;
        const int nkg = (slabs[r].K + KG - 1) / KG;
        const int base = (int)ctas.size();
        for (int jb = 0; jb < njb; ++jb)
            for (int kg = 0; kg < nkc; ++kg) {
                SweepCta c;
                c.slab = r; c.jb = jb; c.kg = kg;
                const bool live = kg < nkg;
                c.up_j = live && jb > 0 ? base + (jb - 1) * nkc + kg : -1;
                c.up_k = live && kg > 0 ? base + jb * nkc + (kg - 1) : -1;
                c.dn_j = live && jb < njb - 1 ? 1 : 0;
                c.dn_k = live && kg < nkg - 1 ? 1 : 0;
                ctas.push_back(c);
            }
    }
    h->sweep_kc = nkc;
    for (auto& prec : h->sweep_cluster)
        for (auto& row : prec)
            for (int& v : row) v = -1;
    h->n_cta = (int)ctas.size();
    TBL_CUDA_TRY(cudaMalloc(&h->ctas, ctas.size() * sizeof(SweepCta)));
    TBL_CUDA_TRY(cudaMemcpy(h->ctas, ctas.data(), ctas.size() * sizeof(SweepCta), cudaMemcpyHostToDevice));
    TBL_CUDA_TRY(cudaMalloc(&h->slabs, slabs.size() * sizeof(SlabDesc)));
    TBL_CUDA_TRY(cudaMemcpy(h->slabs, slabs.data(), slabs.size() * sizeof(SlabDesc), cudaMemcpyHostToDevice));
    // flag sets: three GS components, or up to SSOR_MAX_NIB streamwise SSOR blocks
    const size_t nsets = SSOR_MAX_NIB > 3 ? SSOR_MAX_NIB : 3;
    TBL_CUDA_TRY(cudaMalloc(&h->flags, nsets * h->n_cta * KG * sizeof(unsigned long long)));
    TBL_CUDA_TRY(cudaMemset(h->flags, 0, nsets * h->n_cta * KG * sizeof(unsigned long long)));
    h->epoch = 1;
    return TBL_OK;
}

template <typename T>
static SweepArgs<T> base_args(tbl_handle* h) {
    SweepArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.g = h->g;
    a.ctas = h->ctas;
    a.slabs = h->slabs;
    a.n_cta = h->n_cta;
    a.P = h->P;
    a.C = (h->g.nx - 2) / sweep_ch<T>() + 1;
    a.flags = h->flags;
    a.epoch = h->epoch++;
    a.err = h->err;
    a.Ab = h->Ab; a.At = h->At; a.Ap = h->Ap; a.rAp = h->rAp;
    a.aw = 1.0 / (h->cfg.dx * h->cfg.dx);
    a.as = 1.0 / (h->cfg.dy * h->cfg.dy);
    a.omega = h->cfg.omega;
    a.sw = (2 - h->cfg.omega) / h->cfg.omega;
    a.jb_rows = (h->cfg.flags & TBL_FLAG_SSOR_SPAN_BLOCKS) ? 32 : 0;
    a.nib = h->ssor_nib > 0 ? h->ssor_nib : 1;
    // A row lags the row above by one position.  With 4 span rows or fewer the
    // Gauss-Seidel wrap row (which reads row 1's new values from global
    // memory) would share a step with row 1, so those grids lag by a chunk.
    a.plag = h->g.ny - 2 <= sweep_ch<T>() ? sweep_ch<T>() : 1;
    a.t = -h->cfg.dt / (h->cfg.re);
    return a;
}

template <int MODE, typename T>
static int launch_sweep(tbl_handle* h, SweepArgs<T>& a, int ncomp) {
    void* args[] = {&a};
    dim3 grid(h->n_cta, ncomp), block(KG * 32);
    // (the dynamic shared memory limit of the three sweep kernels of the
    // handle's precision is raised once, in check_cooperative)
    // The CTAs of a slab column form one thread-block cluster when they are
    // 2..8 and the launch's clusters can all be resident at once; the plane
    // hand-off between them then goes through distributed shared memory.
    const int nkc = h->sweep_kc;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = sweep_smem<T>();
    cfg.stream = h->stream;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)nkc;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int& use = h->sweep_cluster[sizeof(T) == 8 ? 1 : 0][MODE][ncomp < 8 ? ncomp : 7];
    if (use < 0) {
        use = 0;
        int ncl = 0;
        if (nkc >= 2 && nkc <= 8) {
            if (cudaOccupancyMaxActiveClusters(&ncl, (const void*)k_sweep<MODE, T>, &cfg) == cudaSuccess)
                use = (long long)ncl * nkc >= (long long)h->n_cta * ncomp ? 1 : 0;
            else
                (void)cudaGetLastError();  // a refused query leaves the cooperative launch
        }
    }
    if (use) {
        a.xk = nkc;
        TBL_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_sweep<MODE, T>, a));
    } else {
        a.xk = 0;
        TBL_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_sweep<MODE, T>, grid, block, args, sweep_smem<T>(), h->stream));
    }
    h->launches++;
    return TBL_OK;
}

template <typename T>
static int gs_pre_and_sweep(tbl_handle* h, T* const F[3], const T* const Q[3], T* const PRE[3], T* halo,
                            const int* comps, int ncomp, int parity) {
    const size_t hsz = (size_t)3 * 2 * h->P * h->g.ps;
    SweepArgs<T> a = base_args<T>(h);
    for (int c = 0; c < 3; ++c) { a.F[c] = F[c]; a.Q[c] = Q[c]; a.PRE[c] = PRE[c]; }
    for (int c = 0; c < ncomp; ++c) a.comp[c] = comps[c];
    a.halo_in = halo + (size_t)(parity & 1) * hsz;
    a.halo_out = halo + (size_t)((parity + 1) & 1) * hsz;
    const Geom& g = h->g;
    Ptr3<T> Fs, Qs, Ps;
    for (int c = 0; c < 3; ++c) { Fs.p[c] = F[c]; Qs.p[c] = Q[c]; Ps.p[c] = PRE[c]; }
    dim3 grid((g.nx - 2 + 255) / 256, (g.ny - 2 + ROWS_PER_BLOCK - 1) / ROWS_PER_BLOCK, (g.nz - 2) * ncomp);
    const T* pc = sizeof(T) == 8 ? (const T*)h->gs_coef : (const T*)h->gs_coef_f;
    k_gs_pre<T><<<grid, 256, 0, h->stream>>>(g, pc, h->slab_of_k, h->slabs, h->P,
                                             comps[0], ncomp > 1 ? comps[1] : 0, ncomp > 2 ? comps[2] : 0, Fs, Qs,
                                             Ps, a.halo_in);
    h->launches++;
    return launch_sweep<SW_GS, T>(h, a, ncomp);
}

// GS sweep for the listed components (old-value terms precomputed first);
// halo buffers ping-pong by `parity`.  When the components' CTAs cannot all
// be resident at once, they sweep in consecutive launches.
static int launch_gs_sweep_chunk(tbl_handle* h, const int* comps, int ncomp, int parity);

template <typename T>
static int rb_gs(tbl_handle* h, T* const F[3], const T* const Q[3], const T* pc, const T* pb, const int* comps,
                 int ncomp) {
    const Geom& g = h->g;
    Ptr3<T> Fs, Qs;
    for (int c = 0; c < 3; ++c) { Fs.p[c] = F[c]; Qs.p[c] = Q[c]; }
    dim3 grid(((g.nx - 1) / 2 + 255) / 256, (g.ny - 2 + ROWS_PER_BLOCK - 1) / ROWS_PER_BLOCK, (g.nz - 2) * ncomp);
    for (int color = 0; color < 2; ++color)
        k_rb_gs<T><<<grid, 256, 0, h->stream>>>(g, pc, pb, Fs, Qs, comps[0], ncomp > 1 ? comps[1] : 0,
                                                ncomp > 2 ? comps[2] : 0, color);
    h->launches += 2;
    return TBL_OK;
}

int launch_gs_sweep(tbl_handle* h, const int* comps, int ncomp, int parity) {
    if (h->cfg.flags & TBL_FLAG_RB_ORDER) {
        const int nz = h->g.nz;
        if (h->cfg.precision == TBL_PREC_MIXED) {
            float* F[3] = {h->Df[0], h->Df[1], h->Df[2]};
            const float* Q[3] = {h->Qf[0], h->Qf[1], h->Qf[2]};
            return rb_gs<float>(h, F, Q, h->gs_coef_f, h->gs_coef_f + 4 * (size_t)nz, comps, ncomp);
        }
        double* F[3] = {h->U[0], h->U[1], h->U[2]};
        const double* Q[3] = {h->Q[0], h->Q[1], h->Q[2]};
        return rb_gs<double>(h, F, Q, h->gs_coef, h->gs_coef + 7 * (size_t)nz, comps, ncomp);
    }
    const int per = h->gs_comps_per_launch > 0 ? h->gs_comps_per_launch : 1;
    for (int c0 = 0; c0 < ncomp; c0 += per) {
        const int n = ncomp - c0 < per ? ncomp - c0 : per;
        const int s = launch_gs_sweep_chunk(h, comps + c0, n, parity);
        if (s != TBL_OK) return s;
    }
    return TBL_OK;
}

static int launch_gs_sweep_chunk(tbl_handle* h, const int* comps, int ncomp, int parity) {
    if (h->cfg.precision == TBL_PREC_MIXED) {  // delta form: iterate on D with r0 in Qf
        float* F[3] = {h->Df[0], h->Df[1], h->Df[2]};
        const float* Q[3] = {h->Qf[0], h->Qf[1], h->Qf[2]};
        float* P[3] = {h->PREf, h->PREf + h->g.vol, h->PREf + 2 * h->g.vol};
        return gs_pre_and_sweep<float>(h, F, Q, P, reinterpret_cast<float*>(h->halo), comps, ncomp, parity);
    }
    double* F[3] = {h->U[0], h->U[1], h->U[2]};
    const double* Q[3] = {h->Q[0], h->Q[1], h->Q[2]};
    double* P[3] = {h->PRE, h->PRE + h->g.vol, h->PRE + 2 * h->g.vol};
    return gs_pre_and_sweep<double>(h, F, Q, P, h->halo, comps, ncomp, parity);
}

// Forward SSOR sweep of r = L7 X (Q8 == nullptr) or r = Q8 - L7 X.
int launch_ssor_fwd(tbl_handle* h, const double* X, const double* Q8, const int* skip) {
    const Geom& g = h->g;
    const double aw = 1.0 / (h->cfg.dx * h->cfg.dx), as = 1.0 / (h->cfg.dy * h->cfg.dy);
    k_lap<double, double, double><<<dim3((g.nx - 2 + 255) / 256, g.ny - 2, g.nz - 2), 256, 0, h->stream>>>(
        g, aw, as, h->Ab, h->At, h->Ap, X, Q8, h->RH, h->lap_scale, skip);
    h->launches++;
    if (h->cfg.flags & TBL_FLAG_RB_PRECOND) return TBL_OK;  // the red-black passes run in launch_ssor_bwd
    SweepArgs<double> a = base_args<double>(h);
    a.RH = h->RH;
    a.skip = skip;
    return launch_sweep<SW_FWD, double>(h, a, a.nib);
}

template <typename T>
static int rb_ssor(tbl_handle* h, T aw, T as, const T* Ab, const T* At, const T* sk, const T* RH, T* out) {
    const Geom& g = h->g;
    const double w = h->cfg.omega;
    const T cfac = (T)(-w * ((2.0 - w) / w));
    dim3 grid(((g.nx - 1) / 2 + 255) / 256, g.ny - 2, g.nz - 2);  // (nx-1)/2 >= the points of a colour on a row
    k_rb_ssor<T><<<grid, 256, 0, h->stream>>>(g, aw, as, Ab, At, sk, cfac, RH, out, 1);
    k_rb_ssor<T><<<grid, 256, 0, h->stream>>>(g, aw, as, Ab, At, sk, cfac, RH, out, 2);
    h->launches += 2;
    return TBL_OK;
}

int launch_ssor_bwd(tbl_handle* h, double* out, const int* skip) {
    if (h->cfg.flags & TBL_FLAG_RB_PRECOND)
        return rb_ssor<double>(h, 1.0 / (h->cfg.dx * h->cfg.dx), 1.0 / (h->cfg.dy * h->cfg.dy), h->Ab, h->At,
                               h->lap_scale, h->RH, out);
    SweepArgs<double> a = base_args<double>(h);
    a.RH = h->RH;
    a.OUT = out;
    a.skip = skip;
    return launch_sweep<SW_BWD, double>(h, a, a.nib);
}

// Mixed precision: FP32 preconditioned matvec of the inner GMRES.  Xd (FP64
// outer residual, r = Q8 - L7 p' computed in FP64) or Xf (inner FP32 vector;
// with denom, the previous Arnoldi vector before its division by *denom,
// which the matvec applies, writing the normalised vector to vout).
int launch_ssor_fwd_f(tbl_handle* h, const float* Xf, const double* PCd, const double* Q8, const int* skip,
                      const double* denom, float* vout) {
    const Geom& g = h->g;
    dim3 grid((g.nx - 2 + 255) / 256, g.ny - 2, g.nz - 2);
    const double aw = 1.0 / (h->cfg.dx * h->cfg.dx), as = 1.0 / (h->cfg.dy * h->cfg.dy);
    if (PCd)
        k_lap<double, float, double><<<grid, 256, 0, h->stream>>>(g, aw, as, h->Ab, h->At, h->Ap, PCd, Q8, h->RHf,
                                                                  h->coef_f + 3 * (size_t)g.nz, skip);
    else {  // the inner Arnoldi matvec: TMA plane tiles
        const int s = launch_lap_tma<float>(h, Xf, h->RHf, (float)aw, (float)as, h->coef_f, h->coef_f + g.nz,
                                            h->coef_f + 2 * (size_t)g.nz, h->coef_f + 3 * (size_t)g.nz, skip, denom,
                                            vout);
        if (s != TBL_OK) return s;
        h->launches--;  // counted by launch_lap_tma
    }
    h->launches++;
    if (h->cfg.flags & TBL_FLAG_RB_PRECOND) return TBL_OK;
    SweepArgs<float> a = base_args<float>(h);
    a.RH = h->RHf;
    a.skip = skip;
    return launch_sweep<SW_FWD, float>(h, a, a.nib);
}

int launch_ssor_bwd_f(tbl_handle* h, float* out, const int* skip) {
    if (h->cfg.flags & TBL_FLAG_RB_PRECOND) {
        const size_t nz = (size_t)h->g.nz;
        return rb_ssor<float>(h, (float)(1.0 / (h->cfg.dx * h->cfg.dx)), (float)(1.0 / (h->cfg.dy * h->cfg.dy)),
                              h->coef_f, h->coef_f + nz, h->coef_f + 3 * nz, h->RHf, out);
    }
    SweepArgs<float> a = base_args<float>(h);
    a.RH = h->RHf;
    a.OUT = out;
    a.skip = skip;
    return launch_sweep<SW_BWD, float>(h, a, a.nib);
}

// Snapshot of the planes every slab reads from its neighbours before the
// first sweep (the end-of-step halo of the previous step).
template <typename T>
__global__ void k_halo_init(Geom g, const SlabDesc* __restrict__ slabs, int P, const T* __restrict__ U0,
                            const T* __restrict__ U1, const T* __restrict__ U2, T* __restrict__ halo) {
    // blockIdx.y = comp*2P + side*P + slab
    const int comp = blockIdx.y / (2 * P), rem = blockIdx.y % (2 * P), side = rem / P, r = rem % P;
    const SlabDesc s = slabs[r];
    if (side == 0 && r == 0) return;
    if (side == 1 && r == P - 1) return;
    const int kk = side == 0 ? s.bn - 1 : s.bn + s.K;
    const T* F = comp == 0 ? U0 : (comp == 1 ? U1 : U2);
    T* dst = halo + (size_t)blockIdx.y * g.ps;
    const T* src = F + (long long)kk * g.ps;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < g.ps; q += (long long)gridDim.x * blockDim.x)
        dst[q] = src[q];
}

int launch_halo_init(tbl_handle* h, int parity) {
    const size_t hsz = (size_t)3 * 2 * h->P * h->g.ps;
    // per-plane GS coefficients of the operator in use (the adjoint swaps in A^T)
    k_gs_coef<<<(h->g.nz + 127) / 128, 128, 0, h->stream>>>(h->g.nz, -h->cfg.dt / (h->cfg.re),
                                                             1.0 / (h->cfg.dx * h->cfg.dx),
                                                             1.0 / (h->cfg.dy * h->cfg.dy), h->Ap, h->At, h->Ab,
                                                             h->gs_coef, h->gs_coef_f);
    h->launches++;
    if (h->cfg.precision == TBL_PREC_MIXED)
        k_halo_init<float><<<dim3(32, 3 * 2 * h->P), 256, 0, h->stream>>>(
            h->g, h->slabs, h->P, h->Df[0], h->Df[1], h->Df[2], reinterpret_cast<float*>(h->halo) + (size_t)(parity & 1) * hsz);
    else
        k_halo_init<double><<<dim3(32, 3 * 2 * h->P), 256, 0, h->stream>>>(h->g, h->slabs, h->P, h->U[0], h->U[1],
                                                                           h->U[2], h->halo + (size_t)(parity & 1) * hsz);
    h->launches++;
    return TBL_OK;
}

int check_cooperative(tbl_handle* h) {
    int dev = 0, sms = 0, coop = 0;
    TBL_CUDA_TRY(cudaGetDevice(&dev));
    TBL_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    TBL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // every CTA of a sweep launch must be resident at once (they wait on one
    // another): the SSOR sweeps need n_cta CTAs, a GS launch n_cta per component
    const bool mx = h->cfg.precision == TBL_PREC_MIXED;
    const void* ks[3] = {mx ? (const void*)k_sweep<SW_GS, float> : (const void*)k_sweep<SW_GS, double>,
                         mx ? (const void*)k_sweep<SW_FWD, float> : (const void*)k_sweep<SW_FWD, double>,
                         mx ? (const void*)k_sweep<SW_BWD, float> : (const void*)k_sweep<SW_BWD, double>};
    long long cap[3];
    for (int q = 0; q < 3; ++q) {
        int per_sm = 0;
        const size_t smem = mx ? sweep_smem<float>() : sweep_smem<double>();
        TBL_CUDA_TRY(cudaFuncSetAttribute(ks[q], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        TBL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks[q], KG * 32, smem));
        cap[q] = (long long)per_sm * sms;
    }
    h->coop_ok = coop && cap[0] >= h->n_cta && cap[1] >= h->n_cta && cap[2] >= h->n_cta;
    h->gs_comps_per_launch = (int)(cap[0] / (h->n_cta > 0 ? h->n_cta : 1));
    if (h->gs_comps_per_launch > 3) h->gs_comps_per_launch = 3;
    // streamwise SSOR blocks: up to SSOR_MAX_NIB, as many as stay co-resident
    h->ssor_nib = 1;
    if (h->cfg.flags & TBL_FLAG_SSOR_STREAM_BLOCKS) {
        const long long fit = (cap[1] < cap[2] ? cap[1] : cap[2]) / (h->n_cta > 0 ? h->n_cta : 1);
        int nib = (int)(fit < SSOR_MAX_NIB ? (fit < 1 ? 1 : fit) : SSOR_MAX_NIB);
        // no empty block: the sweep splits C chunks into blocks of ceil(C/nib)
        const int C = (h->g.nx - 2) / (mx ? sweep_ch<float>() : sweep_ch<double>()) + 1;
        if (nib > C) nib = C;
        const int cb = (C + nib - 1) / nib;
        h->ssor_nib = (C + cb - 1) / cb;
    }
    return h->coop_ok ? TBL_OK : TBL_ERR_BAD_ARG;
}

}  // namespace tbl
