// tbl_internal.cuh -- device state and kernel interfaces of libtblgpu.so.
//
// Layout in HBM: every 3-D field is the reference array Ut(nx,ny,nz,.) with
// i fastest, stored with a row pitch sx = nx+7 rounded up to 8 elements so
// that each row starts on a 32-byte boundary and a 32-byte chunk of a
// wavefront lane never crosses a row.
// Element (i,j,k) (0-based) is at i + sx*(j + ny*k).  Padding columns hold 0.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>

#include "../../include/tbl_gpu.h"

#define TBL_CUDA_TRY(expr)                                                    \
    do {                                                                      \
        cudaError_t e_ = (expr);                                              \
        if (e_ != cudaSuccess) {                                              \
            tbl::set_last_cuda_error(e_, #expr, __FILE__, __LINE__);          \
            return TBL_ERR_CUDA;                                              \
        }                                                                     \
    } while (0)

namespace tbl {

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);

constexpr int KG = 4;             // k-planes (warps) per wavefront CTA
constexpr int SSOR_MAX_NIB = 4;    // streamwise SSOR blocks per line at most
constexpr int RED_THREADS = 256;  // threads per reduction block

// Geometry shared by all kernels (passed by value).
struct Geom {
    int nx, ny, nz;   // reference n3d
    int sx;           // row pitch
    long long ps;     // plane stride sx*ny
    long long vol;    // sx*ny*nz
    int J;            // ny-2 unique spanwise rows
};

// One wavefront CTA: a 32-row x KG-plane block of (j,k) lines of one slab.
struct SweepCta {
    int slab;      // slab index r
    int jb, kg;    // block coordinates inside the slab
    int up_j;      // CTA index of (jb-1, kg) or -1
    int up_k;      // CTA index of (jb, kg-1) or -1
    int dn_j;      // 1 when a CTA (jb+1, kg) exists (it reads this CTA's last rows)
    int dn_k;      // 1 when a CTA (jb, kg+1) exists (its warp 0 reads this CTA's last plane)
};

// Slab s covers interior planes k in [bn, bn+K) (0-based).
struct SlabDesc {
    int bn, K;
};

// Device-side scalars of the recycling bookkeeping and of GMRES.
struct DevScalars {
    double lamda;
    double lamda03;
    int ksep;
    int stop;  // set by k_givens when the Arnoldi estimate reaches its target: the kernels
               // of an Arnoldi step enqueued ahead of the host's check then return at once
    // GMRES
    double rho, sumnor, sumav;
    // reductions (result slots)
    double red[16];
};

// Reduction workspace: partial sums + arrival counters per slot.
struct RedWork {
    double* partial;      // [slots][max_blocks]
    unsigned int* count;  // [slots]
    int max_blocks;
};

struct AdjTape;  // tbl_adjoint.cu

template <typename T>
struct Fields {
    T* U[3];
    T* P;
    T* PC;
    T* Q[3];
    T* Q8;
};

}  // namespace tbl

struct tbl_handle {
    tbl_config cfg;
    tbl::Geom g;
    int P;
    std::vector<int> bn, en;  // 0-based first/last interior plane per slab
    // device arrays (FP64)
    double* U[3];
    double* Pr;
    double* PC;
    double* Q[3];
    double* Q8;
    double* RH;      // SSOR forward result (scaled)
    double* PRE;     // 3 x vol: old-value terms of the GS point updates (FP64)
    float* PREf;     // 3 x vol: the same in mixed precision
    double* gs_coef; // 8 x nz per-plane coefficients of the GS update, residual and red-black update
    float* gs_coef_f;   // 5 x nz: the update coefficients rounded to FP32 (+ the red-black U(k-1) one)
    double* lap_scale;  // nz: -w/Ap(k), the SSOR forward scaling folded into the matvec
    float* coef_f;      // 4 x nz FP32: Ab, At, Ap, -w/Ap (FP32 matvec)
    double* V;       // kmax+1 Krylov vectors, vol each
    double* uold1;   // U1 at i=1 before the inflow update, (ny, nz)
    // mixed precision (TBL_PREC_MIXED): FP32 fields and inner-GMRES vectors
    float* Uf[3];
    float* Pf;
    float* Qf[3];
    float* Df[3];    // GS increments (delta form)
    float* Vf;       // inner Krylov vectors
    float* RHf;      // inner SSOR work
    double* R64;     // FP64 outer residual
    double* lsg_partial;        // low-synch Gram-Schmidt: per-block partials [2*8*groups][max_blocks]
    double *lsg_L, *lsg_d, *lsg_g;  // (K1 x K1) strictly lower Gram matrix, Q^T w, Q^T v_new
    // per-k coefficient arrays and mesh (nz)
    double *x3, *jacinv, *jac2, *Ab, *At, *Ap, *rAp;
    // recycling state
    double *usum2, *vsum2, *wsum2, *wt, *ume1, *bltkns;
    int* newk;
    double* ufl_file;  // 3 x (ny,nz) restart-file copy of Ufluc(irec,:,:,:)
    double* ufl_live;  // 3 x (ny,nz) per-slab live copy
    double* ufl_full;  // 3 x vol uploaded Ufluc (restart output)
    double* usum2_fl;  // 3 x (nx,nz): means used by the last per-step Ufluc update
    // statistics
    double* sums;      // 9 x (nx,nz): usum vsum wsum uusum vvsum wwsum uvsum uwsum vwsum
    double* avg;       // 9 x (nx,nz): sums / cum of the last rescaling, before the reset
    double* bl_out;    // 4 x nx: deltastar theta Ht Reth
    double* ubulk;     // 5: mass flux through the five planes (last step)
    double* sumxz;     // nx: wall-shear accumulator
    double* tauw_win;  // nx: mean of the last completed wall-shear window
    double area_mf;    // Av = x3(nz) (x2(ny-1) - x2(2)) (1-based); dnssetbl (x3(nz-1) - x3(2)) (x2(ny-1) - x2(2))
    double stats_A;    // x2(ny) - x2(2) (dnstbl2/dnstbl.f90:442); dnssetbl ny - 2
    double stats_dA;   // dy; dnssetbl 1 (unweighted)
    std::vector<double> x3h;  // host copy of x3
    int* slab_of_k;    // nz: slab index of each interior plane
    tbl::DevScalars* sc;
    // GMRES small arrays (kmax+1)^2 + 4(kmax+1)
    double *h, *gg, *gc, *gs, *gy;
    // reductions
    tbl::RedWork red;
    // wavefront
    double* halo;                  // [2 buffers][3 comps][2 sides][P] planes
    unsigned long long* flags;     // [3 comps][n_cta]
    tbl::SweepCta* ctas;           // [n_cta]
    tbl::SlabDesc* slabs;          // [P]
    int n_cta;
    int sweep_kc;                  // CTAs of a slab column (plane groups): one thread-block cluster
    int sweep_cluster[2][3][8];    // per precision, sweep mode and grid.y: 1 cluster launch, 0 cooperative, -1 unknown
    unsigned long long epoch;
    int* err;                      // device error word
    // host side
    double* hpin;                  // pinned readback
    cudaEvent_t ahead_ev[2];       // Arnoldi steps enqueued ahead: the copy of step k's estimate done
    cudaStream_t stream;
    int64_t launches;
    double npts;                   // nx*ny*nz reference points (algorithmic byte counts)
    int nstep, cont, nstat;
    int cnt2;  // steps this program has run (originalTBL's inflow ramp)
    double time;
    bool fluc_updated;
    int coop_ok;
    int ssor_nib;                  // streamwise SSOR blocks per line (TBL_FLAG_SSOR_STREAM_BLOCKS), 1..SSOR_MAX_NIB
    int gs_comps_per_launch;       // velocity components one cooperative GS launch can hold (1..3)
    int n_sm;                      // multiprocessors of the device
    // replay
    std::vector<int32_t> replay;
    size_t replay_pos;
    std::vector<int32_t> last_counts;
    double lamda_host;
    // wall control and the adjoint window (tbl_adjoint.cu)
    double* wallw;          // nx*(ny-2) wall-normal wall velocity, null = 0
    double *AbT, *AtT;      // transposed wall-normal coefficients: AbT[k] = At[k-1], AtT[k] = Ab[k+1]
    double* tape_u1;        // when set, one_step copies the post-inflow velocities here (3 x vol)
    unsigned char* conv_bits;  // frozen-branch record of this step (vol bytes), with conv_bits_mode
    int conv_bits_mode;        // TBL_BRANCH_*
    tbl::AdjTape* adj;
    std::vector<double> x1h;  // host copy of x1
    // kernel-group timing (tbl_profile)
    struct ProfMark { int group; int e0, e1; double bytes; int64_t launches; };
    bool prof_on;
    std::vector<cudaEvent_t> prof_ev;
    size_t prof_used;
    std::vector<ProfMark> prof_marks;
    double prof_ms[TBL_PROF_NGROUPS];
    double prof_bytes[TBL_PROF_NGROUPS];
    int64_t prof_n[TBL_PROF_NGROUPS];
};

namespace tbl {
// Records a CUDA event pair around a group of launches when profiling is on.
struct ProfScope {
    tbl_handle* h;
    int group;
    double bytes;
    int e0;
    int64_t l0;  // h->launches when the scope opened
    ProfScope(tbl_handle* h_, int g_, double b_);
    ~ProfScope();
};
int prof_drain(tbl_handle* h);
}  // namespace tbl
