/*
 * tbl_gpu.h -- C ABI of the GB300 (sm_103a) time-step library for the
 * spatially developing turbulent boundary layer DNS of theparvezahmad/turbulentBL.
 *
 * The library replaces the body of the reference's time loop
 *     dnstbl2/dnstbl.f90:538-2375  (do while (nstep < maxstep) ... end do)
 * i.e. the recycling inflow, convection + explicit RHS, Gauss-Seidel implicit
 * diffusion, divergence, SSOR-preconditioned GMRES pressure-Poisson solve,
 * projection, boundary conditions, per-step statistics and the every-`cum`
 * recycling/rescaling bookkeeping.  The reference has no plugin or FFI API of
 * its own: its state is the program-global arrays Ut, Press, PCorr, usum2,
 * vsum2, wsum2, Wt, Ufluc, new, lamda and the mesh x1,x2,x3,Jac,Jac2.  Every
 * entry point below names the reference lines whose state or work it takes
 * over.
 *
 * Conventions (identical to the reference arrays):
 *   - 3-D fields are Fortran column-major, i (streamwise) fastest, then j
 *     (spanwise, periodic, j=1 and j=ny are ghost copies of ny-1 and 2), then
 *     k (wall-normal, wall at k=1).  Size nx*ny*nz doubles.
 *   - 2-D statistics arrays are (nx, nz), i fastest.
 *   - Index arrays (new(k)) hold the reference's 1-based values.
 *   - Host pointers are borrowed for the duration of a call only; the handle
 *     owns all device memory.  One host thread per handle.
 *   - Every function returns TBL_OK (0) or a negative TBL_ERR_* code; nothing
 *     aborts or throws across the ABI.
 */
#ifndef TBL_GPU_H
#define TBL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TBL_ABI_VERSION 1

/* status codes */
#define TBL_OK                 0
#define TBL_ERR_CUDA          -1  /* a CUDA runtime call failed */
#define TBL_ERR_BAD_ARG       -2  /* invalid configuration or pointer */
#define TBL_ERR_NOT_CONVERGED -3  /* GS or GMRES hit mmax (reference continues silently) */
#define TBL_ERR_NAN           -4  /* NaN/Inf found in the state after a step */
#define TBL_ERR_BLOWUP        -5  /* u',v' or w' > 25 (reference STOP, dnstbl2/dnstbl.f90:1749-1775) */
#define TBL_ERR_TIMEOUT       -6  /* a bounded device wait gave up */
#define TBL_ERR_NO_DEVICE     -7  /* no CUDA device / library built without it */
#define TBL_ERR_REPLAY        -8  /* replay counts exhausted or inconsistent */
#define TBL_ERR_ZERO_RHS      -9  /* zero preconditioned PPE residual at restart 1 (reference divides by zero) */

/* precision modes */
#define TBL_PREC_FP64   0   /* the plain method: every field and operation in FP64 */
#define TBL_PREC_MIXED  1   /* FP32 stencils/storage/inner GMRES inside FP64 iterative refinement */

/* Variants: the reference's three programs of the same method.  Their
 * differences on the time step are switched by tbl_config.variant; cum,
 * recycle_after and nproc stay separate parameters (originalTBL: 1000 and
 * 1000, dnssetbl: freqTimAvg = 500 for both).  Adjoint windows and the
 * red-black mode take TBL_VARIANT_DNSTBL2 only. */
#define TBL_VARIANT_DNSTBL2   0  /* dnstbl2/dnstbl.f90 (default) */
#define TBL_VARIANT_ORIGINAL  1  /* originalTBL/fnldnstbl.f90: Peclet windows Pe > 2 without the upper bounds
                                    (:665, :689, :711); inflow u mean ramped from Ume1 to the recycled mean,
                                    eps = min(cnt2 * 5e-5, 1) with cnt2 = tbl_state.cnt2 (:561-587, :2382);
                                    divergence print sqrt(|sum|/N) (:1586); wall-shear window 1000 steps
                                    (:1679-1681) */
#define TBL_VARIANT_DNSSETBL  2  /* dnssetbl/dnssetbl.f90: Pe = |Re u h| > 2 (:311, :323, :335); second-order
                                    central y convection on the first/last span rows (:325-326); inflow
                                    eps = min(nstep * 5e-5, 1) ramp of the u mean, v mean times lamda, blend
                                    weight Wt(1,k) (:259-300); Gauss-Seidel also stops when the L1 residual
                                    sum < 1e-12 (a REAL(4) literal, :392); slabs nz/P from k = 1 with the
                                    remainder on the last ranks (:78-92); unweighted span statistics
                                    (:936-983); rescaling when mod(nstep, cum) = 0 (:986) with the recycled
                                    plane refreshed on rank 0's slab (:1033-1041); fluctuations and KE when
                                    cont > recycle_after over i = 2..nx-1 (:1223-1254); mass flux over each
                                    slab's own planes, divided by (x3(nz-1)-x3(2))(x2(ny-1)-x2(2))
                                    (:884-896) */

/* flags */
#define TBL_FLAG_REPLAY        1  /* follow counts given by tbl_set_replay instead of testing convergence */
#define TBL_FLAG_PPE_RESIDUAL  2  /* compute the true relative PPE residual after each solve */
#define TBL_FLAG_RB_ORDER      8  /* throughput mode, not the reference's sweep order: red-black (i+j+k odd/even)
                                     ordering of the implicit-diffusion Gauss-Seidel sweeps (one global block,
                                     periodic in j), so every sweep is two fully parallel passes; the converged
                                     solves are the same systems */
#define TBL_FLAG_RB_PRECOND   16  /* with TBL_FLAG_RB_ORDER: the SSOR preconditioner of GMRES red-black ordered
                                     too.  A weaker preconditioner (about 2.7x the GMRES iterations at
                                     512x128x128), kept for experiments */
#define TBL_FLAG_SSOR_SPAN_BLOCKS 32  /* throughput mode, not the reference's preconditioner: the block SSOR of
                                     GMRES also splits every slab into blocks of 32 span rows (zero halos
                                     between blocks, as between slabs), so a preconditioner sweep is
                                     nx/4 + 32 + K wavefront steps long instead of nx/4 + (ny-2) + K */
#define TBL_FLAG_SSOR_STREAM_BLOCKS 64  /* throughput mode, not the reference's preconditioner: the block SSOR
                                     also splits every line into up to four streamwise blocks (zero halo
                                     between them), as many as keep the sweep's CTAs co-resident, cutting the
                                     nx/4 part of the wavefront chain */
#define TBL_FLAG_DIAGNOSTICS   4  /* accepted for compatibility: the divergence, mass-flux, wall-shear and
                                     KE diagnostics run every step, as in the reference */

/* Run parameters.  The reference hard-codes all of them as literals
 * (dnstbl2/dnstbl.f90:20-140); here they are one plain struct. */
typedef struct tbl_config {
    int32_t nx, ny, nz;     /* n3d(1..3); ny includes the 2 periodic ghost rows */
    int32_t nproc;          /* virtual MPI ranks P (slab decomposition in k, :469-475) */
    int32_t irec;           /* recycling plane, 1-based (reference: 68, :560) */
    int32_t cum;            /* recycling / statistics window in steps (reference: 5, :115) */
    int32_t istat;          /* statistics period (reference: 1, :28) */
    int32_t recycle_after;  /* recycled inflow when nstep > this (reference: 5, :557) */
    int32_t kmax;           /* GMRES restart length (reference: 50, :138) */
    int32_t mmax;           /* max GS sweeps and max GMRES restarts (reference: 1000, :139) */
    int32_t precision;      /* TBL_PREC_* */
    int32_t flags;          /* TBL_FLAG_* */
    int32_t mixed_kmax;     /* inner FP32 GMRES restart length (mixed mode), 1..63 */
    int32_t mixed_max_outer;/* max FP64 refinement sweeps (mixed mode) */
    double dt;              /* time step (reference: 1e-4, :34) */
    double re;              /* Reynolds number (reference: 150.92, :48) */
    double ue;              /* free-stream velocity (reference: 19.798, :113) */
    double dx, dy, dxi;     /* uniform spacings in x1, x2 and the computational xi (:401-403) */
    double omega;           /* SSOR relaxation w (reference: REAL(4) 1.835, :140) */
    double errtol;          /* GMRES relative tolerance (reference: 1e-5, :137) */
    double errorstop;       /* GS L1 residual ratio (reference: 1e-6, :23) */
    double mixed_inner_tol; /* inner FP32 GMRES relative tolerance (mixed mode) */
    double mixed_outer_tol; /* FP64 refinement residual target, relative (mixed mode) */
    double mixed_true_tol;  /* mixed mode: also refine until ||Q8 - L7 p'||_2 / ||Q8||_2 <= this (0 = off) */
    int32_t variant;        /* TBL_VARIANT_*: which of the reference's programs the step follows */
    int32_t reserved_;      /* zero */
} tbl_config;

/* Mesh, host-computed once (dnstbl2/dnstbl.f90:392-426): x1(nx), x2(ny),
 * x3(nz), Jac(nz) = dx3/dxi and Jac2(nz) = d2x3/dxi2, NOT inverted. */
typedef struct tbl_mesh {
    const double* x1;
    const double* x2;
    const double* x3;
    const double* jac;
    const double* jac2;
} tbl_mesh;

/* The restart state (the 15 columns of 3D.tp, dnstbl2/dnstbl.f90:350-358,
 * plus the scalars the program carries).  Used for upload and download; in
 * download any pointer may be NULL to skip that array. */
typedef struct tbl_state {
    double* u; double* v; double* w;        /* Ut(:,:,:,1..3), nx*ny*nz */
    double* p;                              /* Press */
    double* pcorr;                          /* PCorr (GMRES warm start) */
    double* usum2; double* vsum2; double* wsum2;  /* recycling means (nx,nz) */
    double* wt;                             /* Wt(nx,nz) */
    double* uf; double* vf; double* wf;     /* Ufluc(:,:,:,1..3), nx*ny*nz */
    int32_t* newk;                          /* new(nz), 1-based */
    double* ume1;                           /* Ume1(1,k): fixed inflow mean, nz */
    double* bltkns;                         /* boundary-layer thickness bltkns(nx) */
    double lamda;                           /* u_tau ratio (reset to 1 at start, :441) */
    double time;
    int32_t nstep;                          /* from the 3D.tp header */
    int32_t cont;                           /* steps since program start (drives cum) */
    int32_t ksep;                           /* last inner index of the previous rescaling */
    int32_t cnt2;                           /* steps this program has run (originalTBL's cnt2, :143 :2382);
                                               drives TBL_VARIANT_ORIGINAL's inflow ramp */
} tbl_state;

/* Per-step report (replaces the reference's stdout/ASCII monitors). */
typedef struct tbl_step_stats {
    int32_t nstep;
    int32_t status;
    int32_t gs_sweeps[3];       /* GS sweeps per velocity component */
    int32_t gmres_restarts;     /* GMRES outer restarts m */
    int32_t gmres_iters;        /* total Arnoldi steps over all restarts */
    int32_t cum_step;           /* 1 when the rescaling bookkeeping ran */
    int32_t outer_iters;        /* mixed mode: FP64 refinement sweeps */
    int32_t pad_;
    double gs_resid[3];         /* final GS L1 ratio sumav */
    double gmres_resid;         /* final GMRES estimate |g(kit+1)|/rho_0 */
    double ppe_rel_resid;       /* ||L7 p' - Q8||_2 / ||Q8||_2 (flag TBL_FLAG_PPE_RESIDUAL) */
    double div_diag;            /* |sum div| / N, the reference's printout (:1571-1577) */
    double ke;                  /* kinetic energy of fluctuations (:1724-1741) */
    double lamda;               /* current lamda */
    double time;
} tbl_step_stats;

/* Statistics and rescaling outputs (dnstbl2/dnstbl.f90:1902-2277). */
typedef struct tbl_stats_out {
    double* usum; double* vsum; double* wsum;          /* running sums (nx,nz) */
    double* uusum; double* vvsum; double* wwsum;
    double* uvsum; double* uwsum; double* vwsum;
    double* deltastar; double* theta; double* ht; double* reth;  /* (nx), last rescaling */
    double* tauw_sum;     /* sumxz(nx): span sums of the wall shear, accumulated every step (:1616-1668) */
    double* ubulk;        /* UbDNS(5): mass flux through the planes i = 5,20,40,60,85 (1-based, clamped
                             to nx-1), divided by the cross-section area (:1578-1594), last step */
    double lamda03;
    int32_t nstat;
    int32_t pad_;
    double* tauw_window;  /* sumxz/500 of the last completed 500-step window (:1670-1681); the
                             reference's Cf is 2 tauw_window / (Ue^2 (ny-2)) */
} tbl_stats_out;

typedef struct tbl_handle tbl_handle;

/* Create a handle on the current CUDA device; allocates all device memory,
 * computes the stencil coefficients (dnstbl2/dnstbl.f90:487-536). */
int tbl_create(const tbl_config* cfg, const tbl_mesh* mesh, tbl_handle** out);

/* Upload the restart state (replaces the 3D.tp read, :350-358). */
int tbl_upload_state(tbl_handle* h, const tbl_state* st);

/* Advance nsteps time steps (the loop body :538-2375).  stats may be NULL,
 * else it receives nsteps records. */
int tbl_step(tbl_handle* h, int32_t nsteps, tbl_step_stats* stats);

/* Download the state (replaces the 3D%03d.tp write, :2380-2397). */
int tbl_download_state(tbl_handle* h, tbl_state* st);

/* Download the statistics accumulators and rescaling outputs. */
int tbl_download_stats(tbl_handle* h, tbl_stats_out* out);
/* The statistics of the last rescaling: the running sums divided by cum
 * before they are reset (dnstbl2/dnstbl.f90:2021-2049, :2063-2078) -- u, v,
 * w, uu, vv, ww, uv, uw, vw, nx*nz doubles each (Fortran order), 9*nx*nz in
 * all; zeros before the first rescaling. */
int tbl_download_averages(tbl_handle* h, double* avg);

/* Replay iteration counts (parity runs).  rec is a sequence of per-step
 * records {gs1, gs2, gs3, nrestarts, kit_1 .. kit_nrestarts}; used when
 * TBL_FLAG_REPLAY is set.  The library copies the array. */
int tbl_set_replay(tbl_handle* h, const int32_t* rec, int64_t len);

/* Iteration-count record of the most recent step in the replay format.
 * Returns the record length (>= 4) or a negative status; writes at most cap. */
int tbl_last_counts(tbl_handle* h, int32_t* buf, int32_t cap);

/* Replace only the 3-D fields (u, v, w, p and, when non-NULL, pcorr) and keep
 * the recycling state, statistics accumulators and step counters: the
 * per-step entry of a host driver that owns Ut/Press/PCorr in its own arrays
 * (the reference's program-global arrays, dnstbl2/dnstbl.f90:172-321). */
int tbl_upload_fields(tbl_handle* h, const double* u, const double* v, const double* w, const double* p,
                      const double* pcorr);

/* Kernel-group timing with CUDA events on the library's stream.  enable=1
 * turns it on (and clears the totals), 0 turns it off.  tbl_profile_read
 * copies per-group totals: milliseconds, algorithmic bytes and kernel
 * launches, for TBL_PROF_NGROUPS groups (indices TBL_PROF_*). */
#define TBL_PROF_CONV      0  /* convection + explicit RHS */
#define TBL_PROF_GS_SWEEP  1  /* GS wavefront sweeps */
#define TBL_PROF_GS_RESID  2  /* GS residual checks */
#define TBL_PROF_SSOR_FWD  3  /* fused L7 matvec + forward SSOR sweep */
#define TBL_PROF_SSOR_BWD  4  /* backward SSOR sweep */
#define TBL_PROF_MGS       5  /* Gram-Schmidt passes with fused reductions */
#define TBL_PROF_SMALL     6  /* Givens / back substitution / restart set-up */
#define TBL_PROF_VEC       7  /* normalisation and p' update */
#define TBL_PROF_BC        8  /* divergence, projection, boundary conditions */
#define TBL_PROF_STATS     9  /* statistics, diagnostics, rescaling */
#define TBL_PROF_TOTAL    10  /* whole tbl_step calls, device time between events on the stream */
#define TBL_PROF_NGROUPS  11
int tbl_profile(tbl_handle* h, int enable);
int tbl_profile_read(tbl_handle* h, double* ms, double* bytes, int64_t* launches, int ngroups);

/* ---- Allocation-free divergence diagnostic ------------------------------
 * No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory (a host code whose own pool allocator owns
 * every byte of the GPU, or a time loop in which an allocation could
 * synchronise the device).  It computes the reference's divergence printout
 * |sum div U| / ((nx-2)(ny-2)(nz-2)) (the value tbl_step reports as div_diag;
 * its square root for cfg->variant == TBL_VARIANT_ORIGINAL) for fields the caller already holds on the current device, and allocates
 * nothing: its only scratch is a fixed array of TBL_NOALLOC_BLOCKS doubles in
 * the library image, held by every GPU that loads the library until exit.
 *   cfg     grid sizes, dx, dy, dxi and variant (other fields unused)
 *   jacinv  device, nz doubles: 1/Jac(k)
 *   u,v,w   device, nx*ny*nz doubles each, the reference layout (i fastest)
 *   out     device, one double receiving the result
 * Runs asynchronously on the legacy default stream.  Every call looks up the
 * scratch address on the current device; the first call on a device also
 * loads the library's kernels there (make it before any stream capture).
 * Calls share the scratch: calls that overlap on the GPU race.  Grids with
 * more than TBL_NOALLOC_MAX_POINTS interior points are rejected with
 * TBL_ERR_TOO_LARGE. */
#define TBL_ERR_TOO_LARGE     -10
/* A restart or counter file could not be opened, read, parsed or written. */
#define TBL_ERR_IO            -11
#define TBL_NOALLOC_BLOCKS     4096
#define TBL_NOALLOC_MAX_POINTS ((int64_t)TBL_NOALLOC_BLOCKS * 256 * 64)
int tbl_div_diag_noalloc(const tbl_config* cfg, const double* jacinv, const double* u, const double* v,
                         const double* w, double* out);

/* ---- Wall control and the discrete adjoint of a window of steps ---------
 * The reference has no adjoint; it holds w = 0 at the wall
 * (dnstbl2/dnstbl.f90:1317-1319).  tbl_set_wall_control replaces that value
 * of w with a steady blowing/suction profile c, used by every later step:
 *   w(i, j, k=1) = c[(i-1) + nx*(j-2)]   for i = 1..nx, j = 2..ny-1 (1-based)
 * (nx*(ny-2) doubles; the spanwise ghost rows follow by the periodic copy).
 * c = NULL restores w = 0.  FP64 and mixed handles alike. */
int tbl_set_wall_control(tbl_handle* h, const double* c);

/* Objective of a window of W steps: the time average over the steps of the
 * span- and patch-averaged wall shear (dw/dx + du/dz)/Re at the wall,
 * with the reference's wall-shear stencils (dnstbl2/dnstbl.f90:1636-1660:
 * 6th-order central dw/dx, 2nd order within 3 points of the i ends;
 * one-sided 2nd-order du/dz on the stretched grid) over the columns
 * i = 2..nx-1 whose x1(i) lies in [x_lo, x_hi]. */
typedef struct {
    double x_lo, x_hi;    /* streamwise extent of the wall-shear patch */
    int32_t ckpt_every;   /* checkpoint interval in steps (>= 1) */
    int32_t branch_mode;  /* TBL_BRANCH_*: the convection's data-dependent decisions */
} tbl_window_config;

/* The convection switches stencils on Peclet windows and on the sign of the
 * advecting velocity (:651-713), so the step is only piecewise smooth.  For
 * checking gradients by finite differences a window can record those
 * decisions (one byte per point and step) and later windows of the same
 * length can replay them, which makes the forward map exactly the one the
 * adjoint differentiates.  TBL_BRANCH_FREE is the reference behaviour. */
#define TBL_BRANCH_FREE    0
#define TBL_BRANCH_RECORD  1
#define TBL_BRANCH_REPLAY  2

/* Host field pointers (the reference layout, nx*ny*nz doubles; NULL = none). */
typedef struct {
    double *u, *v, *w, *p;
} tbl_fields;

typedef struct {
    int32_t steps;             /* W */
    int32_t recomputed_steps;  /* forward steps re-run from checkpoints */
    int32_t adj_gs_sweeps;     /* Gauss-Seidel sweeps of the transposed solves */
    int32_t adj_gmres_iters;   /* GMRES iterations of the transposed Poisson solves */
    int32_t status, pad_;
    double max_gs_resid;       /* worst final relative residual of the transposed solves */
    double max_gmres_resid;
    double forward_ms;         /* host wall time of the last tbl_forward_window */
    double backward_ms;        /* host wall time of this tbl_backward_window */
} tbl_adjoint_stats;

/* Advance nsteps steps exactly as tbl_step does (FP64 handles), recording a
 * checkpoint of the state every wc->ckpt_every steps for a later
 * tbl_backward_window, and return the window objective in *objective.  The
 * recycling means, Wt, new(k) and lamda must stay fixed over the window: a
 * window that would reach a rescaling step (every `cum` steps) is rejected
 * with TBL_ERR_BAD_ARG, as are a replay handle, the throughput-mode flags
 * (red-black, span or streamwise SSOR blocks) and variants other than
 * TBL_VARIANT_DNSTBL2. */
int tbl_forward_window(tbl_handle* h, int32_t nsteps, const tbl_window_config* wc, double* objective,
                       tbl_step_stats* stats);

/* Discrete adjoint of the last forward window (reverse sweep over the
 * recorded checkpoints, recomputing each segment's steps).  The map
 * differentiated is the step with converged solves: the implicit-diffusion
 * and pressure-Poisson adjoints are solves with the transposed operators
 * (same Gauss-Seidel / SSOR-GMRES code, transposed wall-normal
 * coefficients, the handle's errorstop / errtol), and the branch decisions
 * (Peclet windows, upwind sides) are those of the recorded trajectory.
 *   dL_dJ       weight of the window objective in the loss L
 *   dL_dfinal   dL/d(state after the window) (u, v, w, p), or NULL
 *   dL_dc       out: dL/dc, nx*(ny-2) doubles (layout of tbl_set_wall_control)
 *   dL_dinitial out: dL/d(state before the window), or NULL
 * Afterwards the handle holds the state at the end of the window again. */
int tbl_backward_window(tbl_handle* h, double dL_dJ, const tbl_fields* dL_dfinal, double* dL_dc,
                        tbl_fields* dL_dinitial, tbl_adjoint_stats* stats);

/* Release everything. */
void tbl_destroy(tbl_handle* h);

const char* tbl_status_string(int status);

/* Number of kernel launches issued by this handle so far (instrumentation). */
int64_t tbl_launch_count(tbl_handle* h);

/* Failure-detection self-test (no handle): one kernel thread waits, with the
 * wavefront sweeps' bounded wait, on a progress flag that nothing sets.  The
 * wait gives up after its poll limit (about a second) and the kernel reports
 * TBL_ERR_TIMEOUT in *observed, as a stalled sweep does in tbl_step; the
 * device stays usable.  Returns TBL_OK when the self-test itself ran;
 * *seconds (may be NULL) receives the time the wait took. */
int tbl_selftest_bounded_wait(int32_t* observed, double* seconds);

/* ------------------------------------------------------------ restart files
 * Host-only readers and writers of the reference's restart files (no device,
 * no handle): Tecplot ASCII POINT, i outermost, then j, then k.  Arrays are
 * those of tbl_state / tbl_mesh (Fortran order, nx*ny*nz and nx*nz); ranges
 * are 1-based and inclusive.  The state's time and nstep go to the title.
 * Values are written with 15 significant digits (E22.15), as the reference
 * writes them. */
#define TBL_TP_DNSTBL2   0  /* 15 columns x y z U V W P Um Vm Wm Uf Vf Wf Wt Nk (dnstbl2/dnstbl.f90:2357-2384) */
#define TBL_TP_ORIGINAL  1  /* 8 columns x y z U V W T P, T written as 0 (originalTBL/fnldnstbl.f90:1696-1717) */
#define TBL_TP_DNSSETBL  2  /* 7 columns x y z U V W P (dnssetbl/dnssetbl.f90:908-932) */

/* One file of points i = 1..nx, j = j0..j1, k = k0..k1.  header: 0 none (the
 * files of ranks > 0), 1 the program's own writer (dnssetbl's title also
 * carries nproc), 2 the merger's.  Replaces the WRITE loops at
 * dnstbl2/dnstbl.f90:2357-2377. */
int tbl_tp_write(const char* path, int32_t format, const tbl_mesh* mesh, const tbl_state* st, int32_t nx,
                 int32_t ny, int32_t nz, int32_t j0, int32_t j1, int32_t k0, int32_t k1, int32_t header,
                 int32_t nproc);
/* The per-rank files dir/3D%03d.tp (dir/3D%03d.dat for dnssetbl) of an
 * nproc-rank run: j = 2..ny-1 and the rank's k range (dnstbl2/dnstbl.f90:
 * 469-485, 2357-2377; dnssetbl/dnssetbl.f90:78-92, 908-932). */
int tbl_tp_write_ranks(const char* dir, int32_t format, const tbl_mesh* mesh, const tbl_state* st, int32_t nx,
                       int32_t ny, int32_t nz, int32_t nproc);
/* Merge the per-rank files in dir into out_path with every j (the periodic
 * ghost rows filled), as dnstbl/restart.f90:17-86, originalTBL/restart.f90
 * and dnssetbl/combineFile.f90 do. */
int tbl_tp_merge(const char* dir, int32_t format, int32_t nz, int32_t nproc, const char* out_path);
/* Read a merged file (every j) into st (any array pointer may be NULL to
 * skip it) and x1/x2/x3 (may be NULL); sets st->time and st->nstep
 * (dnstbl2/dnstbl.f90:147-159, 350-358).  The file's zone must be nx, ny, nz. */
int tbl_tp_read(const char* path, int32_t format, int32_t nx, int32_t ny, int32_t nz, double* x1, double* x2,
                double* x3, tbl_state* st);
/* The counter files dir/cnt ("nz cnt proc") and dir/cnt2 (:147-153, :2054-2056, :2349-2352). */
int tbl_counters_write(const char* dir, int32_t nz, int32_t cnt, int32_t nproc, int32_t cnt2);
int tbl_counters_read(const char* dir, int32_t* nz, int32_t* cnt, int32_t* nproc, int32_t* cnt2);
/* dnssetbl's statData.dat: usum2, vsum2, wsum2 at plane irec, Wt(1,k), new(k)
 * per k, FORMAT(4(1X,F15.7),I5.3) (dnssetbl/dnssetbl.f90:1203-1208, 136-140). */
int tbl_statdata_write(const char* path, int32_t nx, int32_t nz, int32_t irec, const tbl_state* st);
int tbl_statdata_read(const char* path, int32_t nx, int32_t nz, int32_t irec, tbl_state* st);
/* The inflow mean profile file U_innerdns.dat (dnssetbl: Input/initProf.dat):
 * 37 records FORMAT(24X,E18.8), plane 37's value repeated above it
 * (dnstbl2/dnstbl.f90:322-345; originalTBL/fnldnstbl.f90:411-423;
 * dnssetbl/dnssetbl.f90:105-114).  The read fills ume1[0..nz-1] (records
 * beyond nz are read and dropped); the write puts k and x3(k) in the 24
 * skipped columns and needs nz >= 37. */
#define TBL_INFLOW_RECORDS 37
int tbl_inflow_profile_read(const char* path, int32_t nz, double* ume1);
int tbl_inflow_profile_write(const char* path, int32_t nz, const double* x3, const double* ume1);

/* ------------------------------------------------------------ monitor files
 * Host-only writers of the files the reference's rank 0 writes during a run,
 * record for record and in its edit descriptors.  Files the reference opens
 * with ACCESS='APPEND' get the records appended, the others are rewritten.
 * (nx,nz) arrays in Fortran order.  The values come from tbl_step_stats,
 * tbl_download_stats, tbl_download_state and tbl_download_averages; the
 * schedule (every step, every 500 steps, every rescaling, every 100th step
 * of a rescaling) is the caller's, as in turbulentbl_gb300/monitor.py. */
/* massflow.xy: time, UbDNS(1..5), 6(1X,F15.7) (dnstbl2/dnstbl.f90:1613-1615) */
int tbl_monitor_massflow(const char* path, double time, const double* ubulk);
/* numrcltauwall.xy, per i = 2..nx-1: time, x1, tauw/(ny-2), Cf, 4(1X,F15.7)
 * (:1670-1681); tauw_window as in tbl_stats_out */
int tbl_monitor_tauwall(const char* path, double time, int32_t nx, int32_t ny, double ue, const double* x1,
                        const double* tauw_window);
/* kineticenergy.dat: time, ke, 2(2X,E20.10) (:1718-1721) */
int tbl_monitor_kinetic_energy(const char* path, double time, double ke);
/* lamda.dat: time, lamda, lamda03, 3(2X,F20.10) (:2170-2174) */
int tbl_monitor_lamda(const char* path, double time, double lamda, double lamda03);
/* W.dat (rewritten): x1, x3, Wt per (i,k), 3(1X,F15.7) (:2180-2188) */
int tbl_monitor_blend(const char* path, int32_t nx, int32_t nz, const double* x1, const double* x3, const double* wt);
/* boundarylthickness.dat (rewritten): time, x1, bltkns, deltastar, theta,
 * Ht, Reth per i, 7(2X,F20.10) (:2258-2267) */
int tbl_monitor_bl_thickness(const char* path, double time, int32_t nx, const double* x1, const double* bltkns,
                             const double* deltastar, const double* theta, const double* ht, const double* reth);
/* k.dat: k, new(k), eta(k) per k, (I5,2(F20.10)) (:2286-2292) */
int tbl_monitor_knew(const char* path, int32_t nz, const int32_t* newk, const double* eta);
/* meanvalues.dat: x1, x3, usum2, vsum2, wsum2 per (i,k), 5(1X,F15.7)
 * (:2296-2302) */
int tbl_monitor_meanvalues(const char* path, int32_t nx, int32_t nz, const double* x1, const double* x3,
                           const double* usum2, const double* vsum2, const double* wsum2);
/* Umeanvalues.dat (rewritten): the same and x3*Re, 6(1X,F15.7) (:2098-2104) */
int tbl_monitor_umeanvalues(const char* path, int32_t nx, int32_t nz, const double* x1, const double* x3,
                            const double* usum2, const double* vsum2, const double* wsum2, double re);
/* means / medians / taustress (rewritten): one record of a, b, c, 0 per
 * (i,k), 4(1X,F15.7) each (:2021-2049) -- the u v w, uu vv ww or uv uw vw
 * blocks of tbl_download_averages */
int tbl_monitor_averages(const char* path, int32_t nx, int32_t nz, const double* a, const double* b,
                         const double* c);

#ifdef __cplusplus
}
#endif
#endif /* TBL_GPU_H */
