// tbl_kernels.cuh -- host-side launchers shared between translation units.
#pragma once
#include "tbl_internal.cuh"

namespace tbl {

// tbl_stencil.cu
int launch_save_uold(tbl_handle* h);
int launch_inflow(tbl_handle* h);
int launch_conv_q(tbl_handle* h);
int launch_gs_resid(tbl_handle* h, const int* comps, int ncomp, int nblocks);
int launch_div(tbl_handle* h);
int launch_pc_zero_faces(tbl_handle* h);
int launch_project_bcs(tbl_handle* h);
int launch_div_diag(tbl_handle* h, int nblocks, int slot);
int launch_flux_shear(tbl_handle* h);
int launch_fluc_ke(tbl_handle* h, int nblocks, int slot);
int launch_stats(tbl_handle* h);
int launch_rescale(tbl_handle* h);
int launch_gs_delta_init(tbl_handle* h, int comp);
int launch_gs_delta_apply(tbl_handle* h, int comp);
int launch_gs_delta_restart(tbl_handle* h, int comp);

// tbl_sweep.cu
int build_sweep_ctas(tbl_handle* h);
int check_cooperative(tbl_handle* h);
int launch_gs_sweep(tbl_handle* h, const int* comps, int ncomp, int parity);
int launch_halo_init(tbl_handle* h, int parity);
int launch_ssor_fwd(tbl_handle* h, const double* X, const double* Q8, const int* skip = nullptr);
int launch_ssor_bwd(tbl_handle* h, double* out, const int* skip = nullptr);
int launch_ssor_fwd_f(tbl_handle* h, const float* Xf, const double* PCd, const double* Q8, const int* skip = nullptr,
                      const double* denom = nullptr, float* vout = nullptr);
int launch_ssor_bwd_f(tbl_handle* h, float* out, const int* skip = nullptr);
int selftest_bounded_wait(int* observed, double* seconds);

// tbl_lap.cu: R = scale(k) L7 X by TMA plane tiles (the Arnoldi matvec)
template <typename T>
int launch_lap_tma(tbl_handle* h, const T* X, T* R, T aw, T as, const T* Ab, const T* At, const T* Ap, const T* scale,
                   const int* skip, const double* denom = nullptr, T* vout = nullptr);

// tbl_krylov.cu
int launch_dot(tbl_handle* h, const double* a, const double* b, double* out, int op);
int launch_mgs(tbl_handle* h, double* w, const double* vk, const double* hk, const double* vn, double* out, int op,
               const int* skip = nullptr);
int launch_scale_by_inv(tbl_handle* h, double* w, const double* denom, const int* skip = nullptr);
int launch_givens(tbl_handle* h, int kit, const int* skip = nullptr, double stop_at = 0.0);
int launch_backsub_update(tbl_handle* h, int kit);
int launch_restart_init(tbl_handle* h, int first);
int launch_ppe_resid(tbl_handle* h);
int red_blocks(tbl_handle* h);
int launch_dot_f(tbl_handle* h, const float* a, const float* b, double* out, int op);
int launch_scale_by_inv_f(tbl_handle* h, float* w, const double* denom, const int* skip = nullptr);
int launch_backsub_update_f(tbl_handle* h, int kit);
int launch_restart_init_k(tbl_handle* h, int first, int K1);
int launch_givens_k(tbl_handle* h, int kit, int K1, const int* skip = nullptr, double stop_at = 0.0);
int launch_lsg_f(tbl_handle* h, float* W, int kit, double* hcol, const int* skip = nullptr);

// tbl_api.cu
int readback(tbl_handle* h, const void* dev, size_t bytes);
int put3(tbl_handle* h, double* dst, const double* src);
int get3(tbl_handle* h, double* dst, const double* src);
int gs_solve(tbl_handle* h, const int* target, tbl_step_stats& st, bool zero_ok);
int gmres(tbl_handle* h, const int32_t* rec, std::vector<int32_t>& kits, tbl_step_stats& st);
int one_step(tbl_handle* h, tbl_step_stats* out);

// tbl_adjoint.cu
void adj_free(tbl_handle* h);

}  // namespace tbl
