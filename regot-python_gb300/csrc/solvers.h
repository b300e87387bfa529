// Solver entry points behind the C ABI (capi.cu).
#pragma once

#include "internal.h"

namespace regot {

class ErotOps;

void sinkhorn_bcd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                      const regot_opts& o, regot_result* res);
void sinkhorn_newton_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                         const regot_opts& o, regot_result* res);
void sinkhorn_ssns_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                       const regot_opts& o, regot_result* res);
void sinkhorn_sparse_newton_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol,
                                int max_iter, const regot_opts& o, regot_result* res);
void sinkhorn_splr_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                       const regot_opts& o, regot_result* res);
void erot_sparsify_density_gpu(regot_ctx* ctx, regot_dproblem* P, double reg,
                               const double* gamma, double density, long long* nnz, int* mask);
void sinkhorn_lbfgs_dual_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol,
                             int max_iter, const regot_opts& o, regot_result* res);
void sinkhorn_apdagd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                         const regot_opts& o, regot_result* res);
// sparsify_mat3 of T(gamma) (sinkhorn_sparsify3.cpp:276-405): nnz as the
// reference counts it (kept entries including exact zeros of T) and, if mask
// is not NULL, the stored kept entries as a row-major n x (m - 1) 0/1 mask.
void erot_sparsify_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                       double delta, double density_hint, long long* nnz, int* mask);
// Contraction of G = T or T o (u_i + u_j - W_ij) / reg (erot_grad.cu): rows
// (cols = false) sums = G 1, Z = G Y with Y m x d, Z n x d; columns
// (cols = true) sums = G'1, Z = G'Y with Y n x d, Z m x d. All pointers
// device: gamma and u n + m (last 0), W n x m; Z and Y may be NULL when
// d == 0. FP32 storage runs the tensor-core kernel (erot_tc.cu).
void erot_contract_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, const double* d_gamma,
                       const double* d_u, const double* d_W, const double* d_Y, int d, bool cols,
                       double* d_sums, double* d_Z);
// M = scale * squared Euclidean distances of the rows of x (n x d) and y
// (m x d), row-major with stride ldm, FP32 or FP64 (fp64) throughout.
void sqeuclid_gpu(const void* x, const void* y, int n, int m, int d, double scale, bool fp64,
                  void* M, long long ldm, cudaStream_t st);
void erot_contract_tc(regot_ctx* ctx, regot_dproblem* P, double reg, const double* d_gamma,
                      const double* d_u, const double* d_W, const double* d_Y, int d, bool cols,
                      double* d_sums, double* d_Z);
// Half-sweep variant of the batched BCD per dimension class (erot_batch.cu):
// force one for every class (0 CUDA cores, 1 tensor cores, -1 timed
// choice; returns the previous forced value), and the timed choices made on
// this device so far (-1: none yet) for the classes d <= 4, 8, 16.
int force_batch_variant(int v);
// Batched BCD: the number of running problems at or below which the rest of
// the solve runs in the cluster-per-problem tail kernel (0: never); returns
// the previous value (erot_batch.cu).
int set_batch_tail(int max_active);
int force_sparsify_path(int shared_memory);
// QROT Schur CG products: 0 chosen by the entries of sigma, 1 the bitmask,
// 2 the index lists, 3 the index lists with the vectors exchanged through
// global memory; returns the previous setting (qrot.cu)
int force_qrot_cg_path(int mode);
std::vector<int> batch_variants();
// Batched BCD over point-cloud problems (erot_batch.cu).
// cost, grad_x, grad_y (host, optional): each problem's regularised OT cost
// and its gradients with respect to the points (FP32, like the points), at
// the returned duals.
void erot_solve_batched_gpu(regot_ctx* ctx, const regot_batch_desc* D, double reg, double tol,
                            int max_iter, regot_batch_result* res, double* cost = nullptr,
                            float* grad_x = nullptr, float* grad_y = nullptr);
// H x = rhs with the exact dual Hessian at gamma (host vectors, n + m - 1).
void erot_hess_solve_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                         const double* rhs, double tol, int max_iter, double* x, int* iters);
void qrot_lbfgs_dual_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                         const regot_opts& o, regot_result* res);
void qrot_bcd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                  const regot_opts& o, regot_result* res);
void qrot_gd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                 const regot_opts& o, regot_result* res);
void qrot_apdagd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                     const regot_opts& o, regot_result* res);
void qrot_pdaam_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                    const regot_opts& o, regot_result* res);
void qrot_grssn_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                    const regot_opts& o, regot_result* res);
void qrot_lbfgs_semi_dual_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol,
                              int max_iter, const regot_opts& o, regot_result* res);
void qrot_pdip_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                   const regot_pdip_opts& po, const regot_opts& o, regot_result* res,
                   int* converged);
void qrot_assn_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                   const regot_opts& o, regot_result* res);

// Copy an EROT solve out: gamma = (alpha, beta~) with beta_m = 0 held on the
// device as n + m doubles (last one 0); device histories of length hist_len
// (each array hist_cap apart is not assumed: separate pointers).
void finish_erot_result(ErotOps& ops, const double* d_gamma, const double* hobj,
                        const double* hmar, const double* htime, const double* hdens,
                        int hist_len, int hist_cap, int niter, long long passes,
                        const regot_opts& o, regot_result* res);

}  // namespace regot
