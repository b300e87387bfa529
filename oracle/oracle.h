/*
 * FP64 CPU oracle for the RegOT dense dual-evaluation hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path
 * is compared against (and the timed CPU baseline). Product code never
 * links, loads or calls it.
 *
 * It restates, in plain C++17 without Eigen, the math and control flow of
 * the reference solvers of yixuan/regot-python:
 *   src/sinkhorn_problem_bcd.cpp, src/sinkhorn_problem_obj.cpp,
 *   src/sinkhorn_result.h, src/sinkhorn_bcd.cpp, src/sinkhorn_newton.cpp,
 *   src/sinkhorn_lbfgs_dual.cpp, src/sinkhorn_apdagd.cpp,
 *   src/sinkhorn_sparse_newton.cpp, src/sinkhorn_splr.cpp, src/sinkhorn_sparsify4.cpp,
 *   src/sinkhorn_ssns.cpp, src/sinkhorn_problem_ls.cpp, src/sinkhorn_hess.cpp,
 *   src/sinkhorn_sparsify3.cpp, src/sinkhorn_linsolve.cpp, src/sinkhorn_cg.cpp,
 *   src/qrot_problem.cpp, src/approx_proj.h, src/qrot_result.h,
 *   src/qrot_lbfgs_dual.cpp, src/qrot_assn.cpp, src/qrot_hess.cpp,
 *   src/qrot_bcd.cpp, src/qrot_gd.cpp, src/qrot_apdagd.cpp, src/qrot_pdaam.cpp,
 *   src/qrot_grssn.cpp, src/qrot_lbfgs_semi_dual.cpp, src/pdip_cg.cpp, src/pdip_fp.cpp,
 *   src/pdip_transport_ops.hpp, src/pdip_block_operator.h, src/pdip_sparse_chol.cpp,
 *   src/qrot_linsolve.cpp, src/qrot_cg.cpp, src/LBFGSpp/LBFGS.h,
 *   src/LBFGSpp/LBFGSpp/BFGSMat.h, src/LBFGSpp/LBFGSpp/LineSearchNocedalWright.h,
 *   src/LBFGSpp/LBFGSpp/Param.h, src/solvers.cpp (kwargs defaults).
 *
 * Parity status: pinned at 8-bit resolution to the reference's own outputs,
 * and otherwise by known answers. The reference ships no tests, fixtures or
 * golden vectors, and it cannot be compiled here (its numerics need Eigen
 * 5.0.1, which setup.py downloads at build time). Its only outputs are the
 * four plan images of its README (figs/plan_*.png: sinkhorn_bcd reg 0.1,
 * sinkhorn_ssns reg 0.01, qrot_pdip "cg" reg 0.1 and "fp" reg 0.01 on the
 * 100 x 80 README example). The oracle's plans fall, entry for entry, in
 * the colormap bins of those images (tests/test_reference_images_cpu.py).
 * Beyond that the oracle is checked against known-answer problems
 * (separable costs with closed-form plans), KKT conditions, and independent
 * numpy/scipy restatements in tests/.
 *
 * Storage: M is column-major n x m (column j contiguous), like the Eigen
 * MatrixXd the reference computes on; loops run j-outer, i-inner as there.
 * Plans are written row-major n x m (REGOT_USE_ROW_MAJOR_MATRIX, config.h:5).
 */
#ifndef REGOT_ORACLE_H
#define REGOT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Options; defaults of SinkhornSolverOpts (sinkhorn_solvers.h:35-37) and
 * QROTSolverOpts (qrot_solvers.h:28-30). x0 == NULL means "not given". */
typedef struct {
    const double* x0;
    int x0_len;
    int method;
    double mu0;
    double shift;
    double density;
    double tau;
} oracle_opts;

/* Caller-owned result buffers. History arrays have capacity hist_cap.
 * plan may be NULL (skipped). densities / prim_vals may be NULL. */
typedef struct {
    int niter;
    int hist_len;
    int hist_cap;
    double* dual;
    double* plan;
    double* obj_vals;
    double* mar_errs;
    double* run_times;
    double* densities;
    double* prim_vals;
    char err[256];
} oracle_result;

/* ---- EROT problem pieces (M column-major) ---- */
void oracle_erot_optimal_beta(const double* M, int n, int m, const double* b,
                              double reg, const double* alpha, double* beta);
void oracle_erot_optimal_alpha(const double* M, int n, int m, const double* a,
                               double reg, const double* beta, double* alpha);
double oracle_erot_dual_obj(const double* M, int n, int m, const double* a,
                            const double* b, double reg, const double* gamma);
double oracle_erot_dual_obj_grad(const double* M, int n, int m, const double* a,
                                 const double* b, double reg,
                                 const double* gamma, double* grad);
/* y = H x with H the exact dual Hessian (sinkhorn_problem_obj.cpp:396-418). */
void oracle_erot_hvp(const double* M, int n, int m, const double* a,
                     const double* b, double reg, const double* gamma,
                     const double* x, double* y);
/* Newton direction -H^{-1} g by a dense Cholesky of the Schur complement. */
int oracle_erot_newton_direction(const double* M, int n, int m, const double* a,
                                 const double* b, double reg,
                                 const double* gamma, double* direc);
/* T = exp((alpha (+) [beta~, 0] - M)/reg), written column-major. */
double oracle_erot_compute_T(const double* M, int n, int m, double reg,
                             const double* gamma, double* T);
/* sparsify_mat3 (sinkhorn_sparsify3.cpp:276-405). T column-major n x m.
 * Output CSC of the kept entries of the first m-1 columns:
 * outer[m] (m entries: 0..m-1), inner[cap], values[cap]. Returns nnz,
 * or -1 if cap is too small. */
long oracle_sparsify_mat3(const double* T, int n, int m, double delta,
                          double density_hint, int* outer, int* inner,
                          double* values, long cap);
/* sparsify_mat_with_density (sinkhorn_sparsify4.cpp:77-174, preserve =
 * true), same output convention as oracle_sparsify_mat3. */
long oracle_sparsify_density(const double* T, int n, int m, double density,
                             int* outer, int* inner, double* values, long cap);
/* line_search_wolfe (sinkhorn_problem_ls.cpp:226-436) on the quartic with
 * coefficients c[0..4]. */
double oracle_wolfe_poly(const double* c, double init_step, int* recompute,
                         int* nev);
void oracle_erot_plan(const double* M, int n, int m, double reg,
                      const double* gamma, double* plan_rowmajor);

/* ---- EROT solvers ---- */
int oracle_sinkhorn_bcd(const double* M, int n, int m, const double* a,
                        const double* b, double reg, double tol, int max_iter,
                        int verbose, const oracle_opts* opts,
                        oracle_result* res);
int oracle_sinkhorn_newton(const double* M, int n, int m, const double* a,
                           const double* b, double reg, double tol,
                           int max_iter, int verbose, const oracle_opts* opts,
                           oracle_result* res);
int oracle_sinkhorn_ssns(const double* M, int n, int m, const double* a,
                         const double* b, double reg, double tol, int max_iter,
                         int verbose, const oracle_opts* opts,
                         oracle_result* res);
int oracle_sinkhorn_lbfgs_dual(const double* M, int n, int m, const double* a,
                               const double* b, double reg, double tol,
                               int max_iter, int verbose,
                               const oracle_opts* opts, oracle_result* res);
int oracle_sinkhorn_sparse_newton(const double* M, int n, int m,
                                  const double* a, const double* b, double reg,
                                  double tol, int max_iter, int verbose,
                                  const oracle_opts* opts, oracle_result* res);
int oracle_sinkhorn_splr(const double* M, int n, int m, const double* a,
                         const double* b, double reg, double tol, int max_iter,
                         int verbose, const oracle_opts* opts, oracle_result* res);
int oracle_sinkhorn_apdagd(const double* M, int n, int m, const double* a,
                           const double* b, double reg, double tol,
                           int max_iter, int verbose, const oracle_opts* opts,
                           oracle_result* res);

/* ---- QROT problem pieces ---- */
double oracle_qrot_dual_obj(const double* M, int n, int m, const double* a,
                            const double* b, double reg, double tau,
                            const double* gamma);
double oracle_qrot_dual_obj_grad(const double* M, int n, int m,
                                 const double* a, const double* b, double reg,
                                 double tau, const double* gamma, double* grad);
void oracle_qrot_optimal_beta(const double* M, int n, int m, const double* b,
                              double reg, const double* alpha, double* beta);
double oracle_qrot_primal_val(const double* M, int n, int m, const double* a,
                              const double* b, double reg,
                              const double* gamma);
/* Generalized-Jacobian solve (H + shift I)^{-1} rhs by Schur CG
 * (qrot_cg.cpp:9-50); sigma = 1[alpha_i + beta_j - M_ij > 0]. */
int oracle_qrot_hess_cg(const double* M, int n, int m, const double* gamma,
                        const double* rhs, double shift, double tau,
                        double cg_tol, double* res);
void oracle_qrot_plan(const double* M, int n, int m, double reg,
                      const double* gamma, double* plan_rowmajor);

/* ---- QROT solvers ---- */
int oracle_qrot_lbfgs_dual(const double* M, int n, int m, const double* a,
                           const double* b, double reg, double tol,
                           int max_iter, int verbose, const oracle_opts* opts,
                           oracle_result* res);
int oracle_qrot_bcd(const double* M, int n, int m, const double* a,
                    const double* b, double reg, double tol, int max_iter,
                    int verbose, const oracle_opts* opts, oracle_result* res);
int oracle_qrot_gd(const double* M, int n, int m, const double* a,
                   const double* b, double reg, double tol, int max_iter,
                   int verbose, const oracle_opts* opts, oracle_result* res);
int oracle_qrot_apdagd(const double* M, int n, int m, const double* a,
                       const double* b, double reg, double tol, int max_iter,
                       int verbose, const oracle_opts* opts, oracle_result* res);
int oracle_qrot_pdaam(const double* M, int n, int m, const double* a,
                      const double* b, double reg, double tol, int max_iter,
                      int verbose, const oracle_opts* opts, oracle_result* res);
int oracle_qrot_lbfgs_semi_dual(const double* M, int n, int m, const double* a,
                                const double* b, double reg, double tol,
                                int max_iter, int verbose, const oracle_opts* opts,
                                oracle_result* res);
int oracle_qrot_grssn(const double* M, int n, int m, const double* a,
                      const double* b, double reg, double tol, int max_iter,
                      int verbose, const oracle_opts* opts, oracle_result* res);
/* qrot_pdip (pdip_cg.cpp:206-413, pdip_fp.cpp:278-667): inner_solver 0 =
 * "cg", 1 = "fp". Plan row-major; res->dual[0] = converged flag. popts
 * (NULL for the defaults): cg_max_iter, fixed_threshold, fp_max_iter,
 * fp_exit_scale, fp_stop_gap_mu_only, cg_stop_gap_mu_only, cg_mar_tol. */
int oracle_qrot_pdip(const double* M, int n, int m, const double* a,
                     const double* b, double reg, double tol, int max_iter,
                     int inner_solver, const double* popts, oracle_result* res);
/* optimal_alpha: qrot_problem.cpp:409-419. */
void oracle_qrot_optimal_alpha(const double* M, int n, int m, const double* a,
                               double reg, const double* beta, double* alpha);
int oracle_qrot_assn(const double* M, int n, int m, const double* a,
                     const double* b, double reg, double tol, int max_iter,
                     int verbose, const oracle_opts* opts, oracle_result* res);

#ifdef __cplusplus
}
#endif

#endif /* REGOT_ORACLE_H */
