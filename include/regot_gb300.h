/*
 * regot_gb300 -- C ABI of the GB300 (sm_103a) implementation of RegOT's dense
 * dual-evaluation hot path.
 *
 * The reference exposes its solvers through one pybind11 module,
 * regot._internal (src/solvers.cpp:463-569); each solver takes
 * (M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs) and returns a
 * result object with niter / dual / plan / obj_vals / mar_errs / run_times
 * (+ densities for EROT, prim_vals for QROT). The entry points below are what
 * a binding of that module needs: one call per solver with plain pointers and
 * sizes, caller-owned output buffers, an int status and a per-context error
 * string. No torch or CUDA types appear in the signatures; device pointers
 * are accepted where a descriptor says so.
 *
 * Threading: one regot_ctx per host thread; calls on one context are not
 * thread-safe. Every call is synchronous with respect to the host.
 */
#ifndef REGOT_GB300_H
#define REGOT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. Python maps INVALID_ARG to ValueError and the others to
 * RuntimeError, like pybind11 maps the reference's std::invalid_argument and
 * std::runtime_error / std::logic_error (src/solvers.cpp:280,290;
 * src/LBFGSpp/LBFGSpp/LineSearchNocedalWright.h:93-117,227,247,267). */
enum {
    REGOT_OK = 0,
    REGOT_ERR_INVALID_ARG = 1,
    REGOT_ERR_NONFINITE = 2,
    REGOT_ERR_LINESEARCH = 3,
    REGOT_ERR_CUDA = 4,
    REGOT_ERR_TIMEOUT = 5,
    REGOT_ERR_NUMERIC = 6,
    REGOT_ERR_NO_DEVICE = 7,
    REGOT_ERR_TOO_LARGE = 8   /* problem exceeds a fixed scratch maximum */
};

enum { REGOT_F64 = 0, REGOT_F32 = 1 };              /* element type of M */
enum { REGOT_MEM_HOST = 0, REGOT_MEM_DEVICE = 1 };  /* where a buffer lives */
/* Arithmetic of the dense passes. FP64: M stored in FP64 and every
 * element-wise operation in FP64 (the plain comparator). MIXED: M stored in
 * FP32, exponent/relu arguments formed with an exact hi/lo split of the FP64
 * duals, FP32 exp2 and accumulation in short FP32 chunks merged in FP64;
 * duals, objective differences and marginal errors stay FP64. */
enum { REGOT_PREC_FP64 = 0, REGOT_PREC_MIXED = 1 };

typedef struct regot_ctx regot_ctx;
typedef struct regot_dproblem regot_dproblem;

/* Dense problem description. M is n x m row-major with row stride ldm
 * elements (ldm >= m); a has n entries, b has m entries (FP64). */
typedef struct {
    const void* M;
    int M_dtype;     /* REGOT_F64 or REGOT_F32 */
    int M_mem;       /* REGOT_MEM_HOST or REGOT_MEM_DEVICE */
    long long ldm;
    int n, m;
    const double* a;
    const double* b;
    int ab_mem;      /* REGOT_MEM_HOST or REGOT_MEM_DEVICE */
} regot_problem_desc;

/* Solver options. Defaults (regot_opts_init) follow SinkhornSolverOpts
 * (src/sinkhorn_solvers.h:35-37) and QROTSolverOpts (src/qrot_solvers.h:28-30),
 * with the per-solver overrides of src/solvers.cpp:124,415,433,451. */
typedef struct {
    int precision;        /* REGOT_PREC_* (default MIXED) */
    int method;           /* linear solver selector; -1 = solver default */
    double mu0;           /* SSNS initial shift factor (1.0) */
    double shift;         /* (1e-3) */
    double density;       /* (0.01) */
    double tau;           /* QROT extra regularisation (0.0) */
    const double* x0;     /* optional initial duals on the host, or NULL */
    int x0_len;
    double cg_tol;        /* relative residual target of the Newton-CG solve and of the
                             SSNS method-1 solve (1e-10) */
    int cg_max_iter;      /* per linear solve (0 = solver default: Newton 2*(n+m),
                             SSNS method 0 2*(m-1), method 1 10*(m-1)) */
    int verbose;
    int plan;             /* 1 = fill result->plan, 0 = skip */
    int plan_mem;         /* REGOT_MEM_HOST or REGOT_MEM_DEVICE */
    int prim_vals;        /* QROT: 1 = evaluate prim_vals every iteration */
} regot_opts;

/* Caller-owned result buffers (host unless plan_mem says otherwise).
 * History arrays need hist_cap >= max_iter + 2 entries; any may be NULL. */
typedef struct {
    int niter;
    int hist_len;
    int hist_cap;
    double* dual;      /* n+m-1 (EROT, beta_m = 0 gauge) or n+m (QROT) */
    double* plan;      /* n*m row-major FP64, or NULL */
    double* obj_vals;
    double* mar_errs;
    double* run_times; /* cumulative milliseconds, device clock */
    double* densities; /* EROT SSNS */
    double* prim_vals; /* QROT */
    /* statistics of the call */
    long long passes;  /* streamed passes over M */
    double solve_ms;   /* device time of the solve, upload excluded */
} regot_result;

void regot_opts_init(regot_opts* opts);

/* Context: one CUDA device, one stream, a workspace grown on demand. */
int regot_ctx_create(int device, regot_ctx** out);
void regot_ctx_destroy(regot_ctx* ctx);
const char* regot_ctx_last_error(const regot_ctx* ctx);
/* Launch on an external cudaStream_t (as void*). NULL is the CUDA legacy
 * default stream, as in the CUDA runtime; regot_ctx_set_stream(ctx,
 * regot_ctx_own_stream(ctx)) restores the context's own stream. */
int regot_ctx_set_stream(regot_ctx* ctx, void* stream);
void* regot_ctx_own_stream(const regot_ctx* ctx);
/* Number of kernels this context has launched so far. */
long long regot_ctx_kernel_launches(const regot_ctx* ctx);

/* Device-resident problem: M is converted to the storage of `precision`
 * (FP64 or FP32, rows padded to 16 bytes) once; solves reuse it. */
int regot_problem_create(regot_ctx* ctx, const regot_problem_desc* desc, int precision,
                         regot_dproblem** out);
/* Frees the problem's device memory on its context's stream and waits for
 * it. Destroy every problem of a context before the context itself. */
void regot_problem_destroy(regot_dproblem* prob);

/* Page-locked host memory for result buffers (the n x m plan): a device to
 * host copy into it runs at the full link bandwidth, where a copy into
 * pageable memory is staged by the driver. Freed blocks are kept (up to
 * 4 GiB) and reused. No counterpart in the reference, which returns plans in
 * ordinary heap memory (src/sinkhorn_result.h:32-50). */
int regot_host_alloc(size_t bytes, void** out);
void regot_host_free(void* ptr);

/* ---- Solvers (reference: src/solvers.cpp:359-441 and 69-148) ---- */

/* sinkhorn_bcd (src/sinkhorn_bcd.cpp:14-124). */
int regot_sinkhorn_bcd(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                       int max_iter, const regot_opts* opts, regot_result* res);
/* sinkhorn_newton (src/sinkhorn_newton.cpp:17-129); the Newton system is
 * solved matrix-free by CG on the exact Hessian instead of a dense LLT. */
int regot_sinkhorn_newton(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                          int max_iter, const regot_opts* opts, regot_result* res);
/* sinkhorn_ssns (src/sinkhorn_ssns.cpp:16-234). */
int regot_sinkhorn_ssns(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                        int max_iter, const regot_opts* opts, regot_result* res);
/* sinkhorn_sparse_newton (src/sinkhorn_sparse_newton.cpp:24-171): Newton
 * steps on the density-sparsified Hessian (opts->density, default 0.01;
 * shift min(||g||, opts->shift)) with the More-Thuente line search. */
int regot_sinkhorn_sparse_newton(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                                 int max_iter, const regot_opts* opts, regot_result* res);
/* sinkhorn_splr (src/sinkhorn_splr.cpp:24-200): sparse-plus-low-rank
 * quasi-Newton steps (BFGS correction of the sparsified Hessian). */
int regot_sinkhorn_splr(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                        int max_iter, const regot_opts* opts, regot_result* res);
/* sinkhorn_lbfgs_dual (src/sinkhorn_lbfgs_dual.cpp:81-126). */
int regot_sinkhorn_lbfgs_dual(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                              int max_iter, const regot_opts* opts, regot_result* res);
/* sinkhorn_apdagd (src/sinkhorn_apdagd.cpp:14-183); the returned plan is
 * the averaged primal plan, the dual the last extrapolated point. */
int regot_sinkhorn_apdagd(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                          int max_iter, const regot_opts* opts, regot_result* res);
/* qrot_lbfgs_dual (src/qrot_lbfgs_dual.cpp:81-126). */
int regot_qrot_lbfgs_dual(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                          int max_iter, const regot_opts* opts, regot_result* res);
/* qrot_bcd (src/qrot_bcd.cpp:14-103): exact alternating minimisation. */
int regot_qrot_bcd(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol, int max_iter,
                   const regot_opts* opts, regot_result* res);
/* qrot_gd (src/qrot_gd.cpp:14-120): gradient descent with Armijo backtracking. */
int regot_qrot_gd(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol, int max_iter,
                  const regot_opts* opts, regot_result* res);
/* qrot_apdagd (src/qrot_apdagd.cpp:14-179): accelerated primal-dual adaptive
 * gradient descent; the plan output is the averaged plan. */
int regot_qrot_apdagd(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                      int max_iter, const regot_opts* opts, regot_result* res);
/* qrot_pdaam (src/qrot_pdaam.cpp:14-188): primal-dual accelerated
 * alternating minimisation; the plan output is the averaged plan. */
int regot_qrot_pdaam(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                     int max_iter, const regot_opts* opts, regot_result* res);
/* qrot_grssn (src/qrot_grssn.cpp:16-133): regularized semi-smooth Newton with
 * shift opts->shift (default 1e-3) and Armijo backtracking; tau must be 0. */
int regot_qrot_grssn(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                     int max_iter, const regot_opts* opts, regot_result* res);
/* qrot_lbfgs_semi_dual (src/qrot_lbfgs_semi_dual.cpp:84-126): L-BFGS on the
 * semi-dual in alpha, beta = optimal_beta(alpha); dual = (alpha, beta). */
int regot_qrot_lbfgs_semi_dual(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                               int max_iter, const regot_opts* opts, regot_result* res);
/* Options of qrot_pdip (PDIPSolverOpts, src/pdip_solvers.h:16-35, as parsed
 * by parse_pdip_opts, src/solvers.cpp:203-239). */
typedef struct {
    int inner_solver;         /* 0 = "cg" (default), 1 = "fp" */
    int cg_max_iter;          /* 1000 */
    double fixed_threshold;   /* 1e-9 */
    int fp_max_iter;          /* 800 */
    double fp_exit_scale;     /* 1e-2 */
    int fp_stop_gap_mu_only;  /* 1 */
    int cg_stop_gap_mu_only;  /* 0 */
    double cg_mar_tol;        /* 1e-10 */
} regot_pdip_opts;
void regot_pdip_opts_init(regot_pdip_opts* popts);
/* qrot_pdip (src/solvers.cpp:268-292; pdip_cg.cpp:206-413 and
 * pdip_fp.cpp:278-667): primal-dual interior point for QROT. Fills niter,
 * hist_len, obj_vals, mar_errs, run_times and the plan (the primal x) of
 * res (res->dual is not used); *converged (may be NULL) receives the
 * converged flag. Only opts->verbose, plan and plan_mem are read. */
int regot_qrot_pdip(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol, int max_iter,
                    const regot_pdip_opts* popts, const regot_opts* opts, regot_result* res,
                    int* converged);
/* qrot_assn (src/qrot_assn.cpp:16-170). */
int regot_qrot_assn(regot_ctx* ctx, regot_dproblem* prob, double reg, double tol,
                    int max_iter, const regot_opts* opts, regot_result* res);

/* ---- Pass-level entry points (host vectors in and out) ---- */

/* ---- Batched EROT (no reference counterpart: the reference solves one
 * problem per call) ---- */

/* `count` independent problems with squared-Euclidean costs computed on the
 * fly from point clouds: M_ij = s_p sum_k (x_ik - y_jk)^2 in FP32, problem p
 * with n_p rows, m_p columns, d_p <= REGOT_BATCH_MAX_DIM dimensions and cost
 * scale s_p (NULL: 1). Points and marginals are concatenated over the
 * problems: x holds sum n_p d_p floats (problem p's n_p x d_p row-major block
 * after those of problems < p), y likewise, a sum n_p and b sum m_p doubles.
 * Sizes and scales are host arrays; `mem` says where x, y, a and b live. */
#define REGOT_BATCH_MAX_DIM 16
typedef struct {
    int count;
    const int* n;
    const int* m;
    const int* d;
    const double* cost_scale;
    const float* x;
    const float* y;
    const double* a;
    const double* b;
    int mem;
} regot_batch_desc;

/* Results, host buffers: duals concatenated like a and b, gauge-fixed per
 * problem as sinkhorn_bcd returns them (alpha + beta_m, beta - beta_m, so
 * every problem's last beta is 0); per-problem iteration counts and final
 * marginal errors. */
typedef struct {
    double* alpha;
    double* beta;
    int* niter;
    double* mar_err;
    long long sweeps;   /* out: sweeps run by the batch (the slowest problem) */
    double solve_ms;    /* out: device time of the solve */
} regot_batch_result;

/* sinkhorn_bcd (src/sinkhorn_bcd.cpp:14-124) on every problem of the batch
 * at once: one row and one column log-sum-exp kernel per sweep over all
 * problems still running, each problem stopping at its own iteration with
 * the reference's test (marginal error < tol, or max_iter). The sweeps run
 * as a device-side loop; the last few problems finish in the tail kernel
 * (regot_set_batch_tail). */
int regot_erot_solve_batched(regot_ctx* ctx, const regot_batch_desc* desc, double reg, double tol,
                             int max_iter, regot_batch_result* res);
/* The half-sweeps of a dimension class (d <= 4, <= 8, <= 16) run either on
 * the CUDA cores (direct differences, FP32) or with the cost tile x y' on
 * the tensor cores (tcgen05, TF32 hi/lo split operands, FP32 accumulation,
 * M = s (|x|^2 + |y|^2 - 2 x.y)): about 2^-21 s (|x|^2 + |y|^2) absolute
 * error in M instead of the direct difference's relative FP32 rounding.
 * The first batch with problems of a class on a device times one row
 * half-sweep of each and keeps the faster for the process.
 * regot_force_batch_variant(0 | 1) forces one for every class (-1: the timed
 * choice) and returns the previous forced value; regot_batch_variants
 * fills out[3] with the timed choices so far (-1: not yet timed). No
 * counterpart in the reference. */
int regot_force_batch_variant(int variant);
int regot_batch_variants(regot_ctx* ctx, int* out);
/* The last problems of a batch: once at most `max_active` problems are still
 * running, the remaining sweeps run in one launch of thread-block clusters,
 * one cluster of 16 CTAs (8 where the device cannot hold clusters of 16) per
 * running problem, each running its problem's
 * sweeps to its stop with cluster barriers between the half-sweeps (the
 * same arithmetic and stopping test as the per-sweep kernels). 0 keeps the
 * per-sweep kernels to the end; a value >= the batch size runs the whole
 * solve this way after the first two sweeps. Returns the previous setting
 * (default REGOT_BATCH_TAIL_DEFAULT). No counterpart in the reference. */
#define REGOT_BATCH_TAIL_DEFAULT 64
int regot_set_batch_tail(int max_active);

/* regot_erot_solve_batched followed by its backward (no counterpart in the
 * reference, which has no derivatives): at each problem's returned duals,
 * cost[p] = a'alpha + b'beta - reg sum T (the regularised OT cost, the
 * negated dual objective of src/sinkhorn_problem_obj.cpp:324-342) and, by
 * the envelope theorem dL/dM = T with M_ij = s |x_i - y_j|^2,
 * grad_x = 2 s sum_j T_ij (x_i - y_j), grad_y = 2 s sum_i T_ij (y_j - x_i),
 * laid out like desc->x and desc->y and, like the points, FP32 (they are
 * accumulated in FP32). Host buffers, each optional (NULL); res->solve_ms
 * then covers the solve and the backward. */
int regot_erot_solve_batched_grad(regot_ctx* ctx, const regot_batch_desc* desc, double reg,
                                  double tol, int max_iter, regot_batch_result* res, double* cost,
                                  float* grad_x, float* grad_y);

/* ---- Derivatives of EROT solves (no reference counterpart) ---- */

/* Solve H x = rhs with the exact dual Hessian at gamma, the matrix that
 * sinkhorn_newton factors (src/sinkhorn_newton.cpp:91-92; H from
 * src/sinkhorn_problem_obj.cpp:396-418), by Jacobi-preconditioned CG to
 * ||H x - rhs|| < tol ||rhs|| (max_iter <= 0: 2 (n + m - 1) steps). Host
 * vectors of n + m - 1 entries; *iters receives the CG steps taken. */
int regot_erot_hess_solve(regot_ctx* ctx, regot_dproblem* prob, double reg, const double* gamma,
                          const double* rhs, double tol, int max_iter, double* x, int* iters);
/* Weighted plan contraction without an n x m intermediate:
 *   G_ij = T_ij                               (u == NULL), or
 *   G_ij = T_ij (u_i + u_{n+j} - W_ij) / reg   (u given; W may be NULL),
 *   rows_i = sum_j G_ij (rows may be NULL), Z = G Y (Y m x d, Z n x d, row-major),
 * with T = exp((alpha (+) [beta~, 0] - M)/reg). gamma and u have n + m - 1
 * entries, W is n x m row-major. mem (REGOT_MEM_HOST / DEVICE) applies to
 * every array argument. */
int regot_erot_tyy(regot_ctx* ctx, regot_dproblem* prob, double reg, const double* gamma,
                   const double* u, const double* W, const double* Y, int d, double* rows,
                   double* Z, int mem);
/* M = scale * (squared Euclidean distance of row i of x and row j of y), by
 * direct differences (no |x|^2 + |y|^2 - 2 x.y cancellation): x n x d, y
 * m x d, M n x m with row stride ldm, all row-major DEVICE arrays of dtype
 * (REGOT_F32 or REGOT_F64). Enqueued on the context's stream, not
 * synchronised. The cost of the point-cloud losses of the torch wrapper; no
 * counterpart in the reference, which takes M as given. */
int regot_sqeuclid_cost(regot_ctx* ctx, const void* x, const void* y, int n, int m, int d,
                        double scale, int dtype, void* M, long long ldm);
/* The column-side contraction of the same G: cols_j = sum_i G_ij (cols may
 * be NULL) and Z = G'X (X n x d, Z m x d, row-major); the dL/dy of a
 * squared-Euclidean cost is 2 (cols o y - Z) / scale. FP32 storage runs both
 * contractions on the tensor cores (tcgen05, BF16 hi/lo split operands,
 * FP32 accumulation: about 1e-5 relative per product); FP64 storage on the
 * CUDA cores in FP64. No counterpart in the reference. */
int regot_erot_tty(regot_ctx* ctx, regot_dproblem* prob, double reg, const double* gamma,
                   const double* u, const double* W, const double* X, int d, double* cols,
                   double* Z, int mem);

/* Problem::optimal_beta / optimal_alpha (src/sinkhorn_problem_bcd.cpp:149-201). */
int regot_erot_optimal_beta(regot_ctx* ctx, regot_dproblem* prob, double reg,
                            const double* alpha, double* beta);
int regot_erot_optimal_alpha(regot_ctx* ctx, regot_dproblem* prob, double reg,
                             const double* beta, double* alpha);
/* Problem::dual_obj_grad (src/sinkhorn_problem_obj.cpp:363-393);
 * gamma has n+m-1 entries (beta_m = 0). */
int regot_erot_dual_obj_grad(regot_ctx* ctx, regot_dproblem* prob, double reg,
                             const double* gamma, double* obj, double* grad);
/* y = H x with H the dual Hessian of dual_obj_grad_densehess
 * (src/sinkhorn_problem_obj.cpp:396-418), without forming H. */
int regot_erot_hvp(regot_ctx* ctx, regot_dproblem* prob, double reg, const double* gamma,
                   const double* x, double* y);
/* SinkhornResult::get_plan (src/sinkhorn_result.h:32-50); plan row-major. */
int regot_erot_plan(regot_ctx* ctx, regot_dproblem* prob, double reg, const double* gamma,
                    double* plan, int plan_mem);
/* sparsify_mat3 (src/sinkhorn_sparsify3.cpp:276-405) of T(gamma) with the
 * threshold delta and the density hint that selects find_small (> 0.2) or
 * find_large, as dual_sparsified_hess calls it (src/sinkhorn_problem_obj.cpp:432-443).
 * *nnz = number of kept entries of the first m-1 columns, exact zeros of T
 * included (the reference's SparseMatrix::nonZeros()). If mask is not NULL it
 * receives the kept nonzero entries as a row-major n x (m-1) array of 0/1. */
int regot_erot_sparsify(regot_ctx* ctx, regot_dproblem* prob, double reg, const double* gamma,
                        double delta, double density_hint, long long* nnz, int* mask);
/* sparsify_mat_with_density (src/sinkhorn_sparsify4.cpp:77-174, preserve =
 * true) of T(gamma), as dual_sparsified_hess_with_density calls it
 * (src/sinkhorn_problem_obj.cpp:446-457): the largest floor(n (m-1) density)
 * entries of the first m-1 columns plus the first row and column. Entries
 * tied with the threshold value are all kept. *nnz = number of kept nonzero
 * entries; mask as for regot_erot_sparsify. */
int regot_erot_sparsify_density(regot_ctx* ctx, regot_dproblem* prob, double reg,
                                const double* gamma, double density, long long* nnz, int* mask);
/* The selection stages of both sparsifications run with each row and column
 * in registers when n and m - 1 are at most 16384 (FP32) or 8192 (FP64),
 * else from shared memory; the two give the same thresholds and the same
 * kept entries. regot_force_sparsify_path(1) makes every later
 * sparsification take the shared-memory path (0: the default choice) and
 * returns the previous setting. No counterpart in the reference. */
int regot_force_sparsify_path(int shared_memory);
/* The Schur-complement CG of qrot_assn and qrot_grssn (hess_cg,
 * src/qrot_cg.cpp:9-50) multiplies by sigma either from the n x m bitmask
 * of the generalized Jacobian pass or from row and column index lists built
 * from it, with the whole CG in one thread-block cluster; the lists are
 * taken when sigma holds at most n m / 64 entries. The cluster exchanges
 * the CG vectors through distributed shared memory when 8 (n + m) bytes fit
 * in 200 KB, else through global memory. regot_force_qrot_cg_path forces a
 * path (1: bitmask, 2: index lists, 3: index lists with the global-memory
 * exchange, 0: the choice by size) and returns the previous setting. All
 * give the same directions up to rounding. No counterpart in the
 * reference. */
int regot_force_qrot_cg_path(int mode);
/* QROT Problem::dual_obj_grad (src/qrot_problem.cpp:226-253). */
int regot_qrot_dual_obj_grad(regot_ctx* ctx, regot_dproblem* prob, double reg,
                             const double* gamma, double* obj, double* grad);
/* QROT Problem::optimal_beta (src/qrot_problem.cpp:397-404). */
int regot_qrot_optimal_beta(regot_ctx* ctx, regot_dproblem* prob, double reg,
                            const double* alpha, double* beta);
/* QROT Problem::optimal_alpha (src/qrot_problem.cpp:409-419). */
int regot_qrot_optimal_alpha(regot_ctx* ctx, regot_dproblem* prob, double reg,
                             const double* beta, double* alpha);
/* QROT Problem::primal_val (src/qrot_problem.cpp:10-24, src/approx_proj.h:6-26). */
int regot_qrot_primal_val(regot_ctx* ctx, regot_dproblem* prob, double reg,
                          const double* gamma, double* value);
/* QROTResult::get_plan (src/qrot_result.h:31-43). */
int regot_qrot_plan(regot_ctx* ctx, regot_dproblem* prob, double reg, const double* gamma,
                    double* plan, int plan_mem);

/* ---- Measurement ---- */

/* Kinds of dense pass for regot_time_pass (each is one streamed read of M,
 * plus the writes noted). */
enum {
    REGOT_PASS_EROT_ROW = 0,      /* row log-sum-exp pass of sinkhorn_bcd */
    REGOT_PASS_EROT_COL = 1,      /* column log-sum-exp pass of sinkhorn_bcd */
    REGOT_PASS_EROT_GRAD = 2,     /* fused row+column sums (objective / gradient) */
    REGOT_PASS_EROT_HVP = 3,      /* Hessian-vector product */
    REGOT_PASS_QROT_GRAD = 4,     /* QROT relu objective / gradient */
    REGOT_PASS_EROT_LS = 5,       /* objective changes at 4 step sizes (Armijo, line_selection) */
    REGOT_PASS_EROT_GRADLS = 6,   /* L-BFGS / More-Thuente trial: gradient + exact change */
    REGOT_PASS_EROT_AVG = 7,      /* APDAGD averaged plan (X read and written) */
    REGOT_PASS_EROT_PLAN = 8,     /* FP64 plan written to device memory */
    REGOT_PASS_EROT_ROWMAX = 9,   /* optimal_alpha anchor (row max) */
    REGOT_PASS_EROT_COLMAX = 10,  /* optimal_beta anchor (column max) */
    REGOT_PASS_QROT_GRADMASK = 11,/* QROT gradient + Jacobian bitmask written */
    REGOT_PASS_QROT_GRADLS = 12,  /* QROT line-search trial */
    REGOT_PASS_QROT_OBJ = 13,     /* QROT objective only */
    REGOT_PASS_QROT_P1 = 14,      /* primal_val pass 1 (row sums) */
    REGOT_PASS_QROT_P2 = 15,      /* primal_val pass 2 (weighted column sums) */
    REGOT_PASS_QROT_P3 = 16,      /* primal_val pass 3 (value terms) */
    REGOT_PASS_QROT_COLROOT = 17, /* optimal_beta Newton round (FP64 accumulation) */
    REGOT_PASS_QROT_ROWROOT = 18, /* optimal_alpha Newton round (FP64 accumulation) */
    REGOT_PASS_QROT_AVG = 19,     /* QROT averaged plan (X read and written) */
    REGOT_PASS_QROT_PLAN = 20,    /* FP64 QROT plan written to device memory */
    REGOT_PASS_COUNT = 21
};
/* Enqueue `reps` launches of one dense pass over M on the context's stream
 * and return without synchronising, so that the caller can bracket them
 * with its own events. The inputs are fixed, deterministic vectors (duals 0
 * for the EROT passes and 0.1 for the QROT passes). The first call for a
 * (problem, kind, reg) also prepares the pass inputs (in mixed precision
 * the FP32 split and one pass) and synchronises before enqueueing; later
 * calls enqueue the `reps` passes only. No counterpart in the reference: it
 * measures the kernels behind the solvers above. */
int regot_time_pass(regot_ctx* ctx, regot_dproblem* prob, int kind, double reg, int reps);
/* Algorithmic bytes of one pass of `kind` over prob (M read once in its
 * storage type, plus the plan, averaged-plan or bitmask traffic the pass
 * writes); -1 for an invalid argument. */
long long regot_pass_bytes(regot_dproblem* prob, int kind);
/* Limit (polls of about 200 us) of the dense passes' bounded waits on their
 * parameter copies; returns the previous limit, and a negative value
 * restores the default (16384). A pass whose wait gives up drains the copy
 * under the default limit, marks its result invalid and the call returns
 * REGOT_ERR_TIMEOUT; 0 makes every such wait give up at once. Process-wide;
 * for exercising the timeout path. No counterpart in the reference. */
long long regot_set_wait_limit(long long spins);

/* ---- Autotuner of the dense passes (no counterpart in the reference,
 * whose passes are fixed Eigen loops, e.g. src/sinkhorn_problem_bcd.cpp:82-146
 * and src/sinkhorn_problem_obj.cpp:16-136) ----
 * Every dense pass has two launch configurations with the same tile shape:
 * 0 = two CTAs per SM (128 registers a thread) with a 4-deep ring of row
 * buffers per warp, 1 = one CTA per SM (255 registers) with an 8-deep ring.
 * regot_autotune times every pass kind under both on a synthetic n x m
 * problem of the given storage precision (`reps` back-to-back launches,
 * CUDA events) and keeps the faster one for (this GPU, precision, pass,
 * size class floor(log2(n m))); later passes of that class (or of the
 * nearest tuned class within two) use it. Choices persist through
 * regot_autotune_save / _load (NULL path: $REGOT_GB300_AUTOTUNE, else
 * ~/.cache/regot_gb300_autotune.tsv, read on the first launch of a process).
 * Untuned passes use configuration 0. */
int regot_autotune(regot_ctx* ctx, int n, int m, int precision, int reps);
int regot_autotune_save(const char* path);   /* entries written, or -1 */
int regot_autotune_load(const char* path);   /* entries read */
void regot_autotune_clear(void);
/* The table as text (one tab-separated line per entry: device, precision,
 * pass, size class, configuration, microseconds of each configuration);
 * copies at most len - 1 bytes and returns the full length. */
size_t regot_autotune_entries(char* buf, size_t len);
/* Force configuration cfg (0 or 1) for every pass; -1 restores the tuned
 * choices. Returns the previous forced value. */
int regot_force_pass_config(int cfg);
/* The configuration a pass of `kind` (REGOT_PASS_*) would use now for an
 * n x m problem of `precision`; -1 on error. */
int regot_pass_config(regot_ctx* ctx, int kind, int precision, int n, int m);

/* ---- Allocation-free variant ----
 * No counterpart in the reference. regot_erot_dual_obj_grad for callers that
 * cannot allocate device memory: code running while another framework
 * captures a CUDA graph (cudaMalloc is not allowed inside such a capture),
 * custom-call hooks of frameworks that own all device memory, and loops that
 * cannot afford cudaMalloc's implicit device synchronisation. It allocates
 * nothing: its scratch is one static device array of
 * REGOT_NOALLOC_SCRATCH_BYTES (16 MiB) that every GPU loading the library
 * holds until exit; a problem that needs more (about 32 (n + m) +
 * 4 n m (1/512 + 1/64) bytes: beyond about n = m = 15400, while n = m = 14000
 * always fits) returns REGOT_ERR_TOO_LARGE. All pointers are device pointers: M is n x m
 * FP32 row-major with row stride ldm (a multiple of 4, 16-byte aligned
 * base), gamma = (alpha, beta~) has n+m-1 entries (beta_m = 0), grad has
 * n+m-1 entries, obj one. The work is enqueued on `stream` (a cudaStream_t,
 * NULL = legacy default) and not synchronised. The first call on a device
 * looks up the scratch address (cudaGetSymbolAddress) and should come before
 * any stream capture. All calls share the scratch: calls that overlap on the
 * GPU race and must be serialised by the caller. A failure on the GPU after
 * the call has returned (a bounded wait of the dense pass that gave up)
 * shows as NaN in grad and *obj; the status only reports argument, size and
 * launch errors. */
#define REGOT_NOALLOC_SCRATCH_BYTES (16u << 20)
int regot_erot_dual_obj_grad_noalloc(const float* M, long long ldm, int n, int m,
                                     const double* gamma, const double* a, const double* b,
                                     double reg, double* grad, double* obj, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* REGOT_GB300_H */
