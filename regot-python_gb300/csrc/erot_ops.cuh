// EROT building blocks on top of the dense passes: robust log-sum-exp
// updates (optimal_alpha / optimal_beta), the fused objective/gradient,
// the Hessian-vector product and the plan, plus the small vector kernels
// that merge pass partials in FP64.
#pragma once

#include "device_util.cuh"
#include "internal.h"

namespace regot {

// Partial-sum buffers of one problem shape (sized for the widest pass).
struct PassBuffers {
    PassShape shape{};
    bool mixed = true;
    DBuf<char> rowpart, colpart;
    DBuf<double> totpart;
    void init(int n, int m, bool mixed_, int max_nr, int max_nc, int max_nt, cudaStream_t st) {
        mixed = mixed_;
        shape = mixed ? pass_shape<float>(n, m) : pass_shape<double>(n, m);
        // column partials of the FP64 root-finding pass are FP64 in both modes
        const size_t acc = 8;
        rowpart.alloc((size_t)max_nr * shape.nslabs * n * acc, st);
        colpart.alloc((size_t)max_nc * shape.nrb * m * acc, st);
        totpart.alloc((size_t)max_nt * shape.nblocks, st);
    }
};

// Engine bound to one device problem and one regularisation value.
class ErotOps {
public:
    ErotOps(regot_dproblem* P, double reg, cudaStream_t st);

    int n() const { return n_; }
    int m() const { return m_; }
    bool mixed() const { return mixed_; }
    cudaStream_t stream() const { return st_; }
    const double* a() const { return P_->a; }
    const double* b() const { return P_->b; }
    regot_dproblem* problem() const { return P_; }
    const double* loga() const { return P_->loga; }
    const double* logb() const { return P_->logb; }
    double sum_a() const { return sum_a_; }
    double sum_bt() const { return sum_bt_; }
    double reg() const { return reg_; }
    PassBuffers& buf() { return buf_; }
    // FP32 split of the row / column vectors of the last mixed pass
    // (x = hi, y = lo, z = rx, w = rd), valid until the next pass.
    const float4* rsplit() const { return rsplit_.get(); }
    const float4* csplit() const { return csplit_.get(); }

    // Dense pass with this problem's M, reg and partial buffers.
    void pass(int op, PassParams p);
    // Throw REGOT_ERR_TIMEOUT if a pass gave up a bounded wait (synchronises).
    void check_err();
    int* err_flag() const { return err_.get(); }
    // Dense pass reusing the FP32 split of the previous pass (mixed mode).
    void pass_presplit(int op, PassParams p);
    // The FP32 split of p's vectors alone (mixed mode; no-op in FP64), for
    // passes that follow with pass_presplit.
    void split(const PassParams& p);
    // Writable split arrays, for kernels that update one component (the
    // z = rx / cx entries of a CG vector) between passes.
    float4* rsplit_mut() { return rsplit_.get(); }
    float4* csplit_mut() { return csplit_.get(); }
    PassParams base_params() const;

    // Maximum of |x| over up to two device vectors, into *out (device).
    void maxabs(const double* x, int nx, const double* y, int ny, double* out);

    // beta = optimal_beta(alpha) (robust: column max anchor, then sums).
    void optimal_beta(const double* alpha, double* beta, double* maxabs_scratch);
    // alpha = optimal_alpha(beta).
    void optimal_alpha(const double* beta, double* alpha, double* maxabs_scratch);
    // Row sums r[n] and column sums c[m] of T(alpha, beta) (beta full length).
    void row_col_sums(const double* alpha, const double* beta, double* r, double* c,
                      double* maxabs_scratch);
    // y_r = T x_c (rows), y_c = T' x_r (cols), for T(alpha, beta).
    void tmatvec(const double* alpha, const double* beta, const double* xr, const double* xc,
                 double* yr, double* yc, double* maxabs_scratch);
    // plan = T(alpha, beta) (device output, row-major, stride m).
    void plan(const double* alpha, const double* beta, double* out, double* maxabs_scratch);
    // At the trial point (alpha, beta), reached from a base point by `step`
    // along (dr, dc): row sums r[n] and column sums c[m] of T, and
    // total[0] = sum T e^(-step w) phi(step w), w = (dr_i + dc_j)/reg,
    // phi(x) = e^x - 1 - x. reg * total is the objective change from the
    // base point minus its linear part step * g'd, with no cancellation.
    void grad_ls(const double* alpha, const double* beta, const double* dr, const double* dc,
                 double step, double* r, double* c, double* total, double* maxabs_scratch);
    // Averaged plan X <- (1 - tau) X + tau T(alpha, beta) (X <- T when init):
    // X is n x m row-major in the pass's element type (FP32 mixed, FP64
    // otherwise). Row sums r[n], column sums c[m] of the new X, and
    // totals[0] = sum M X, totals[1] = sum X (1 - log X).
    void avg_plan(const double* alpha, const double* beta, void* X, double tau, bool init,
                  double* r, double* c, double* totals, double* maxabs_scratch);
    // out[t] = sum over the CTAs of total t of the last pass `op` (t < nt).
    void merge_totals(int op, int nt, double* out);

    // Merge helpers (FP64 outputs).
    void merge_rows(int nr, double* out);  // out[r*n + i]
    void merge_cols(int nc, double* out);  // out[c*m + j]

private:
    regot_dproblem* P_;
    cudaStream_t st_;
    int n_, m_;
    bool mixed_;
    double reg_;
    double sum_a_ = 0, sum_bt_ = 0;
    PassBuffers buf_;
    DBuf<double> anchor_;
    DBuf<float4> rsplit_, csplit_;
    DBuf<float> cdsplit_;
    DBuf<int> err_;
};

}  // namespace regot
