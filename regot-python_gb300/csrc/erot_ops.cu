// EROT building blocks (see erot_ops.cuh).
#include <cmath>

#include "erot_ops.cuh"

namespace regot {

namespace {

template <typename Acc>
__device__ __forceinline__ double merge_row(const Acc* rp, int nslabs, int n, int i, int r = 0) {
    return merge_strided(rp + (size_t)r * nslabs * n + i, nslabs, (size_t)n);
}

template <typename Acc>
__device__ __forceinline__ double merge_col(const Acc* cp, int nrb, int m, int j, int c = 0) {
    return merge_strided(cp + (size_t)c * nrb * m + j, nrb, (size_t)m);
}

template <typename Acc>
__device__ __forceinline__ double max_row(const Acc* rp, int nslabs, int n, int i) {
    return max_strided(rp + i, nslabs, (size_t)n);
}

template <typename Acc>
__device__ __forceinline__ double max_col(const Acc* cp, int nrb, int m, int j) {
    return max_strided(cp + j, nrb, (size_t)m);
}

__global__ void k_log(const double* x, int len, double* y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) y[i] = log(x[i]);
}

__global__ void k_maxabs(const double* x, int nx, const double* y, int ny, double* out) {
    double v = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nx + ny; i += gridDim.x * blockDim.x) {
        const double t = i < nx ? x[i] : y[i - nx];
        if (isfinite(t)) v = fmax(v, fabs(t));
    }
    block_atomic_max_abs(out, v);
}

// anchor = -max partials (row or column direction).
template <typename Acc>
__global__ void k_row_anchor(const Acc* rp, int nslabs, int n, double* anchor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) anchor[i] = -max_row(rp, nslabs, n, i);
}
template <typename Acc>
__global__ void k_col_anchor(const Acc* cp, int nrb, int m, double* anchor) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) anchor[j] = -max_col(cp, nrb, m, j);
}

// out = anchor + reg (logw - log S'), S' from the partial sums.
template <typename Acc>
__global__ void k_row_lse(const Acc* rp, int nslabs, int n, const double* anchor,
                          const double* logw, double reg, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = anchor[i] + reg * (logw[i] - log(merge_row(rp, nslabs, n, i)));
}
template <typename Acc>
__global__ void k_col_lse(const Acc* cp, int nrb, int m, const double* anchor,
                          const double* logw, double reg, double* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) out[j] = anchor[j] + reg * (logw[j] - log(merge_col(cp, nrb, m, j)));
}

template <typename Acc>
__global__ void k_merge_rows(const Acc* rp, int nslabs, int n, int nr, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        for (int r = 0; r < nr; ++r) out[(size_t)r * n + i] = merge_row(rp, nslabs, n, i, r);
}
template <typename Acc>
__global__ void k_merge_cols(const Acc* cp, int nrb, int m, int nc, double* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m)
        for (int c = 0; c < nc; ++c) out[(size_t)c * m + j] = merge_col(cp, nrb, m, j, c);
}

}  // namespace

ErotOps::ErotOps(regot_dproblem* P, double reg, cudaStream_t st)
    : P_(P), st_(st), n_(P->n), m_(P->m), mixed_(P->prec == REGOT_PREC_MIXED), reg_(reg) {
    loga_.alloc(n_, st_);
    logb_.alloc(m_, st_);
    k_log<<<cdiv(n_, 256), 256, 0, st_>>>(P->a, n_, loga_.get());
    k_log<<<cdiv(m_, 256), 256, 0, st_>>>(P->b, m_, logb_.get());
    count_launch(2);
    REGOT_CHECK_LAUNCH();
    for (int i = 0; i < n_; ++i) sum_a_ += P->ha[i];
    for (int j = 0; j < m_ - 1; ++j) sum_bt_ += P->hb[j];
    buf_.init(n_, m_, mixed_, 3, 2, 4, st_);
    anchor_.alloc((size_t)(n_ > m_ ? n_ : m_), st_);
    err_.alloc(1, st_);
    err_.zero();
    if (mixed_) {
        rsplit_.alloc(n_, st_);
        csplit_.alloc(m_, st_);
        cdsplit_.alloc(m_, st_);
    }
}

PassParams ErotOps::base_params() const {
    PassParams p;
    p.err = err_.get();
    p.M = P_->M;
    p.ldm = P_->ldm;
    p.n = n_;
    p.m = m_;
    p.reg = reg_;
    p.rowpart = buf_.rowpart.get();
    p.colpart = buf_.colpart.get();
    p.totpart = buf_.totpart.get();
    return p;
}

void ErotOps::check_err() {
    int e = 0;
    d2h(&e, err_.get(), sizeof(int), st_);
    sync(st_);
    if (e) throw Error(REGOT_ERR_TIMEOUT, "a dense pass gave up waiting for its tile copies");
}

void ErotOps::pass(int op, PassParams p) {
    if (!p.err) p.err = err_.get();
    if (mixed_) {
        launch_split(p, rsplit_.get(), csplit_.get(), cdsplit_.get(), st_);
        p.rsplit = rsplit_.get();
        p.csplit = csplit_.get();
        p.cdsplit = cdsplit_.get();
        launch_pass<float>(op, p, st_);
    } else {
        launch_pass<double>(op, p, st_);
    }
}

void ErotOps::pass_presplit(int op, PassParams p) {
    if (!p.err) p.err = err_.get();
    if (mixed_) {
        p.rsplit = rsplit_.get();
        p.csplit = csplit_.get();
        p.cdsplit = cdsplit_.get();
        launch_pass<float>(op, p, st_);
    } else {
        launch_pass<double>(op, p, st_);
    }
}

void ErotOps::maxabs(const double* x, int nx, const double* y, int ny, double* out) {
    REGOT_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st_));
    k_maxabs<<<64, 256, 0, st_>>>(x, nx, y, ny, out);
    count_launch();
    REGOT_CHECK_LAUNCH();
}

// Launch a partial-merging kernel with the accumulator type of the pass.
#define REGOT_LAUNCH_ACC(KERNEL, LEN, PART, ...)                                   \
    do {                                                                           \
        if (mixed_)                                                                \
            KERNEL<float><<<cdiv(LEN, 64), 64, 0, st_>>>(                          \
                reinterpret_cast<const float*>(PART), __VA_ARGS__);                \
        else                                                                       \
            KERNEL<double><<<cdiv(LEN, 64), 64, 0, st_>>>(                         \
                reinterpret_cast<const double*>(PART), __VA_ARGS__);               \
        count_launch();                                                            \
        REGOT_CHECK_LAUNCH();                                                      \
    } while (0)

void ErotOps::merge_rows(int nr, double* out) {
    REGOT_LAUNCH_ACC(k_merge_rows, n_, buf_.rowpart.get(), buf_.shape.nslabs, n_, nr, out);
}

void ErotOps::merge_cols(int nc, double* out) {
    REGOT_LAUNCH_ACC(k_merge_cols, m_, buf_.colpart.get(), buf_.shape.nrb, m_, nc, out);
}

// sinkhorn_problem_bcd.cpp:149-174: beta_j = reg (log b_j - LSE_i (alpha_i - M_ij)/reg),
// evaluated as anchor_j + reg (log b_j - log sum_i exp((alpha_i + anchor_j - M_ij)/reg))
// with anchor_j = -max_i (alpha_i - M_ij), so no term exceeds 1.
void ErotOps::optimal_beta(const double* alpha, double* beta, double* mx) {
    PassParams p = base_params();
    p.ra = alpha;
    maxabs(alpha, n_, nullptr, 0, mx);
    p.grid = mx;
    pass(OP_E_COLMAX, p);
    REGOT_LAUNCH_ACC(k_col_anchor, m_, buf_.colpart.get(), buf_.shape.nrb, m_, anchor_.get());
    maxabs(alpha, n_, anchor_.get(), m_, mx);
    p.cb = anchor_.get();
    pass(OP_E_COL, p);
    REGOT_LAUNCH_ACC(k_col_lse, m_, buf_.colpart.get(), buf_.shape.nrb, m_, anchor_.get(),
                     logb_.get(), reg_, beta);
}

// sinkhorn_problem_bcd.cpp:177-201, the row analogue of optimal_beta.
void ErotOps::optimal_alpha(const double* beta, double* alpha, double* mx) {
    PassParams p = base_params();
    p.cb = beta;
    maxabs(beta, m_, nullptr, 0, mx);
    p.grid = mx;
    pass(OP_E_ROWMAX, p);
    REGOT_LAUNCH_ACC(k_row_anchor, n_, buf_.rowpart.get(), buf_.shape.nslabs, n_, anchor_.get());
    maxabs(beta, m_, anchor_.get(), n_, mx);
    p.ra = anchor_.get();
    pass(OP_E_ROW, p);
    REGOT_LAUNCH_ACC(k_row_lse, n_, buf_.rowpart.get(), buf_.shape.nslabs, n_, anchor_.get(),
                     loga_.get(), reg_, alpha);
}

void ErotOps::row_col_sums(const double* alpha, const double* beta, double* r, double* c,
                           double* mx) {
    PassParams p = base_params();
    p.ra = alpha;
    p.cb = beta;
    maxabs(alpha, n_, beta, m_, mx);
    p.grid = mx;
    pass(OP_E_ROWCOL, p);
    merge_rows(1, r);
    merge_cols(1, c);
}

void ErotOps::tmatvec(const double* alpha, const double* beta, const double* xr, const double* xc,
                      double* yr, double* yc, double* mx) {
    PassParams p = base_params();
    p.ra = alpha;
    p.cb = beta;
    p.rx = xr;
    p.cx = xc;
    maxabs(alpha, n_, beta, m_, mx);
    p.grid = mx;
    pass(OP_E_HVP, p);
    merge_rows(1, yr);
    merge_cols(1, yc);
}

void ErotOps::plan(const double* alpha, const double* beta, double* out, double* mx) {
    PassParams p = base_params();
    p.ra = alpha;
    p.cb = beta;
    p.out = out;
    maxabs(alpha, n_, beta, m_, mx);
    p.grid = mx;
    pass(OP_E_PLAN, p);
}

}  // namespace regot
