// EROT building blocks (see erot_ops.cuh).
#include <cmath>

#include "erot_ops.cuh"

namespace regot {

namespace {

// Partial-merging kernels: (32, 8) blocks, 32 rows (columns) per block with
// their partials split over threadIdx.y (merge_2d / max_2d), so that a merge
// is not bound by one thread's chain of loads and FP32 partials are summed
// without FP64 arithmetic.
constexpr int kMergeItems = 32;

__global__ void k_log(const double* x, int len, double* y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) y[i] = log(x[i]);
}

__global__ void k_maxabs(const double* x, int nx, const double* y, int ny, double* out) {
    unsigned long long v = 0ULL;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nx + ny; i += gridDim.x * blockDim.x) {
        const unsigned long long t = abs_bits(i < nx ? x[i] : y[i - nx]);
        v = t > v ? t : v;
    }
    block_atomic_max_bits(out, v);
}

// anchor = -max partials (row or column direction); *mx is raised to
// max |anchor| as well.
template <typename Acc>
__global__ void k_row_anchor(const Acc* rp, int nslabs, int n, double* anchor, double* mx) {
    const int i = blockIdx.x * kMergeItems + threadIdx.x;
    const double v = max_2d(rp + i, nslabs, (size_t)n, i < n);
    const bool own = threadIdx.y == 0 && i < n;
    if (own) anchor[i] = -v;
    block_atomic_max_bits(mx, own ? abs_bits(v) : 0ULL);
}
template <typename Acc>
__global__ void k_col_anchor(const Acc* cp, int nrb, int m, double* anchor, double* mx) {
    const int j = blockIdx.x * kMergeItems + threadIdx.x;
    const double v = max_2d(cp + j, nrb, (size_t)m, j < m);
    const bool own = threadIdx.y == 0 && j < m;
    if (own) anchor[j] = -v;
    block_atomic_max_bits(mx, own ? abs_bits(v) : 0ULL);
}

// out = anchor + reg (logw - log S'), S' from the partial sums.
template <typename Acc>
__global__ void k_row_lse(const Acc* rp, int nslabs, int n, const double* anchor,
                          const double* logw, double reg, double* out) {
    const int i = blockIdx.x * kMergeItems + threadIdx.x;
    const double S = merge_2d(rp + i, nslabs, (size_t)n, i < n);
    if (threadIdx.y == 0 && i < n) out[i] = anchor[i] + reg * (logw[i] - log(S));
}
template <typename Acc>
__global__ void k_col_lse(const Acc* cp, int nrb, int m, const double* anchor,
                          const double* logw, double reg, double* out) {
    const int j = blockIdx.x * kMergeItems + threadIdx.x;
    const double S = merge_2d(cp + j, nrb, (size_t)m, j < m);
    if (threadIdx.y == 0 && j < m) out[j] = anchor[j] + reg * (logw[j] - log(S));
}

// out[r][i] = merged partial r of row i (r < nr); columns likewise.
template <typename Acc>
__global__ void k_merge_rows(const Acc* rp, int nslabs, int n, int nr, double* out) {
    const int i = blockIdx.x * kMergeItems + threadIdx.x;
    for (int r = 0; r < nr; ++r) {
        const double S = merge_2d(rp + (size_t)r * nslabs * n + i, nslabs, (size_t)n, i < n);
        if (threadIdx.y == 0 && i < n) out[(size_t)r * n + i] = S;
        __syncthreads();  // merge_2d's shared buffer is reused
    }
}
template <typename Acc>
__global__ void k_merge_cols(const Acc* cp, int nrb, int m, int nc, double* out) {
    const int j = blockIdx.x * kMergeItems + threadIdx.x;
    for (int c = 0; c < nc; ++c) {
        const double S = merge_2d(cp + (size_t)c * nrb * m + j, nrb, (size_t)m, j < m);
        if (threadIdx.y == 0 && j < m) out[(size_t)c * m + j] = S;
        __syncthreads();
    }
}

// out[t] = sum of the per-CTA totals of a pass, in CTA order.
__global__ void k_sum_totals(const double* totpart, int nblocks, int nt, double* out) {
    const int t = threadIdx.x;
    if (t >= nt) return;
    double acc = 0.0;
    for (int k = 0; k < nblocks; ++k) acc += totpart[(size_t)t * nblocks + k];
    out[t] = acc;
}

}  // namespace

ErotOps::ErotOps(regot_dproblem* P, double reg, cudaStream_t st)
    : P_(P), st_(st), n_(P->n), m_(P->m), mixed_(P->prec == REGOT_PREC_MIXED), reg_(reg) {
    if (!P->loga) {  // once per problem, kept with it
        P->loga = static_cast<double*>(dev_alloc(n_ * sizeof(double), st_));
        P->logb = static_cast<double*>(dev_alloc(m_ * sizeof(double), st_));
        k_log<<<cdiv(n_, 256), 256, 0, st_>>>(P->a, n_, P->loga);
        k_log<<<cdiv(m_, 256), 256, 0, st_>>>(P->b, m_, P->logb);
        count_launch(2);
        REGOT_CHECK_LAUNCH();
    }
    sum_a_ = P->sum_a;
    sum_bt_ = P->sum_bt;
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
    read_small(P_->ctx, &e, err_.get(), sizeof(int), st_);
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

void ErotOps::split(const PassParams& p) {
    if (mixed_) launch_split(p, rsplit_.get(), csplit_.get(), cdsplit_.get(), st_);
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
            KERNEL<float><<<cdiv(LEN, kMergeItems), dim3(32, 8), 0, st_>>>(        \
                reinterpret_cast<const float*>(PART), __VA_ARGS__);                \
        else                                                                       \
            KERNEL<double><<<cdiv(LEN, kMergeItems), dim3(32, 8), 0, st_>>>(       \
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
    // mx = max(|alpha|, |anchor|): the anchor kernel raises max |alpha|
    REGOT_LAUNCH_ACC(k_col_anchor, m_, buf_.colpart.get(), buf_.shape.nrb, m_, anchor_.get(), mx);
    p.cb = anchor_.get();
    pass(OP_E_COL, p);
    REGOT_LAUNCH_ACC(k_col_lse, m_, buf_.colpart.get(), buf_.shape.nrb, m_, anchor_.get(),
                     P_->logb, reg_, beta);
}

// sinkhorn_problem_bcd.cpp:177-201, the row analogue of optimal_beta.
void ErotOps::optimal_alpha(const double* beta, double* alpha, double* mx) {
    PassParams p = base_params();
    p.cb = beta;
    maxabs(beta, m_, nullptr, 0, mx);
    p.grid = mx;
    pass(OP_E_ROWMAX, p);
    REGOT_LAUNCH_ACC(k_row_anchor, n_, buf_.rowpart.get(), buf_.shape.nslabs, n_, anchor_.get(), mx);
    p.ra = anchor_.get();
    pass(OP_E_ROW, p);
    REGOT_LAUNCH_ACC(k_row_lse, n_, buf_.rowpart.get(), buf_.shape.nslabs, n_, anchor_.get(),
                     P_->loga, reg_, alpha);
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

void ErotOps::merge_totals(int op, int nt, double* out) {
    k_sum_totals<<<1, 32, 0, st_>>>(buf_.totpart.get(), pass_blocks(op, mixed_, n_, m_), nt, out);
    count_launch();
    REGOT_CHECK_LAUNCH();
}

void ErotOps::grad_ls(const double* alpha, const double* beta, const double* dr, const double* dc,
                      double step, double* r, double* c, double* total, double* mx) {
    PassParams p = base_params();
    p.ra = alpha;
    p.cb = beta;
    p.rd = dr;
    p.cd = dc;
    p.steps[0] = step;
    p.nsteps = 1;
    maxabs(alpha, n_, beta, m_, mx);
    p.grid = mx;
    pass(OP_E_GRADLS, p);
    merge_rows(1, r);
    merge_cols(1, c);
    merge_totals(OP_E_GRADLS, 1, total);
}

void ErotOps::avg_plan(const double* alpha, const double* beta, void* X, double tau, bool init,
                       double* r, double* c, double* totals, double* mx) {
    PassParams p = base_params();
    p.ra = alpha;
    p.cb = beta;
    p.xavg = X;
    p.steps[0] = tau;
    p.nsteps = init ? 0 : 1;
    maxabs(alpha, n_, beta, m_, mx);
    p.grid = mx;
    pass(OP_E_AVG, p);
    merge_rows(1, r);
    merge_cols(1, c);
    merge_totals(OP_E_AVG, 2, totals);
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
