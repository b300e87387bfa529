// FP64 oracle: entropic-regularised OT (EROT) problem pieces and the
// sinkhorn_bcd / sinkhorn_newton / sinkhorn_ssns solvers.
// Test infrastructure only (see oracle.h). Each function cites the reference
// file:line whose math and control flow it restates.
#include "oracle_lbfgs.h"
#include "oracle_util.h"

namespace oracle {
namespace erot {

struct Problem {
    int n, m;
    const double* M;  // column-major n x m
    const double* a;
    const double* b;
    double reg;
    Vec loga, logb;
    // sinkhorn_problem.h:36-44
    Problem(const double* M_, int n_, int m_, const double* a_, const double* b_, double reg_)
        : n(n_), m(m_), M(M_), a(a_), b(b_), reg(reg_), loga(n_), logb(m_) {
        for (int i = 0; i < n; i++) loga[i] = std::log(a[i]);
        for (int j = 0; j < m; j++) logb[j] = std::log(b[j]);
    }
    double Mij(int i, int j) const { return M[(size_t)j * n + i]; }
};

// optimal_beta: sinkhorn_problem_bcd.cpp:149-174 with log_sum_exp_colwise
// (111-146): D = (alpha - M)/reg, beta_j = reg (log b_j - LSE_i D_ij),
// LSE with the column max as shift.
static void optimal_beta(const Problem& p, const double* alpha, double* beta) {
    const int n = p.n;
    Vec D(n);
    for (int j = 0; j < p.m; j++) {
        const double* Mj = p.M + (size_t)j * n;
        double c = -std::numeric_limits<double>::infinity();
        for (int i = 0; i < n; i++) {
            D[i] = (alpha[i] - Mj[i]) / p.reg;
            c = std::max(c, D[i]);
        }
        double s = 0.0;
        for (int i = 0; i < n; i++) s += std::exp(D[i] - c);
        const double lse = c + std::log(s);
        beta[j] = p.reg * (p.logb[j] - lse);
    }
}

// optimal_alpha: sinkhorn_problem_bcd.cpp:177-201 with log_sum_exp_rowwise
// (82-108): row max first, then exp sums accumulated column by column.
static void optimal_alpha(const Problem& p, const double* beta, double* alpha) {
    const int n = p.n, m = p.m;
    Vec c(n, -std::numeric_limits<double>::infinity()), res(n, 0.0);
    for (int j = 0; j < m; j++) {
        const double* Mj = p.M + (size_t)j * n;
        for (int i = 0; i < n; i++) c[i] = std::max(c[i], (beta[j] - Mj[i]) / p.reg);
    }
    for (int j = 0; j < m; j++) {
        const double* Mj = p.M + (size_t)j * n;
        for (int i = 0; i < n; i++) res[i] += std::exp((beta[j] - Mj[i]) / p.reg - c[i]);
    }
    for (int i = 0; i < n; i++) alpha[i] = p.reg * (p.loga[i] - (c[i] + std::log(res[i])));
}

// compute_T: sinkhorn_problem_obj.cpp:139-188 (with compute_column_helper
// 16-136): T_ij = exp((alpha_i + beta_j - M_ij)/reg), last column with
// beta_m = 0 ("NoBeta"); returns sum(T).
static double compute_T(const Problem& p, const double* gamma, double* T) {
    const int n = p.n, m = p.m;
    const double* alpha = gamma;
    const double* beta = gamma + n;
    double Tsum = 0.0;
    for (int j = 0; j < m; j++) {
        const double* Mj = p.M + (size_t)j * n;
        double* Tj = T + (size_t)j * n;
        double colsum = 0.0;
        if (j < m - 1) {
            const double bj = beta[j];
            for (int i = 0; i < n; i++) {
                const double t = std::exp((alpha[i] + bj - Mj[i]) / p.reg);
                colsum += t;
                Tj[i] = t;
            }
        } else {
            for (int i = 0; i < n; i++) {
                const double t = std::exp((alpha[i] - Mj[i]) / p.reg);
                colsum += t;
                Tj[i] = t;
            }
        }
        Tsum += colsum;
    }
    return Tsum;
}

// compute_sums: sinkhorn_problem_obj.cpp:192-297. Row sums in sums[0:n],
// column sums of the first m-1 columns in sums[n:n+m-1].
static void compute_sums(const Problem& p, const double* T, double* sums) {
    const int n = p.n, m = p.m;
    double* rs = sums;
    double* cs = sums + n;
    std::fill(rs, rs + n, 0.0);
    for (int j = 0; j < m; j++) {
        const double* Tj = T + (size_t)j * n;
        double c = 0.0;
        for (int i = 0; i < n; i++) {
            c += Tj[i];
            rs[i] += Tj[i];
        }
        if (j < m - 1) cs[j] = c;
    }
}

// dual_obj: sinkhorn_problem_obj.cpp:324-342.
static double dual_obj(const Problem& p, const double* gamma, double* T) {
    const double Tsum = compute_T(p, gamma, T);
    return p.reg * Tsum - dot(gamma, p.a, p.n) - dot(gamma + p.n, p.b, p.m - 1);
}

// dual_obj_grad: sinkhorn_problem_obj.cpp:371-393 (computeT selects whether
// T is recomputed or reused).
static double dual_obj_grad(const Problem& p, const double* gamma, double* grad, double* T,
                            bool computeT) {
    const int n = p.n, m = p.m;
    if (computeT) compute_T(p, gamma, T);
    compute_sums(p, T, grad);
    const double Tsum = sum(grad, n);
    for (int i = 0; i < n; i++) grad[i] -= p.a[i];
    for (int j = 0; j < m - 1; j++) grad[n + j] -= p.b[j];
    return p.reg * Tsum - dot(gamma, p.a, n) - dot(gamma + n, p.b, m - 1);
}

// Gauge fix of sinkhorn_bcd.cpp:50-51: gamma = (alpha + beta_m, beta~ - beta_m).
static void gauge(int n, int m, const double* alpha, const double* beta, double* gamma) {
    for (int i = 0; i < n; i++) gamma[i] = alpha[i] + beta[m - 1];
    for (int j = 0; j < m - 1; j++) gamma[n + j] = beta[j] - beta[m - 1];
}

// Recovered plan, sinkhorn_result.h:32-50, written row-major.
static void get_plan(const Problem& p, const double* gamma, double* plan) {
    const int n = p.n, m = p.m;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < m; j++) {
            const double bj = (j < m - 1) ? gamma[n + j] : 0.0;
            plan[(size_t)i * m + j] = std::exp((gamma[i] + bj - p.Mij(i, j)) / p.reg);
        }
}

// ---------------- sparsify_mat3 (sinkhorn_sparsify3.cpp) ----------------
// The non-AVX2 build of the reference (what runs on Arm hosts) selects with
// std::nth_element and sorts with std::sort; the same calls are used here.

// select_and_find: sinkhorn_sparsify3.cpp:35-64.
static int select_and_find(double* x, int n, int k, double target, double& block_sum) {
    std::nth_element(x, x + k, x + n);
    block_sum = 0.0;
    for (int i = 0; i < k; i++) block_sum += x[i];
    if (block_sum <= target) return k;
    std::sort(x, x + k);
    double s = 0.0;
    for (int i = 0; i < k; i++) {
        s += x[i];
        if (s > target) return i;
    }
    return k - 1;
}

// select_and_find_reverse: sinkhorn_sparsify3.cpp:73-102.
static int select_and_find_reverse(double* x, int n, int k, double target, double& block_sum) {
    std::nth_element(x, x + k, x + n);
    block_sum = 0.0;
    for (int i = k; i < n; i++) block_sum += x[i];
    if (block_sum < target) return k - 1;
    std::sort(x + k, x + n);
    double s = 0.0;
    for (int i = n - 1; i >= k; i--) {
        s += x[i];
        if (s >= target) return i;
    }
    return k;
}

static int block_size(int n) {
    int b = n / 32;
    b = std::max(b, 32);
    return std::min(b, n);
}

// find_small: sinkhorn_sparsify3.cpp:112-148 (blocks of max(n/32, 32)
// smallest elements, scanned from the left).
static int find_small(double* x, int n, double delta) {
    const int blk = block_size(n);
    int found = n;
    double target = delta;
    for (int w = 0; w < n; w += blk) {
        const int len = n - w;
        const int bs = std::min(len, blk);
        double block_sum;
        const int L = select_and_find(x + w, len, bs, target, block_sum);
        if (L < bs) {
            found = w + L;
            break;
        }
        target -= block_sum;
    }
    return found;
}

// find_large: sinkhorn_sparsify3.cpp:160-196 (blocks of the largest
// elements, scanned from the right; target = sum - delta).
static int find_large(double* x, int n, double target) {
    const int blk = block_size(n);
    int found = 0;
    for (int w = n; w >= 0; w -= (blk > 0 ? blk : 1)) {
        const int len = w;
        const int bs = std::min(len, blk);
        const int k = len - bs;
        double block_sum;
        const int L = select_and_find_reverse(x, len, k, target, block_sum);
        if (L >= k) {
            found = L;
            break;
        }
        target -= block_sum;
        if (blk == 0) break;
    }
    return found;
}

struct CSC {
    int n = 0, ncol = 0;
    std::vector<int> outer;   // ncol + 1
    std::vector<int> inner;
    std::vector<double> val;
    long nnz() const { return (long)val.size(); }
};

// sparsify_mat3: sinkhorn_sparsify3.cpp:276-405.
static CSC sparsify_mat3(const double* T, int n, int m, double delta, double density_hint) {
    const double Inf = std::numeric_limits<double>::infinity();
    std::vector<double> Delta(T, T + (size_t)n * m);
    std::fill(Delta.begin() + (size_t)(m - 1) * n, Delta.end(), 0.0);
    // Column stage (lines 295-319).
    for (int j = 0; j < m - 1; j++) {
        const double* Tj = T + (size_t)j * n;
        double* data = Delta.data() + (size_t)j * n;
        int L;
        if (density_hint > 0.2) {
            L = find_small(data, n, delta);
        } else {
            const double s = sum(Tj, n);
            L = find_large(data, n, s - delta);
        }
        const double thresh = (L >= n) ? Inf : data[L];
        for (int i = 0; i < n; i++) data[i] = (Tj[i] >= thresh) ? 0.0 : Tj[i];
    }
    // Row stage (lines 333-353).
    std::vector<double> row(m);
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < m; j++) row[j] = Delta[(size_t)j * n + i];
        const double rowsum = sum(row.data(), m);
        if (rowsum > 2.0 * delta) {
            const double target = rowsum - 2.0 * delta;
            const int L = find_large(row.data(), m - 1, target);
            const double thresh = (L >= m - 1) ? Inf : row[L];
            for (int j = 0; j < m - 1; j++) {
                double& d = Delta[(size_t)j * n + i];
                d = (d >= thresh) ? 0.0 : d;
            }
        }
    }
    // Kept entries are those with Delta == 0 (line 378), exact zeros of T
    // included.
    CSC sp;
    sp.n = n;
    sp.ncol = m - 1;
    sp.outer.assign(m, 0);
    for (int j = 0; j < m - 1; j++) {
        const double* Tj = T + (size_t)j * n;
        const double* Dj = Delta.data() + (size_t)j * n;
        for (int i = 0; i < n; i++) {
            if (Dj[i] == 0.0) {
                sp.val.push_back(Tj[i]);
                sp.inner.push_back(i);
            }
        }
        sp.outer[j + 1] = (int)sp.val.size();
    }
    return sp;
}

// Sparsified Hessian: sinkhorn_hess.h:46-158, sinkhorn_hess.cpp:15-164.
struct Hessian {
    int n = 0, m = 0;
    Vec h1, h2;
    CSC sigmad;  // values already divided by reg
    double density() const {
        const long nnz = 2 * sigmad.nnz() + n + m - 1;
        const double d = (double)(n + m - 1);
        return (double)nnz / d / d;
    }
    // res = sigmad * x, x [m-1], res [n]
    void apply_sigmadx(const double* x, double* res) const {
        std::fill(res, res + n, 0.0);
        for (int j = 0; j < m - 1; j++)
            for (int k = sigmad.outer[j]; k < sigmad.outer[j + 1]; k++)
                res[sigmad.inner[k]] += sigmad.val[k] * x[j];
    }
    // res = sigmad' * x, x [n], res [m-1]
    void apply_sigmadtx(const double* x, double* res) const {
        for (int j = 0; j < m - 1; j++) {
            double s = 0.0;
            for (int k = sigmad.outer[j]; k < sigmad.outer[j + 1]; k++)
                s += sigmad.val[k] * x[sigmad.inner[k]];
            res[j] = s;
        }
    }
    // apply_Deltax: sinkhorn_hess.cpp:136-148.
    void apply_Deltax(const Vec& x, double shift, Vec& res) const {
        Vec sx(n), t(n), stx(m - 1);
        apply_sigmadx(x.data(), sx.data());
        for (int i = 0; i < n; i++) t[i] = sx[i] / (h1[i] + shift);
        apply_sigmadtx(t.data(), stx.data());
        res.resize(m - 1);
        for (int j = 0; j < m - 1; j++) res[j] = h2[j] * x[j] + shift * x[j] - stx[j];
    }
    // apply_Hsx: sinkhorn_hess.cpp:151-164.
    void apply_Hsx(const Vec& x, Vec& res) const {
        res.resize(n + m - 1);
        apply_sigmadx(x.data() + n, res.data());
        apply_sigmadtx(x.data(), res.data() + n);
        for (int i = 0; i < n; i++) res[i] += h1[i] * x[i];
        for (int j = 0; j < m - 1; j++) res[n + j] += h2[j] * x[n + j];
    }
};

// dual_sparsified_hess: sinkhorn_problem_obj.cpp:432-443 + compute_hess
// sinkhorn_hess.cpp:15-33.
static void sparsified_hess(const Problem& p, const double* T, const Vec& grad, double delta,
                            double density_hint, Hessian& H) {
    const int n = p.n, m = p.m;
    H.n = n;
    H.m = m;
    H.h1.resize(n);
    H.h2.resize(m - 1);
    for (int i = 0; i < n; i++) H.h1[i] = (grad[i] + p.a[i]) / p.reg;
    for (int j = 0; j < m - 1; j++) H.h2[j] = (grad[n + j] + p.b[j]) / p.reg;
    H.sigmad = sparsify_mat3(T, n, m, delta, density_hint);
    for (auto& v : H.sigmad.val) v /= p.reg;
}

// hess_cg: sinkhorn_cg.cpp:9-50 (Schur complement on the beta block).
static int hess_cg(const Hessian& H, const Vec& rhs, double shift, const Vec* guess, double tol,
                   Vec& res) {
    const int n = H.n, m = H.m;
    res.assign(n + m - 1, 0.0);
    Vec v(n), y(m - 1), zy(m - 1);
    for (int i = 0; i < n; i++) v[i] = rhs[i] / (H.h1[i] + shift);
    H.apply_sigmadtx(v.data(), y.data());
    for (int j = 0; j < m - 1; j++) zy[j] = rhs[n + j] - y[j];
    Vec r2;
    const int it = cg_solve([&](const Vec& x, Vec& out) { H.apply_Deltax(x, shift, out); }, zy, r2,
                            tol, guess);
    std::copy(r2.begin(), r2.end(), res.begin() + n);
    Vec bx(n);
    H.apply_sigmadx(r2.data(), bx.data());
    for (int i = 0; i < n; i++) res[i] = (rhs[i] - bx[i]) / (H.h1[i] + shift);
    return it;
}

// Direct solve of (Hs + shift I) x = rhs. The reference factors the sparse
// matrix with SimplicialLDLT/LLT/SparseLU (sinkhorn_linsolve.cpp:58-106);
// the oracle solves the same SPD system exactly through a dense Cholesky of
// its Schur complement on the beta block.
static bool hess_direct(const Hessian& H, const Vec& rhs, double shift, Vec& res) {
    const int n = H.n, m1 = H.m - 1;
    // CSR view of sigmad.
    std::vector<std::vector<std::pair<int, double>>> rows(n);
    for (int j = 0; j < m1; j++)
        for (int k = H.sigmad.outer[j]; k < H.sigmad.outer[j + 1]; k++)
            rows[H.sigmad.inner[k]].push_back({j, H.sigmad.val[k]});
    std::vector<double> S((size_t)m1 * m1, 0.0);
    for (int j = 0; j < m1; j++) S[(size_t)j * m1 + j] = H.h2[j] + shift;
    for (int i = 0; i < n; i++) {
        const double w = 1.0 / (H.h1[i] + shift);
        const auto& r = rows[i];
        for (size_t p = 0; p < r.size(); p++)
            for (size_t q = 0; q <= p; q++) {
                const int j = r[p].first, k = r[q].first;
                const double v = r[p].second * r[q].second * w;
                S[(size_t)std::max(j, k) * m1 + std::min(j, k)] -= v;
            }
    }
    if (!cholesky(S, m1)) return false;
    Vec t(n), y(m1);
    for (int i = 0; i < n; i++) t[i] = rhs[i] / (H.h1[i] + shift);
    H.apply_sigmadtx(t.data(), y.data());
    Vec r2(m1);
    for (int j = 0; j < m1; j++) r2[j] = rhs[n + j] - y[j];
    cholesky_solve(S, m1, r2);
    res.assign(n + m1, 0.0);
    Vec bx(n);
    H.apply_sigmadx(r2.data(), bx.data());
    for (int i = 0; i < n; i++) res[i] = (rhs[i] - bx[i]) / (H.h1[i] + shift);
    for (int j = 0; j < m1; j++) res[n + j] = r2[j];
    return true;
}

// Newton direction -H^{-1} g for the dense dual Hessian
// H = [diag(r) T~; T~' diag(c~)]/reg (sinkhorn_problem_obj.cpp:396-418),
// solved exactly (the reference uses Eigen::LLT on H, sinkhorn_newton.cpp:91)
// via a dense Cholesky of the Schur complement
// diag(c~) - T~' diag(1/r) T~ (all divided by reg).
static bool newton_direction(const Problem& p, const double* T, const Vec& g, Vec& direc) {
    const int n = p.n, m1 = p.m - 1;
    Vec r(n), c(m1);
    for (int i = 0; i < n; i++) r[i] = g[i] + p.a[i];
    for (int j = 0; j < m1; j++) c[j] = g[n + j] + p.b[j];
    const double reg = p.reg;
    // Columns of T~/reg scaled by sqrt(reg/r_i), so S = diag(c~)/reg - U'U.
    std::vector<double> U((size_t)m1 * n);
    for (int j = 0; j < m1; j++)
        for (int i = 0; i < n; i++)
            U[(size_t)j * n + i] = (T[(size_t)j * n + i] / reg) * std::sqrt(reg / r[i]);
    std::vector<double> S((size_t)m1 * m1, 0.0);
    for (int j = 0; j < m1; j++) {
        const double* Uj = U.data() + (size_t)j * n;
        for (int k = 0; k <= j; k++) {
            const double* Uk = U.data() + (size_t)k * n;
            double s = 0.0;
            for (int i = 0; i < n; i++) s += Uj[i] * Uk[i];
            S[(size_t)j * m1 + k] = (j == k ? c[j] / reg : 0.0) - s;
        }
    }
    if (!cholesky(S, m1)) return false;
    // rhs = -g; x_b = S^{-1}(-g_b + B' A^{-1} g_a); x_a = A^{-1}(-g_a - B x_b)
    Vec xb(m1);
    for (int j = 0; j < m1; j++) {
        const double* Tj = T + (size_t)j * n;
        double s = 0.0;
        for (int i = 0; i < n; i++) s += (Tj[i] / reg) * (g[i] / (r[i] / reg));
        xb[j] = -g[n + j] + s;
    }
    cholesky_solve(S, m1, xb);
    direc.assign(n + m1, 0.0);
    for (int i = 0; i < n; i++) {
        double s = 0.0;
        for (int j = 0; j < m1; j++) s += (T[(size_t)j * n + i] / reg) * xb[j];
        direc[i] = (-g[i] - s) / (r[i] / reg);
    }
    for (int j = 0; j < m1; j++) direc[n + j] = xb[j];
    return true;
}

// line_selection: sinkhorn_problem_ls.cpp:13-41. T is left holding the last
// candidate evaluated.
static double line_selection(const Problem& p, const std::vector<double>& candid, const Vec& gamma,
                             const Vec& direc, double curobj, double* T, double& objval) {
    double best = 1.0;
    objval = std::numeric_limits<double>::infinity();
    Vec ng(gamma.size());
    for (double alpha : candid) {
        for (size_t k = 0; k < gamma.size(); k++) ng[k] = gamma[k] + alpha * direc[k];
        const double f = dual_obj(p, ng.data(), T);
        if (f < objval) {
            best = alpha;
            objval = f;
        }
        if (objval < curobj) return best;
    }
    return best;
}

static void init_gamma(const Problem& p, const oracle_opts* opts, Vec& gamma) {
    const int n = p.n, m = p.m;
    gamma.assign(n + m - 1, 0.0);
    if (opts && opts->x0 && opts->x0_len == n + m - 1) {
        std::copy(opts->x0, opts->x0 + n + m - 1, gamma.begin());
        return;
    }
    Vec alpha(n, 0.0), beta(m);
    optimal_beta(p, alpha.data(), beta.data());
    gauge(n, m, alpha.data(), beta.data(), gamma.data());
}

static void finish(const Problem& p, int niter, const Vec& gamma, History& h, oracle_result* r) {
    r->niter = niter;
    r->hist_len = h.len;
    std::copy(gamma.begin(), gamma.end(), r->dual);
    if (r->plan) get_plan(p, gamma.data(), r->plan);
}

// ------------- sparsify_mat_with_density (sinkhorn_sparsify4.cpp) -------------
// sinkhorn_sparsify4.cpp:77-174 with preserve = true (sinkhorn_sparsify.h:22):
// the largest k = floor(n (m-1) density) entries of T[:, :m-1] (selected with
// std::nth_element, the reference's non-AVX2 path), plus the first column and
// the first row of T[:, :m-1].
static CSC sparsify_with_density(const double* T, int n, int m, double density) {
    const size_t len = (size_t)n * (m - 1);
    density = std::min(std::max(density, 0.0), 1.0);
    const size_t k = (size_t)(len * density);
    std::vector<size_t> ind(len);
    for (size_t q = 0; q < len; q++) ind[q] = q;
    if (k > 0 && k < len)
        std::nth_element(ind.begin(), ind.begin() + (len - k), ind.end(),
                         [T](size_t x, size_t y) { return T[x] < T[y]; });
    std::vector<char> keep(len, 0);
    for (int i = 0; i < n; i++) keep[i] = 1;                          // column 0
    for (int j = 1; j < m - 1; j++) keep[(size_t)j * n] = 1;          // row 0
    for (size_t q = len - k; q < len; q++) keep[ind[q]] = 1;
    CSC sp;
    sp.n = n;
    sp.ncol = m - 1;
    sp.outer.assign(m, 0);
    for (int j = 0; j < m - 1; j++) {
        for (int i = 0; i < n; i++) {
            const size_t q = (size_t)j * n + i;
            if (keep[q]) {
                sp.val.push_back(T[q]);
                sp.inner.push_back(i);
            }
        }
        sp.outer[j + 1] = (int)sp.val.size();
    }
    return sp;
}

// dual_sparsified_hess_with_density: sinkhorn_problem_obj.cpp:446-457 with
// compute_hess_with_density (sinkhorn_hess.cpp:37-55).
static void sparsified_hess_density(const Problem& p, const double* T, const Vec& grad,
                                    double density, Hessian& H) {
    const int n = p.n, m = p.m;
    H.n = n;
    H.m = m;
    H.h1.resize(n);
    H.h2.resize(m - 1);
    for (int i = 0; i < n; i++) H.h1[i] = (grad[i] + p.a[i]) / p.reg;
    for (int j = 0; j < m - 1; j++) H.h2[j] = (grad[n + j] + p.b[j]) / p.reg;
    H.sigmad = sparsify_with_density(T, n, m, density);
    for (auto& v : H.sigmad.val) v /= p.reg;
}

// density_T2H: sinkhorn_sparse_newton.cpp:17-22 (sinkhorn_splr.cpp:16-21).
static double density_T2H(double denT, int n, int m) {
    const double nnz = 2.0 * denT * n * (m - 1) + n + m - 1;
    return nnz / double(n + m - 1) / double(n + m - 1);
}

// ---------------- More-Thuente line search (sinkhorn_problem_ls.cpp) ----------------
// quadratic_minimizer (fa, ga, fb): lines 68-75.
static double qmin_fgf(double a, double b, double fa, double ga, double fb) {
    const double ba = b - a;
    const double w = 0.5 * ba * ga / (fa - fb + ba * ga);
    return a + w * ba;
}
// quadratic_minimizer (ga, gb): lines 83-87.
static double qmin_gg(double a, double b, double ga, double gb) {
    const double w = ga / (ga - gb);
    return a + w * (b - a);
}
// cubic_minimizer: lines 92-150.
static double cmin(double a, double b, double fa, double fb, double ga, double gb, bool& exists) {
    const double apb = a + b, ba = b - a, ba2 = ba * ba;
    const double fba = fb - fa, gba = gb - ga;
    const double z3 = (ga + gb) * ba - 2.0 * fba;
    const double z2 = 0.5 * (gba * ba2 - 3.0 * apb * z3);
    const double z1 = fba * ba2 - apb * z2 - (a * apb + b * b) * z3;
    const double eps = std::numeric_limits<double>::epsilon();
    if (std::abs(z3) < eps * std::abs(z2) || std::abs(z3) < eps * std::abs(z1)) {
        exists = (z2 * ba > 0.0);
        return exists ? (-0.5 * z1 / z2) : b;
    }
    const double u = z2 / (3.0 * z3), v = z1 / z2;
    const double vu = v / u;
    exists = (vu <= 1.0);
    if (!exists) return b;
    double r1, r2;
    if (std::abs(u) >= std::abs(v)) {
        const double w = 1.0 + std::sqrt(1.0 - vu);
        r1 = -u * w;
        r2 = -v / w;
    } else {
        const double sd = std::sqrt(std::abs(u)) * std::sqrt(std::abs(v)) * std::sqrt(1 - u / v);
        r1 = -u - sd;
        r2 = -u + sd;
    }
    return (z3 * ba > 0.0) ? std::max(r1, r2) : std::min(r1, r2);
}
// step_selection: lines 154-222.
static double step_select(double al, double au, double at, double fl, double fu, double ft,
                          double gl, double gu, double gt) {
    if (al == au) return al;
    if (!std::isfinite(ft) || !std::isfinite(gt)) return (al + at) / 2.0;
    bool ac_ok;
    const double ac = cmin(al, at, fl, ft, gl, gt, ac_ok);
    const double aq = qmin_fgf(al, at, fl, gl, ft);
    if (ft > fl) {
        if (!ac_ok) return aq;
        return (std::abs(ac - al) < std::abs(aq - al)) ? ac : ((aq + ac) / 2.0);
    }
    const double as = qmin_gg(al, at, gl, gt);
    if (gt * gl < 0.0) return (std::abs(ac - at) >= std::abs(as - at)) ? ac : as;
    const double deltal = 1.1, deltau = 0.66;
    if (std::abs(gt) < std::abs(gl)) {
        const bool use_ac = ac_ok && ((ac - at) * (at - al) > 0.0) &&
                            (std::abs(ac - at) < std::abs(as - at));
        const double r = use_ac ? ac : as;
        return (at > al) ? std::min(at + deltau * (au - at), r)
                         : std::max(at + deltau * (au - at), r);
    }
    if (!std::isfinite(au) || !std::isfinite(fu) || !std::isfinite(gu))
        return at + deltal * (at - al);
    bool ae_ok;
    const double ae = cmin(at, au, ft, fu, gt, gu, ae_ok);
    return (at > al) ? std::min(at + deltau * (au - at), ae) : std::max(at + deltau * (au - at), ae);
}

// line_search_wolfe: sinkhorn_problem_ls.cpp:226-436 (c1 = 1e-4, c2 = 0.9,
// 20 trials, steps in [1e-10, 2]). eval(step, &f, &dg) evaluates the
// objective and its directional derivative at gamma + step d (leaving T
// there). Sets recompute when the returned step is not the last evaluated.
template <typename Eval>
static double wolfe_search(double init_step, double f0, double dg0, Eval&& eval,
                           bool& recompute) {
    const double c1 = 1e-4, c2 = 0.9;
    const int max_iter = 20;
    recompute = false;
    const double step_min = 1e-10, step_max = 2.0;
    init_step = std::min(std::max(init_step, step_min), step_max);
    double step = init_step;
    if (dg0 > 0.0) {
        recompute = true;
        return init_step;
    }
    const double test_decr = c1 * dg0, test_curv = -c2 * dg0;
    const double Inf = std::numeric_limits<double>::infinity();
    double I_lo = 0.0, I_hi = Inf, fI_lo = 0.0, fI_hi = Inf;
    double gI_lo = (1.0 - c1) * dg0, gI_hi = Inf, psiI_lo = 0.0;
    bool bracketed = false, guard_min = true;
    double width = Inf, width_prev = Inf;
    int shrink_fails = 0;
    const double delta_max = 1.1, delta_min = 7.0 / 12, shrink = 0.66;
    double fx = f0;
    for (int it = 0; it < max_iter; it++) {
        double dg;
        eval(step, &fx, &dg);
        const double psit = fx - f0 - step * test_decr;
        const double dpsit = dg - test_decr;
        if (psit <= 0.0 && std::abs(dg) <= test_curv) return step;
        if (step <= step_min && (psit > 0.0 || dpsit >= 0.0)) return step;
        if (step >= step_max && (psit <= 0.0 && dpsit < 0.0)) return step;
        const double ft = psit, gt = dpsit;  // f is psi throughout (line 329)
        if (guard_min && (psit <= 0.0 && dpsit < 0.0)) guard_min = false;
        double next;
        const bool case2 = (psit <= psiI_lo) && (dpsit * (I_lo - step) > 0.0);
        if (case2) {
            next = std::min(step_max, step + delta_max * (step - I_lo));
        } else {
            next = step_select(I_lo, I_hi, step, fI_lo, fI_hi, ft, gI_lo, gI_hi, gt);
            next = std::min(std::max(next, step_min), step_max);
            if (guard_min) {
                next = std::max(next, step_min);
                next = std::min(next, std::max(step_min, delta_min * step));
            }
        }
        if (psit > psiI_lo) {
            I_hi = step;
            fI_hi = ft;
            gI_hi = gt;
        } else if (case2) {
            I_lo = step;
            fI_lo = ft;
            gI_lo = gt;
            psiI_lo = psit;
        } else {
            I_hi = I_lo;
            fI_hi = fI_lo;
            gI_hi = gI_lo;
            I_lo = step;
            fI_lo = ft;
            gI_lo = gt;
            psiI_lo = psit;
        }
        if (!bracketed && !case2) {
            const double l = std::min(I_lo, I_hi), r = std::max(I_lo, I_hi);
            bracketed = (l >= step_min && r <= step_max);
        }
        if (bracketed) {
            width_prev = width;
            width = std::abs(I_hi - I_lo);
            if (width_prev < Inf && width > shrink * width_prev) shrink_fails += 1;
            else shrink_fails = 0;
            if (shrink_fails >= 2) {
                next = (I_lo + I_hi) / 2.0;
                shrink_fails = 0;
            }
        }
        step = next;
    }
    // Trials used up (lines 417-435): the psi of the last evaluated value at
    // the step chosen next decides between that step and I_lo.
    const double psit = fx - f0 - step * test_decr;
    if (psit <= psiI_lo) return step;
    recompute = true;
    if (I_lo <= 0.0) return init_step;
    return I_lo;
}

}  // namespace erot
}  // namespace oracle

using namespace oracle;
using namespace oracle::erot;

extern "C" {

void oracle_erot_optimal_beta(const double* M, int n, int m, const double* b, double reg,
                              const double* alpha, double* beta) {
    std::vector<double> ones(n, 1.0);
    Problem p(M, n, m, ones.data(), b, reg);
    optimal_beta(p, alpha, beta);
}

void oracle_erot_optimal_alpha(const double* M, int n, int m, const double* a, double reg,
                               const double* beta, double* alpha) {
    std::vector<double> ones(m, 1.0);
    Problem p(M, n, m, a, ones.data(), reg);
    optimal_alpha(p, beta, alpha);
}

double oracle_erot_dual_obj(const double* M, int n, int m, const double* a, const double* b,
                            double reg, const double* gamma) {
    Problem p(M, n, m, a, b, reg);
    std::vector<double> T((size_t)n * m);
    return dual_obj(p, gamma, T.data());
}

double oracle_erot_dual_obj_grad(const double* M, int n, int m, const double* a, const double* b,
                                 double reg, const double* gamma, double* grad) {
    Problem p(M, n, m, a, b, reg);
    std::vector<double> T((size_t)n * m);
    return dual_obj_grad(p, gamma, grad, T.data(), true);
}

void oracle_erot_hvp(const double* M, int n, int m, const double* a, const double* b, double reg,
                     const double* gamma, const double* x, double* y) {
    Problem p(M, n, m, a, b, reg);
    std::vector<double> T((size_t)n * m);
    Vec g(n + m - 1);
    dual_obj_grad(p, gamma, g.data(), T.data(), true);
    for (int i = 0; i < n; i++) y[i] = (g[i] + a[i]) * x[i];
    for (int j = 0; j < m - 1; j++) y[n + j] = (g[n + j] + b[j]) * x[n + j];
    for (int j = 0; j < m - 1; j++) {
        const double* Tj = T.data() + (size_t)j * n;
        double s = 0.0;
        for (int i = 0; i < n; i++) {
            y[i] += Tj[i] * x[n + j];
            s += Tj[i] * x[i];
        }
        y[n + j] += s;
    }
    for (int k = 0; k < n + m - 1; k++) y[k] /= reg;
}

int oracle_erot_newton_direction(const double* M, int n, int m, const double* a, const double* b,
                                 double reg, const double* gamma, double* direc) {
    Problem p(M, n, m, a, b, reg);
    std::vector<double> T((size_t)n * m);
    Vec g(n + m - 1), d;
    dual_obj_grad(p, gamma, g.data(), T.data(), true);
    if (!newton_direction(p, T.data(), g, d)) return 1;
    std::copy(d.begin(), d.end(), direc);
    return 0;
}

double oracle_erot_compute_T(const double* M, int n, int m, double reg, const double* gamma,
                             double* T) {
    std::vector<double> ones(std::max(n, m), 1.0);
    Problem p(M, n, m, ones.data(), ones.data(), reg);
    return compute_T(p, gamma, T);
}

long oracle_sparsify_mat3(const double* T, int n, int m, double delta, double density_hint,
                          int* outer, int* inner, double* values, long cap) {
    CSC sp = sparsify_mat3(T, n, m, delta, density_hint);
    if (sp.nnz() > cap) return -1;
    std::copy(sp.outer.begin(), sp.outer.end(), outer);
    std::copy(sp.inner.begin(), sp.inner.end(), inner);
    std::copy(sp.val.begin(), sp.val.end(), values);
    return sp.nnz();
}

void oracle_erot_plan(const double* M, int n, int m, double reg, const double* gamma,
                      double* plan) {
    std::vector<double> ones(std::max(n, m), 1.0);
    Problem p(M, n, m, ones.data(), ones.data(), reg);
    get_plan(p, gamma, plan);
}

// sinkhorn_bcd_internal: sinkhorn_bcd.cpp:14-124.
int oracle_sinkhorn_bcd(const double* M, int n, int m, const double* a, const double* b,
                        double reg, double tol, int max_iter, int verbose,
                        const oracle_opts* opts, oracle_result* res) {
    try {
        Problem p(M, n, m, a, b, reg);
        Vec alpha(n), beta(m), gamma(n + m - 1), grad(n + m - 1);
        std::vector<double> T((size_t)n * m);
        History h(res);
        if (opts && opts->x0 && opts->x0_len == n + m - 1) {
            std::copy(opts->x0, opts->x0 + n, alpha.begin());
            std::copy(opts->x0 + n, opts->x0 + n + m - 1, beta.begin());
            beta[m - 1] = 0.0;
        } else {
            std::fill(alpha.begin(), alpha.end(), 0.0);
            optimal_beta(p, alpha.data(), beta.data());
        }
        Timer timer;
        timer.tic();
        gauge(n, m, alpha.data(), beta.data(), gamma.data());
        double f = dual_obj_grad(p, gamma.data(), grad.data(), T.data(), true);
        double gnorm = norm(grad);
        h.push(f, gnorm, timer.toc());
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if (gnorm < tol) break;
            optimal_alpha(p, beta.data(), alpha.data());
            optimal_beta(p, alpha.data(), beta.data());
            gauge(n, m, alpha.data(), beta.data(), gamma.data());
            f = dual_obj_grad(p, gamma.data(), grad.data(), T.data(), true);
            gnorm = norm(grad);
            const double d = timer.toc();
            h.push(f, gnorm, h.last_time() + d);
        }
        finish(p, i, gamma, h, res);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// sinkhorn_lbfgs_dual_internal: sinkhorn_lbfgs_dual.cpp:81-126 (SinkhornDual
// 18-79): L-BFGS on the dual objective with LBFGSParam() defaults except
// epsilon = tol, epsilon_rel = 0, max_iterations = max_iter (101-104).
int oracle_sinkhorn_lbfgs_dual(const double* M, int n, int m, const double* a, const double* b,
                               double reg, double tol, int max_iter, int verbose,
                               const oracle_opts* opts, oracle_result* res) {
    try {
        Problem p(M, n, m, a, b, reg);
        oracle::lbfgs::LbfgsParam param;
        param.epsilon = tol;
        param.epsilon_rel = 0.0;
        param.max_iterations = max_iter;
        Vec gamma;
        init_gamma(p, opts, gamma);
        std::vector<double> T((size_t)n * m);
        History h(res);
        Timer timer;
        double last_obj = std::numeric_limits<double>::infinity();
        int it = 0;
        oracle::lbfgs::FunGrad fg = [&](const Vec& x, Vec& g) {
            last_obj = dual_obj_grad(p, x.data(), g.data(), T.data(), true);
            return last_obj;
        };
        // SinkhornDual::iterate (58-78): objective of the last evaluation,
        // final_grad_norm, cumulative time; prim_vals are not recorded.
        auto iterate = [&](const Vec&, double gnorm) {
            const double d = timer.toc();
            h.push(last_obj, gnorm, h.last_time() + d);
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", it, last_obj, gnorm);
            it++;
            timer.tic();
        };
        timer.tic();
        double fx;
        const int niter = oracle::lbfgs::lbfgs_minimize(fg, iterate, param, gamma, fx);
        finish(p, niter, gamma, h, res);
        return 0;
    } catch (const std::invalid_argument& e) {
        set_err(res, e.what());
        return 2;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// sinkhorn_apdagd_internal: sinkhorn_apdagd.cpp:14-183. Accelerated
// primal-dual adaptive gradient descent on phi = -f over dual = -gamma, with
// the primal plan averaged over the iterations; stops when the duality gap
// and the marginal error of the averaged plan are both <= tol. The reported
// dual is -dualt of the last iteration and the plan is the averaged one.
int oracle_sinkhorn_apdagd(const double* M, int n, int m, const double* a, const double* b,
                           double reg, double tol, int max_iter, int verbose,
                           const oracle_opts* opts, oracle_result* res) {
    try {
        constexpr double L0 = 1.0;
        constexpr int max_inner = 20;
        Problem p(M, n, m, a, b, reg);
        const int N = n + m - 1;
        Vec gamma, grad(N), dual(N), dual_new(N), dualp(N), dualp_new(N), dualt(N), diff(N);
        std::vector<double> T((size_t)n * m);
        // averaged plan and the plan of the current dualt, row-major
        std::vector<double> plan((size_t)n * m), plan_t((size_t)n * m);
        History h(res);
        init_gamma(p, opts, gamma);
        for (int q = 0; q < N; q++) dual[q] = -gamma[q];
        dualp = dual;
        dualt = dual;
        get_plan(p, gamma.data(), plan.data());

        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), grad.data(), T.data(), true);
        double gnorm = norm(grad);
        h.push(f, gnorm, timer.toc());

        int i;
        double L = L0, pbeta = 0.0;
        for (i = 0; i < max_iter; i++) {
            timer.tic();
            L *= 0.5;
            double ptau = 0.0, phi_new = 0.0;
            for (int j = 0; j < max_inner; j++) {
                const double palpha = (1.0 + std::sqrt(4.0 * L * pbeta + 1.0)) / (2.0 * L);
                const double pbeta_new = pbeta + palpha;
                ptau = palpha / pbeta_new;
                for (int q = 0; q < N; q++) dualt[q] = (1.0 - ptau) * dual[q] + ptau * dualp[q];
                for (int q = 0; q < N; q++) gamma[q] = -dualt[q];
                f = dual_obj_grad(p, gamma.data(), grad.data(), T.data(), true);
                const double phit = -f;
                for (int q = 0; q < N; q++) dualp_new[q] = dualp[q] + palpha * grad[q];
                for (int q = 0; q < N; q++)
                    dual_new[q] = (1.0 - ptau) * dual[q] + ptau * dualp_new[q];
                for (int q = 0; q < N; q++) gamma[q] = -dual_new[q];
                f = dual_obj(p, gamma.data(), T.data());
                phi_new = -f;
                for (int q = 0; q < N; q++) diff[q] = dual_new[q] - dualt[q];
                const double rhs = phit + dot(grad, diff) - 0.5 * L * sqnorm(diff);
                if (verbose >= 2)
                    std::printf("j = %d, palpha = %g, pbeta = %g, phit = %g, phi_new = %g, rhs = %g\n",
                                j, palpha, pbeta_new, phit, phi_new, rhs);
                if (phi_new >= rhs || j >= max_inner - 1) {
                    pbeta = pbeta_new;
                    dualp.swap(dualp_new);
                    dual.swap(dual_new);
                    break;
                }
                L *= 2.0;
            }
            // plan = (1 - ptau) plan + ptau plan(-dualt)
            for (int q = 0; q < N; q++) gamma[q] = -dualt[q];
            get_plan(p, gamma.data(), plan_t.data());
            for (size_t e = 0; e < plan.size(); e++)
                plan[e] = (1.0 - ptau) * plan[e] + ptau * plan_t[e];
            // statistics of the averaged plan (0 * log 0 gives NaN, as in
            // the reference's array expression)
            double entropy = 0.0, mp = 0.0;
            std::vector<double> ra(n, 0.0), rb(m, 0.0);
            for (int jj = 0; jj < m; jj++)
                for (int ii = 0; ii < n; ii++) {
                    const double x = plan[(size_t)ii * m + jj];
                    entropy += x * (1.0 - std::log(x));
                    mp += p.Mij(ii, jj) * x;
                    ra[ii] += x;
                    rb[jj] += x;
                }
            const double primal_obj = mp - reg * entropy;
            double r2 = 0.0;
            for (int ii = 0; ii < n; ii++) r2 += (ra[ii] - a[ii]) * (ra[ii] - a[ii]);
            for (int jj = 0; jj < m; jj++) r2 += (rb[jj] - b[jj]) * (rb[jj] - b[jj]);
            const double mar_err = std::sqrt(r2);
            h.push(f, mar_err, h.last_time() + timer.toc());
            if (verbose >= 1)
                std::printf("iter = %d, primal_obj = %g, phi_new = %g, mar_err = %g\n", i,
                            primal_obj, phi_new, mar_err);
            if (primal_obj - phi_new <= tol && mar_err <= tol) break;
        }
        res->niter = i;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) std::copy(plan.begin(), plan.end(), res->plan);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// sinkhorn_newton_internal: sinkhorn_newton.cpp:17-129.
int oracle_sinkhorn_newton(const double* M, int n, int m, const double* a, const double* b,
                           double reg, double tol, int max_iter, int verbose,
                           const oracle_opts* opts, oracle_result* res) {
    try {
        constexpr double theta = 0.5, kappa = 0.5;
        constexpr int nlinesearch = 20;
        Problem p(M, n, m, a, b, reg);
        Vec gamma, newgamma(n + m - 1), direc, g(n + m - 1);
        std::vector<double> T((size_t)n * m), Tls((size_t)n * m);
        History h(res);
        init_gamma(p, opts, gamma);
        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), g.data(), T.data(), true);
        double gnorm = norm(g);
        h.push(f, gnorm, timer.toc());
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if ((gnorm < tol) || (!std::isfinite(f))) break;
            if (!newton_direction(p, T.data(), g, direc))
                throw std::runtime_error("Newton Hessian is not positive definite");
            double step = 1.0;
            const double thresh = theta * dot(g, direc);
            for (int k = 0; k < nlinesearch; k++) {
                for (int q = 0; q < n + m - 1; q++) newgamma[q] = gamma[q] + step * direc[q];
                const double newf = dual_obj(p, newgamma.data(), Tls.data());
                if (newf <= f + step * thresh) break;
                step *= kappa;
            }
            gamma.swap(newgamma);
            f = dual_obj_grad(p, gamma.data(), g.data(), T.data(), true);
            gnorm = norm(g);
            const double d = timer.toc();
            h.push(f, gnorm, h.last_time() + d);
        }
        finish(p, i, gamma, h, res);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// sinkhorn_ssns_internal: sinkhorn_ssns.cpp:16-234.
int oracle_sinkhorn_ssns(const double* M, int n, int m, const double* a, const double* b,
                         double reg, double tol, int max_iter, int verbose,
                         const oracle_opts* opts, oracle_result* res) {
    try {
        const int method = opts ? opts->method : 1;
        const double mu0 = opts ? opts->mu0 : 1.0;
        constexpr double rho_t1 = 0.25, rho_t2 = 0.75, mu_s1 = 4.0, mu_s2 = 0.5, kappa = 0.001,
                         cg_tol = 1e-8, nu0 = 0.01;
        double mu = mu0, rho = 1.0;
        Problem p(M, n, m, a, b, reg);
        Vec gamma, step(n + m - 1), Hstep, direc(n + m - 1, 0.0), g(n + m - 1);
        std::vector<double> T((size_t)n * m);
        History h(res);
        init_gamma(p, opts, gamma);
        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), g.data(), T.data(), true);
        double gnorm = norm(g);
        double delta = nu0 * gnorm;
        Hessian H;
        sparsified_hess(p, T.data(), g, delta, 0.001, H);
        h.push(f, gnorm, timer.toc(), H.density());
        const std::vector<double> alphas{1.0, 0.5, 0.25, 0.1};
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if (gnorm < tol) break;
            const double shift = mu * gnorm;
            // The warm start the reference sets here has length m while the
            // CG solves a system of size m-1, so it is never used
            // (sinkhorn_ssns.cpp:124 vs sinkhorn_cg.cpp:35).
            Vec rhs(n + m - 1);
            for (int q = 0; q < n + m - 1; q++) rhs[q] = -g[q];
            if (method == 0) {
                hess_cg(H, rhs, shift, nullptr, cg_tol, direc);
            } else {
                if (!hess_direct(H, rhs, shift, direc))
                    throw std::runtime_error("sparse factorization failed");
            }
            double newf;
            const double alpha = line_selection(p, alphas, gamma, direc, f, T.data(), newf);
            for (int q = 0; q < n + m - 1; q++) step[q] = alpha * direc[q];
            H.apply_Hsx(step, Hstep);
            const double numer = f - newf;
            const double denom = -dot(g, step) - 0.5 * dot(step, Hstep);
            rho = numer / denom;
            if (rho > 0.0)
                for (int q = 0; q < n + m - 1; q++) gamma[q] += step[q];
            if (rho < rho_t1) {
                mu = mu_s1 * mu;
            } else if (rho > rho_t2) {
                mu = std::max(mu_s2 * mu, kappa);
            }
            if (rho > 0.0) {
                f = dual_obj_grad(p, gamma.data(), g.data(), T.data(), false);
                gnorm = norm(g);
                delta = nu0 * gnorm;
                const double dens = H.density();
                sparsified_hess(p, T.data(), g, delta, dens, H);
            }
            const double d = timer.toc();
            h.push(f, gnorm, h.last_time() + d, H.density());
        }
        finish(p, i, gamma, h, res);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}


// Shared loop of sinkhorn_sparse_newton (sinkhorn_sparse_newton.cpp:24-171)
// and sinkhorn_splr (sinkhorn_splr.cpp:24-200): sparsified Hessian with a
// target density, shift min(gnorm, shift), More-Thuente line search from
// min(1, 1.5 alpha). SPLR adds the BFGS correction of solve_low_rank
// (sinkhorn_linsolve.cpp:160-225, always a direct factorization) when
// y's > 1e-6 y'y, and adapts the density more gently.
static int sparse_newton_loop(bool splr, const double* M, int n, int m, const double* a,
                              const double* b, double reg, double tol, int max_iter, int verbose,
                              const oracle_opts* opts, oracle_result* res) {
    try {
        const int method = opts ? opts->method : 1;
        const double density_max = opts ? opts->density : 0.01;
        const double density_min = 0.01 * density_max;
        double density = 0.1 * density_max;
        const double shift_max = opts ? opts->shift : 1e-3;
        const double cg_tol = 1e-8, eps = 1e-6;
        const int N = n + m - 1;
        Problem p(M, n, m, a, b, reg);
        Vec gamma, gamma_pre(N, 0.0), g(N), g_pre(N, 0.0), direc(N), x(N), gx(N), rhs(N);
        std::vector<double> T((size_t)n * m);
        History h(res);
        init_gamma(p, opts, gamma);
        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), g.data(), T.data(), true);
        double gnorm = norm(g);
        const double gnorm_init = gnorm;
        Hessian H;
        sparsified_hess_density(p, T.data(), g, density, H);
        h.push(f, gnorm, timer.toc(), density_T2H(density, n, m));
        double alpha = 1.0;
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if (gnorm < tol || !std::isfinite(f)) break;
            for (int q = 0; q < N; q++) rhs[q] = -g[q];
            const double shift = std::min(gnorm, shift_max);
            bool low_rank = false;
            Vec y(N), sv(N);
            double ys = 0.0;
            if (splr) {
                double yy = 0.0;
                for (int q = 0; q < N; q++) {
                    y[q] = g[q] - g_pre[q];
                    sv[q] = gamma[q] - gamma_pre[q];
                    ys += y[q] * sv[q];
                    yy += y[q] * y[q];
                }
                low_rank = (i > 0) && (ys > eps * yy);
            }
            if (low_rank) {
                Vec ir, iy;
                if (!hess_direct(H, rhs, shift, ir) || !hess_direct(H, y, shift, iy))
                    throw std::runtime_error("sparse factorization failed");
                const double rs = dot(sv, rhs), yiy = dot(y, iy), yir = dot(y, ir);
                const double rs_ys = rs / ys;
                const double cs = (1.0 + yiy / ys) * rs_ys - yir / ys;
                for (int q = 0; q < N; q++) direc[q] = ir[q] + cs * sv[q] - rs_ys * iy[q];
            } else if (method == 0) {
                hess_cg(H, rhs, shift, nullptr, cg_tol, direc);
            } else if (!hess_direct(H, rhs, shift, direc)) {
                throw std::runtime_error("sparse factorization failed");
            }
            bool recompute = true;
            auto eval = [&](double st, double* fx, double* dg) {
                for (int q = 0; q < N; q++) x[q] = gamma[q] + st * direc[q];
                *fx = dual_obj_grad(p, x.data(), gx.data(), T.data(), true);
                *dg = dot(gx, direc);
            };
            alpha = wolfe_search(std::min(1.0, 1.5 * alpha), f, dot(g, direc), eval, recompute);
            gamma_pre = gamma;
            for (int q = 0; q < N; q++) gamma[q] += alpha * direc[q];
            g_pre = g;
            // T is the last line-search evaluation unless recompute is set
            f = dual_obj_grad(p, gamma.data(), g.data(), T.data(), recompute);
            const double gnorm_pre = gnorm;
            gnorm = norm(g);
            if (splr) {
                const bool bad = (gnorm_pre < gnorm_init) && (gnorm > gnorm_pre);
                density *= bad ? 1.1 : 0.99;
            } else {
                const bool bad = (gnorm_pre < gnorm_init) && (gnorm > 1.1 * gnorm_pre);
                density *= bad ? 2.0 : 0.9;
            }
            density = std::min(density_max, std::max(density_min, density));
            sparsified_hess_density(p, T.data(), g, density, H);
            const double d = timer.toc();
            h.push(f, gnorm, h.last_time() + d, density_T2H(density, n, m));
        }
        finish(p, i, gamma, h, res);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

int oracle_sinkhorn_sparse_newton(const double* M, int n, int m, const double* a,
                                  const double* b, double reg, double tol, int max_iter,
                                  int verbose, const oracle_opts* opts, oracle_result* res) {
    return sparse_newton_loop(false, M, n, m, a, b, reg, tol, max_iter, verbose, opts, res);
}

int oracle_sinkhorn_splr(const double* M, int n, int m, const double* a, const double* b,
                         double reg, double tol, int max_iter, int verbose,
                         const oracle_opts* opts, oracle_result* res) {
    return sparse_newton_loop(true, M, n, m, a, b, reg, tol, max_iter, verbose, opts, res);
}

// sparsify_mat_with_density (sinkhorn_sparsify4.cpp:77-174, preserve = true)
// of a column-major n x m T into CSC of its first m-1 columns; returns nnz or
// -1 if cap is too small.
long oracle_sparsify_density(const double* T, int n, int m, double density, int* outer,
                             int* inner, double* values, long cap) {
    const CSC sp = sparsify_with_density(T, n, m, density);
    if (sp.nnz() > cap) return -1;
    std::copy(sp.outer.begin(), sp.outer.end(), outer);
    std::copy(sp.inner.begin(), sp.inner.end(), inner);
    std::copy(sp.val.begin(), sp.val.end(), values);
    return sp.nnz();
}

// line_search_wolfe on f(s) = c0 + c1 s + c2 s^2 + c3 s^3 + c4 s^4 (tests of
// the More-Thuente restatement); returns the step, recompute in *flag and the
// number of evaluations in *nev.
double oracle_wolfe_poly(const double* c, double init_step, int* flag, int* nev) {
    auto poly = [c](double s) { return c[0] + s * (c[1] + s * (c[2] + s * (c[3] + s * c[4]))); };
    auto dpoly = [c](double s) { return c[1] + s * (2 * c[2] + s * (3 * c[3] + s * 4 * c[4])); };
    int count = 0;
    auto eval = [&](double st, double* fx, double* dg) {
        *fx = poly(st);
        *dg = dpoly(st);
        count++;
    };
    bool recompute = false;
    const double step = wolfe_search(init_step, poly(0.0), dpoly(0.0), eval, recompute);
    *flag = recompute ? 1 : 0;
    *nev = count;
    return step;
}

}  // extern "C"
