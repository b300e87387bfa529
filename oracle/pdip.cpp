// FP64 oracle: the primal-dual interior-point method for QROT (qrot_pdip,
// inner_solver "cg" and "fp"). Test infrastructure only (see oracle.h).
//
// Restates src/pdip_cg.cpp:206-413 and src/pdip_fp.cpp:278-667 with the
// transport operators of src/pdip_transport_ops.hpp. Storage follows the
// reference: x, s and the cost are row-major n x m vectors (index i*m + j),
// the equality stack is A x = (column sums [m]; row sums of rows < n-1).
// M is passed column-major like the rest of the oracle; run_pdip
// (solvers.cpp:240-266) transposes it so that the cost is row-major.
//
// Linear algebra. The reference factors the (m+n-1)-square block matrix
// B = [diag(B11) D; D' diag(B22)] with Eigen (SimplicialLDLT for the CG
// preconditioner, dense LLT or SimplicialLLT for FP). The oracle factors the
// same matrix exactly by eliminating the diagonal demand block first and
// Cholesky-factoring the Schur complement diag(B22) - D' diag(1/B11) D
// densely; the solves agree with the reference's up to rounding.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <vector>

#include "oracle.h"
#include "oracle_util.h"

namespace oracle {
namespace pdip {

using Vec = std::vector<double>;
constexpr double SMALL = 1e-50;

struct Dims {
    int n, m;
    size_t nv() const { return (size_t)n * m; }
    int nc() const { return m + n - 1; }
};

// A x: column sums (m) then row sums of rows 0..n-2 (pdip_transport_ops.hpp:14-28),
// of x * scale when scale is given.
static void A_mul(const Dims& d, const double* x, const double* scale, double* y) {
    std::fill(y, y + d.nc(), 0.0);
    for (int i = 0; i < d.n; i++) {
        double r = 0.0;
        for (int j = 0; j < d.m; j++) {
            const size_t k = (size_t)i * d.m + j;
            const double v = scale ? x[k] * scale[k] : x[k];
            y[j] += v;
            r += v;
        }
        if (i < d.n - 1) y[d.m + i] = r;
    }
}

// A' lambda: Y(i, j) = lambda_j + (i < n-1 ? lambda_{m+i} : 0) (lines 31-40).
static void AT_mul(const Dims& d, const double* lam, double* y) {
    for (int i = 0; i < d.n; i++) {
        const double li = i < d.n - 1 ? lam[d.m + i] : 0.0;
        for (int j = 0; j < d.m; j++) y[(size_t)i * d.m + j] = lam[j] + li;
    }
}

// solve_AAT (lines 43-52).
static void solve_AAT(const Dims& d, const double* r, double* out) {
    const int n = d.n, m = d.m;
    double sum_d = 0.0;
    for (int j = 0; j < m; j++) sum_d += r[j];
    Vec tmp(n - 1);
    for (int i = 0; i < n - 1; i++) tmp[i] = sum_d / (double)n - r[m + i];
    double sum_t = 0.0;
    for (double v : tmp) sum_t += v;
    for (int i = 0; i < n - 1; i++) out[m + i] = (tmp[i] + sum_t) / (double)m;
    double sum_x2 = 0.0;
    for (int i = 0; i < n - 1; i++) sum_x2 += out[m + i];
    for (int j = 0; j < m; j++) out[j] = (r[j] - sum_x2) / (double)n;
}

static double step_size(const Vec& x, const Vec& dx) {
    double mn = 1.0;
    for (size_t k = 0; k < x.size(); k++) {
        const double c = dx[k] < 0 ? -x[k] / (dx[k] + SMALL) : 1.0;
        mn = std::min(mn, c);
    }
    return std::min(1.0, mn);
}

static double nrm(const double* v, size_t len) {
    double s = 0.0;
    for (size_t k = 0; k < len; k++) s += v[k] * v[k];
    return std::sqrt(s);
}

// marginal error: max of the row and column residual norms, a's last entry
// replaced by 1 - sum of the others (pdip_cg.cpp:71-83, pdip_fp.cpp:155-166).
static double mar_err(const Dims& d, const Vec& x, const Vec& eq) {
    const int n = d.n, m = d.m;
    Vec rs(n, 0.0), cs(m, 0.0);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < m; j++) {
            rs[i] += x[(size_t)i * m + j];
            cs[j] += x[(size_t)i * m + j];
        }
    double alast = 1.0;
    for (int i = 0; i < n - 1; i++) alast -= eq[m + i];
    double e1 = 0.0, e2 = 0.0;
    for (int i = 0; i < n; i++) {
        const double ai = i < n - 1 ? eq[m + i] : alast;
        e1 += (rs[i] - ai) * (rs[i] - ai);
    }
    for (int j = 0; j < m; j++) e2 += (cs[j] - eq[j]) * (cs[j] - eq[j]);
    return std::max(std::sqrt(e1), std::sqrt(e2));
}

// Block matrix [diag(B11) D; D' diag(B22)], D (m x n12) given by columns of
// supply rows: D(j, i) = scale(i, j), i < n-1. `keep` selects the stored
// off-diagonal entries (all for the dense operator).
struct Block {
    int m = 0, n12 = 0;
    Vec B11, B22;
    // sparse off-diagonal part by supply row i: (j, value)
    std::vector<std::vector<std::pair<int, double>>> rows;
};

static void block_diag(const Dims& d, const Vec& scale, Block& B) {
    const int n = d.n, m = d.m;
    B.m = m;
    B.n12 = n - 1;
    B.B11.assign(m, 0.0);
    B.B22.assign(n - 1, 0.0);
    for (int i = 0; i < n; i++) {
        double r = 0.0;
        for (int j = 0; j < m; j++) {
            const double v = scale[(size_t)i * m + j];
            B.B11[j] += v;
            r += v;
        }
        if (i < n - 1) B.B22[i] = r;
    }
}

// y = [diag(B11) w + D z ; diag(B22) z + D' w] with the full D (BlockACG,
// pdip_block_operator.h:88-96; matvec_A_block, pdip_fp.cpp:126-135).
static void full_mul(const Dims& d, const Vec& scale, const Block& B, const double* x, double* y) {
    const int m = d.m, n12 = d.n - 1;
    for (int j = 0; j < m; j++) y[j] = B.B11[j] * x[j];
    for (int i = 0; i < n12; i++) {
        double s = B.B22[i] * x[m + i];
        for (int j = 0; j < m; j++) {
            const double v = scale[(size_t)i * m + j];
            y[j] += v * x[m + i];
            s += v * x[j];
        }
        y[m + i] = s;
    }
}

// y = B_sparse x (matvec_B_block, pdip_fp.cpp:137-153).
static void sparse_mul(const Block& B, const double* x, double* y) {
    const int m = B.m;
    for (int j = 0; j < m; j++) y[j] = B.B11[j] * x[j];
    for (int i = 0; i < B.n12; i++) {
        double s = B.B22[i] * x[m + i];
        for (const auto& e : B.rows[i]) {
            y[e.first] += e.second * x[m + i];
            s += e.second * x[e.first];
        }
        y[m + i] = s;
    }
}

// Exact factorization of B + shift I: the demand block is diagonal, so
// B^-1 r follows from the dense Cholesky factor of the Schur complement
// S = diag(B22 + shift) - D' diag(1 / (B11 + shift)) D.
struct BlockChol {
    int m = 0, n12 = 0;
    Vec d1;   // B11 + shift
    Vec L;    // Cholesky factor of S (row-major, lower)
    const Block* B = nullptr;
    bool factor(const Block& blk, double shift) {
        B = &blk;
        m = blk.m;
        n12 = blk.n12;
        d1.resize(m);
        for (int j = 0; j < m; j++) {
            d1[j] = blk.B11[j] + shift;
            if (!(d1[j] > 0.0)) return false;
        }
        L.assign((size_t)n12 * n12, 0.0);
        for (int i = 0; i < n12; i++) L[(size_t)i * n12 + i] = blk.B22[i] + shift;
        // subtract D' diag(1/d1) D: by demand j over the supply rows touching it
        std::vector<std::vector<std::pair<int, double>>> cols(m);
        for (int i = 0; i < n12; i++)
            for (const auto& e : blk.rows[i]) cols[e.first].push_back({i, e.second});
        for (int j = 0; j < m; j++) {
            const auto& c = cols[j];
            for (size_t p = 0; p < c.size(); p++)
                for (size_t q = 0; q <= p; q++) {
                    const int a = c[p].first, b = c[q].first;
                    L[(size_t)std::max(a, b) * n12 + std::min(a, b)] -=
                        c[p].second * c[q].second / d1[j];
                }
        }
        return cholesky(L, n12);
    }
    void solve(const double* r, double* x) const {
        Vec t(n12);
        for (int i = 0; i < n12; i++) {
            double s = r[m + i];
            for (const auto& e : B->rows[i]) s -= e.second * r[e.first] / d1[e.first];
            t[i] = s;
        }
        cholesky_solve(L, n12, t);
        for (int j = 0; j < m; j++) x[j] = r[j];
        for (int i = 0; i < n12; i++)
            for (const auto& e : B->rows[i]) x[e.first] -= e.second * t[i];
        for (int j = 0; j < m; j++) x[j] /= d1[j];
        for (int i = 0; i < n12; i++) x[m + i] = t[i];
    }
};

// Factor with the shift retries of the reference (0, 1e-12, 1e-10, 1e-8;
// pdip_cg.cpp:262-268, pdip_sparse_chol.cpp:40-60).
static void factor_retry(const Block& blk, BlockChol& ch) {
    const double shifts[] = {0.0, 1e-12, 1e-10, 1e-8};
    for (double s : shifts)
        if (ch.factor(blk, s)) return;
    throw std::runtime_error("pdip: block factorization failed");
}

// dynamic_threshold: pdip_cg.cpp:95-143 (default keep factor 3).
static double dynamic_threshold(const Vec& scale, const Dims& d, int iter, double reg) {
    const int n = d.n, m = d.m;
    std::vector<double> pos;
    for (size_t k = 0; k < (size_t)(n - 1) * m; k++)
        if (scale[k] > 0) pos.push_back(scale[k]);
    if (pos.empty()) return 1e-9;
    double scale_ref = reg > 0 ? 1.0 / reg : 0.0;
    if (scale_ref < 1e-16) {
        const size_t mid = pos.size() / 2;
        std::nth_element(pos.begin(), pos.begin() + mid, pos.end());
        scale_ref = pos[mid];
    }
    scale_ref = std::max(scale_ref, 1e-16);
    const double keep_factor = 3.0;
    const int k0 = 15;
    const double progress = std::min((double)iter / k0, 1.0);
    const double eff = 1.0 + (keep_factor - 1.0) * progress;
    const double keep_ratio = std::min(1.0, eff / std::max(n, 1));
    size_t idx = (size_t)((1.0 - keep_ratio) * pos.size());
    if (idx >= pos.size()) idx = 0;
    std::nth_element(pos.begin(), pos.begin() + idx, pos.end());
    const double pct = pos[idx];
    const int iv = std::min(std::max(iter, 0), 52);
    const double t_fac = std::pow(1.48, iv);
    const double blend = std::min(1.0, (iter + 1) / 20.0);
    double th = (scale_ref / std::max(n, 1)) * t_fac * (1.0 - 0.52 * blend) + pct * 0.52 * blend;
    th = std::min(th, pct);
    const double min_th = std::max(1e-9, std::min(scale_ref * 1e-6, pct));
    th = std::max(th, min_th);
    th = std::min(th, scale_ref * 0.5);
    return th;
}

// Off-diagonal entries scale(i, j) >= th of the supply rows i < n-1.
static void block_pattern(const Dims& d, const Vec& scale, double th, Block& B) {
    B.rows.assign(d.n - 1, {});
    for (int i = 0; i < d.n - 1; i++)
        for (int j = 0; j < d.m; j++) {
            const double v = scale[(size_t)i * d.m + j];
            if (v >= th) B.rows[i].push_back({j, v});
        }
}

// Eigen::ConjugateGradient with a preconditioner (the textbook PCG loop of
// Eigen's conjugate_gradient): relative tolerance tol on ||r|| / ||b||.
template <typename Mul, typename Pre>
static void pcg(int N, Mul&& mul, Pre&& pre, const Vec& rhs, Vec& x, double tol, int max_iter) {
    Vec r(N), p(N), z(N), t(N);
    mul(x.data(), t.data());
    for (int q = 0; q < N; q++) r[q] = rhs[q] - t[q];
    double rhs2 = 0.0;
    for (double v : rhs) rhs2 += v * v;
    if (rhs2 == 0.0) {
        std::fill(x.begin(), x.end(), 0.0);
        return;
    }
    const double thresh = std::max(tol * tol * rhs2, std::numeric_limits<double>::min());
    double r2 = 0.0;
    for (double v : r) r2 += v * v;
    if (r2 < thresh) return;
    pre(r.data(), p.data());
    double absnew = 0.0;
    for (int q = 0; q < N; q++) absnew += r[q] * p[q];
    for (int it = 0; it < max_iter; it++) {
        mul(p.data(), t.data());
        double pt = 0.0;
        for (int q = 0; q < N; q++) pt += p[q] * t[q];
        const double alpha = absnew / pt;
        for (int q = 0; q < N; q++) {
            x[q] += alpha * p[q];
            r[q] -= alpha * t[q];
        }
        r2 = 0.0;
        for (double v : r) r2 += v * v;
        if (r2 < thresh) break;
        pre(r.data(), z.data());
        const double absold = absnew;
        absnew = 0.0;
        for (int q = 0; q < N; q++) absnew += r[q] * z[q];
        const double beta = absnew / absold;
        for (int q = 0; q < N; q++) p[q] = z[q] + beta * p[q];
    }
}

struct Opts {
    int cg_max_iter = 1000;
    double fixed_threshold = 1e-9;
    int fp_max_iter = 800;
    double fp_exit_scale = 1e-2;
    bool fp_stop_gap_mu_only = true;
    bool cg_stop_gap_mu_only = false;
    double cg_mar_tol = 1e-10;
};

// Shared PDIP loop; fp selects the inner solver of pdip_fp.cpp.
static int run(bool fp, const double* Mcol, int n, int m, const double* a, const double* b,
               double reg, double tol, int max_iter, const Opts& o, oracle_result* res) {
    const Dims d{n, m};
    const size_t nv = d.nv();
    const int nc = d.nc(), N = nc;
    const double reg_val = reg > 0 ? reg : 1e-6, barrier = reg_val;
    Vec cost(nv), eq(nc);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < m; j++) cost[(size_t)i * m + j] = Mcol[(size_t)j * n + i];
    for (int j = 0; j < m; j++) eq[j] = b[j];
    for (int i = 0; i < n - 1; i++) eq[m + i] = a[i];
    const auto t_start = std::chrono::steady_clock::now();

    // Phase 1: initial point (pdip_cg.cpp:240-262, pdip_fp.cpp:319-356)
    Vec lam(nc), x(nv), s(nv), at(nv), b2(nc), t(nc);
    solve_AAT(d, eq.data(), lam.data());
    AT_mul(d, lam.data(), x.data());
    A_mul(d, x.data(), nullptr, b2.data());
    A_mul(d, cost.data(), nullptr, t.data());
    for (int q = 0; q < nc; q++) b2[q] = -barrier * b2[q] - t[q];
    solve_AAT(d, b2.data(), lam.data());
    AT_mul(d, lam.data(), at.data());
    for (size_t k = 0; k < nv; k++) s[k] = barrier * x[k] + cost[k] + at[k];
    double dxs = 0.0, dss = 0.0;
    for (size_t k = 0; k < nv; k++) {
        if (x[k] < 0) dxs = std::max(dxs, -1.5 * x[k]);
        if (s[k] < 0) dss = std::max(dss, -1.5 * s[k]);
    }
    for (size_t k = 0; k < nv; k++) {
        x[k] += dxs;
        s[k] += dss;
    }
    {
        double xs = 0.0, ss = 0.0, xx = 0.0;
        for (size_t k = 0; k < nv; k++) {
            xs += x[k] * s[k];
            ss += s[k];
            xx += x[k];
        }
        const double ax = fp ? 0.5 * xs / ss : 0.5 * xs / (ss + SMALL);
        for (size_t k = 0; k < nv; k++) x[k] += ax;
        xs = 0.0;
        double sx = 0.0;
        for (size_t k = 0; k < nv; k++) {
            xs += x[k] * s[k];
            sx += x[k];
        }
        // pdip_fp.cpp:353 accumulates the new sum onto the old one
        xx = fp ? xx + sx : sx;
        const double as = fp ? 0.5 * xs / xx : 0.5 * xs / (xx + SMALL);
        for (size_t k = 0; k < nv; k++) {
            s[k] += as;
            x[k] = std::max(x[k], 1e-10);
            s[k] = std::max(s[k], 1e-10);
        }
    }

    Vec scale(nv), r_dual(nv), r_pri(nc), b1(nv), c(nc), dlam(nc, 0.0), dlam2(nc, 0.0),
        dlam_prev, dx(nv), ds(nv), rcc(nv), at_l(nv);
    History h(res);
    std::vector<double> mar_hist;
    double norm_eq = nrm(eq.data(), nc), norm_cost = nrm(cost.data(), nv);
    int niter = 0;
    bool converged = false;
    for (int it = 0; it < max_iter; it++) {
        // 2.1 residuals and scaling
        for (size_t k = 0; k < nv; k++) scale[k] = x[k] / (barrier * x[k] + s[k] + SMALL);
        AT_mul(d, lam.data(), at_l.data());
        for (size_t k = 0; k < nv; k++) r_dual[k] = barrier * x[k] + cost[k] + at_l[k] - s[k];
        A_mul(d, x.data(), nullptr, r_pri.data());
        for (int q = 0; q < nc; q++) r_pri[q] -= eq[q];

        // 2.2 the block matrix and its factorization
        Block blk;
        block_diag(d, scale, blk);
        BlockChol ch;
        bool use_fp_iter = false;
        if (!fp) {
            block_pattern(d, scale, dynamic_threshold(scale, d, it, reg_val), blk);
            factor_retry(blk, ch);
        } else {
            bool dense = it < 3;
            if (!dense) {
                long kept = 0;
                for (size_t k = 0; k < (size_t)(n - 1) * m; k++)
                    if (scale[k] >= o.fixed_threshold) kept++;
                const long total = (long)m * (n - 1);
                const double sparsity = total == 0 ? 1.0 : 1.0 - (double)kept / (double)total;
                use_fp_iter = o.fixed_threshold > 0.0 && sparsity >= 0.99;
                dense = !use_fp_iter;
            }
            if (use_fp_iter) block_pattern(d, scale, o.fixed_threshold, blk);
            else block_pattern(d, scale, -std::numeric_limits<double>::infinity(), blk);
            factor_retry(blk, ch);
        }

        // inner solve of B dlam = rhs (guess: the previous or the first solve)
        double cg_tol = 0.0;
        if (!fp) {
            const double rp = nrm(r_pri.data(), nc);
            const double tb = std::min((double)it, 40.0) / 40.0;
            const double rel = 0.1 * std::pow(0.01 / 0.1, tb);
            cg_tol = std::max(rel * rp, 1e-12);
        }
        auto inner = [&](const Vec& rhs, Vec& out, const Vec* guess) {
            if (!fp) {
                // solve_block_schur_cg (pdip_cg.cpp:157-176)
                if (guess && (int)guess->size() == N) out = *guess;
                else out.assign(N, 0.0);
                const double cn = nrm(rhs.data(), N) + 1e-50;
                const double rtol = std::min(cg_tol / cn, 0.1);
                const double bn = nrm(rhs.data(), N) + 1e-50;
                const double rel_eff = std::max(rtol, cg_tol / bn);
                pcg(N, [&](const double* xx, double* yy) { full_mul(d, scale, blk, xx, yy); },
                    [&](const double* rr, double* zz) { ch.solve(rr, zz); }, rhs, out, rel_eff,
                    o.cg_max_iter);
            } else if (!use_fp_iter) {
                out.resize(N);
                ch.solve(rhs.data(), out.data());
            } else {
                // fixed_point_solve_block_sparse (pdip_fp.cpp:232-276)
                Vec xk(N), xt(N), rw(N), rh(N);
                if (guess && !guess->empty()) xk = *guess;
                else ch.solve(rhs.data(), xk.data());
                full_mul(d, scale, blk, xk.data(), rw.data());
                double rpk = 0.0;
                for (int q = 0; q < N; q++) rpk += (rhs[q] - rw[q]) * (rhs[q] - rw[q]);
                rpk = std::sqrt(rpk) + 1e-20;
                const double exit_scale = o.fp_exit_scale <= 0 ? 1e-2 : o.fp_exit_scale;
                for (int k = 0; k < o.fp_max_iter; k++) {
                    full_mul(d, scale, blk, xk.data(), rw.data());
                    for (int q = 0; q < N; q++) rh[q] = rhs[q] - rw[q];
                    sparse_mul(blk, xk.data(), rw.data());
                    for (int q = 0; q < N; q++) rh[q] += rw[q];
                    ch.solve(rh.data(), xt.data());
                    full_mul(d, scale, blk, xt.data(), rw.data());
                    double rn = 0.0;
                    for (int q = 0; q < N; q++) rn += (rhs[q] - rw[q]) * (rhs[q] - rw[q]);
                    rn = std::sqrt(rn);
                    if (rn < exit_scale * rpk) break;
                    rpk = rn;
                    xk = xt;
                }
                out = xt;
            }
        };

        // 2.3 predictor
        for (size_t k = 0; k < nv; k++) b1[k] = -s[k] - r_dual[k];
        A_mul(d, b1.data(), scale.data(), c.data());
        for (int q = 0; q < nc; q++) c[q] += r_pri[q];
        inner(c, dlam, dlam_prev.size() == (size_t)N ? &dlam_prev : nullptr);
        AT_mul(d, dlam.data(), b1.data());
        for (size_t k = 0; k < nv; k++) {
            ds[k] = (1.0 - barrier * scale[k]) * (b1[k] + r_dual[k] - barrier * x[k]);
            dx[k] = (-x[k] * s[k] - x[k] * ds[k]) / (s[k] + SMALL);
        }
        double a1 = std::min(step_size(x, dx), 1.0);
        a1 = std::min(a1, step_size(s, ds));
        a1 = std::min(a1, 1.0);
        double mu = 0.0, mu_aff = 0.0;
        for (size_t k = 0; k < nv; k++) mu += x[k] * s[k];
        mu /= (double)nv;
        for (size_t k = 0; k < nv; k++) mu_aff += (x[k] + a1 * dx[k]) * (s[k] + a1 * ds[k]);
        mu_aff /= (double)nv;
        const double sigma = std::min(std::pow(mu_aff / mu, 3.0), 1.0);

        // 2.4 corrector
        for (size_t k = 0; k < nv; k++) {
            rcc[k] = x[k] * s[k] + dx[k] * ds[k] - sigma * mu;
            b1[k] = -rcc[k] / (x[k] + SMALL) - r_dual[k];
        }
        A_mul(d, b1.data(), scale.data(), c.data());
        for (int q = 0; q < nc; q++) c[q] += r_pri[q];
        inner(c, dlam2, &dlam);
        AT_mul(d, dlam2.data(), b1.data());
        for (size_t k = 0; k < nv; k++) {
            ds[k] = (1.0 - barrier * scale[k]) *
                    (b1[k] + r_dual[k] - barrier * rcc[k] / (s[k] + SMALL));
            dx[k] = (-rcc[k] - x[k] * ds[k]) / (s[k] + SMALL);
        }
        double a2 = std::min(step_size(x, dx), step_size(s, ds));
        a2 = std::min(0.99 * a2, 1.0);
        for (size_t k = 0; k < nv; k++) {
            x[k] += a2 * dx[k];
            s[k] += a2 * ds[k];
        }
        for (int q = 0; q < nc; q++) lam[q] += a2 * dlam2[q];
        dlam_prev = dlam2;

        // 2.5 convergence and history. PDIP-CG forms r_dual with the
        // multipliers' image from before the update (pdip_cg.cpp:352-356);
        // PDIP-FP with the updated one (pdip_fp.cpp:602-608).
        Vec at_new(nv);
        AT_mul(d, lam.data(), at_new.data());
        const Vec& at_rd = fp ? at_new : at_l;
        for (size_t k = 0; k < nv; k++) r_dual[k] = barrier * x[k] + cost[k] + at_rd[k] - s[k];
        A_mul(d, x.data(), nullptr, r_pri.data());
        for (int q = 0; q < nc; q++) r_pri[q] -= eq[q];
        const double primal_gap = nrm(r_pri.data(), nc) / (1.0 + norm_eq);
        const double dual_gap = nrm(r_dual.data(), nv) / (1.0 + norm_cost + nrm(at_new.data(), nv));
        mu = 0.0;
        for (size_t k = 0; k < nv; k++) mu += x[k] * s[k];
        mu /= (double)nv;
        const double me = mar_err(d, x, eq);
        double obj = 0.0, xx = 0.0;
        for (size_t k = 0; k < nv; k++) {
            obj += cost[k] * x[k];
            xx += x[k] * x[k];
        }
        obj += reg_val / 2.0 * xx;
        const double ms = std::chrono::duration<double, std::milli>(
                              std::chrono::steady_clock::now() - t_start).count();
        if (!fp) {
            if (!std::isfinite(me) || !std::isfinite(primal_gap) || !std::isfinite(dual_gap) ||
                !std::isfinite(mu))
                break;
            bool finite = true;
            for (size_t k = 0; k < nv && finite; k++) finite = std::isfinite(x[k]) && std::isfinite(s[k]);
            if (me > 1e3 || !finite) {
                niter = it + 1;
                break;
            }
        }
        h.push(obj, me, ms);
        mar_hist.push_back(me);
        const bool by_gap = primal_gap < tol && dual_gap < tol && mu < tol;
        bool stop;
        if (fp) {
            stop = o.fp_stop_gap_mu_only ? by_gap : (by_gap || me < tol);
        } else {
            bool stable = false;
            const int len = (int)mar_hist.size();
            if (len >= 30) {
                double mx = -1e30, mn = 1e30;
                for (int q = std::max(0, len - 30); q < len; q++) {
                    const double v = std::log10(std::max(mar_hist[q], 1e-20));
                    mx = std::max(mx, v);
                    mn = std::min(mn, v);
                }
                stable = mx - mn <= 0.1;
            }
            const bool by_mar = me < o.cg_mar_tol;
            stop = o.cg_stop_gap_mu_only ? by_gap : (by_gap || by_mar || (stable && by_mar));
        }
        niter = it + 1;
        if (stop) {
            converged = true;
            break;
        }
    }
    res->niter = niter;
    res->hist_len = h.len;
    if (res->dual) res->dual[0] = converged ? 1.0 : 0.0;  // converged flag
    if (res->plan) std::copy(x.begin(), x.end(), res->plan);
    return 0;
}

}  // namespace pdip
}  // namespace oracle

extern "C" {

// qrot_pdip (solvers.cpp:268-292): inner_solver 0 = "cg", 1 = "fp". M is
// column-major n x m; the plan is written row-major; res->dual[0] receives
// the converged flag. popts (may be NULL): cg_max_iter, fixed_threshold,
// fp_max_iter, fp_exit_scale, fp_stop_gap_mu_only, cg_stop_gap_mu_only,
// cg_mar_tol as doubles.
int oracle_qrot_pdip(const double* M, int n, int m, const double* a, const double* b, double reg,
                     double tol, int max_iter, int inner_solver, const double* popts,
                     oracle_result* res) {
    try {
        oracle::pdip::Opts o;
        if (popts) {
            o.cg_max_iter = (int)popts[0];
            o.fixed_threshold = popts[1];
            o.fp_max_iter = (int)popts[2];
            o.fp_exit_scale = popts[3];
            o.fp_stop_gap_mu_only = popts[4] != 0.0;
            o.cg_stop_gap_mu_only = popts[5] != 0.0;
            o.cg_mar_tol = popts[6];
        }
        return oracle::pdip::run(inner_solver == 1, M, n, m, a, b, reg, tol, max_iter, o, res);
    } catch (const std::exception& e) {
        oracle::set_err(res, e.what());
        return 1;
    }
}

}  // extern "C"
