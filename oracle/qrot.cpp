// FP64 oracle: quadratically regularised OT (QROT) problem pieces and the
// qrot_lbfgs_dual / qrot_assn solvers, including a restatement of the
// L-BFGS driver, two-loop recursion and Nocedal-Wright line search of the
// vendored LBFGS++ (MIT). Test infrastructure only (see oracle.h).
#include "oracle_lbfgs.h"
#include "oracle_util.h"

namespace oracle {
namespace qrot {

using namespace oracle::lbfgs;

struct Problem {
    int n, m;
    const double* M;  // column-major
    const double* a;
    const double* b;
    double reg, tau;
    double Mij(int i, int j) const { return M[(size_t)j * n + i]; }
};

// compute_D_stats: qrot_problem.cpp:36-94. C = alpha_i + beta_j - M_ij,
// D = C+ ; returns ||D||^2 and fills row/column sums of D when requested.
static double D_stats(const Problem& p, const double* gamma, double* rs, double* cs) {
    const int n = p.n, m = p.m;
    const double* alpha = gamma;
    const double* beta = gamma + n;
    double sq = 0.0;
    if (rs) std::fill(rs, rs + n, 0.0);
    for (int j = 0; j < m; j++) {
        const double* Mj = p.M + (size_t)j * n;
        const double bj = beta[j];
        double c = 0.0;
        for (int i = 0; i < n; i++) {
            const double C = alpha[i] + bj - Mj[i];
            if (C > 0.0) {
                sq += C * C;
                if (rs) rs[i] += C;
                c += C;
            }
        }
        if (cs) cs[j] = c;
    }
    return sq;
}

static double tau_diff(const Problem& p, const double* gamma) {
    return sum(gamma, p.n) - sum(gamma + p.n, p.m);
}

// dual_obj: qrot_problem.cpp:118-198.
static double dual_obj(const Problem& p, const double* gamma) {
    const double sq = D_stats(p, gamma, nullptr, nullptr);
    double obj = 0.5 * sq - p.reg * (dot(gamma, p.a, p.n) + dot(gamma + p.n, p.b, p.m));
    if (p.tau > 0.0) {
        const double d = tau_diff(p, gamma);
        obj += 0.5 * p.tau * d * d;
    }
    return obj;
}

// dual_obj_grad: qrot_problem.cpp:226-253; dual_grad 201-223.
static double dual_obj_grad(const Problem& p, const double* gamma, double* grad) {
    const int n = p.n, m = p.m;
    const double sq = D_stats(p, gamma, grad, grad + n);
    for (int i = 0; i < n; i++) grad[i] -= p.reg * p.a[i];
    for (int j = 0; j < m; j++) grad[n + j] -= p.reg * p.b[j];
    double obj = 0.5 * sq - p.reg * (dot(gamma, p.a, n) + dot(gamma + n, p.b, m));
    if (p.tau > 0.0) {
        const double d = tau_diff(p, gamma);
        obj += 0.5 * p.tau * d * d;
        for (int i = 0; i < n; i++) grad[i] += p.tau * d;
        for (int j = 0; j < m; j++) grad[n + j] -= p.tau * d;
    }
    return obj;
}

// piecewise_linear_equation: qrot_problem.cpp:368-392. Solves
// sum_i (x - y_i)+ = b for x from the sorted y.
static double piecewise_linear_equation(std::vector<double>& y, double b) {
    const int n = (int)y.size();
    std::sort(y.begin(), y.end());
    double cs = 0.0, f = 0.0;
    for (int i = 0; i < n - 1; i++) {
        cs += y[i];
        const double fnext = (i + 1) * y[i + 1] - cs;
        if (b >= f && b < fnext) return (b + cs) / (i + 1);
        f = fnext;
    }
    cs += y[n - 1];
    return (b + cs) / n;
}

// optimal_beta: qrot_problem.cpp:397-404.
static void optimal_beta(const Problem& p, const double* alpha, double* beta) {
    std::vector<double> y(p.n);
    for (int j = 0; j < p.m; j++) {
        const double* Mj = p.M + (size_t)j * p.n;
        for (int i = 0; i < p.n; i++) y[i] = Mj[i] - alpha[i];
        beta[j] = piecewise_linear_equation(y, p.reg * p.b[j]);
    }
}

// optimal_alpha: qrot_problem.cpp:409-419, the row analogue.
static void optimal_alpha(const Problem& p, const double* beta, double* alpha) {
    std::vector<double> y(p.m);
    for (int i = 0; i < p.n; i++) {
        for (int j = 0; j < p.m; j++) y[j] = p.Mij(i, j) - beta[j];
        alpha[i] = piecewise_linear_equation(y, p.reg * p.a[i]);
    }
}

// primal_val: qrot_problem.cpp:10-24 with approx_proj (approx_proj.h:6-26).
static double primal_val(const Problem& p, const double* gamma) {
    const int n = p.n, m = p.m;
    std::vector<double> P((size_t)n * m);  // column-major
    for (int j = 0; j < m; j++)
        for (int i = 0; i < n; i++) {
            const double C = gamma[i] + gamma[n + j] - p.Mij(i, j);
            P[(size_t)j * n + i] = std::max(C, 0.0) / p.reg;
        }
    Vec rs(n, 0.0), x(n), cs(m), y(m);
    for (int j = 0; j < m; j++)
        for (int i = 0; i < n; i++) rs[i] += P[(size_t)j * n + i];
    for (int i = 0; i < n; i++) x[i] = std::min(p.a[i] / rs[i], 1.0);
    for (int j = 0; j < m; j++)
        for (int i = 0; i < n; i++) P[(size_t)j * n + i] *= x[i];
    for (int j = 0; j < m; j++) {
        double c = 0.0;
        for (int i = 0; i < n; i++) c += P[(size_t)j * n + i];
        cs[j] = c;
    }
    for (int j = 0; j < m; j++) y[j] = std::min(p.b[j] / cs[j], 1.0);
    for (int j = 0; j < m; j++)
        for (int i = 0; i < n; i++) P[(size_t)j * n + i] *= y[j];
    Vec ea(n), eb(m);
    std::fill(rs.begin(), rs.end(), 0.0);
    for (int j = 0; j < m; j++) {
        double c = 0.0;
        for (int i = 0; i < n; i++) {
            rs[i] += P[(size_t)j * n + i];
            c += P[(size_t)j * n + i];
        }
        eb[j] = p.b[j] - c;
    }
    double l1 = 0.0;
    for (int i = 0; i < n; i++) {
        ea[i] = p.a[i] - rs[i];
        l1 += std::abs(ea[i]);
    }
    double val = 0.0, sq = 0.0;
    for (int j = 0; j < m; j++)
        for (int i = 0; i < n; i++) {
            const double v = P[(size_t)j * n + i] + ea[i] * eb[j] / l1;
            val += v * p.Mij(i, j);
            sq += v * v;
        }
    return val + 0.5 * p.reg * sq;
}

// Generalized Hessian: qrot_hess.h:37-176, qrot_hess.cpp:41-216.
// sigma = 1[C > 0] kept as per-row and per-column index lists.
struct Hessian {
    int n = 0, m = 0;
    Vec h1, h2;
    std::vector<std::vector<int>> sigma, sigmat;
    void apply_sigmax(const double* x, double* res) const {
        for (int i = 0; i < n; i++) {
            double s = 0.0;
            for (int j : sigma[i]) s += x[j];
            res[i] = s;
        }
    }
    void apply_sigmatx(const double* x, double* res) const {
        for (int j = 0; j < m; j++) {
            double s = 0.0;
            for (int i : sigmat[j]) s += x[i];
            res[j] = s;
        }
    }
    // solve_Ax: qrot_hess.cpp:127-142.
    void solve_Ax(const double* x, double shift, double tau, double* res) const {
        if (tau > 0.0) {
            double c1 = 1.0 / tau, c2 = 0.0;
            Vec xh(n);
            for (int i = 0; i < n; i++) {
                xh[i] = x[i] / (h1[i] + shift);
                c1 += 1.0 / (h1[i] + shift);
                c2 += xh[i];
            }
            for (int i = 0; i < n; i++) res[i] = xh[i] - (c2 / c1) / (h1[i] + shift);
        } else {
            for (int i = 0; i < n; i++) res[i] = x[i] / (h1[i] + shift);
        }
    }
    void apply_Bx(const double* x, double tau, double* res) const {
        apply_sigmax(x, res);
        if (tau > 0.0) {
            const double s = sum(x, m);
            for (int i = 0; i < n; i++) res[i] -= tau * s;
        }
    }
    void apply_Cx(const double* x, double tau, double* res) const {
        apply_sigmatx(x, res);
        if (tau > 0.0) {
            const double s = sum(x, n);
            for (int j = 0; j < m; j++) res[j] -= tau * s;
        }
    }
    // apply_Deltax: qrot_hess.cpp:173-189.
    void apply_Deltax(const Vec& x, double shift, double tau, Vec& res) const {
        Vec bx(n), t(n), ct(m);
        apply_Bx(x.data(), tau, bx.data());
        solve_Ax(bx.data(), shift, tau, t.data());
        apply_Cx(t.data(), tau, ct.data());
        res.resize(m);
        for (int j = 0; j < m; j++) res[j] = h2[j] * x[j] + shift * x[j] - ct[j];
        if (tau > 0.0) {
            const double s = sum(x.data(), m);
            for (int j = 0; j < m; j++) res[j] += tau * s;
        }
    }
};

// compute_D_hess: qrot_hess.cpp:41-96 (also gives ||D||^2 and D sums).
static double D_hess(const Problem& p, const double* gamma, double* rs, double* cs, Hessian& H) {
    const int n = p.n, m = p.m;
    H.n = n;
    H.m = m;
    H.h1.assign(n, 0.0);
    H.h2.assign(m, 0.0);
    H.sigma.assign(n, {});
    H.sigmat.assign(m, {});
    std::fill(rs, rs + n, 0.0);
    double sq = 0.0;
    for (int j = 0; j < m; j++) {
        const double* Mj = p.M + (size_t)j * n;
        const double bj = gamma[n + j];
        double c = 0.0;
        int h2j = 0;
        for (int i = 0; i < n; i++) {
            const double C = gamma[i] + bj - Mj[i];
            if (C > 0.0) {
                H.sigma[i].push_back(j);
                H.sigmat[j].push_back(i);
                sq += C * C;
                rs[i] += C;
                c += C;
                H.h1[i] += 1;
                h2j++;
            }
        }
        cs[j] = c;
        H.h2[j] = h2j;
    }
    return sq;
}

// dual_obj_grad_hess: qrot_problem.cpp:262-290.
static double dual_obj_grad_hess(const Problem& p, const double* gamma, double* grad, Hessian& H) {
    const int n = p.n, m = p.m;
    const double sq = D_hess(p, gamma, grad, grad + n, H);
    double obj = 0.5 * sq - p.reg * (dot(gamma, p.a, n) + dot(gamma + n, p.b, m));
    for (int i = 0; i < n; i++) grad[i] -= p.reg * p.a[i];
    for (int j = 0; j < m; j++) grad[n + j] -= p.reg * p.b[j];
    if (p.tau > 0.0) {
        const double d = tau_diff(p, gamma);
        obj += 0.5 * p.tau * d * d;
        for (int i = 0; i < n; i++) grad[i] += p.tau * d;
        for (int j = 0; j < m; j++) grad[n + j] -= p.tau * d;
    }
    return obj;
}

// hess_cg: qrot_cg.cpp:9-50 (Schur complement on the beta block).
static int hess_cg(const Hessian& H, const Vec& rhs, double shift, double tau, double tol,
                   Vec& res) {
    const int n = H.n, m = H.m;
    res.assign(n + m, 0.0);
    Vec v(n), y(m), zy(m);
    H.solve_Ax(rhs.data(), shift, tau, v.data());
    H.apply_Cx(v.data(), tau, y.data());
    for (int j = 0; j < m; j++) zy[j] = rhs[n + j] - y[j];
    Vec r2;
    const int it = cg_solve([&](const Vec& x, Vec& out) { H.apply_Deltax(x, shift, tau, out); },
                            zy, r2, tol, nullptr);
    std::copy(r2.begin(), r2.end(), res.begin() + n);
    Vec bx(n), t(n);
    H.apply_Bx(r2.data(), tau, bx.data());
    for (int i = 0; i < n; i++) t[i] = rhs[i] - bx[i];
    H.solve_Ax(t.data(), shift, tau, res.data());
    return it;
}

// Direct solve used for method != 0 (the reference factors the sparse
// matrix, qrot_linsolve.cpp:72-105): dense Cholesky of the Schur
// complement, exact for the same SPD system (tau = 0 only).
static bool hess_direct(const Hessian& H, const Vec& rhs, double shift, Vec& res) {
    const int n = H.n, m = H.m;
    std::vector<double> S((size_t)m * m, 0.0);
    for (int j = 0; j < m; j++) S[(size_t)j * m + j] = H.h2[j] + shift;
    for (int i = 0; i < n; i++) {
        const double w = 1.0 / (H.h1[i] + shift);
        const auto& r = H.sigma[i];
        for (size_t p = 0; p < r.size(); p++)
            for (size_t q = 0; q <= p; q++) {
                const int j = r[p], k = r[q];
                S[(size_t)std::max(j, k) * m + std::min(j, k)] -= w;
            }
    }
    if (!cholesky(S, m)) return false;
    Vec v(n), y(m), r2(m);
    for (int i = 0; i < n; i++) v[i] = rhs[i] / (H.h1[i] + shift);
    H.apply_sigmatx(v.data(), y.data());
    for (int j = 0; j < m; j++) r2[j] = rhs[n + j] - y[j];
    cholesky_solve(S, m, r2);
    res.assign(n + m, 0.0);
    Vec bx(n);
    H.apply_sigmax(r2.data(), bx.data());
    for (int i = 0; i < n; i++) res[i] = (rhs[i] - bx[i]) / (H.h1[i] + shift);
    for (int j = 0; j < m; j++) res[n + j] = r2[j];
    return true;
}

static void get_plan(const Problem& p, const double* gamma, double* plan) {
    // qrot_result.h:31-43, written row-major.
    for (int i = 0; i < p.n; i++)
        for (int j = 0; j < p.m; j++) {
            const double C = gamma[i] + gamma[p.n + j] - p.Mij(i, j);
            plan[(size_t)i * p.m + j] = std::max(C, 0.0) / p.reg;
        }
}

static void init_gamma(const Problem& p, const oracle_opts* opts, Vec& gamma) {
    gamma.assign(p.n + p.m, 0.0);
    if (opts && opts->x0 && opts->x0_len == p.n + p.m) {
        std::copy(opts->x0, opts->x0 + p.n + p.m, gamma.begin());
        return;
    }
    optimal_beta(p, gamma.data(), gamma.data() + p.n);
}

}  // namespace qrot
}  // namespace oracle

using namespace oracle;
using namespace oracle::qrot;

static Problem make_problem(const double* M, int n, int m, const double* a, const double* b,
                            double reg, double tau) {
    Problem p;
    p.n = n;
    p.m = m;
    p.M = M;
    p.a = a;
    p.b = b;
    p.reg = reg;
    p.tau = tau;
    return p;
}

extern "C" {

double oracle_qrot_dual_obj(const double* M, int n, int m, const double* a, const double* b,
                            double reg, double tau, const double* gamma) {
    return dual_obj(make_problem(M, n, m, a, b, reg, tau), gamma);
}

double oracle_qrot_dual_obj_grad(const double* M, int n, int m, const double* a, const double* b,
                                 double reg, double tau, const double* gamma, double* grad) {
    return dual_obj_grad(make_problem(M, n, m, a, b, reg, tau), gamma, grad);
}

void oracle_qrot_optimal_alpha(const double* M, int n, int m, const double* a, double reg,
                               const double* beta, double* alpha) {
    Problem p = make_problem(M, n, m, a, a, reg, 0.0);
    optimal_alpha(p, beta, alpha);
}

void oracle_qrot_optimal_beta(const double* M, int n, int m, const double* b, double reg,
                              const double* alpha, double* beta) {
    Problem p = make_problem(M, n, m, nullptr, b, reg, 0.0);
    optimal_beta(p, alpha, beta);
}

double oracle_qrot_primal_val(const double* M, int n, int m, const double* a, const double* b,
                              double reg, const double* gamma) {
    return primal_val(make_problem(M, n, m, a, b, reg, 0.0), gamma);
}

int oracle_qrot_hess_cg(const double* M, int n, int m, const double* gamma, const double* rhs,
                        double shift, double tau, double cg_tol, double* res) {
    std::vector<double> ones(std::max(n, m), 1.0);
    Problem p = make_problem(M, n, m, ones.data(), ones.data(), 1.0, tau);
    Hessian H;
    Vec g(n + m), r(rhs, rhs + n + m), out;
    D_hess(p, gamma, g.data(), g.data() + n, H);
    const int it = hess_cg(H, r, shift, tau, cg_tol, out);
    std::copy(out.begin(), out.end(), res);
    return it;
}

void oracle_qrot_plan(const double* M, int n, int m, double reg, const double* gamma,
                      double* plan) {
    get_plan(make_problem(M, n, m, nullptr, nullptr, reg, 0.0), gamma, plan);
}

// qrot_bcd_internal: qrot_bcd.cpp:14-103 (block coordinate descent: alpha
// then beta exactly; the problem is built with tau = 0).
int oracle_qrot_bcd(const double* M, int n, int m, const double* a, const double* b, double reg,
                    double tol, int max_iter, int verbose, const oracle_opts* opts,
                    oracle_result* res) {
    try {
        Problem p = make_problem(M, n, m, a, b, reg, 0.0);
        Vec gamma, grad(n + m);
        init_gamma(p, opts, gamma);
        History h(res);
        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), grad.data());
        double gnorm = norm(grad);
        h.push(f, gnorm / reg, timer.toc(), 0.0, primal_val(p, gamma.data()));
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if (gnorm < tol) break;
            optimal_alpha(p, gamma.data() + n, gamma.data());
            optimal_beta(p, gamma.data(), gamma.data() + n);
            f = dual_obj_grad(p, gamma.data(), grad.data());
            gnorm = norm(grad);
            const double d = timer.toc();
            h.push(f, gnorm / reg, h.last_time() + d, 0.0, primal_val(p, gamma.data()));
        }
        res->niter = i;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) get_plan(p, gamma.data(), res->plan);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// qrot_gd_internal: qrot_gd.cpp:14-120 (gradient descent with Armijo
// backtracking: theta = kappa = 0.5, at most 20 trials; the last trial is
// kept when none is accepted).
int oracle_qrot_gd(const double* M, int n, int m, const double* a, const double* b, double reg,
                   double tol, int max_iter, int verbose, const oracle_opts* opts,
                   oracle_result* res) {
    try {
        constexpr double theta = 0.5, kappa = 0.5;
        constexpr int nlinesearch = 20;
        const double tau = opts ? opts->tau : 0.0;
        Problem p = make_problem(M, n, m, a, b, reg, tau);
        Vec gamma, newgamma(n + m), grad(n + m);
        init_gamma(p, opts, gamma);
        History h(res);
        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), grad.data());
        double gnorm = norm(grad);
        h.push(f, gnorm / reg, timer.toc(), 0.0, primal_val(p, gamma.data()));
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if (gnorm < tol) break;
            double step = 1.0;
            const double thresh = theta * gnorm * gnorm;
            for (int k = 0; k < nlinesearch; k++) {
                for (int q = 0; q < n + m; q++) newgamma[q] = gamma[q] - step * grad[q];
                const double newf = dual_obj(p, newgamma.data());
                if (newf <= f - step * thresh) break;
                step *= kappa;
            }
            gamma.swap(newgamma);
            f = dual_obj_grad(p, gamma.data(), grad.data());
            gnorm = norm(grad);
            const double d = timer.toc();
            h.push(f, gnorm / reg, h.last_time() + d, 0.0, primal_val(p, gamma.data()));
        }
        res->niter = i;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) get_plan(p, gamma.data(), res->plan);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// Primal objective <M, X> + reg/2 ||X||^2 and marginal error of an averaged
// plan X (row-major), as qrot_apdagd.cpp:141-146 / qrot_pdaam.cpp:150-155.
static void plan_stats(const Problem& p, const Vec& X, double* primal, double* mar_err) {
    const int n = p.n, m = p.m;
    Vec rs(n, 0.0), cs(m, 0.0);
    double mx = 0.0, xx = 0.0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < m; j++) {
            const double x = X[(size_t)i * m + j];
            mx += p.Mij(i, j) * x;
            xx += x * x;
            rs[i] += x;
            cs[j] += x;
        }
    double r2 = 0.0;
    for (int i = 0; i < n; i++) r2 += (rs[i] - p.a[i]) * (rs[i] - p.a[i]);
    for (int j = 0; j < m; j++) r2 += (cs[j] - p.b[j]) * (cs[j] - p.b[j]);
    *primal = mx + 0.5 * p.reg * xx;
    *mar_err = std::sqrt(r2);
}

// qrot_apdagd_internal: qrot_apdagd.cpp:14-179 (accelerated primal-dual
// adaptive gradient descent on dual = -gamma, phi = -f / reg; L0 = 1, at
// most 20 line-search trials, plan averaged with weight ptau).
int oracle_qrot_apdagd(const double* M, int n, int m, const double* a, const double* b,
                       double reg, double tol, int max_iter, int verbose,
                       const oracle_opts* opts, oracle_result* res) {
    try {
        constexpr double L0 = 1.0;
        constexpr int max_inner = 20;
        const int N = n + m;
        Problem p = make_problem(M, n, m, a, b, reg, 0.0);
        Vec gamma, grad(N), dual(N), dual_new(N), dualp(N), dualp_new(N), dualt(N);
        init_gamma(p, opts, gamma);
        for (int q = 0; q < N; q++) dual[q] = -gamma[q];
        dualp = dual;
        dualt = dual;
        Vec X((size_t)n * m), Xn((size_t)n * m);
        get_plan(p, gamma.data(), X.data());
        History h(res);
        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), grad.data());
        h.push(f, norm(grad) / reg, timer.toc(), 0.0, primal_val(p, gamma.data()));
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
                f = dual_obj_grad(p, gamma.data(), grad.data());
                const double phit = -f / reg;
                for (int q = 0; q < N; q++) dualp_new[q] = dualp[q] + (palpha / reg) * grad[q];
                for (int q = 0; q < N; q++)
                    dual_new[q] = (1.0 - ptau) * dual[q] + ptau * dualp_new[q];
                for (int q = 0; q < N; q++) gamma[q] = -dual_new[q];
                f = dual_obj(p, gamma.data());
                phi_new = -f / reg;
                double gd = 0.0, dd = 0.0;
                for (int q = 0; q < N; q++) {
                    const double df = dual_new[q] - dualt[q];
                    gd += grad[q] * df;
                    dd += df * df;
                }
                const double rhs = phit + gd / reg - 0.5 * L * dd;
                if (verbose >= 2)
                    std::printf("j = %d, palpha = %g, pbeta = %g, phit = %g, phi_new = %g, "
                                "rhs = %g\n", j, palpha, pbeta_new, phit, phi_new, rhs);
                if (phi_new >= rhs || j >= max_inner - 1) {
                    pbeta = pbeta_new;
                    dualp.swap(dualp_new);
                    dual.swap(dual_new);
                    break;
                }
                L *= 2.0;
            }
            for (int q = 0; q < N; q++) gamma[q] = -dualt[q];
            get_plan(p, gamma.data(), Xn.data());
            for (size_t e = 0; e < X.size(); e++) X[e] = (1.0 - ptau) * X[e] + ptau * Xn[e];
            double primal_obj, mar_err;
            plan_stats(p, X, &primal_obj, &mar_err);
            const double d = timer.toc();
            h.push(f, mar_err, h.last_time() + d, 0.0, primal_val(p, gamma.data()));
            if (verbose >= 1)
                std::printf("iter = %d, primal_obj = %g, phi_new = %g, mar_err = %g\n", i,
                            primal_obj, phi_new, mar_err);
            if (primal_obj - phi_new <= tol && mar_err <= tol) break;
        }
        res->niter = i;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) std::copy(X.begin(), X.end(), res->plan);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// qrot_pdaam_internal: qrot_pdaam.cpp:14-188 (primal-dual accelerated
// alternating minimisation: the block with the larger gradient norm is
// minimised exactly at the extrapolated point; L0 = 1, at most 20 trials).
int oracle_qrot_pdaam(const double* M, int n, int m, const double* a, const double* b,
                      double reg, double tol, int max_iter, int verbose,
                      const oracle_opts* opts, oracle_result* res) {
    try {
        constexpr double L0 = 1.0;
        constexpr int max_inner = 20;
        const int N = n + m;
        Problem p = make_problem(M, n, m, a, b, reg, 0.0);
        Vec gamma, grad(N), dual(N), dual_new(N), dualp(N), dualt(N);
        init_gamma(p, opts, gamma);
        for (int q = 0; q < N; q++) dual[q] = -gamma[q];
        dualp = dual;
        dualt = dual;
        Vec X((size_t)n * m), Xn((size_t)n * m);
        get_plan(p, gamma.data(), X.data());
        History h(res);
        Timer timer;
        timer.tic();
        double f = dual_obj_grad(p, gamma.data(), grad.data());
        h.push(f, norm(grad) / reg, timer.toc(), 0.0, primal_val(p, gamma.data()));
        int i;
        double L = L0, palpha = 0.0;
        for (i = 0; i < max_iter; i++) {
            timer.tic();
            double L_new = 0.5 * L, phi_new = 0.0, tau_old = 0.0, tau_new = 0.0;
            for (int j = 0; j < max_inner; j++) {
                const double palpha_new =
                    (1.0 + std::sqrt(4.0 * palpha * palpha * L * L_new + 1.0)) / (2.0 * L_new);
                const double ptau = 1.0 / (palpha_new * L_new);
                for (int q = 0; q < N; q++) dualt[q] = (1.0 - ptau) * dual[q] + ptau * dualp[q];
                for (int q = 0; q < N; q++) gamma[q] = -dualt[q];
                f = dual_obj_grad(p, gamma.data(), grad.data());
                const double phit = -f / reg;
                double lam = 0.0, mu = 0.0;
                for (int q = 0; q < n; q++) lam += grad[q] * grad[q];
                for (int q = 0; q < m; q++) mu += grad[n + q] * grad[n + q];
                if (lam > mu) optimal_alpha(p, gamma.data() + n, gamma.data());
                else optimal_beta(p, gamma.data(), gamma.data() + n);
                for (int q = 0; q < N; q++) dual_new[q] = -gamma[q];
                f = dual_obj(p, gamma.data());
                phi_new = -f / reg;
                const double rhs = phit + (lam + mu) / (2.0 * L_new * reg * reg);
                if (verbose >= 2)
                    std::printf("j = %d, L = %g, palpha = %g, phit = %g, phi_new = %g, rhs = %g\n",
                                j, L_new, palpha, phit, phi_new, rhs);
                if (phi_new >= rhs || j >= max_inner - 1) {
                    const double ar = palpha / palpha_new, lr = L / L_new;
                    tau_old = ar * ar * lr;
                    tau_new = ptau;
                    palpha = palpha_new;
                    L = L_new;
                    dual.swap(dual_new);
                    break;
                }
                L_new *= 2.0;
            }
            for (int q = 0; q < N; q++) dualp[q] += (palpha / reg) * grad[q];
            for (int q = 0; q < N; q++) gamma[q] = -dualt[q];
            get_plan(p, gamma.data(), Xn.data());
            for (size_t e = 0; e < X.size(); e++) X[e] = tau_old * X[e] + tau_new * Xn[e];
            double primal_obj, mar_err;
            plan_stats(p, X, &primal_obj, &mar_err);
            const double d = timer.toc();
            h.push(f, mar_err, h.last_time() + d, 0.0, primal_val(p, gamma.data()));
            if (verbose >= 1)
                std::printf("iter = %d, primal_obj = %g, phi_new = %g, mar_err = %g\n", i,
                            primal_obj, phi_new, mar_err);
            if (primal_obj - phi_new <= tol && mar_err <= tol) break;
        }
        res->niter = i;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) std::copy(X.begin(), X.end(), res->plan);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// semi_dual_obj_grad: qrot_problem.cpp:420-442. beta = optimal_beta(alpha),
// f = 0.5 ||D||^2 - reg (a'alpha + b'beta), grad = D 1 - reg a.
static double semi_dual_obj_grad(const Problem& p, const double* alpha, double* grad,
                                 double* beta) {
    const int n = p.n, m = p.m;
    optimal_beta(p, alpha, beta);
    Vec gamma(n + m);
    std::copy(alpha, alpha + n, gamma.begin());
    std::copy(beta, beta + m, gamma.begin() + n);
    const double sq = D_stats(p, gamma.data(), grad, nullptr);
    for (int i = 0; i < n; i++) grad[i] -= p.reg * p.a[i];
    return 0.5 * sq - p.reg * (dot(alpha, p.a, n) + dot(beta, p.b, m));
}

// qrot_lbfgs_semi_dual_internal: qrot_lbfgs_semi_dual.cpp:84-126
// (QROTSemiDual 18-82): L-BFGS on alpha with epsilon = epsilon_rel = tol;
// alpha0 = 0 or the first n entries of x0; the result is
// (alpha, optimal_beta(alpha)).
int oracle_qrot_lbfgs_semi_dual(const double* M, int n, int m, const double* a,
                                const double* b, double reg, double tol, int max_iter,
                                int verbose, const oracle_opts* opts, oracle_result* res) {
    try {
        Problem p = make_problem(M, n, m, a, b, reg, 0.0);
        LbfgsParam param;
        param.epsilon = tol;
        param.epsilon_rel = tol;
        param.max_iterations = max_iter;
        Vec alpha(n, 0.0), beta(m);
        if (opts && opts->x0 && opts->x0_len == n + m) std::copy(opts->x0, opts->x0 + n, alpha.begin());
        History h(res);
        Timer timer;
        double last_obj = std::numeric_limits<double>::infinity();
        int it = 0;
        FunGrad fg = [&](const Vec& x, Vec& g) {
            last_obj = semi_dual_obj_grad(p, x.data(), g.data(), beta.data());
            return last_obj;
        };
        Vec gamma(n + m);
        auto iterate = [&](const Vec& x, double gnorm) {
            const double d = timer.toc();
            std::copy(x.begin(), x.end(), gamma.begin());
            optimal_beta(p, x.data(), gamma.data() + n);
            const double prim = primal_val(p, gamma.data());
            h.push(last_obj, gnorm / reg, h.last_time() + d, 0.0, prim);
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", it, last_obj, gnorm);
            it++;
            timer.tic();
        };
        timer.tic();
        double fx;
        const int niter = lbfgs_minimize(fg, iterate, param, alpha, fx);
        std::copy(alpha.begin(), alpha.end(), gamma.begin());
        optimal_beta(p, alpha.data(), gamma.data() + n);
        res->niter = niter;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) get_plan(p, gamma.data(), res->plan);
        return 0;
    } catch (const std::invalid_argument& e) {
        set_err(res, e.what());
        return 2;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// qrot_grssn_internal: qrot_grssn.cpp:16-133 (regularized semi-smooth Newton:
// direction (H + shift I)^{-1}(-g) by the Schur CG of hess_cg with tolerance
// 1e-8, Armijo backtracking theta = kappa = 0.5, at most 20 trials).
int oracle_qrot_grssn(const double* M, int n, int m, const double* a, const double* b,
                      double reg, double tol, int max_iter, int verbose,
                      const oracle_opts* opts, oracle_result* res) {
    try {
        constexpr double theta = 0.5, kappa = 0.5, cg_tol = 1e-8;
        constexpr int nlinesearch = 20;
        const double tau = opts ? opts->tau : 0.0;
        const double shift = opts ? opts->shift : 1e-3;
        Problem p = make_problem(M, n, m, a, b, reg, tau);
        Vec gamma, newgamma(n + m), grad(n + m), direc, rhs(n + m);
        init_gamma(p, opts, gamma);
        History h(res);
        Timer timer;
        timer.tic();
        Hessian H;
        double f = dual_obj_grad_hess(p, gamma.data(), grad.data(), H);
        double gnorm = norm(grad);
        h.push(f, gnorm / reg, timer.toc(), 0.0, primal_val(p, gamma.data()));
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if (gnorm < tol) break;
            for (int q = 0; q < n + m; q++) rhs[q] = -grad[q];
            hess_cg(H, rhs, shift, tau, cg_tol, direc);
            double step = 1.0;
            const double thresh = theta * dot(grad, direc);
            for (int k = 0; k < nlinesearch; k++) {
                for (int q = 0; q < n + m; q++) newgamma[q] = gamma[q] + step * direc[q];
                const double newf = dual_obj(p, newgamma.data());
                if (newf <= f + step * thresh) break;
                step *= kappa;
            }
            gamma.swap(newgamma);
            f = dual_obj_grad_hess(p, gamma.data(), grad.data(), H);
            gnorm = norm(grad);
            const double d = timer.toc();
            h.push(f, gnorm / reg, h.last_time() + d, 0.0, primal_val(p, gamma.data()));
        }
        res->niter = i;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) get_plan(p, gamma.data(), res->plan);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// qrot_lbfgs_dual_internal: qrot_lbfgs_dual.cpp:81-126 (QROTDual 18-79).
int oracle_qrot_lbfgs_dual(const double* M, int n, int m, const double* a, const double* b,
                           double reg, double tol, int max_iter, int verbose,
                           const oracle_opts* opts, oracle_result* res) {
    try {
        const double tau = opts ? opts->tau : 0.0;
        Problem p = make_problem(M, n, m, a, b, reg, tau);
        LbfgsParam param;
        param.epsilon = tol;
        param.epsilon_rel = tol;
        param.max_iterations = max_iter;
        Vec gamma;
        init_gamma(p, opts, gamma);
        History h(res);
        Timer timer;
        double last_obj = std::numeric_limits<double>::infinity();
        int it = 0;
        FunGrad fg = [&](const Vec& x, Vec& g) {
            last_obj = dual_obj_grad(p, x.data(), g.data());
            return last_obj;
        };
        auto iterate = [&](const Vec& x, double gnorm) {
            const double d = timer.toc();
            const double prim = primal_val(p, x.data());
            h.push(last_obj, gnorm / reg, h.last_time() + d, 0.0, prim);
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", it, last_obj, gnorm);
            it++;
            timer.tic();
        };
        timer.tic();
        double fx;
        const int niter = lbfgs_minimize(fg, iterate, param, gamma, fx);
        res->niter = niter;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) get_plan(p, gamma.data(), res->plan);
        return 0;
    } catch (const std::invalid_argument& e) {
        set_err(res, e.what());
        return 2;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

// qrot_assn_internal: qrot_assn.cpp:16-170.
int oracle_qrot_assn(const double* M, int n, int m, const double* a, const double* b, double reg,
                     double tol, int max_iter, int verbose, const oracle_opts* opts,
                     oracle_result* res) {
    try {
        const double tau = opts ? opts->tau : 0.0;
        const int method = opts ? opts->method : 0;
        constexpr double nu = 0.99, eta1 = 0.25, eta2 = 0.75, gamma1 = 2.0, gamma2 = 4.0,
                         lam_min = 0.01, beta = 0.5, cg_tol = 1e-8;
        double xi = 0.0, lam = 1.0;
        Problem p = make_problem(M, n, m, a, b, reg, tau);
        const int N = n + m;
        Vec gamma, u(N), gu(N), v(N), gv(N), direc, g(N);
        init_gamma(p, opts, gamma);
        History h(res);
        Timer timer;
        timer.tic();
        Hessian H;
        double f = dual_obj_grad_hess(p, gamma.data(), g.data(), H);
        double gnorm = norm(g);
        double d = timer.toc();
        h.push(f, gnorm / reg, d, 0.0, primal_val(p, gamma.data()));
        int i;
        for (i = 0; i < max_iter; i++) {
            if (verbose >= 1)
                std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
            timer.tic();
            if (gnorm < tol) break;
            if (i == 0) xi = gnorm;
            const double mu = lam * gnorm;
            Vec rhs(N);
            for (int q = 0; q < N; q++) rhs[q] = -g[q];
            if (method == 0 || tau > 0.0) {
                hess_cg(H, rhs, mu, tau, cg_tol, direc);
            } else if (!hess_direct(H, rhs, mu, direc)) {
                throw std::runtime_error("sparse factorization failed");
            }
            for (int q = 0; q < N; q++) u[q] = gamma[q] + direc[q];
            dual_obj_grad(p, u.data(), gu.data());
            const double gunorm = norm(gu);
            if (gunorm <= nu * xi) {
                gamma.swap(u);
                xi = gunorm;
            } else {
                const double numer = -dot(gu, direc);
                const double denom = sqnorm(direc);
                const double rho = numer / denom;
                for (int q = 0; q < N; q++) v[q] = gamma[q] + (-numer) / (gunorm * gunorm) * gu[q];
                dual_obj_grad(p, v.data(), gv.data());
                const double gvnorm = norm(gv);
                if (rho >= eta1 && gvnorm <= gnorm) {
                    gamma.swap(v);
                } else {
                    for (int q = 0; q < N; q++) gamma[q] -= beta * g[q];
                }
                if (rho >= eta2) {
                    lam = 0.5 * (lam_min + lam);
                } else if (rho >= eta1) {
                    lam *= gamma1;
                } else {
                    lam *= gamma2;
                }
            }
            f = dual_obj_grad_hess(p, gamma.data(), g.data(), H);
            gnorm = norm(g);
            d = timer.toc();
            h.push(f, gnorm / reg, h.last_time() + d, 0.0, primal_val(p, gamma.data()));
        }
        res->niter = i;
        res->hist_len = h.len;
        std::copy(gamma.begin(), gamma.end(), res->dual);
        if (res->plan) get_plan(p, gamma.data(), res->plan);
        return 0;
    } catch (const std::exception& e) {
        set_err(res, e.what());
        return 1;
    }
}

}  // extern "C"
