// sinkhorn_lbfgs_dual (src/sinkhorn_lbfgs_dual.cpp:81-126) and
// sinkhorn_apdagd (src/sinkhorn_apdagd.cpp:14-183) on the dense passes.
//
// Both are first-order methods on the EROT dual f(gamma) = reg sum T -
// a'alpha - b~'beta~ (sinkhorn_problem_obj.cpp:324-393). The drivers run on
// the host in FP64, like the reference's; every objective/gradient is one
// dense pass (row and column sums of T, OP_E_ROWCOL), read back as n + m
// sums. In mixed precision, differences of objective values that the
// algorithms compare are formed without cancellation:
//   - L-BFGS line-search trials (OP_E_GRADLS): f(xp + s d) - f(xp) =
//     s g'd + reg sum T(xp) phi(s w), phi(x) = e^x - 1 - x >= 0, evaluated
//     at the trial point together with its gradient;
//   - the APDAGD line-search test phi_new >= phit + g'diff - L/2 |diff|^2,
//     which is reg sum T(t) phi(w) <= L/2 |diff|^2 (OP_E_LS at the point t).
// FP64 storage evaluates the objectives directly, as the reference does.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "lbfgs.h"
#include "solvers.h"

namespace regot {

namespace {

using Clock = std::chrono::steady_clock;
using Vec = std::vector<double>;

double ms_since(Clock::time_point t) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t).count();
}

// Objective and gradient of the EROT dual from one row/column-sums pass.
class ErotDual {
public:
    ErotDual(regot_ctx* ctx, regot_dproblem* P, ErotOps& ops)
        : ctx_(ctx), P_(P), ops_(ops), st_(ops.stream()), n_(P->n), m_(P->m),
          g_(n_ + m_, st_), d_(n_ + m_, st_), sums_(n_ + m_, st_), tot_(2, st_), mx_(1, st_),
          hsums_(n_ + m_ + 2) {
        g_.zero();  // beta_m slots stay 0
        d_.zero();
    }

    double* alpha() { return g_.get(); }
    double* beta() { return g_.get() + n_; }
    double* dir_alpha() { return d_.get(); }
    double* dir_beta() { return d_.get() + n_; }
    long long passes() const { return passes_; }

    // gamma = (alpha, beta~) to the device (beta_m = 0 is kept).
    void upload(const Vec& x) { h2d(g_.get(), x.data(), x.size() * sizeof(double), st_); }
    void upload_dir(const Vec& x) { h2d(d_.get(), x.data(), x.size() * sizeof(double), st_); }

    // f and gradient at the uploaded point (sinkhorn_problem_obj.cpp:363-393).
    double value_grad(const Vec& x, Vec& g) {
        ops_.row_col_sums(alpha(), beta(), sums_.get(), sums_.get() + n_, mx_.get());
        ++passes_;
        read(n_ + m_);
        return from_sums(x, g);
    }

    // Trial point of the L-BFGS line search, uploaded, reached by `step`
    // along the uploaded direction: gradient there and reg * the
    // second-order part of the change (OP_E_GRADLS).
    double trial_grad(const Vec& x, double step, Vec& g, double* rem) {
        ops_.grad_ls(alpha(), beta(), dir_alpha(), dir_beta(), step, sums_.get(),
                     sums_.get() + n_, tot_.get(), mx_.get());
        ++passes_;
        read(n_ + m_ + 1);
        *rem = ops_.reg() * hsums_[n_ + m_];
        return from_sums(x, g);
    }

    // reg * sum T phi(w) at the uploaded point along the uploaded direction
    // with step 1 (OP_E_LS).
    double ls_remainder() {
        PassParams p = ops_.base_params();
        p.ra = alpha();
        p.cb = beta();
        p.rd = dir_alpha();
        p.cd = dir_beta();
        p.steps[0] = 1.0;
        p.nsteps = 1;
        ops_.maxabs(alpha(), n_, beta(), m_, mx_.get());
        p.grid = mx_.get();
        ops_.pass(OP_E_LS, p);
        ops_.merge_totals(OP_E_LS, 1, tot_.get());
        ++passes_;
        double t = 0.0;
        read_small(ctx_, &t, tot_.get(), sizeof(double), st_);
        return ops_.reg() * t;
    }

    // Averaged-plan pass at the uploaded point; returns the primal objective
    // <M, X> - reg sum X (1 - log X) and the marginal error of X
    // (sinkhorn_apdagd.cpp:150-159).
    void avg_plan(void* X, double tau, bool init, double* primal, double* mar_err) {
        ops_.avg_plan(alpha(), beta(), X, tau, init, sums_.get(), sums_.get() + n_, tot_.get(),
                      mx_.get());
        ++passes_;
        read(n_ + m_ + 2);
        double r2 = 0.0;
        for (int i = 0; i < n_; ++i) {
            const double e = hsums_[i] - P_->ha[i];
            r2 += e * e;
        }
        for (int j = 0; j < m_; ++j) {
            const double e = hsums_[n_ + j] - P_->hb[j];
            r2 += e * e;
        }
        *mar_err = std::sqrt(r2);
        *primal = hsums_[n_ + m_] - ops_.reg() * hsums_[n_ + m_ + 1];
    }

private:
    // sums (and, past them, the totals) back to the host behind one
    // synchronisation
    void read(int count) {
        double* h = static_cast<double*>(ctx_stage(ctx_, (size_t)count * sizeof(double)));
        d2h(h, sums_.get(), (size_t)std::min(count, n_ + m_) * sizeof(double), st_);
        if (count > n_ + m_)
            d2h(h + n_ + m_, tot_.get(), (size_t)(count - n_ - m_) * sizeof(double), st_);
        sync(st_);
        std::memcpy(hsums_.data(), h, (size_t)count * sizeof(double));
    }

    // g = [T1 - a ; (T'1 - b)_{0..m-2}], f = reg sum T - a'alpha - b~'beta~.
    double from_sums(const Vec& x, Vec& g) {
        double tsum = 0.0;
        for (int i = 0; i < n_; ++i) {
            tsum += hsums_[i];
            g[i] = hsums_[i] - P_->ha[i];
        }
        for (int j = 0; j < m_ - 1; ++j) g[n_ + j] = hsums_[n_ + j] - P_->hb[j];
        double da = 0.0, db = 0.0;
        for (int i = 0; i < n_; ++i) da += x[i] * P_->ha[i];
        for (int j = 0; j < m_ - 1; ++j) db += x[n_ + j] * P_->hb[j];
        return ops_.reg() * tsum - da - db;
    }

    regot_ctx* ctx_;
    regot_dproblem* P_;
    ErotOps& ops_;
    cudaStream_t st_;
    int n_, m_;
    DBuf<double> g_, d_, sums_, tot_, mx_;
    Vec hsums_;
    long long passes_ = 0;
};

// Initial value of sinkhorn_lbfgs_dual.cpp:108-117 and
// sinkhorn_apdagd.cpp:45-54: x0, or (0 + beta_m, beta~ - beta_m) with
// beta = optimal_beta(alpha = 0).
void initial_gamma(ErotOps& ops, const regot_opts& o, int n, int m, Vec& gamma) {
    cudaStream_t st = ops.stream();
    gamma.assign(n + m - 1, 0.0);
    if (o.x0 && o.x0_len == n + m - 1) {
        std::copy(o.x0, o.x0 + n + m - 1, gamma.begin());
        return;
    }
    DBuf<double> beta(m, st), zero(n, st), mx(1, st);
    zero.zero();
    ops.optimal_beta(zero.get(), beta.get(), mx.get());
    Vec hb(m);
    read_small(ops.problem()->ctx, hb.data(), beta.get(), m * sizeof(double), st);
    for (int i = 0; i < n; ++i) gamma[i] = hb[m - 1];
    for (int j = 0; j < m - 1; ++j) gamma[n + j] = hb[j] - hb[m - 1];
}

// Result with host histories: dual, histories, and the plan produced by
// plan_fn(dst) into an n x m FP64 destination (device or host view).
template <typename F>
void finish_host(ErotOps& ops, const Vec& gamma, const Vec& hobj, const Vec& hmar,
                 const Vec& htime, int niter, long long passes, const regot_opts& o,
                 regot_result* res, F&& plan_fn) {
    const int n = ops.n(), m = ops.m();
    cudaStream_t st = ops.stream();
    const int L = (int)hobj.size();
    res->niter = niter;
    res->hist_len = L;
    res->passes = passes;
    std::memcpy(res->dual, gamma.data(), (size_t)(n + m - 1) * sizeof(double));
    if (res->obj_vals) std::memcpy(res->obj_vals, hobj.data(), L * sizeof(double));
    if (res->mar_errs) std::memcpy(res->mar_errs, hmar.data(), L * sizeof(double));
    if (res->run_times) std::memcpy(res->run_times, htime.data(), L * sizeof(double));
    if (o.plan && res->plan) emit_plan(res->plan, o.plan_mem, (size_t)n * m, st, plan_fn);
    ops.check_err();  // synchronises
}

}  // namespace

// sinkhorn_lbfgs_dual_internal: sinkhorn_lbfgs_dual.cpp:81-126 (SinkhornDual
// 18-79). LBFGSParam() defaults except epsilon = tol, epsilon_rel = 0,
// max_iterations = max_iter (101-104).
void sinkhorn_lbfgs_dual_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol,
                             int max_iter, const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m - 1;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    ErotOps ops(P, reg, st);
    ErotDual E(ctx, P, ops);
    lbfgs::Param param;
    param.epsilon = tol;
    param.epsilon_rel = 0.0;
    param.max_iterations = max_iter;
    Vec gamma;
    initial_gamma(ops, o, n, m, gamma);

    Vec hobj, hmar, htime;
    double last_obj = std::numeric_limits<double>::infinity();
    int it = 0;
    lbfgs::FunGrad fg = [&](const lbfgs::Vec& x, lbfgs::Vec& g) {
        E.upload(x);
        last_obj = E.value_grad(x, g);
        return last_obj;
    };
    // In mixed precision f(x) - f(xp) is far below the FP32 rounding of f
    // near convergence: the trial returns f(xp) + s g'd + reg sum T phi, with
    // the remainder from the trial pass itself. The history records f(x)
    // evaluated directly, as the reference's operator() does.
    lbfgs::TrialFn trial = [&](const lbfgs::Vec& xp, const lbfgs::Vec& drt, double step,
                               double fx_init, double dg_init, lbfgs::Vec& x, lbfgs::Vec& g) {
        for (int k = 0; k < N; ++k) x[k] = xp[k] + step * drt[k];
        if (!mixed) return fg(x, g);
        E.upload(x);
        E.upload_dir(drt);
        double rem = 0.0;
        last_obj = E.trial_grad(x, step, g, &rem);
        return fx_init + (step * dg_init + rem);
    };
    auto t_prev = Clock::now();
    auto iterate = [&](const lbfgs::Vec&, double gnorm) {
        const double d = ms_since(t_prev);
        hobj.push_back(last_obj);
        hmar.push_back(gnorm);
        htime.push_back((htime.empty() ? 0.0 : htime.back()) + d);
        if (o.verbose >= 1)
            std::printf("iter = %d, objval = %g, ||grad|| = %g\n", it, last_obj, gnorm);
        it++;
        t_prev = Clock::now();
    };
    double fx;
    const int niter = lbfgs::minimize(fg, trial, iterate, param, gamma, fx);
    E.upload(gamma);
    DBuf<double> mx(1, st);
    finish_host(ops, gamma, hobj, hmar, htime, niter, E.passes(), o, res,
                [&](double* dst) { ops.plan(E.alpha(), E.beta(), dst, mx.get()); });
}

// sinkhorn_apdagd_internal: sinkhorn_apdagd.cpp:14-183. dual = -gamma;
// phi = -f. The averaged plan lives on the device in the pass's element type.
void sinkhorn_apdagd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                         const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m - 1;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    constexpr double L0 = 1.0;
    constexpr int max_inner = 20;
    ErotOps ops(P, reg, st);
    ErotDual E(ctx, P, ops);
    const size_t es = mixed ? sizeof(float) : sizeof(double);
    DBuf<char> X((size_t)n * m * es, st);

    Vec gamma, grad(N), dual(N), dual_new(N), dualp(N), dualp_new(N), dualt(N), diff(N), d(N);
    initial_gamma(ops, o, n, m, gamma);
    for (int q = 0; q < N; ++q) dual[q] = -gamma[q];
    dualp = dual;
    dualt = dual;
    // result.get_plan(gamma) before the timer (sinkhorn_apdagd.cpp:58)
    E.upload(gamma);
    double primal = 0.0, mar_err = 0.0;
    E.avg_plan(X.get(), 1.0, true, &primal, &mar_err);

    Vec hobj, hmar, htime;
    auto t0 = Clock::now();
    double f = E.value_grad(gamma, grad);
    hobj.push_back(f);
    hmar.push_back(lbfgs::norm(grad));
    htime.push_back(ms_since(t0));

    int i;
    double L = L0, pbeta = 0.0;
    for (i = 0; i < max_iter; i++) {
        t0 = Clock::now();
        L *= 0.5;
        double ptau = 0.0, phi_new = 0.0;
        for (int j = 0; j < max_inner; j++) {
            const double palpha = (1.0 + std::sqrt(4.0 * L * pbeta + 1.0)) / (2.0 * L);
            const double pbeta_new = pbeta + palpha;
            ptau = palpha / pbeta_new;
            for (int q = 0; q < N; ++q) dualt[q] = (1.0 - ptau) * dual[q] + ptau * dualp[q];
            for (int q = 0; q < N; ++q) gamma[q] = -dualt[q];
            E.upload(gamma);
            const double ft = E.value_grad(gamma, grad);
            const double phit = -ft;
            for (int q = 0; q < N; ++q) dualp_new[q] = dualp[q] + palpha * grad[q];
            for (int q = 0; q < N; ++q)
                dual_new[q] = (1.0 - ptau) * dual[q] + ptau * dualp_new[q];
            for (int q = 0; q < N; ++q) diff[q] = dual_new[q] - dualt[q];
            const double dd = lbfgs::dot(diff, diff);
            bool accept;
            if (mixed) {
                // gamma_new - gamma_t = -diff: f_new = f_t - g'diff + reg sum T phi
                for (int q = 0; q < N; ++q) d[q] = -diff[q];
                E.upload_dir(d);
                const double rem = E.ls_remainder();
                f = ft - lbfgs::dot(grad, diff) + rem;
                phi_new = -f;
                accept = rem <= 0.5 * L * dd;
                if (o.verbose >= 2)
                    std::printf("j = %d, palpha = %g, pbeta = %g, phit = %g, phi_new = %g\n", j,
                                palpha, pbeta_new, phit, phi_new);
            } else {
                Vec gn(N);
                for (int q = 0; q < N; ++q) gamma[q] = -dual_new[q];
                E.upload(gamma);
                f = E.value_grad(gamma, gn);
                phi_new = -f;
                const double rhs = phit + lbfgs::dot(grad, diff) - 0.5 * L * dd;
                accept = phi_new >= rhs;
                if (o.verbose >= 2)
                    std::printf("j = %d, palpha = %g, pbeta = %g, phit = %g, phi_new = %g, "
                                "rhs = %g\n", j, palpha, pbeta_new, phit, phi_new, rhs);
            }
            if (accept || j >= max_inner - 1) {
                pbeta = pbeta_new;
                dualp.swap(dualp_new);
                dual.swap(dual_new);
                break;
            }
            L *= 2.0;
        }
        // plan = (1 - ptau) plan + ptau plan(-dualt), statistics of it
        for (int q = 0; q < N; ++q) gamma[q] = -dualt[q];
        E.upload(gamma);
        E.avg_plan(X.get(), ptau, false, &primal, &mar_err);
        hobj.push_back(f);
        hmar.push_back(mar_err);
        htime.push_back(htime.back() + ms_since(t0));
        if (o.verbose >= 1)
            std::printf("iter = %d, primal_obj = %g, phi_new = %g, mar_err = %g\n", i, primal,
                        phi_new, mar_err);
        if (primal - phi_new <= tol && mar_err <= tol) break;
    }
    const long long count = (long long)n * m;
    finish_host(ops, gamma, hobj, hmar, htime, i, E.passes(), o, res, [&](double* dst) {
        if (mixed) {
            k_widen<float><<<1024, 256, 0, st>>>(reinterpret_cast<const float*>(X.get()), count, dst);
            count_launch();
            REGOT_CHECK_LAUNCH();
        } else {
            REGOT_CUDA(cudaMemcpyAsync(dst, X.get(), (size_t)count * sizeof(double),
                                       cudaMemcpyDefault, st));
        }
    });
}

}  // namespace regot
