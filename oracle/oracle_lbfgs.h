// FP64 oracle: restatement of the L-BFGS driver, two-loop recursion and
// Nocedal-Wright line search of the vendored LBFGS++ (MIT), shared by the
// qrot_lbfgs_dual and sinkhorn_lbfgs_dual restatements. Test infrastructure
// only (see oracle.h).
// The L-BFGS control flow, line search and error messages below follow
// LBFGS++, which carries this notice:
//
//   Copyright (C) 2016-2026 Yixuan Qiu <yixuan.qiu@cos.name>
//   Copyright (C) 2016-2026 Dirk Toewe <DirkToewe@GoogleMail.com>
//   MIT License
//
//   Permission is hereby granted, free of charge, to any person obtaining a
//   copy of this software and associated documentation files (the
//   "Software"), to deal in the Software without restriction, including
//   without limitation the rights to use, copy, modify, merge, publish,
//   distribute, sublicense, and/or sell copies of the Software, and to
//   permit persons to whom the Software is furnished to do so, subject to
//   the following conditions:
//
//   The above copyright notice and this permission notice shall be included
//   in all copies or substantial portions of the Software.
//
//   THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS
//   OR IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF
//   MERCHANTABILITY, FITNESS FOR A PARTICULAR PURPOSE AND NONINFRINGEMENT.
//   IN NO EVENT SHALL THE AUTHORS OR COPYRIGHT HOLDERS BE LIABLE FOR ANY
//   CLAIM, DAMAGES OR OTHER LIABILITY, WHETHER IN AN ACTION OF CONTRACT,
//   TORT OR OTHERWISE, ARISING FROM, OUT OF OR IN CONNECTION WITH THE
//   SOFTWARE OR THE USE OR OTHER DEALINGS IN THE SOFTWARE.
#ifndef REGOT_ORACLE_LBFGS_H
#define REGOT_ORACLE_LBFGS_H

#include <functional>
#include <limits>
#include <stdexcept>

#include "oracle_util.h"

namespace oracle {
namespace lbfgs {

// ---------------- L-BFGS (LBFGS++ restated) ----------------

struct LineSearchError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// L-BFGS parameters: LBFGSParam() defaults (Param.h:168-182); the solvers
// override epsilon, epsilon_rel and max_iterations (qrot_lbfgs_dual.cpp:100-103,
// sinkhorn_lbfgs_dual.cpp:101-104).
struct LbfgsParam {
    int m = 6;
    double epsilon = 1e-5, epsilon_rel = 1e-5;
    int max_iterations = 0;
    int max_linesearch = 20;
    double ftol = 1e-4, wolfe = 0.9;
};

// Compact two-loop storage: BFGSMat.h:61-100 (reset/add_correction) and
// apply_Hv 276-302.
struct BfgsMat {
    int mm = 0, ncorr = 0, ptr = 0;
    double theta = 1.0;
    std::vector<Vec> s, y;
    Vec ys, alpha;
    void reset(int n, int m_) {
        mm = m_;
        theta = 1.0;
        s.assign(mm, Vec(n));
        y.assign(mm, Vec(n));
        ys.assign(mm, 0.0);
        alpha.assign(mm, 0.0);
        ncorr = 0;
        ptr = mm;
    }
    void add_correction(const Vec& sv, const Vec& yv) {
        const int loc = ptr % mm;
        s[loc] = sv;
        y[loc] = yv;
        const double yts = dot(s[loc], y[loc]);
        ys[loc] = yts;
        theta = sqnorm(y[loc]) / yts;
        if (ncorr < mm) ncorr++;
        ptr = loc + 1;
    }
    void apply_Hv(const Vec& v, double a, Vec& res) {
        const size_t n = v.size();
        res.resize(n);
        for (size_t k = 0; k < n; k++) res[k] = a * v[k];
        int j = ptr % mm;
        for (int i = 0; i < ncorr; i++) {
            j = (j + mm - 1) % mm;
            alpha[j] = dot(s[j], res) / ys[j];
            for (size_t k = 0; k < n; k++) res[k] -= alpha[j] * y[j][k];
        }
        for (size_t k = 0; k < n; k++) res[k] /= theta;
        for (int i = 0; i < ncorr; i++) {
            const double beta = dot(y[j], res) / ys[j];
            for (size_t k = 0; k < n; k++) res[k] += (alpha[j] - beta) * s[j][k];
            j = (j + 1) % mm;
        }
    }
};

using FunGrad = std::function<double(const Vec&, Vec&)>;

// quad_interp: LineSearchNocedalWright.h:30-60.
inline double quad_interp(double step_lo, double step_hi, double fx_lo, double fx_hi,
                          double dg_lo) {
    const double fdiff = fx_hi - fx_lo;
    const double sdiff = step_hi - step_lo;
    const double smid = (step_hi + step_lo) / 2.0;
    double cand = fdiff * step_lo - smid * sdiff * dg_lo;
    cand = cand / (fdiff - sdiff * dg_lo);
    const bool cand_nan = !std::isfinite(cand);
    const double end_dist = std::min(std::abs(cand - step_lo), std::abs(cand - step_hi));
    const bool near_end = end_dist < 0.01 * std::abs(sdiff);
    const bool bisect = cand_nan || (cand <= std::min(step_lo, step_hi)) ||
                        (cand >= std::max(step_lo, step_hi)) || near_end;
    return bisect ? smid : cand;
}

// LineSearchNocedalWright::LineSearch: LineSearchNocedalWright.h:85-280
// (bracketing, then zoom with quadratic interpolation).
inline void line_search_nw(const FunGrad& f, const LbfgsParam& param, const Vec& xp,
                           const Vec& drt, double& step, double& fx, Vec& grad, double& dg,
                           Vec& x) {
    const size_t n = xp.size();
    if (step <= 0.0) throw std::invalid_argument("'step' must be positive");
    const double expansion = 2.0;
    const double fx_init = fx;
    const double dg_init = dg;
    if (dg_init > 0.0)
        throw std::logic_error("the moving direction increases the objective function value");
    const double test_decr = param.ftol * dg_init, test_curv = -param.wolfe * dg_init;
    double step_hi = 0.0, fx_hi = 0.0;
    double step_lo = 0.0, fx_lo = fx_init, dg_lo = dg_init;
    Vec x_lo = xp, grad_lo = grad;
    int iter = 0;
    for (;;) {
        for (size_t k = 0; k < n; k++) x[k] = xp[k] + step * drt[k];
        fx = f(x, grad);
        dg = dot(grad, drt);
        if (fx - fx_init > step * test_decr || (0.0 < step_lo && fx >= fx_lo)) {
            step_hi = step;
            fx_hi = fx;
            break;
        }
        if (std::abs(dg) <= test_curv) return;
        step_hi = step_lo;
        fx_hi = fx_lo;
        step_lo = step;
        fx_lo = fx;
        dg_lo = dg;
        x_lo.swap(x);
        grad_lo.swap(grad);
        if (dg >= 0.0) break;
        iter++;
        if (iter >= param.max_linesearch) {
            x.swap(x_lo);
            grad.swap(grad_lo);
            return;
        }
        step *= expansion;
    }
    for (;;) {
        step = quad_interp(step_lo, step_hi, fx_lo, fx_hi, dg_lo);
        for (size_t k = 0; k < n; k++) x[k] = xp[k] + step * drt[k];
        fx = f(x, grad);
        dg = dot(grad, drt);
        if (fx - fx_init > step * test_decr || fx >= fx_lo) {
            if (step == step_hi)
                throw LineSearchError(
                    "the line search routine failed, possibly due to insufficient numeric precision");
            step_hi = step;
            fx_hi = fx;
        } else {
            if (std::abs(dg) <= test_curv) return;
            if (dg * (step_hi - step_lo) >= 0.0) {
                step_hi = step_lo;
                fx_hi = fx_lo;
            }
            if (step == step_lo)
                throw LineSearchError(
                    "the line search routine failed, possibly due to insufficient numeric precision");
            step_lo = step;
            fx_lo = fx;
            dg_lo = dg;
            x_lo.swap(x);
            grad_lo.swap(grad);
        }
        iter++;
        if (iter >= param.max_linesearch) {
            if (step_lo <= 0.0)
                throw LineSearchError(
                    "the line search routine failed, unable to sufficiently decrease the function value");
            step = step_lo;
            fx = fx_lo;
            dg = dg_lo;
            x.swap(x_lo);
            grad.swap(grad_lo);
            return;
        }
    }
}

// LBFGSSolver::minimize: LBFGS.h:79-175. `iterate` is called after the
// initial evaluation and after every line search (QROTDual::iterate,
// SinkhornDual::iterate).
inline int lbfgs_minimize(const FunGrad& f, const std::function<void(const Vec&, double)>& iterate,
                          const LbfgsParam& param, Vec& x, double& fx) {
    const size_t n = x.size();
    BfgsMat bfgs;
    bfgs.reset((int)n, param.m);
    Vec xp(n), grad(n), gradp(n), drt(n);
    fx = f(x, grad);
    double gnorm = norm(grad);
    iterate(x, gnorm);
    if (gnorm <= param.epsilon || gnorm <= param.epsilon_rel * norm(x)) return 1;
    for (size_t k = 0; k < n; k++) drt[k] = -grad[k];
    double step = 1.0 / norm(drt);
    const double eps = std::numeric_limits<double>::epsilon();
    Vec vs(n), vy(n);
    int k = 1;
    for (;;) {
        xp = x;
        gradp = grad;
        double dg = dot(grad, drt);
        line_search_nw(f, param, xp, drt, step, fx, grad, dg, x);
        gnorm = norm(grad);
        iterate(x, gnorm);
        if (gnorm <= param.epsilon || gnorm <= param.epsilon_rel * norm(x)) return k;
        if (param.max_iterations != 0 && k >= param.max_iterations) return k;
        for (size_t q = 0; q < n; q++) {
            vs[q] = x[q] - xp[q];
            vy[q] = grad[q] - gradp[q];
        }
        if (dot(vs, vy) > eps * sqnorm(vy)) bfgs.add_correction(vs, vy);
        bfgs.apply_Hv(grad, -1.0, drt);
        step = 1.0;
        k++;
    }
}

}  // namespace lbfgs
}  // namespace oracle

#endif
