// L-BFGS with the Nocedal-Wright strong-Wolfe line search, restating the
// vendored LBFGS++ (MIT) that the reference's qrot_lbfgs_dual and
// sinkhorn_lbfgs_dual use:
// LBFGSSolver::minimize (src/LBFGSpp/LBFGS.h:79-175), the two-loop recursion
// BFGSMat::apply_Hv (src/LBFGSpp/LBFGSpp/BFGSMat.h:61-100, 276-302),
// LineSearchNocedalWright::LineSearch (LineSearchNocedalWright.h:30-280) and
// the defaults of LBFGSParam (Param.h:168-182). The driver runs on the host in
// FP64; every function evaluation is one dense GPU pass (the caller's
// callback). Vectors have n + m entries (QROT) or n + m - 1 (EROT).
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
#pragma once

#include <algorithm>
#include <cmath>
#include <functional>
#include <limits>
#include <stdexcept>
#include <vector>

#include "internal.h"

namespace regot {
namespace lbfgs {

using Vec = std::vector<double>;

inline double dot(const Vec& x, const Vec& y) {
    double s = 0.0;
    for (size_t i = 0; i < x.size(); ++i) s += x[i] * y[i];
    return s;
}
inline double norm(const Vec& x) { return std::sqrt(dot(x, x)); }

struct Param {
    int m = 6;
    double epsilon = 1e-5, epsilon_rel = 1e-5;
    int max_iterations = 0;
    int max_linesearch = 20;
    double ftol = 1e-4, wolfe = 0.9;
};

class BfgsMat {
public:
    void reset(size_t n, int m) {
        mm_ = m;
        theta_ = 1.0;
        s_.assign(m, Vec(n));
        y_.assign(m, Vec(n));
        ys_.assign(m, 0.0);
        alpha_.assign(m, 0.0);
        ncorr_ = 0;
        ptr_ = m;
    }
    void add_correction(const Vec& s, const Vec& y) {
        const int loc = ptr_ % mm_;
        s_[loc] = s;
        y_[loc] = y;
        const double ys = dot(s_[loc], y_[loc]);
        ys_[loc] = ys;
        theta_ = dot(y_[loc], y_[loc]) / ys;
        if (ncorr_ < mm_) ncorr_++;
        ptr_ = loc + 1;
    }
    // res = a * H v (two-loop recursion)
    void apply_Hv(const Vec& v, double a, Vec& res) {
        const size_t n = v.size();
        res.resize(n);
        for (size_t k = 0; k < n; ++k) res[k] = a * v[k];
        int j = ptr_ % mm_;
        for (int i = 0; i < ncorr_; ++i) {
            j = (j + mm_ - 1) % mm_;
            alpha_[j] = dot(s_[j], res) / ys_[j];
            for (size_t k = 0; k < n; ++k) res[k] -= alpha_[j] * y_[j][k];
        }
        for (size_t k = 0; k < n; ++k) res[k] /= theta_;
        for (int i = 0; i < ncorr_; ++i) {
            const double beta = dot(y_[j], res) / ys_[j];
            for (size_t k = 0; k < n; ++k) res[k] += (alpha_[j] - beta) * s_[j][k];
            j = (j + 1) % mm_;
        }
    }

private:
    int mm_ = 6, ncorr_ = 0, ptr_ = 6;
    double theta_ = 1.0;
    std::vector<Vec> s_, y_;
    Vec ys_, alpha_;
};

using FunGrad = std::function<double(const Vec&, Vec&)>;
// Line-search trial: set x = xp + step * drt and grad = grad f(x), return
// f(x). fx_init and dg_init are f(xp) and grad f(xp)' drt, so an
// implementation may evaluate f(x) as fx_init + (f(x) - f(xp)) with the
// difference computed directly.
using TrialFn = std::function<double(const Vec& xp, const Vec& drt, double step, double fx_init,
                                     double dg_init, Vec& x, Vec& grad)>;

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

// Errors of the line search map to REGOT_ERR_LINESEARCH / INVALID_ARG, which
// Python raises as RuntimeError / ValueError like pybind11 does for the
// reference's std::runtime_error / std::invalid_argument.
inline void line_search(const TrialFn& f, const Param& param, const Vec& xp, const Vec& drt,
                        double& step, double& fx, Vec& grad, double& dg, Vec& x) {
    if (step <= 0.0) throw Error(REGOT_ERR_INVALID_ARG, "'step' must be positive");
    const double expansion = 2.0;
    const double fx_init = fx;
    const double dg_init = dg;
    if (dg_init > 0.0)
        throw Error(REGOT_ERR_LINESEARCH,
                    "the moving direction increases the objective function value");
    const double test_decr = param.ftol * dg_init, test_curv = -param.wolfe * dg_init;
    double step_hi = 0.0, fx_hi = 0.0;
    double step_lo = 0.0, fx_lo = fx_init, dg_lo = dg_init;
    Vec x_lo = xp, grad_lo = grad;
    int iter = 0;
    for (;;) {
        fx = f(xp, drt, step, fx_init, dg_init, x, grad);
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
        fx = f(xp, drt, step, fx_init, dg_init, x, grad);
        dg = dot(grad, drt);
        if (fx - fx_init > step * test_decr || fx >= fx_lo) {
            if (step == step_hi)
                throw Error(REGOT_ERR_LINESEARCH,
                            "the line search routine failed, possibly due to insufficient "
                            "numeric precision");
            step_hi = step;
            fx_hi = fx;
        } else {
            if (std::abs(dg) <= test_curv) return;
            if (dg * (step_hi - step_lo) >= 0.0) {
                step_hi = step_lo;
                fx_hi = fx_lo;
            }
            if (step == step_lo)
                throw Error(REGOT_ERR_LINESEARCH,
                            "the line search routine failed, possibly due to insufficient "
                            "numeric precision");
            step_lo = step;
            fx_lo = fx;
            dg_lo = dg;
            x_lo.swap(x);
            grad_lo.swap(grad);
        }
        iter++;
        if (iter >= param.max_linesearch) {
            if (step_lo <= 0.0)
                throw Error(REGOT_ERR_LINESEARCH,
                            "the line search routine failed, unable to sufficiently decrease "
                            "the function value");
            step = step_lo;
            fx = fx_lo;
            dg = dg_lo;
            x.swap(x_lo);
            grad.swap(grad_lo);
            return;
        }
    }
}

// Returns the number of iterations (LBFGSSolver::minimize).
inline int minimize(const FunGrad& f, const TrialFn& trial,
                    const std::function<void(const Vec&, double)>& iterate, const Param& param,
                    Vec& x, double& fx) {
    const size_t n = x.size();
    BfgsMat bfgs;
    bfgs.reset(n, param.m);
    Vec xp(n), grad(n), gradp(n), drt(n);
    fx = f(x, grad);
    double gnorm = norm(grad);
    iterate(x, gnorm);
    if (gnorm <= param.epsilon || gnorm <= param.epsilon_rel * norm(x)) return 1;
    for (size_t k = 0; k < n; ++k) drt[k] = -grad[k];
    double step = 1.0 / norm(drt);
    const double eps = std::numeric_limits<double>::epsilon();
    Vec vs(n), vy(n);
    int k = 1;
    for (;;) {
        xp = x;
        gradp = grad;
        double dg = dot(grad, drt);
        line_search(trial, param, xp, drt, step, fx, grad, dg, x);
        gnorm = norm(grad);
        iterate(x, gnorm);
        if (gnorm <= param.epsilon || gnorm <= param.epsilon_rel * norm(x)) return k;
        if (param.max_iterations != 0 && k >= param.max_iterations) return k;
        for (size_t q = 0; q < n; ++q) {
            vs[q] = x[q] - xp[q];
            vy[q] = grad[q] - gradp[q];
        }
        if (dot(vs, vy) > eps * dot(vy, vy)) bfgs.add_correction(vs, vy);
        bfgs.apply_Hv(grad, -1.0, drt);
        step = 1.0;
        k++;
    }
}

}  // namespace lbfgs
}  // namespace regot
