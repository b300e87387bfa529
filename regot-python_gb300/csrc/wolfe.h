// More-Thuente line search with strong Wolfe conditions, as the reference's
// Problem::line_search_wolfe (src/sinkhorn_problem_ls.cpp:226-436, with the
// interpolation helpers of lines 68-222): c1 = 1e-4, c2 = 0.9, at most 20
// trials, steps in [1e-10, 2], the auxiliary function psi(s) = f(s) - f(0)
// - s c1 f'(0) throughout (line 329). Host code: each trial is one dense
// pass run by the caller.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>

namespace regot {
namespace wolfe {

// Minimiser of the quadratic through (a, fa, ga) and (b, fb).
inline double quad_fgf(double a, double b, double fa, double ga, double fb) {
    const double ba = b - a;
    return a + (0.5 * ba * ga / (fa - fb + ba * ga)) * ba;
}

// Minimiser of the quadratic with slopes ga at a and gb at b.
inline double quad_gg(double a, double b, double ga, double gb) {
    return a + (ga / (ga - gb)) * (b - a);
}

// Local minimiser of the cubic through (a, fa, ga) and (b, fb, gb), in the
// scaled coefficients z_k = c_k (b - a)^3; `ok` tells whether one exists.
inline double cubic(double a, double b, double fa, double fb, double ga, double gb, bool& ok) {
    const double sum = a + b, ba = b - a, ba2 = ba * ba;
    const double df = fb - fa, dg = gb - ga;
    const double z3 = (ga + gb) * ba - 2.0 * df;
    const double z2 = 0.5 * (dg * ba2 - 3.0 * sum * z3);
    const double z1 = df * ba2 - sum * z2 - (a * sum + b * b) * z3;
    const double eps = std::numeric_limits<double>::epsilon();
    if (std::abs(z3) < eps * std::abs(z2) || std::abs(z3) < eps * std::abs(z1)) {
        ok = z2 * ba > 0.0;  // a quadratic with positive curvature
        return ok ? -0.5 * z1 / z2 : b;
    }
    const double u = z2 / (3.0 * z3), v = z1 / z2, vu = v / u;
    ok = vu <= 1.0;
    if (!ok) return b;
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
    return z3 * ba > 0.0 ? std::max(r1, r2) : std::min(r1, r2);
}

// Next trial from the interval ends (l, u) and the current trial t.
inline double select(double al, double au, double at, double fl, double fu, double ft, double gl,
                     double gu, double gt) {
    if (al == au) return al;
    if (!std::isfinite(ft) || !std::isfinite(gt)) return (al + at) / 2.0;
    bool c_ok;
    const double ac = cubic(al, at, fl, ft, gl, gt, c_ok);
    const double aq = quad_fgf(al, at, fl, gl, ft);
    if (ft > fl) {
        if (!c_ok) return aq;
        return std::abs(ac - al) < std::abs(aq - al) ? ac : (aq + ac) / 2.0;
    }
    const double as = quad_gg(al, at, gl, gt);
    if (gt * gl < 0.0) return std::abs(ac - at) >= std::abs(as - at) ? ac : as;
    constexpr double dl = 1.1, du = 0.66;
    if (std::abs(gt) < std::abs(gl)) {
        const bool take_c = c_ok && (ac - at) * (at - al) > 0.0 &&
                            std::abs(ac - at) < std::abs(as - at);
        const double r = take_c ? ac : as;
        return at > al ? std::min(at + du * (au - at), r) : std::max(at + du * (au - at), r);
    }
    if (!std::isfinite(au) || !std::isfinite(fu) || !std::isfinite(gu)) return at + dl * (at - al);
    bool e_ok;
    const double ae = cubic(at, au, ft, fu, gt, gu, e_ok);
    return at > al ? std::min(at + du * (au - at), ae) : std::max(at + du * (au - at), ae);
}

struct Outcome {
    double step;
    bool recompute;   // the returned step is not the last evaluated one
    double last_eval; // the last evaluated step (where the caller's T is)
};

// eval(step, &f, &dg): objective and directional derivative at x0 + step d.
template <typename Eval>
Outcome search(double init_step, double f0, double dg0, Eval&& eval) {
    constexpr double c1 = 1e-4, c2 = 0.9, smin = 1e-10, smax = 2.0;
    constexpr int max_trials = 20;
    constexpr double grow = 1.1, dmin = 7.0 / 12, shrink = 0.66;
    constexpr double Inf = std::numeric_limits<double>::infinity();
    Outcome out{0.0, false, 0.0};
    init_step = std::min(std::max(init_step, smin), smax);
    if (dg0 > 0.0) return Outcome{init_step, true, 0.0};  // not a descent direction
    const double decr = c1 * dg0, curv = -c2 * dg0;
    // interval ends: lo (best psi so far) and hi, with psi and psi' values
    double lo = 0.0, hi = Inf, f_lo = 0.0, f_hi = Inf, g_lo = (1.0 - c1) * dg0, g_hi = Inf;
    double psi_lo = 0.0;
    bool bracketed = false, min_guard = true;
    double width = Inf;
    int slow = 0;
    double step = init_step, fx = f0;
    for (int it = 0; it < max_trials; ++it) {
        double dg;
        eval(step, &fx, &dg);
        out.last_eval = step;
        const double psi = fx - f0 - step * decr, dpsi = dg - decr;
        if (psi <= 0.0 && std::abs(dg) <= curv) return Outcome{step, false, step};
        if (step <= smin && (psi > 0.0 || dpsi >= 0.0)) return Outcome{step, false, step};
        if (step >= smax && psi <= 0.0 && dpsi < 0.0) return Outcome{step, false, step};
        if (min_guard && psi <= 0.0 && dpsi < 0.0) min_guard = false;
        const bool extrapolate = psi <= psi_lo && dpsi * (lo - step) > 0.0;
        double next;
        if (extrapolate) {
            next = std::min(smax, step + grow * (step - lo));
        } else {
            next = select(lo, hi, step, f_lo, f_hi, psi, g_lo, g_hi, dpsi);
            next = std::min(std::max(next, smin), smax);
            if (min_guard) next = std::min(std::max(next, smin), std::max(smin, dmin * step));
        }
        if (psi > psi_lo) {
            hi = step;
            f_hi = psi;
            g_hi = dpsi;
        } else {
            if (!extrapolate) {
                hi = lo;
                f_hi = f_lo;
                g_hi = g_lo;
            }
            lo = step;
            f_lo = psi;
            g_lo = dpsi;
            psi_lo = psi;
        }
        if (!bracketed && !extrapolate)
            bracketed = std::min(lo, hi) >= smin && std::max(lo, hi) <= smax;
        if (bracketed) {
            const double prev = width;
            width = std::abs(hi - lo);
            if (prev < Inf && width > shrink * prev) ++slow;
            else slow = 0;
            if (slow >= 2) {
                next = (lo + hi) / 2.0;
                slow = 0;
            }
        }
        step = next;
    }
    // Trials used up: the psi of the last value at the next step decides
    // between that step and the best one (sinkhorn_problem_ls.cpp:417-435).
    if (fx - f0 - step * decr <= psi_lo) {
        out.step = step;
        out.recompute = false;
        return out;
    }
    out.recompute = true;
    out.step = lo <= 0.0 ? init_step : lo;
    return out;
}

}  // namespace wolfe
}  // namespace regot
