// Shared helpers of the FP64 oracle (test infrastructure only; see oracle.h).
#ifndef REGOT_ORACLE_UTIL_H
#define REGOT_ORACLE_UTIL_H

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "oracle.h"

namespace oracle {

using Vec = std::vector<double>;

inline double dot(const double* x, const double* y, size_t n) {
    double s = 0.0;
    for (size_t i = 0; i < n; i++) s += x[i] * y[i];
    return s;
}
inline double dot(const Vec& x, const Vec& y) { return dot(x.data(), y.data(), x.size()); }
inline double sqnorm(const Vec& x) { return dot(x, x); }
inline double norm(const Vec& x) { return std::sqrt(sqnorm(x)); }
inline double sum(const double* x, size_t n) {
    double s = 0.0;
    for (size_t i = 0; i < n; i++) s += x[i];
    return s;
}

// Millisecond wall clock with the tic/toc semantics of timer.h:9-54
// (toc returns the time since the last tic or toc and restarts the clock).
class Timer {
    using Clock = std::chrono::steady_clock;
    Clock::time_point m_start;
public:
    void tic() { m_start = Clock::now(); }
    double toc() {
        auto now = Clock::now();
        double d = std::chrono::duration<double, std::milli>(now - m_start).count();
        m_start = now;
        return d;
    }
};

// History recorder writing into caller buffers (capacity-checked).
struct History {
    oracle_result* r;
    int len = 0;
    explicit History(oracle_result* res) : r(res) {}
    void push(double obj, double mar, double time, double dens = 0.0, double prim = 0.0) {
        if (len >= r->hist_cap) throw std::runtime_error("history capacity exceeded");
        if (r->obj_vals) r->obj_vals[len] = obj;
        if (r->mar_errs) r->mar_errs[len] = mar;
        if (r->run_times) r->run_times[len] = time;
        if (r->densities) r->densities[len] = dens;
        if (r->prim_vals) r->prim_vals[len] = prim;
        len++;
    }
    double last_time() const { return len > 0 ? r->run_times[len - 1] : 0.0; }
};

// Conjugate gradient with identity preconditioner, restating the textbook
// Hestenes-Stiefel iteration that Eigen::ConjugateGradient runs
// (sinkhorn_cg.cpp:31-38, qrot_cg.cpp:31-38): stop when ||r||^2 <
// max(tol^2 ||b||^2, DBL_MIN); at most 2*dim iterations; x0 = 0 unless a
// guess of the right length is given.
inline int cg_solve(const std::function<void(const Vec&, Vec&)>& apply,
                    const Vec& rhs, Vec& x, double tol, const Vec* guess) {
    const size_t n = rhs.size();
    const int max_iter = 2 * static_cast<int>(n);
    x.assign(n, 0.0);
    if (guess && guess->size() == n) x = *guess;
    Vec r(n), p(n), tmp(n);
    apply(x, tmp);
    for (size_t i = 0; i < n; i++) r[i] = rhs[i] - tmp[i];
    const double rhs_norm2 = sqnorm(rhs);
    if (rhs_norm2 == 0.0) { std::fill(x.begin(), x.end(), 0.0); return 0; }
    const double threshold = std::max(tol * tol * rhs_norm2, std::numeric_limits<double>::min());
    double res_norm2 = sqnorm(r);
    if (res_norm2 < threshold) return 0;
    p = r;
    double abs_new = dot(r, p);
    int i = 0;
    while (i < max_iter) {
        apply(p, tmp);
        const double alpha = abs_new / dot(p, tmp);
        for (size_t k = 0; k < n; k++) x[k] += alpha * p[k];
        for (size_t k = 0; k < n; k++) r[k] -= alpha * tmp[k];
        res_norm2 = sqnorm(r);
        if (res_norm2 < threshold) break;
        const double abs_old = abs_new;
        abs_new = dot(r, r);
        const double beta = abs_new / abs_old;
        for (size_t k = 0; k < n; k++) p[k] = r[k] + beta * p[k];
        i++;
    }
    return i;
}

// In-place dense Cholesky A = L L^T of a row-major SPD matrix (lower part
// used). Returns false if a pivot is not positive.
inline bool cholesky(std::vector<double>& A, int n) {
    for (int j = 0; j < n; j++) {
        double* Aj = &A[(size_t)j * n];
        double d = Aj[j];
        for (int k = 0; k < j; k++) d -= Aj[k] * Aj[k];
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        Aj[j] = d;
        for (int i = j + 1; i < n; i++) {
            double* Ai = &A[(size_t)i * n];
            double s = Ai[j];
            for (int k = 0; k < j; k++) s -= Ai[k] * Aj[k];
            Ai[j] = s / d;
        }
    }
    return true;
}

// Solve L L^T x = b given the factor from cholesky().
inline void cholesky_solve(const std::vector<double>& L, int n, Vec& x) {
    for (int i = 0; i < n; i++) {
        const double* Li = &L[(size_t)i * n];
        double s = x[i];
        for (int k = 0; k < i; k++) s -= Li[k] * x[k];
        x[i] = s / Li[i];
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = x[i];
        for (int k = i + 1; k < n; k++) s -= L[(size_t)k * n + i] * x[k];
        x[i] = s / L[(size_t)i * n + i];
    }
}

inline void set_err(oracle_result* r, const char* msg) {
    if (!r) return;
    std::snprintf(r->err, sizeof(r->err), "%s", msg);
}

}  // namespace oracle

#endif  // REGOT_ORACLE_UTIL_H
