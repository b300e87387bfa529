// qrot_pdip: the primal-dual interior-point method for QROT with the CG
// inner solver (reference src/pdip_cg.cpp:206-413) or the fixed-point /
// Cholesky inner solver (src/pdip_fp.cpp:278-667), and the transport
// operators of src/pdip_transport_ops.hpp.
//
// Layout. The primal x, the slack s, the cost c, the scaling
// scale = x / (barrier x + s), the dual residual and the step directions are
// n x m row-major FP64 arrays on the device (index i*m + j), as in the
// reference. Every primal-sized operation is a device kernel: the fused
// element updates, row and column sums (the operator A: column sums, then
// row sums of rows < n-1), A' lambda formed on the fly, the step-length
// minima and the inner products. The equality-sized (m + n - 1) linear
// algebra runs on the host in FP64, as in the reference: the block matrix
// B = [diag(B11) D; D' diag(B22)] (D = scale on the supply rows < n-1) is
// factored exactly by eliminating its diagonal demand block and
// Cholesky-factoring the Schur complement diag(B22) - D' diag(1/B11) D;
// the reference factors the same matrix with Eigen's SimplicialLDLT
// (preconditioner of PDIP-CG), dense LLT or SimplicialLLT (PDIP-FP). The
// products with the full D inside the inner solves are device passes over
// scale.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#include "device_util.cuh"
#include "solvers.h"

namespace regot {

namespace {

constexpr double kSmall = 1e-50;
constexpr int kEw = 256;        // element kernels
constexpr int kRedBlocks = 304; // scalar reductions: fixed grid, host-side final sum

__device__ __forceinline__ double at_of(const double* lam, int i, int j, int n, int m) {
    return lam[j] + (i < n - 1 ? lam[m + i] : 0.0);
}

template <typename TM>
__global__ void k_pd_cost(const TM* M, long long ldm, int n, int m, double* c) {
    const long long nv = (long long)n * m;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / m), j = (int)(k - (long long)i * m);
        c[k] = (double)M[(long long)i * ldm + j];
    }
}

// out = base_coef * base + A' lam (+ c) over the n x m grid:
//   mode 0: out = A' lam
//   mode 1: out = barrier x + c + A' lam  (initial slack)
__global__ void k_pd_at(int n, int m, int mode, double barrier, const double* lam,
                        const double* x, const double* c, double* out) {
    const long long nv = (long long)n * m;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / m), j = (int)(k - (long long)i * m);
        const double at = at_of(lam, i, j, n, m);
        out[k] = mode == 0 ? at : barrier * x[k] + c[k] + at;
    }
}

// x += ax, s += as, then both clamped below at 1e-10 (clamp != 0), or plain
// shifts (clamp == 0).
__global__ void k_pd_shift(long long nv, double ax, double as, int clamp, double* x, double* s) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        double xv = x[k] + ax, sv = s[k] + as;
        if (clamp) {
            xv = fmax(xv, 1e-10);
            sv = fmax(sv, 1e-10);
        }
        x[k] = xv;
        s[k] = sv;
    }
}

// 2.1: scale, r_dual = barrier x + c + A' lam - s, and
// tmp = scale * (-s - r_dual) (the predictor right-hand side before A).
__global__ void k_pd_start(int n, int m, double barrier, const double* x, const double* s,
                           const double* c, const double* lam, double* scale, double* rd,
                           double* tmp) {
    const long long nv = (long long)n * m;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / m), j = (int)(k - (long long)i * m);
        const double xv = x[k], sv = s[k];
        const double sc = xv / (barrier * xv + sv + kSmall);
        const double r = barrier * xv + c[k] + at_of(lam, i, j, n, m) - sv;
        scale[k] = sc;
        rd[k] = r;
        tmp[k] = sc * (-sv - r);
    }
}

// 2.3: ds = (1 - barrier scale)(A' dlam + r_dual - barrier x),
//      dx = (-x s - x ds) / (s + SMALL).
__global__ void k_pd_pred(int n, int m, double barrier, const double* x, const double* s,
                          const double* scale, const double* rd, const double* dlam, double* dx,
                          double* ds) {
    const long long nv = (long long)n * m;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / m), j = (int)(k - (long long)i * m);
        const double xv = x[k], sv = s[k];
        const double d_s = (1.0 - barrier * scale[k]) *
                           (at_of(dlam, i, j, n, m) + rd[k] - barrier * xv);
        ds[k] = d_s;
        dx[k] = (-xv * sv - xv * d_s) / (sv + kSmall);
    }
}

// 2.4: r_c = x s + dx ds - sigma mu, tmp = scale * (-r_c / (x + SMALL) - r_dual).
__global__ void k_pd_corr(long long nv, double smu, const double* x, const double* s,
                          const double* dx, const double* ds, const double* scale,
                          const double* rd, double* rcc, double* tmp) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        const double xv = x[k];
        const double r = xv * s[k] + dx[k] * ds[k] - smu;
        rcc[k] = r;
        tmp[k] = scale[k] * (-r / (xv + kSmall) - rd[k]);
    }
}

// 2.4 final: ds = (1 - barrier scale)(A' dlam + r_dual - barrier r_c / (s + SMALL)),
//            dx = (-r_c - x ds) / (s + SMALL).
__global__ void k_pd_final(int n, int m, double barrier, const double* x, const double* s,
                           const double* scale, const double* rd, const double* rcc,
                           const double* dlam, double* dx, double* ds) {
    const long long nv = (long long)n * m;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / m), j = (int)(k - (long long)i * m);
        const double sv = s[k];
        const double d_s = (1.0 - barrier * scale[k]) *
                           (at_of(dlam, i, j, n, m) + rd[k] - barrier * rcc[k] / (sv + kSmall));
        ds[k] = d_s;
        dx[k] = (-rcc[k] - x[k] * d_s) / (sv + kSmall);
    }
}

// Step: x += a dx, s += a ds; then r_dual = barrier x + c + A' lam_rd - s
// and at = A' lam_new (for the dual-gap denominator).
__global__ void k_pd_update(int n, int m, double barrier, double a, const double* dx,
                            const double* ds, const double* c, const double* lam_rd,
                            const double* lam_new, double* x, double* s, double* rd,
                            double* at) {
    const long long nv = (long long)n * m;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / m), j = (int)(k - (long long)i * m);
        const double xv = x[k] + a * dx[k], sv = s[k] + a * ds[k];
        x[k] = xv;
        s[k] = sv;
        rd[k] = barrier * xv + c[k] + at_of(lam_rd, i, j, n, m) - sv;
        at[k] = at_of(lam_new, i, j, n, m);
    }
}

// Row sums (one warp per row) and column sums (one thread per column) of
// A (times w along the other index when given), deterministic order.
__global__ void k_pd_rowsum(int n, int m, const double* A, const double* wcol, double* out) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const double* r = A + (long long)i * m;
    double s = 0.0;
    for (int j = lane; j < m; j += 32) s += wcol ? r[j] * wcol[j] : r[j];
    s = warp_sum_d(s);
    if (lane == 0) out[i] = s;
}

__global__ void k_pd_colsum(int n, int m, const double* A, const double* wrow, double* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
        const double v = A[(long long)i * m + j];
        s += wrow ? v * wrow[i] : v;
    }
    out[j] = s;
}

// Scalar reductions over nv entries into per-block partials (summed on the
// host in block order): op 0 sum a b; 1 sum a; 2 min step (dx < 0 ?
// -x / (dx + SMALL) : 1); 3 max(-1.5 a); 4 sum (x + t dx)(s + t ds);
// 5 count of non-finite entries of a or b.
__global__ void __launch_bounds__(kEw) k_pd_reduce(int op, long long nv, const double* a,
                                                   const double* b, const double* c,
                                                   const double* d, double t, double* part) {
    double acc = (op == 2) ? 1.0 : (op == 3 ? -INFINITY : 0.0);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nv;
         k += (long long)gridDim.x * blockDim.x) {
        switch (op) {
            case 0: acc += a[k] * b[k]; break;
            case 1: acc += a[k]; break;
            case 2: {
                const double dv = b[k];
                acc = fmin(acc, dv < 0 ? -a[k] / (dv + kSmall) : 1.0);
                break;
            }
            case 3: acc = fmax(acc, -1.5 * a[k]); break;
            case 4: acc += (a[k] + t * b[k]) * (c[k] + t * d[k]); break;
            default: acc += (isfinite(a[k]) && isfinite(b[k])) ? 0.0 : 1.0; break;
        }
    }
    __shared__ double sh[kEw / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double v = __shfl_xor_sync(0xffffffffu, acc, o);
        acc = op == 2 ? fmin(acc, v) : (op == 3 ? fmax(acc, v) : acc + v);
    }
    if (lane == 0) sh[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = sh[0];
        for (int q = 1; q < kEw / 32; ++q)
            r = op == 2 ? fmin(r, sh[q]) : (op == 3 ? fmax(r, sh[q]) : r + sh[q]);
        part[blockIdx.x] = r;
    }
}

// ------------------------------------------------------------ host algebra --
using HVec = std::vector<double>;

// B = [diag(B11) D; D' diag(B22)] with the off-diagonal entries kept by
// supply row i < n-1: (demand j, value).
struct PdBlock {
    int m = 0, n12 = 0;
    HVec B11, B22;
    std::vector<std::vector<std::pair<int, double>>> rows;
};

// In-place Cholesky of a dense SPD matrix (row-major, lower triangle used).
bool pd_cholesky(HVec& A, int n) {
    for (int j = 0; j < n; ++j) {
        double* rj = A.data() + (size_t)j * n;
        double d = rj[j];
        for (int k = 0; k < j; ++k) d -= rj[k] * rj[k];
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        rj[j] = d;
        for (int i = j + 1; i < n; ++i) {
            double* ri = A.data() + (size_t)i * n;
            double v = ri[j];
            for (int k = 0; k < j; ++k) v -= ri[k] * rj[k];
            ri[j] = v / d;
        }
    }
    return true;
}

void pd_chol_solve(const HVec& L, int n, double* x) {
    for (int i = 0; i < n; ++i) {
        const double* ri = L.data() + (size_t)i * n;
        double v = x[i];
        for (int k = 0; k < i; ++k) v -= ri[k] * x[k];
        x[i] = v / ri[i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double v = x[i];
        for (int k = i + 1; k < n; ++k) v -= L[(size_t)k * n + i] * x[k];
        x[i] = v / L[(size_t)i * n + i];
    }
}

// Exact solves with B + shift I: the demand block is diagonal, the supply
// block is the Schur complement S = diag(B22 + shift) - D' diag(1/(B11 + shift)) D.
struct PdFactor {
    const PdBlock* B = nullptr;
    HVec d1, L;
    bool factor(const PdBlock& blk, double shift) {
        B = &blk;
        const int m = blk.m, n12 = blk.n12;
        d1.resize(m);
        for (int j = 0; j < m; ++j) {
            d1[j] = blk.B11[j] + shift;
            if (!(d1[j] > 0.0)) return false;
        }
        L.assign((size_t)n12 * n12, 0.0);
        for (int i = 0; i < n12; ++i) L[(size_t)i * n12 + i] = blk.B22[i] + shift;
        std::vector<std::vector<std::pair<int, double>>> cols(m);
        for (int i = 0; i < n12; ++i)
            for (const auto& e : blk.rows[i]) cols[e.first].push_back({i, e.second});
        for (int j = 0; j < m; ++j) {
            const auto& c = cols[j];
            const double inv = 1.0 / d1[j];
            for (size_t p = 0; p < c.size(); ++p)
                for (size_t q = 0; q <= p; ++q)
                    L[(size_t)c[p].first * n12 + c[q].first] -= c[p].second * c[q].second * inv;
        }
        return pd_cholesky(L, n12);
    }
    void solve(const double* r, double* x) const {
        const int m = B->m, n12 = B->n12;
        HVec t(n12);
        for (int i = 0; i < n12; ++i) {
            double v = r[m + i];
            for (const auto& e : B->rows[i]) v -= e.second * r[e.first] / d1[e.first];
            t[i] = v;
        }
        pd_chol_solve(L, n12, t.data());
        for (int j = 0; j < m; ++j) x[j] = r[j];
        for (int i = 0; i < n12; ++i)
            for (const auto& e : B->rows[i]) x[e.first] -= e.second * t[i];
        for (int j = 0; j < m; ++j) x[j] /= d1[j];
        for (int i = 0; i < n12; ++i) x[m + i] = t[i];
    }
};

// The shift retries of pdip_cg.cpp:262-268 and pdip_sparse_chol.cpp:40-60.
void pd_factor(const PdBlock& blk, PdFactor& f) {
    const double shifts[] = {0.0, 1e-12, 1e-10, 1e-8};
    for (double sh : shifts)
        if (f.factor(blk, sh)) return;
    throw Error(REGOT_ERR_NUMERIC, "qrot_pdip: block factorization failed");
}

// dynamic_threshold (pdip_cg.cpp:95-143) with the default keep factor 3, from
// the entries of scale on the supply rows (host copy, n12 x m row-major).
double pd_threshold(const double* sc, size_t count, int n, int iter, double reg) {
    std::vector<double> pos;
    pos.reserve(count);
    for (size_t k = 0; k < count; ++k)
        if (sc[k] > 0) pos.push_back(sc[k]);
    if (pos.empty()) return 1e-9;
    double ref = reg > 0 ? 1.0 / reg : 0.0;
    if (ref < 1e-16) {
        const size_t mid = pos.size() / 2;
        std::nth_element(pos.begin(), pos.begin() + mid, pos.end());
        ref = pos[mid];
    }
    ref = std::max(ref, 1e-16);
    const double progress = std::min((double)iter / 15.0, 1.0);
    const double keep = std::min(1.0, (1.0 + 2.0 * progress) / std::max(n, 1));
    size_t idx = (size_t)((1.0 - keep) * pos.size());
    if (idx >= pos.size()) idx = 0;
    std::nth_element(pos.begin(), pos.begin() + idx, pos.end());
    const double pct = pos[idx];
    const double t_fac = std::pow(1.48, std::min(std::max(iter, 0), 52));
    const double blend = std::min(1.0, (iter + 1) / 20.0);
    double th = (ref / std::max(n, 1)) * t_fac * (1.0 - 0.52 * blend) + pct * 0.52 * blend;
    th = std::min(th, pct);
    th = std::max(th, std::max(1e-9, std::min(ref * 1e-6, pct)));
    return std::min(th, ref * 0.5);
}

// ------------------------------------------------------------------ engine --
class PdipEngine {
public:
    PdipEngine(regot_ctx* ctx, regot_dproblem* P)
        : ctx_(ctx), st_(ctx->stream), n_(P->n), m_(P->m), nv_((long long)P->n * P->m) {
        const size_t nv = (size_t)nv_;
        for (DBuf<double>* b : {&c_, &x_, &s_, &scale_, &rd_, &dx_, &ds_, &rcc_, &tmp_, &at_})
            b->alloc(nv, st_);
        const int nc = m_ + n_ - 1;
        lam_.alloc(nc, st_);
        lam2_.alloc(nc, st_);
        rows_.alloc(n_, st_);
        cols_.alloc(m_, st_);
        wz_.alloc(m_ + n_, st_);
        part_.alloc(kRedBlocks, st_);
        hrows_.resize(n_);
        hcols_.resize(m_);
        const int g = grid();
        if (P->prec == REGOT_PREC_MIXED)
            k_pd_cost<float><<<g, kEw, 0, st_>>>(static_cast<const float*>(P->M), P->ldm, n_, m_,
                                                  c_.get());
        else
            k_pd_cost<double><<<g, kEw, 0, st_>>>(static_cast<const double*>(P->M), P->ldm, n_,
                                                   m_, c_.get());
        count_launch();
        REGOT_CHECK_LAUNCH();
    }

    int grid() const {
        const long long want = (nv_ + kEw - 1) / kEw;
        return (int)std::max(1LL, std::min<long long>(want, (long long)device_sm_count() * 8));
    }
    long long nv() const { return nv_; }
    cudaStream_t stream() const { return st_; }
    double* c() { return c_.get(); }
    double* x() { return x_.get(); }
    double* s() { return s_.get(); }
    double* scale() { return scale_.get(); }
    double* rd() { return rd_.get(); }
    double* dx() { return dx_.get(); }
    double* ds() { return ds_.get(); }
    double* rcc() { return rcc_.get(); }
    double* tmp() { return tmp_.get(); }
    double* at() { return at_.get(); }
    double* lam() { return lam_.get(); }
    double* lam2() { return lam2_.get(); }

    void upload(double* dst, const HVec& v) {
        h2d(dst, v.data(), v.size() * sizeof(double), st_);
    }

    // A arr (scaled by `sc` elementwise when given): [column sums; row sums of rows < n-1]
    void A_of(const double* arr, HVec& y) {
        const double* src = arr;
        k_pd_rowsum<<<cdiv((long long)n_ * 32, 256), 256, 0, st_>>>(n_, m_, src, nullptr,
                                                                   rows_.get());
        k_pd_colsum<<<cdiv(m_, 128), 128, 0, st_>>>(n_, m_, src, nullptr, cols_.get());
        count_launch(2);
        REGOT_CHECK_LAUNCH();
        read_rc();
        y.resize(m_ + n_ - 1);
        for (int j = 0; j < m_; ++j) y[j] = hcols_[j];
        for (int i = 0; i < n_ - 1; ++i) y[m_ + i] = hrows_[i];
    }
    // Row and column sums of arr into the host copies.
    void rc_of(const double* arr) {
        k_pd_rowsum<<<cdiv((long long)n_ * 32, 256), 256, 0, st_>>>(n_, m_, arr, nullptr,
                                                                   rows_.get());
        k_pd_colsum<<<cdiv(m_, 128), 128, 0, st_>>>(n_, m_, arr, nullptr, cols_.get());
        count_launch(2);
        REGOT_CHECK_LAUNCH();
        read_rc();
    }
    const HVec& hrows() const { return hrows_; }
    const HVec& hcols() const { return hcols_; }

    // y = [D z ; D' w] parts of the block product with the full D = scale
    // on the supply rows: y1_j = sum_{i<n-1} scale_ij z_i, y2_i = sum_j scale_ij w_j.
    void d_mul(const double* v, const PdBlock& B, double* y) {
        HVec wz(m_ + n_, 0.0);
        std::memcpy(wz.data(), v, (size_t)m_ * sizeof(double));        // w
        std::memcpy(wz.data() + m_, v + m_, (size_t)(n_ - 1) * sizeof(double));  // z, z_{n-1} = 0
        h2d(wz_.get(), wz.data(), wz.size() * sizeof(double), st_);
        k_pd_colsum<<<cdiv(m_, 128), 128, 0, st_>>>(n_, m_, scale_.get(), wz_.get() + m_,
                                                   cols_.get());
        k_pd_rowsum<<<cdiv((long long)n_ * 32, 256), 256, 0, st_>>>(n_, m_, scale_.get(),
                                                                   wz_.get(), rows_.get());
        count_launch(2);
        REGOT_CHECK_LAUNCH();
        read_rc();
        for (int j = 0; j < m_; ++j) y[j] = B.B11[j] * v[j] + hcols_[j];
        for (int i = 0; i < n_ - 1; ++i) y[m_ + i] = B.B22[i] * v[m_ + i] + hrows_[i];
    }

    // Scalar reduction (op as k_pd_reduce), summed / min / max on the host in
    // block order.
    double reduce(int op, const double* a, const double* b = nullptr, const double* c = nullptr,
                  const double* d = nullptr, double t = 0.0) {
        k_pd_reduce<<<kRedBlocks, kEw, 0, st_>>>(op, nv_, a, b, c, d, t, part_.get());
        count_launch();
        REGOT_CHECK_LAUNCH();
        double h[kRedBlocks];
        d2h(h, part_.get(), sizeof(h), st_);
        sync(st_);
        double r = h[0];
        for (int q = 1; q < kRedBlocks; ++q)
            r = op == 2 ? std::min(r, h[q]) : (op == 3 ? std::max(r, h[q]) : r + h[q]);
        return r;
    }

    void host_copy(const double* src, HVec& dst) {
        dst.resize((size_t)nv_);
        d2h(dst.data(), src, (size_t)nv_ * sizeof(double), st_);
        sync(st_);
    }

private:
    void read_rc() {
        d2h(hrows_.data(), rows_.get(), (size_t)n_ * sizeof(double), st_);
        d2h(hcols_.data(), cols_.get(), (size_t)m_ * sizeof(double), st_);
        sync(st_);
    }

    regot_ctx* ctx_;
    cudaStream_t st_;
    int n_, m_;
    long long nv_;
    DBuf<double> c_, x_, s_, scale_, rd_, dx_, ds_, rcc_, tmp_, at_, lam_, lam2_, rows_, cols_,
        wz_, part_;
    HVec hrows_, hcols_;
};

// solve_AAT (pdip_transport_ops.hpp:43-52).
void pd_solve_AAT(int n, int m, const HVec& r, HVec& out) {
    out.assign(m + n - 1, 0.0);
    double sum_d = 0.0;
    for (int j = 0; j < m; ++j) sum_d += r[j];
    HVec tmp(n - 1);
    double sum_t = 0.0;
    for (int i = 0; i < n - 1; ++i) {
        tmp[i] = sum_d / (double)n - r[m + i];
        sum_t += tmp[i];
    }
    double sum_x2 = 0.0;
    for (int i = 0; i < n - 1; ++i) {
        out[m + i] = (tmp[i] + sum_t) / (double)m;
        sum_x2 += out[m + i];
    }
    for (int j = 0; j < m; ++j) out[j] = (r[j] - sum_x2) / (double)n;
}

double pd_norm(const HVec& v) {
    double s = 0.0;
    for (double e : v) s += e * e;
    return std::sqrt(s);
}

// ------------------------------------------------------------------ driver --
// pdip_cg_internal (pdip_cg.cpp:206-413) when !fp, pdip_fp_internal
// (pdip_fp.cpp:278-667) when fp.
void pdip_run(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter, bool fp,
              const regot_pdip_opts& po, const regot_opts& o, regot_result* res, int* converged) {
    using clock = std::chrono::steady_clock;
    const int n = P->n, m = P->m, nc = m + n - 1, N = nc;
    require(n >= 2 && m >= 1, "qrot_pdip: n must be at least 2");
    PdipEngine E(ctx, P);
    cudaStream_t st = E.stream();
    const long long nv = E.nv();
    const int g = E.grid();
    const double reg_val = reg > 0 ? reg : 1e-6, barrier = reg_val;
    HVec eq(nc);
    for (int j = 0; j < m; ++j) eq[j] = P->hb[j];
    for (int i = 0; i < n - 1; ++i) eq[m + i] = P->ha[i];
    const auto t_start = clock::now();

    // Phase 1: initial point (pdip_cg.cpp:240-262, pdip_fp.cpp:319-356)
    HVec lam, b2, t, tmpv;
    pd_solve_AAT(n, m, eq, lam);
    E.upload(E.lam(), lam);
    k_pd_at<<<g, kEw, 0, st>>>(n, m, 0, barrier, E.lam(), nullptr, nullptr, E.x());
    count_launch();
    E.A_of(E.x(), b2);
    E.A_of(E.c(), t);
    for (int q = 0; q < nc; ++q) b2[q] = -barrier * b2[q] - t[q];
    pd_solve_AAT(n, m, b2, lam);
    E.upload(E.lam(), lam);
    k_pd_at<<<g, kEw, 0, st>>>(n, m, 1, barrier, E.lam(), E.x(), E.c(), E.s());
    count_launch();
    REGOT_CHECK_LAUNCH();
    const double dxs = std::max(0.0, E.reduce(3, E.x()));
    const double dss = std::max(0.0, E.reduce(3, E.s()));
    k_pd_shift<<<g, kEw, 0, st>>>(nv, dxs, dss, 0, E.x(), E.s());
    count_launch();
    {
        double xs = E.reduce(0, E.x(), E.s()), ss = E.reduce(1, E.s()), xx = E.reduce(1, E.x());
        const double ax = fp ? 0.5 * xs / ss : 0.5 * xs / (ss + kSmall);
        k_pd_shift<<<g, kEw, 0, st>>>(nv, ax, 0.0, 0, E.x(), E.s());
        count_launch();
        xs = E.reduce(0, E.x(), E.s());
        const double sx = E.reduce(1, E.x());
        // pdip_fp.cpp:353 adds the new sum to the old one
        xx = fp ? xx + sx : sx;
        const double as = fp ? 0.5 * xs / xx : 0.5 * xs / (xx + kSmall);
        k_pd_shift<<<g, kEw, 0, st>>>(nv, 0.0, as, 1, E.x(), E.s());
        count_launch();
        REGOT_CHECK_LAUNCH();
    }

    const double norm_eq = pd_norm(eq);
    const double norm_cost = std::sqrt(E.reduce(0, E.c(), E.c()));
    HVec r_pri(nc), c(nc), dlam, dlam2, dlam_prev, hscale, mar_hist, hobj, hmar, htime;
    int niter = 0;
    bool conv = false;
    for (int it = 0; it < max_iter; ++it) {
        // 2.1 residuals and scaling
        k_pd_start<<<g, kEw, 0, st>>>(n, m, barrier, E.x(), E.s(), E.c(), E.lam(), E.scale(),
                                      E.rd(), E.tmp());
        count_launch();
        REGOT_CHECK_LAUNCH();
        E.A_of(E.x(), r_pri);
        for (int q = 0; q < nc; ++q) r_pri[q] -= eq[q];

        // 2.2 the block matrix: diagonals from the sums of scale, the
        // off-diagonal pattern from a host copy of it
        PdBlock blk;
        blk.m = m;
        blk.n12 = n - 1;
        E.rc_of(E.scale());
        blk.B11 = E.hcols();
        blk.B22.assign(E.hrows().begin(), E.hrows().begin() + (n - 1));
        E.host_copy(E.scale(), hscale);
        const size_t supply = (size_t)(n - 1) * m;
        bool use_fp_iter = false;
        double th;
        if (!fp) {
            th = pd_threshold(hscale.data(), supply, n, it, reg_val);
        } else {
            bool dense = it < 3;
            if (!dense) {
                long long kept = 0;
                for (size_t k = 0; k < supply; ++k) kept += hscale[k] >= po.fixed_threshold;
                const double sparsity =
                    supply == 0 ? 1.0 : 1.0 - (double)kept / (double)supply;
                use_fp_iter = po.fixed_threshold > 0.0 && sparsity >= 0.99;
            }
            th = use_fp_iter ? po.fixed_threshold : -std::numeric_limits<double>::infinity();
        }
        blk.rows.assign(n - 1, {});
        for (int i = 0; i < n - 1; ++i)
            for (int j = 0; j < m; ++j) {
                const double v = hscale[(size_t)i * m + j];
                if (v >= th) blk.rows[i].push_back({j, v});
            }
        PdFactor F;
        pd_factor(blk, F);

        double cg_tol = 0.0;
        if (!fp) {
            const double rp = pd_norm(r_pri);
            const double tb = std::min((double)it, 40.0) / 40.0;
            cg_tol = std::max(0.1 * std::pow(0.1, tb) * rp, 1e-12);
        }
        auto mul = [&](const double* v, double* y) { E.d_mul(v, blk, y); };
        // inner solve of B dlam = rhs
        auto inner = [&](const HVec& rhs, HVec& out, const HVec* guess) {
            if (!fp) {
                // solve_block_schur_cg (pdip_cg.cpp:157-176): Eigen's PCG with
                // the factor of the thresholded B as preconditioner
                if (guess && (int)guess->size() == N) out = *guess;
                else out.assign(N, 0.0);
                const double cn = pd_norm(rhs) + 1e-50;
                const double rtol = std::min(cg_tol / cn, 0.1);
                const double rel = std::max(rtol, cg_tol / cn);
                HVec r(N), p(N), z(N), tv(N);
                mul(out.data(), tv.data());
                double rhs2 = 0.0;
                for (int q = 0; q < N; ++q) {
                    r[q] = rhs[q] - tv[q];
                    rhs2 += rhs[q] * rhs[q];
                }
                if (rhs2 == 0.0) {
                    std::fill(out.begin(), out.end(), 0.0);
                    return;
                }
                const double thresh =
                    std::max(rel * rel * rhs2, std::numeric_limits<double>::min());
                double r2 = 0.0;
                for (double v : r) r2 += v * v;
                if (r2 < thresh) return;
                F.solve(r.data(), p.data());
                double absnew = 0.0;
                for (int q = 0; q < N; ++q) absnew += r[q] * p[q];
                for (int k = 0; k < po.cg_max_iter; ++k) {
                    mul(p.data(), tv.data());
                    double pt = 0.0;
                    for (int q = 0; q < N; ++q) pt += p[q] * tv[q];
                    const double alpha = absnew / pt;
                    r2 = 0.0;
                    for (int q = 0; q < N; ++q) {
                        out[q] += alpha * p[q];
                        r[q] -= alpha * tv[q];
                        r2 += r[q] * r[q];
                    }
                    if (r2 < thresh) break;
                    F.solve(r.data(), z.data());
                    const double absold = absnew;
                    absnew = 0.0;
                    for (int q = 0; q < N; ++q) absnew += r[q] * z[q];
                    const double beta = absnew / absold;
                    for (int q = 0; q < N; ++q) p[q] = z[q] + beta * p[q];
                }
            } else if (!use_fp_iter) {
                out.resize(N);
                F.solve(rhs.data(), out.data());
            } else {
                // fixed_point_solve_block_sparse (pdip_fp.cpp:232-276)
                HVec xk(N), xt(N, 0.0), rw(N), rh(N);
                if (guess && !guess->empty()) xk = *guess;
                else F.solve(rhs.data(), xk.data());
                auto resid = [&](const HVec& v) {
                    mul(v.data(), rw.data());
                    double e = 0.0;
                    for (int q = 0; q < N; ++q) e += (rhs[q] - rw[q]) * (rhs[q] - rw[q]);
                    return std::sqrt(e);
                };
                double rpk = resid(xk) + 1e-20;
                const double exit_scale = po.fp_exit_scale <= 0 ? 1e-2 : po.fp_exit_scale;
                for (int k = 0; k < po.fp_max_iter; ++k) {
                    mul(xk.data(), rw.data());
                    for (int q = 0; q < N; ++q) rh[q] = rhs[q] - rw[q];
                    // + B_sparse xk
                    for (int j = 0; j < m; ++j) rh[j] += blk.B11[j] * xk[j];
                    for (int i = 0; i < n - 1; ++i) {
                        double v = blk.B22[i] * xk[m + i];
                        for (const auto& e : blk.rows[i]) {
                            rh[e.first] += e.second * xk[m + i];
                            v += e.second * xk[e.first];
                        }
                        rh[m + i] += v;
                    }
                    F.solve(rh.data(), xt.data());
                    const double rn = resid(xt);
                    if (rn < exit_scale * rpk) break;
                    rpk = rn;
                    xk = xt;
                }
                out = xt;
            }
        };

        // 2.3 predictor: c = A(scale (-s - r_dual)) + r_pri
        E.A_of(E.tmp(), c);
        for (int q = 0; q < nc; ++q) c[q] += r_pri[q];
        inner(c, dlam, dlam_prev.size() == (size_t)N ? &dlam_prev : nullptr);
        E.upload(E.lam2(), dlam);
        k_pd_pred<<<g, kEw, 0, st>>>(n, m, barrier, E.x(), E.s(), E.scale(), E.rd(), E.lam2(),
                                     E.dx(), E.ds());
        count_launch();
        REGOT_CHECK_LAUNCH();
        double a1 = std::min(E.reduce(2, E.x(), E.dx()), 1.0);
        a1 = std::min(a1, E.reduce(2, E.s(), E.ds()));
        a1 = std::min(a1, 1.0);
        const double mu = E.reduce(0, E.x(), E.s()) / (double)nv;
        const double mu_aff = E.reduce(4, E.x(), E.dx(), E.s(), E.ds(), a1) / (double)nv;
        const double sigma = std::min(std::pow(mu_aff / mu, 3.0), 1.0);

        // 2.4 corrector
        k_pd_corr<<<g, kEw, 0, st>>>(nv, sigma * mu, E.x(), E.s(), E.dx(), E.ds(), E.scale(),
                                     E.rd(), E.rcc(), E.tmp());
        count_launch();
        E.A_of(E.tmp(), c);
        for (int q = 0; q < nc; ++q) c[q] += r_pri[q];
        inner(c, dlam2, &dlam);
        E.upload(E.lam2(), dlam2);
        k_pd_final<<<g, kEw, 0, st>>>(n, m, barrier, E.x(), E.s(), E.scale(), E.rd(), E.rcc(),
                                      E.lam2(), E.dx(), E.ds());
        count_launch();
        REGOT_CHECK_LAUNCH();
        double a2 = std::min(E.reduce(2, E.x(), E.dx()), E.reduce(2, E.s(), E.ds()));
        a2 = std::min(0.99 * a2, 1.0);
        HVec lam_new(nc);
        for (int q = 0; q < nc; ++q) lam_new[q] = lam[q] + a2 * dlam2[q];
        // 2.5: PDIP-CG forms r_dual with the multipliers' image from before
        // the update (pdip_cg.cpp:352-356), PDIP-FP with the new one
        // (pdip_fp.cpp:602-608); lam2 holds the new multipliers.
        E.upload(E.lam2(), lam_new);
        k_pd_update<<<g, kEw, 0, st>>>(n, m, barrier, a2, E.dx(), E.ds(), E.c(),
                                       fp ? E.lam2() : E.lam(), E.lam2(), E.x(), E.s(), E.rd(),
                                       E.at());
        count_launch();
        REGOT_CHECK_LAUNCH();
        lam.swap(lam_new);
        E.upload(E.lam(), lam);
        dlam_prev = dlam2;

        E.A_of(E.x(), r_pri);
        for (int q = 0; q < nc; ++q) r_pri[q] -= eq[q];
        const double primal_gap = pd_norm(r_pri) / (1.0 + norm_eq);
        const double dual_gap = std::sqrt(E.reduce(0, E.rd(), E.rd())) /
                                (1.0 + norm_cost + std::sqrt(E.reduce(0, E.at(), E.at())));
        const double mu_stop = E.reduce(0, E.x(), E.s()) / (double)nv;
        // marginal error from the row and column sums of x (already read)
        double e1 = 0.0, e2 = 0.0, alast = 1.0;
        for (int i = 0; i < n - 1; ++i) alast -= eq[m + i];
        const HVec& rs = E.hrows();
        const HVec& cs = E.hcols();
        for (int i = 0; i < n; ++i) {
            const double ai = i < n - 1 ? eq[m + i] : alast;
            e1 += (rs[i] - ai) * (rs[i] - ai);
        }
        for (int j = 0; j < m; ++j) e2 += (cs[j] - eq[j]) * (cs[j] - eq[j]);
        const double me = std::max(std::sqrt(e1), std::sqrt(e2));
        const double obj = E.reduce(0, E.c(), E.x()) + reg_val / 2.0 * E.reduce(0, E.x(), E.x());
        const double ms =
            std::chrono::duration<double, std::milli>(clock::now() - t_start).count();
        if (!fp) {
            if (!std::isfinite(me) || !std::isfinite(primal_gap) || !std::isfinite(dual_gap) ||
                !std::isfinite(mu_stop))
                break;
            if (me > 1e3 || E.reduce(5, E.x(), E.s()) > 0.0) {
                niter = it + 1;
                break;
            }
        }
        hobj.push_back(obj);
        hmar.push_back(me);
        htime.push_back(ms);
        mar_hist.push_back(me);
        if (o.verbose >= 1)
            std::printf("iter = %d, obj = %g, mar_err = %g, primal_gap = %g, dual_gap = %g, "
                        "mu = %g\n", it, obj, me, primal_gap, dual_gap, mu_stop);
        const bool by_gap = primal_gap < tol && dual_gap < tol && mu_stop < tol;
        bool stop;
        if (fp) {
            stop = po.fp_stop_gap_mu_only ? by_gap : (by_gap || me < tol);
        } else {
            // by_stable (pdip_cg.cpp:85-93) implies by_mar_tol
            stop = po.cg_stop_gap_mu_only ? by_gap : (by_gap || me < po.cg_mar_tol);
        }
        niter = it + 1;
        if (stop) {
            conv = true;
            break;
        }
    }
    const int L = (int)hobj.size();
    res->niter = niter;
    res->hist_len = L;
    if (res->obj_vals) std::memcpy(res->obj_vals, hobj.data(), L * sizeof(double));
    if (res->mar_errs) std::memcpy(res->mar_errs, hmar.data(), L * sizeof(double));
    if (res->run_times) std::memcpy(res->run_times, htime.data(), L * sizeof(double));
    if (o.plan && res->plan)
        emit_plan(res->plan, o.plan_mem, (size_t)nv, st, [&](double* dst) {
            REGOT_CUDA(cudaMemcpyAsync(dst, E.x(), (size_t)nv * sizeof(double),
                                       cudaMemcpyDefault, st));
        });
    sync(st);
    if (converged) *converged = conv ? 1 : 0;
}

}  // namespace

void qrot_pdip_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                   const regot_pdip_opts& po, const regot_opts& o, regot_result* res,
                   int* converged) {
    require(po.inner_solver == 0 || po.inner_solver == 1,
            "qrot_pdip: inner_solver must be \"cg\" or \"fp\"");
    pdip_run(ctx, P, reg, tol, max_iter, po.inner_solver == 1, po, o, res, converged);
}

}  // namespace regot
