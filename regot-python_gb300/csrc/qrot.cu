// QROT on the GPU: qrot_lbfgs_dual (reference src/qrot_lbfgs_dual.cpp:81-126),
// qrot_assn (src/qrot_assn.cpp:16-170), qrot_grssn (src/qrot_grssn.cpp:16-133),
// qrot_lbfgs_semi_dual (src/qrot_lbfgs_semi_dual.cpp:84-126), qrot_bcd
// (src/qrot_bcd.cpp:14-103), qrot_gd (src/qrot_gd.cpp:14-120), qrot_apdagd
// (src/qrot_apdagd.cpp:14-179) and qrot_pdaam (src/qrot_pdaam.cpp:14-188),
// with the dense passes of src/qrot_problem.cpp and src/qrot_hess.cpp.
//
//   grad / obj   one pass: D = (alpha_i + beta_j - M_ij)+, row and column sums
//                of D and sum D^2 (compute_D_stats, qrot_problem.cpp:36-94).
//   Jacobian     the same pass also writes sigma = 1[C > 0] as a bitmask
//                (one bit per entry, 32x smaller than FP32 M and L2-resident
//                for the benchmark sizes) plus the row/column counts
//                h1 = sigma 1, h2 = sigma' 1 (compute_D_hess, qrot_hess.cpp:41-96).
//                sigma x and sigma' y then read the bitmask only.
//   primal_val   three passes (row sums of P; column sums of P x; per-row
//                sums of P y, P y f, M f and the totals <R, M>, ||R||^2),
//                the rank-one correction of approx_proj (approx_proj.h:6-26)
//                expanded analytically, so no n x m plan is materialised.
//   optimal_beta per column, Newton's method from above on the convex
//                piecewise-linear sum_i (x - y_i)+ = reg b_j (y = M_:j - alpha):
//                x <- (reg b_j + sum_{y_i < x} y_i) / #{y_i < x}, one pass per
//                step until no active set changes; the fixed point is the root
//                that piecewise_linear_equation (qrot_problem.cpp:368-392) finds
//                by sorting.
// The L-BFGS driver and the ASSN outer loop run on the host in FP64; the
// ASSN Schur-complement CG (qrot_cg.cpp:9-50: identity preconditioner,
// relative tolerance 1e-8, at most 2m steps) runs on the device: with few
// entries in sigma (the usual case: a couple per row) over row and column
// index lists in a single thread-block-cluster launch, else over the
// bitmask in a CUDA graph of its steps.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "device_util.cuh"
#include "sm100_util.cuh"
#include "erot_ops.cuh"
#include "lbfgs.h"
#include "solvers.h"

namespace regot {

namespace {

constexpr int kVT = 64;           // vector-kernel block size
constexpr int kColChunks = 32;    // row chunks of the sigma' y kernel

// Schur CG path: 0 chooses by the number of entries of sigma, 1 always the
// bitmask products, 2 always the index lists, 3 the index lists with the
// vectors exchanged through global memory even where shared memory would
// hold them (force_qrot_cg_path)
std::atomic<int> g_qrot_cg_path{0};

struct QState {
    unsigned counter;
    int cg_done;
    int cg_it;
    int cg_max;
    int changed;
    int pad;
    double dot_ab;   // alpha' a + beta' b
    double sum_a;    // 1' alpha
    double sum_b;    // 1' beta
    double sq;       // sum D^2
    double rr;       // CG r'r
    double alpha;
    double beta;
    double thresh2;
    double prim[6];  // primal-value scalars
    double maxabs;
    double mu;       // shift of the Schur CG (read by its captured steps)
    int root_rounds; // Newton rounds of the last optimal_alpha / optimal_beta
    int root_unconverged;
};

// ---- gradient / objective merge ----
// Blocks of (32, 8) threads: the first cdiv(n, 32) blocks own 32 rows each,
// the rest 32 columns each; the eight threads of a row or column merge its
// partials together (merge_2d), then warp 0 carries on.
template <typename Acc>
__global__ void __launch_bounds__(256) k_q_grad(const Acc* rp, int nslabs, const Acc* cp, int nrb,
                                               int n, int m, int with_counts,
                                               const double* gamma, const double* a,
                                               const double* b, double reg, double* grad,
                                               double* h1, double* h2, double* parts,
                                               QState* st) {
    const int nbr = (n + 31) / 32;
    const bool rows = (int)blockIdx.x < nbr;
    const int t = (rows ? (int)blockIdx.x : (int)blockIdx.x - nbr) * 32 + threadIdx.x;
    const bool valid = rows ? t < n : t < m;
    double sum, cnt = 0.0;
    if (rows) {
        sum = merge_2d(rp + t, nslabs, (size_t)n, valid);
        if (with_counts) {
            __syncthreads();
            cnt = merge_2d(rp + (size_t)nslabs * n + t, nslabs, (size_t)n, valid);
        }
    } else {
        sum = merge_2d(cp + t, nrb, (size_t)m, valid);
        if (with_counts) {
            __syncthreads();
            cnt = merge_2d(cp + (size_t)nrb * m + t, nrb, (size_t)m, valid);
        }
    }
    if (threadIdx.y != 0) return;
    double v[3] = {0.0, 0.0, 0.0};
    if (valid && rows) {
        grad[t] = sum - reg * a[t];
        if (with_counts) h1[t] = cnt;
        v[0] = gamma[t] * a[t];
        v[1] = gamma[t];
    } else if (valid) {
        grad[n + t] = sum - reg * b[t];
        if (with_counts) h2[t] = cnt;
        v[0] = gamma[n + t] * b[t];
        v[2] = gamma[n + t];
    }
    double out[3];
    __threadfence();
    if (warp_grid_reduce<3>(v, parts, &st->counter, out) && threadIdx.x == 0) {
        st->dot_ab = out[0];
        st->sum_a = out[1];
        st->sum_b = out[2];
    }
}

// Sum of one row of per-CTA totals into *out (single block).
__global__ void k_sum_totals(const double* totpart, int nblocks, double* out) {
    double v = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) v += totpart[k];
    __shared__ double s[32];
    v = warp_sum_d(v);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += s[w];
        *out = r;
    }
}

// ---- optimal_beta by Newton's method from above (per column) ----
__global__ void k_root_init(int m, double* x, double* prev_cnt) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) {
        x[j] = INFINITY;
        prev_cnt[j] = -1.0;
    }
}

// Blocks of (32, 8) threads own 32 columns; the eight threads of a column
// merge its row-block partials together (a serial chain of FP64 adds per
// column was latency-bound). The counts are exact in any order.
__global__ void __launch_bounds__(256) k_root_update(const double* cp, int nrb, int m,
                                                     const double* b, double reg, double* x,
                                                     double* prev_cnt, QState* st) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const bool valid = j < m;
    const double cnt = merge_2d(cp + j, nrb, (size_t)m, valid);
    __syncthreads();
    const double sum = merge_2d(cp + (size_t)nrb * m + j, nrb, (size_t)m, valid);
    if (threadIdx.y != 0 || !valid) return;
    if (cnt != prev_cnt[j]) {
        prev_cnt[j] = cnt;
        x[j] = (reg * b[j] + sum) / cnt;
        atomicOr(&st->changed, 1);
    }
}

// Row analogue for optimal_alpha (qrot_problem.cpp:409-419): rows' count
// and sum of y = M_ij - beta_j below the current root x_i.
__global__ void k_rowroot_update(const double* rp, int nslabs, int n, const double* a, double reg,
                                 double* x, double* prev_cnt, QState* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double cnt = merge_strided(rp + i, nslabs, (size_t)n);
    const double sum = merge_strided(rp + (size_t)nslabs * n + i, nslabs, (size_t)n);
    if (cnt != prev_cnt[i]) {
        prev_cnt[i] = cnt;
        x[i] = (reg * a[i] + sum) / cnt;
        atomicOr(&st->changed, 1);
    }
}

// Start and condition of the device-side loop of root rounds (the last node
// of its body): continue while some row or column changed its active set,
// for at most cap rounds.
__global__ void k_root_begin(QState* st) {
    st->changed = 0;
    st->root_rounds = 0;
    st->root_unconverged = 0;
}
__global__ void k_root_loop(QState* st, int cap, cudaGraphConditionalHandle h) {
    const int rounds = ++st->root_rounds;
    const bool changed = st->changed != 0;
    st->changed = 0;
    if (changed && rounds >= cap) st->root_unconverged = 1;
    cudaGraphSetConditional(h, changed && rounds < cap ? 1u : 0u);
}

// ---- primal value (approx_proj) ----
// P1 merge: x_i = min(a_i / (rowsum(D)_i / reg), 1)
template <typename Acc>
__global__ void k_prim1(const Acc* rp, int nslabs, int n, const double* a, double reg,
                        double* xr, float4* rs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double x = fmin(a[i] / (merge_strided(rp + i, nslabs, (size_t)n) / reg), 1.0);
        xr[i] = x;
        if (rs) rs[i].z = (float)x;  // the next passes' row operand, in place
    }
}
// P2 merge: c_j = colsum(D x)/reg; y_j = min(b_j / c_j, 1); f_j = b_j - y_j c_j
template <typename Acc>
__global__ void k_prim2(const Acc* cp, int nrb, int m, const double* b, double reg, double* yc,
                        double* fc, double* parts, QState* st, float4* cs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (j < m) {
        const double c = merge_strided(cp + j, nrb, (size_t)m) / reg;
        const double y = fmin(b[j] / c, 1.0);
        const double f = b[j] - y * c;
        yc[j] = y;
        fc[j] = f;
        if (cs) {  // the P3 pass's column operands, in place
            cs[j].z = (float)y;
            cs[j].w = (float)f;
        }
        v[0] = f * f;
    }
    double out[1];
    __threadfence();
    if (grid_reduce<1>(v, parts, &st->counter, out)) st->prim[0] = out[0];  // ||f||^2
}
// P3 merge: e_i = a_i - x_i A_i; sums |e|, e . Cc, x e B, e^2
template <typename Acc>
__global__ void k_prim3(const Acc* rp, int nslabs, int n, const double* a, const double* xr,
                        double reg, double* parts, QState* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (i < n) {
        const double A = merge_strided(rp + i, nslabs, (size_t)n) / reg;
        const double B = merge_strided(rp + (size_t)nslabs * n + i, nslabs, (size_t)n) / reg;
        const double Cc = merge_strided(rp + 2 * (size_t)nslabs * n + i, nslabs, (size_t)n);
        const double e = a[i] - xr[i] * A;
        v[0] = fabs(e);
        v[1] = e * Cc;
        v[2] = xr[i] * e * B;
        v[3] = e * e;
    }
    double out[4];
    __threadfence();
    if (grid_reduce<4>(v, parts, &st->counter, out)) {
        st->prim[1] = out[0];
        st->prim[2] = out[1];
        st->prim[3] = out[2];
        st->prim[4] = out[3];
    }
}

// ---- sigma x and sigma' y from the bitmask ----
// The bitmask follows the dense-pass tiling: for row i and column slab s,
// LC words; bit L of word q covers column s*CW + ((q/VW)*32 + L)*VW + q%VW.
template <int CW, int VW, int LC>
__device__ __forceinline__ int bit_col(int s, int q, int L) {
    return s * CW + ((q / VW) * 32 + L) * VW + (q % VW);
}

// out_i = scale_i * sum_j sigma_ij x_j, scale_i = 1 / (h1_i + mu) (or 1).
template <int CW, int VW, int LC>
__global__ void k_sigma_rows(const uint32_t* bm, int n, int m, int nslabs, const double* x,
                             const double* h1, double mu, const double* mu_dev, int divide,
                             double* out, const int* done) {
    if (done && *done) return;
    if (mu_dev) mu = *mu_dev;
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    double acc = 0.0;
    const uint32_t* row = bm + (size_t)i * nslabs * LC;
    for (int s = 0; s < nslabs; ++s) {
#pragma unroll
        for (int q = 0; q < LC; ++q) {
            const uint32_t w = row[s * LC + q];
            if ((w >> lane) & 1u) {
                const int j = bit_col<CW, VW, LC>(s, q, lane);
                acc += x[j];
            }
        }
    }
    acc = warp_sum_d(acc);
    if (lane == 0) out[i] = divide ? acc / (h1[i] + mu) : acc;
}

// Mixed engine: the same products with the vector given as FP32 (hi, lo)
// pairs and summed in compensated FP32 (TwoSum), converted to FP64 once per
// row. One FP64 add per set bit made these products FP64-bound on this part;
// the compensated sums stay within about 2^-44 of sum |x_j| over the row.
__device__ __forceinline__ float2 split_f2(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ void cadd(float& s, float& e, float2 x) {
    float t, te;
    two_sum_f(s, x.x, t, te);
    s = t;
    e += te + x.y;
}

template <int CW, int VW, int LC>
__global__ void k_sigma_rows_f(const uint32_t* bm, int n, int m, int nslabs, const float2* x2,
                               const double* h1, double mu, const double* mu_dev, int divide,
                               double* out, float2* out2, const int* done) {
    if (done && *done) return;
    if (mu_dev) mu = *mu_dev;
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    float s = 0.f, e = 0.f;
    const uint32_t* row = bm + (size_t)i * nslabs * LC;
    for (int sl = 0; sl < nslabs; ++sl) {
#pragma unroll
        for (int q = 0; q < LC; ++q) {
            const uint32_t w = row[sl * LC + q];
            if ((w >> lane) & 1u) cadd(s, e, x2[bit_col<CW, VW, LC>(sl, q, lane)]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float so = __shfl_xor_sync(0xffffffffu, s, o);
        const float eo = __shfl_xor_sync(0xffffffffu, e, o);
        float t, te;
        two_sum_f(s, so, t, te);
        s = t;
        e += eo + te;
    }
    if (lane == 0) {
        const double acc = (double)s + (double)e;
        const double r = divide ? acc / (h1[i] + mu) : acc;
        out[i] = r;
        if (out2) out2[i] = split_f2(r);
    }
}

template <int CW, int VW, int LC>
__global__ void k_sigma_cols_f(const uint32_t* bm, int n, int m, int nslabs, const float2* y2,
                               double* partial, const int* done) {
    if (done && *done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (j >= m) return;
    const int sl = j / CW, o = j - sl * CW;
    const int L = (o % (32 * VW)) / VW;
    const int q = (o / (32 * VW)) * VW + (o % VW);
    const int rows_per = (n + gridDim.y - 1) / gridDim.y;
    const int i0 = c * rows_per, i1 = min(n, i0 + rows_per);
    float s = 0.f, e = 0.f;
    int i = i0;
    for (; i + 8 <= i1; i += 8) {
        // eight rows' words and values in flight at once
        uint32_t w[8];
        float2 yv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            w[u] = bm[((size_t)(i + u) * nslabs + sl) * LC + q];
            yv[u] = y2[i + u];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if ((w[u] >> L) & 1u) cadd(s, e, yv[u]);
    }
    for (; i < i1; ++i) {
        const uint32_t w = bm[((size_t)i * nslabs + sl) * LC + q];
        if ((w >> L) & 1u) cadd(s, e, y2[i]);
    }
    partial[(size_t)c * m + j] = (double)s + (double)e;
}

// partial[c][j] = sum_{i in chunk c} sigma_ij y_i
template <int CW, int VW, int LC>
__global__ void k_sigma_cols(const uint32_t* bm, int n, int m, int nslabs, const double* y,
                             double* partial, const int* done) {
    if (done && *done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (j >= m) return;
    const int s = j / CW, o = j - s * CW;
    const int L = (o % (32 * VW)) / VW;
    const int q = (o / (32 * VW)) * VW + (o % VW);
    const int rows_per = (n + gridDim.y - 1) / gridDim.y;
    const int i0 = c * rows_per, i1 = min(n, i0 + rows_per);
    double acc = 0.0;
    int i = i0;
    for (; i + 8 <= i1; i += 8) {
        uint32_t w[8];
        double yv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            w[u] = bm[((size_t)(i + u) * nslabs + s) * LC + q];
            yv[u] = y[i + u];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if ((w[u] >> L) & 1u) acc += yv[u];
    }
    for (; i < i1; ++i) {
        const uint32_t w = bm[((size_t)i * nslabs + s) * LC + q];
        if ((w >> L) & 1u) acc += y[i];
    }
    partial[(size_t)c * m + j] = acc;
}

// ---- ASSN Schur-complement CG: Delta x = h2 o x + mu x - sigma' ((sigma x) / (h1 + mu)) ----
// The float2 arguments (mixed engine, else null) receive the FP32 (hi, lo)
// copies of the vectors the sigma products read.
__global__ void k_acg_init(int m, const double* zy, double tol, double* x, double* r, double* p,
                           double* parts, QState* st, float2* x2, float2* p2) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (j < m) {
        x[j] = 0.0;
        r[j] = zy[j];
        p[j] = zy[j];
        if (x2) x2[j] = make_float2(0.f, 0.f);
        if (p2) p2[j] = split_f2(zy[j]);
        v[0] = zy[j] * zy[j];
    }
    double out[1];
    __threadfence();
    if (grid_reduce<1>(v, parts, &st->counter, out)) {
        st->rr = out[0];
        st->thresh2 = fmax(tol * tol * out[0], 2.2250738585072014e-308);
        st->cg_it = 0;
        st->cg_done = (out[0] == 0.0 || out[0] < st->thresh2) ? 1 : 0;
    }
}

// Blocks of (32, 8) threads own 32 columns; the eight threads of a column
// merge its chunk partials together, then warp 0 carries on.
__global__ void __launch_bounds__(256) k_acg_a(int m, const double* partial, int chunks,
                                               const double* h2, const double* p, double* y,
                                               double* parts, QState* st) {
    if (st->cg_done) return;
    const double mu = st->mu;
    const int j = blockIdx.x * 32 + threadIdx.x;
    const double u = merge_2d(partial + j, chunks, (size_t)m, j < m);
    if (threadIdx.y != 0) return;
    double v[1] = {0.0};
    if (j < m) {
        const double yj = h2[j] * p[j] + mu * p[j] - u;
        y[j] = yj;
        v[0] = p[j] * yj;
    }
    double out[1];
    __threadfence();
    if (warp_grid_reduce<1>(v, parts, &st->counter, out) && threadIdx.x == 0)
        st->alpha = st->rr / out[0];
}

__global__ void k_acg_b(int m, const double* p, const double* y, double* x, double* r,
                        double* parts, QState* st, float2* x2) {
    if (st->cg_done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const double al = st->alpha;
    double v[1] = {0.0};
    if (j < m) {
        const double xj = x[j] + al * p[j];
        x[j] = xj;
        if (x2) x2[j] = split_f2(xj);
        const double rj = r[j] - al * y[j];
        r[j] = rj;
        v[0] = rj * rj;
    }
    double out[1];
    __threadfence();
    if (grid_reduce<1>(v, parts, &st->counter, out)) {
        st->cg_it += 1;
        if (out[0] < st->thresh2 || st->cg_it >= st->cg_max || !(out[0] == out[0])) {
            st->cg_done = 1;
        } else {
            st->beta = out[0] / st->rr;
            st->rr = out[0];
        }
    }
}

__global__ void k_acg_c(int m, const double* r, double* p, QState* st, float2* p2) {
    if (st->cg_done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) {
        const double pj = r[j] + st->beta * p[j];
        p[j] = pj;
        if (p2) p2[j] = split_f2(pj);
    }
}

// w / (h1 + mu) for the Schur right-hand side
__global__ void k_div_h1(int n, const double* w, const double* h1, double mu, double* out,
                         float2* out2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double v = w[i] / (h1[i] + mu);
        out[i] = v;
        if (out2) out2[i] = split_f2(v);
    }
}
// zy_j = rhs_j - sum_c partial[c][j]
__global__ void k_sub_partial(int m, const double* rhs, const double* partial, int chunks,
                              double* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    double u = 0.0;
#pragma unroll 8
    for (int c = 0; c < chunks; ++c) u += partial[(size_t)c * m + j];
    out[j] = rhs[j] - u;
}
// r1_i = (w_i - (sigma r2)_i) / (h1_i + mu)
__global__ void k_backsub(int n, const double* w, const double* sr2, const double* h1, double mu,
                          double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (w[i] - sr2[i]) / (h1[i] + mu);
}

// ---- compact sigma: row and column index lists built from the bitmask ----
// At the points ASSN and GRSSN visit, sigma holds a few entries per row
// (D > 0 on a small fraction of the plan), so the CG products run over
// index lists instead of testing every bit of the n x m mask at each step.
// rcnt_i = number of set bits of row i (one warp per row)
template <int CW, int VW, int LC>
__global__ void k_cs_row_counts(const uint32_t* bm, int n, int nslabs, int* rcnt) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    const int W = nslabs * LC;
    const uint32_t* row = bm + (size_t)i * W;
    int c = 0;
    for (int k = lane; k < W; k += 32) c += __popc(row[k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) rcnt[i] = c;
}

// Column j's bit position in the mask (as k_sigma_cols_f reads it).
template <int CW, int VW>
__device__ __forceinline__ void bit_of_col(int j, int& sl, int& q, int& L) {
    sl = j / CW;
    const int o = j - sl * CW;
    L = (o % (32 * VW)) / VW;
    q = (o / (32 * VW)) * VW + (o % VW);
}

// ccnt[c][j] = set bits of column j among the rows of chunk c
template <int CW, int VW, int LC>
__global__ void k_cs_col_counts(const uint32_t* bm, int n, int m, int nslabs, int* ccnt) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (j >= m) return;
    int sl, q, L;
    bit_of_col<CW, VW>(j, sl, q, L);
    const int rows_per = (n + gridDim.y - 1) / gridDim.y;
    const int i0 = c * rows_per, i1 = min(n, i0 + rows_per);
    int cnt = 0;
    int i = i0;
    for (; i + 8 <= i1; i += 8) {
        uint32_t w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) w[u] = bm[((size_t)(i + u) * nslabs + sl) * LC + q];
#pragma unroll
        for (int u = 0; u < 8; ++u) cnt += (w[u] >> L) & 1u;
    }
    for (; i < i1; ++i) cnt += (bm[((size_t)i * nslabs + sl) * LC + q] >> L) & 1u;
    ccnt[(size_t)c * m + j] = cnt;
}

// Per column: the chunk counts become exclusive offsets within the column,
// ccol_j = the column's total.
__global__ void k_cs_col_offsets(int m, int chunks, int* ccnt, int* ccol) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    int run = 0;
    for (int c = 0; c < chunks; ++c) {
        const int v = ccnt[(size_t)c * m + j];
        ccnt[(size_t)c * m + j] = run;
        run += v;
    }
    ccol[j] = run;
}

// One block: ptr = exclusive scan of cnt (len + 1 entries, 64-bit running
// sums; *total = the sum). Entries past 2^31 - 1 are not used: the caller
// takes the index lists only for totals far below that.
__device__ void block_excl_scan(const int* cnt, int len, int* ptr, long long* total) {
    __shared__ long long wsum[32];
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = (len + T - 1) / T;
    const int b = min(len, t * per), e = min(len, b + per);
    long long s = 0;
    for (int k = b; k < e; ++k) s += cnt[k];
    // inclusive scan of the per-thread sums
    long long inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        long long v = lane < (T >> 5) ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        wsum[lane] = v;
    }
    __syncthreads();
    long long run = inc - s + (w > 0 ? wsum[w - 1] : 0);
    for (int k = b; k < e; ++k) {
        ptr[k] = (int)run;
        run += cnt[k];
    }
    if (t == T - 1) {
        ptr[len] = (int)run;
        *total = run;
    }
    __syncthreads();
}

__global__ void k_cs_scan(const int* rcnt, int n, int* rowptr, const int* ccol, int m,
                          int* colptr, long long* nnz) {
    block_excl_scan(rcnt, n, rowptr, nnz);
    block_excl_scan(ccol, m, colptr, nnz + 1);
}

// colidx: the columns of row i's set bits in mask order (one warp per row)
template <int CW, int VW, int LC>
__global__ void k_cs_row_fill(const uint32_t* bm, int n, int nslabs, const int* rowptr,
                              int* colidx) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    const int W = nslabs * LC;
    const uint32_t* row = bm + (size_t)i * W;
    int base = rowptr[i];
    for (int k0 = 0; k0 < W; k0 += 32) {
        const int k = k0 + lane;
        uint32_t w = k < W ? row[k] : 0u;
        const int c = __popc(w);
        int inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        int pos = base + inc - c;
        const int sl = k / LC, q = k - (k / LC) * LC;
        while (w) {
            const int L = __ffs(w) - 1;
            w &= w - 1;
            colidx[pos++] = bit_col<CW, VW, LC>(sl, q, L);
        }
        base += __shfl_sync(0xffffffffu, inc, 31);
    }
}

// rowidx: the rows of column j's set bits in increasing order; chunk c of
// the rows starts at colptr_j + ccnt[c][j].
template <int CW, int VW, int LC>
__global__ void k_cs_col_fill(const uint32_t* bm, int n, int m, int nslabs, const int* colptr,
                              const int* ccnt, int* rowidx) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (j >= m) return;
    int sl, q, L;
    bit_of_col<CW, VW>(j, sl, q, L);
    const int rows_per = (n + gridDim.y - 1) / gridDim.y;
    const int i0 = c * rows_per, i1 = min(n, i0 + rows_per);
    int pos = colptr[j] + ccnt[(size_t)c * m + j];
    int i = i0;
    for (; i + 8 <= i1; i += 8) {
        uint32_t w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) w[u] = bm[((size_t)(i + u) * nslabs + sl) * LC + q];
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if ((w[u] >> L) & 1u) rowidx[pos++] = i + u;
    }
    for (; i < i1; ++i)
        if ((bm[((size_t)i * nslabs + sl) * LC + q] >> L) & 1u) rowidx[pos++] = i;
}

// ---- the whole Schur CG of hess_cg in one thread-block cluster ----
// The cluster's CTAs split the rows and the columns into contiguous ranges.
// Phases are separated by the hardware cluster barrier (release / acquire).
// A dot product is summed per CTA by one warp from the threads' values in
// shared memory, then over the CTAs from their totals read through
// distributed shared memory, always in the same order, so every thread of
// every CTA holds the same bits and takes the same branch. FP64 issues at
// a small fraction of the FP32 rate on this part, so the kernel keeps its
// FP64 instructions few: one row and one column per thread at the sizes
// the list path serves, the reductions on one warp, and 1 / (h1 + mu)
// formed once per solve.
constexpr int kCgT = 256;

struct ClusterCgArgs {
    int n, m, cg_max;
    double mu, tol;
    const int *rowptr, *colidx, *colptr, *rowidx;
    const double *h1, *h2, *w, *z;  // w: the first n entries of the right-hand side, z: the rest
    double *dinv, *t, *p, *r, *y, *x, *r1;
    float2 *t2, *p2;                // mixed engine: FP32 (hi, lo) pairs the products read
    int* it_out;
};

__device__ __forceinline__ void cluster_barrier() {
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n\t"
        "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_nctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ double ld_dsmem(const double* p, unsigned rank) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
    return v;
}
// Butterfly sum: each step adds the same two values in both lanes of a
// pair, so all 32 lanes end with the same bits.
__device__ __forceinline__ double warp_allsum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// Shared memory of one reduction slot. Two slots alternate (p'q, r'r): a
// CTA may write a slot again only after a cluster barrier that follows
// every remote read of it.
struct CgSlot {
    double cta;    // this CTA's total, read by the others
    double total;  // the cluster total, for this CTA's threads
};
// Sum over the cluster of one value per thread; contains a cluster barrier,
// which also publishes every global store made before the call.
__device__ __forceinline__ double cluster_sum(double v, double* vals, CgSlot& slot, unsigned nc) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    vals[threadIdx.x] = v;
    __syncthreads();
    if (warp == 0) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < kCgT / 32; ++k) s += vals[k * 32 + lane];
        s = warp_allsum_d(s);
        if (lane == 0) slot.cta = s;
    }
    cluster_barrier();
    if (warp == 0) {
        double c = lane < (int)nc ? ld_dsmem(&slot.cta, lane) : 0.0;
        c = warp_allsum_d(c);
        if (lane == 0) slot.total = c;
    }
    __syncthreads();
    return slot.total;
}

// sum_{k in [ptr[i], ptr[i+1])} v[idx[k]]; v written by other CTAs of the
// cluster, so it is read from L2 (ld.global.cg).
template <bool MIXED>
__device__ __forceinline__ double list_sum(const int* ptr, const int* idx, int i, const double* v,
                                           const float2* v2) {
    const int b = __ldg(ptr + i), e = __ldg(ptr + i + 1);
    int k = b;
    if (MIXED) {
        float s = 0.f, er = 0.f;
        for (; k + 4 <= e; k += 4) {
            float2 u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) u[q] = __ldcg(v2 + __ldg(idx + k + q));
#pragma unroll
            for (int q = 0; q < 4; ++q) cadd(s, er, u[q]);
        }
        for (; k < e; ++k) cadd(s, er, __ldcg(v2 + __ldg(idx + k)));
        return (double)s + (double)er;
    } else {
        double acc = 0.0;
        for (; k + 4 <= e; k += 4) {
            double u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) u[q] = __ldcg(v + __ldg(idx + k + q));
#pragma unroll
            for (int q = 0; q < 4; ++q) acc += u[q];
        }
        for (; k < e; ++k) acc += __ldcg(v + __ldg(idx + k));
        return acc;
    }
}

// hess_cg (qrot_cg.cpp:9-50) for Delta = h2 o x + mu x - sigma' ((sigma x) /
// (h1 + mu)): v = w / (h1 + mu), zy = z - sigma' v, identity-preconditioned
// CG on zy from 0 to ||r||^2 < tol^2 ||zy||^2 or cg_max steps, then
// r1 = (w - sigma x) / (h1 + mu). The divisions by h1 + mu are products with
// its reciprocal (within an ulp of the quotient).
template <bool MIXED>
__global__ void __launch_bounds__(kCgT, 1) k_schur_cg_cluster(ClusterCgArgs a) {
    __shared__ double vals[kCgT];
    __shared__ CgSlot slot_pq, slot_rr;
    const unsigned nc = cluster_nctarank(), rk = cluster_ctarank();
    const int tid = threadIdx.x;
    const int n = a.n, m = a.m;
    const double mu = a.mu;
    const int r0 = (int)((long long)rk * n / nc), r1 = (int)((long long)(rk + 1) * n / nc);
    const int c0 = (int)((long long)rk * m / nc), c1 = (int)((long long)(rk + 1) * m / nc);
    // every CTA of the cluster is running before any shared memory is read remotely
    cluster_barrier();
    for (int i = r0 + tid; i < r1; i += kCgT) {
        const double di = 1.0 / (a.h1[i] + mu);
        a.dinv[i] = di;
        const double v = a.w[i] * di;
        if (MIXED) a.t2[i] = split_f2(v);
        else a.t[i] = v;
    }
    cluster_barrier();
    double part = 0.0;
    for (int j = c0 + tid; j < c1; j += kCgT) {
        const double zy = a.z[j] - list_sum<MIXED>(a.colptr, a.rowidx, j, a.t, a.t2);
        a.x[j] = 0.0;
        a.r[j] = zy;
        a.p[j] = zy;
        if (MIXED) a.p2[j] = split_f2(zy);
        part += zy * zy;
    }
    double rr = cluster_sum(part, vals, slot_rr, nc);
    const double thresh2 = fmax(a.tol * a.tol * rr, 2.2250738585072014e-308);
    bool done = rr == 0.0 || rr < thresh2;
    int it = 0;
    while (!done) {
        for (int i = r0 + tid; i < r1; i += kCgT) {
            const double v = list_sum<MIXED>(a.rowptr, a.colidx, i, a.p, a.p2) * a.dinv[i];
            if (MIXED) a.t2[i] = split_f2(v);
            else a.t[i] = v;
        }
        cluster_barrier();
        part = 0.0;
        for (int j = c0 + tid; j < c1; j += kCgT) {
            const double u = list_sum<MIXED>(a.colptr, a.rowidx, j, a.t, a.t2);
            const double pj = a.p[j];
            const double yj = a.h2[j] * pj + mu * pj - u;
            a.y[j] = yj;
            part += pj * yj;
        }
        const double alpha = rr / cluster_sum(part, vals, slot_pq, nc);
        part = 0.0;
        for (int j = c0 + tid; j < c1; j += kCgT) {
            a.x[j] += alpha * a.p[j];
            const double rj = a.r[j] - alpha * a.y[j];
            a.r[j] = rj;
            part += rj * rj;
        }
        const double rn = cluster_sum(part, vals, slot_rr, nc);
        ++it;
        if (rn < thresh2 || it >= a.cg_max || !(rn == rn)) {
            done = true;
        } else {
            const double beta = rn / rr;
            rr = rn;
            for (int j = c0 + tid; j < c1; j += kCgT) {
                const double pj = a.r[j] + beta * a.p[j];
                a.p[j] = pj;
                if (MIXED) a.p2[j] = split_f2(pj);
            }
            cluster_barrier();
        }
    }
    // r1 = (w - sigma x) / (h1 + mu); the mixed products read x's pairs
    if (MIXED)
        for (int j = c0 + tid; j < c1; j += kCgT) a.p2[j] = split_f2(a.x[j]);
    cluster_barrier();
    for (int i = r0 + tid; i < r1; i += kCgT)
        a.r1[i] = (a.w[i] - list_sum<MIXED>(a.rowptr, a.colidx, i, a.x, a.p2)) * a.dinv[i];
    if (rk == 0 && tid == 0) *a.it_out = it;
    // no CTA leaves while another may still read its shared memory
    cluster_barrier();
}

// ---- the same CG with its vectors exchanged through distributed shared
// memory ----
// Every CTA keeps a full copy of the two vectors the sigma products gather
// from (t = (sigma p) / (h1 + mu) over the rows, p over the columns; FP32
// (hi, lo) pairs in the mixed engine, FP64 otherwise) in its own shared
// memory. After forming its slice, a CTA sends the slice to every other
// CTA with one bulk copy each (cp.async.bulk shared::cta -> shared::cluster)
// and CTA totals of the dot products go out with st.async; each transfer
// completes on an mbarrier of the receiving CTA. No step then needs a
// cluster barrier or a global-memory round trip, and every gather reads
// local shared memory. One buffer per vector suffices: a CTA can send step
// k + 1's slice only after every CTA has sent its step-k dot-product
// totals, that is, after every CTA has finished reading the step-k copy.
// Waits are bounded (the library's wait limit); a CTA that gives up sets
// *err and leaves the loop, the others then give up in turn, and all meet
// at the final cluster barrier.
constexpr int kDsT = 256;
constexpr int kDsMaxBytes = 200 * 1024;  // both vectors' copies

struct DsmCgArgs {
    ClusterCgArgs c;
    long long polls;
    int* err;
};

__device__ __forceinline__ uint32_t mapa_u32(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void bulk_s2cluster(uint32_t dst, uint32_t src, uint32_t bytes,
                                               uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "r"(src), "r"(bytes), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void st_async_f64(uint32_t dst, double v, uint32_t bar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];"
                 ::"r"(dst), "l"(__double_as_longlong(v)), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void st_async_f2(uint32_t dst, float2 v, uint32_t bar) {
    const unsigned long long bits =
        ((unsigned long long)__float_as_uint(v.y) << 32) | __float_as_uint(v.x);
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];"
                 ::"r"(dst), "l"(bits), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t* bar, uint32_t parity, long long polls) {
    const uint32_t a = sm100::smem_u32(bar);
    for (long long s = 0; s < polls; ++s) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity), "r"(100000u)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Slice of CTA k (of nc) over len entries: starts at an even index, so that
// its copy starts on a 16-byte boundary; its copy covers an even number of
// 8-byte entries (the last slice may carry one unused pad entry).
struct DsSlices {
    int per;
    __device__ DsSlices(int len, unsigned nc) : per(((len + 2 * (int)nc - 1) / (2 * (int)nc)) * 2) {}
    __device__ int begin(int len, unsigned k) const { return min(len, (int)k * per); }
    __device__ int end(int len, unsigned k) const { return min(len, (int)k * per + per); }
    __device__ uint32_t bytes(int len, unsigned k) const {
        const int c = end(len, k) - begin(len, k);
        return (uint32_t)(((c + 1) & ~1) * 8);
    }
};

// sum_{k in [ptr[i], ptr[i+1])} v[idx[k]] with v in this CTA's shared memory
template <bool MIXED>
__device__ __forceinline__ double list_sum_s(const int* ptr, const int* idx, int i,
                                             const void* vs) {
    const int b = __ldg(ptr + i), e = __ldg(ptr + i + 1);
    int k = b;
    if (MIXED) {
        const float2* v2 = static_cast<const float2*>(vs);
        float s = 0.f, er = 0.f;
        for (; k + 4 <= e; k += 4) {
            float2 u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) u[q] = v2[__ldg(idx + k + q)];
#pragma unroll
            for (int q = 0; q < 4; ++q) cadd(s, er, u[q]);
        }
        for (; k < e; ++k) cadd(s, er, v2[__ldg(idx + k)]);
        return (double)s + (double)er;
    } else {
        const double* v = static_cast<const double*>(vs);
        double acc = 0.0;
        for (; k + 4 <= e; k += 4) {
            double u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) u[q] = v[__ldg(idx + k + q)];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc += u[q];
        }
        for (; k < e; ++k) acc += v[__ldg(idx + k)];
        return acc;
    }
}
template <bool MIXED>
__device__ __forceinline__ void put_slot(void* vs, int j, double v) {
    if (MIXED) static_cast<float2*>(vs)[j] = split_f2(v);
    else static_cast<double*>(vs)[j] = v;
}

struct DsShared {
    double vals[kDsT];
    double red[2][16];  // CTA totals of p'q and r'r, by sending CTA
    double bc[2];       // the cluster total and the quotient formed from it
    uint64_t bar[4];    // arrivals of t, p, the p'q totals, the r'r totals
    int abort;
};

template <bool MIXED>
__global__ void __launch_bounds__(kDsT, 1) k_schur_cg_dsm(DsmCgArgs da) {
    extern __shared__ __align__(16) unsigned char ds_dyn[];
    __shared__ DsShared sh;
    const ClusterCgArgs& a = da.c;
    const unsigned nc = cluster_nctarank(), rk = cluster_ctarank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n = a.n, m = a.m;
    const double mu = a.mu;
    void* Ts = ds_dyn;                                        // (n + 1) & ~1 slots
    void* Ps = ds_dyn + (size_t)((n + 1) & ~1) * 8;           // (m + 1) & ~1 slots
    const DsSlices rs(n, nc), cs(m, nc);
    const int r0 = rs.begin(n, rk), r1 = rs.end(n, rk);
    const int c0 = cs.begin(m, rk), c1 = cs.end(m, rk);
    uint32_t t_in = 0, p_in = 0;
    for (unsigned k = 0; k < nc; ++k)
        if (k != rk) {
            t_in += rs.bytes(n, k);
            p_in += cs.bytes(m, k);
        }
    if (tid == 0) {
        for (int q = 0; q < 4; ++q) sm100::mbar_init(&sh.bar[q], 1);
        sm100::fence_mbar_init();
        sh.abort = 0;
    }
    uint32_t ph = 0u;  // bit q: the parity barrier q waits for next
    // barriers initialised and every CTA running before any remote access
    cluster_barrier();

    // Sends this CTA's slice [b, b + bytes) of vector buffer `vs` to every
    // other CTA, then waits for theirs (barrier q).
    auto exchange = [&](void* vs, int b, uint32_t bytes, uint32_t in_bytes, int q) -> bool {
        sm100::fence_proxy_async_smem();
        __syncthreads();
        if (warp == 0) {
            const uint32_t src = sm100::smem_u32(vs) + (uint32_t)b * 8u;
            const uint32_t bar = sm100::smem_u32(&sh.bar[q]);
            if (bytes > 0 && lane < (int)nc && lane != (int)rk)
                bulk_s2cluster(mapa_u32(src, lane), src, bytes, mapa_u32(bar, lane));
            if (lane == 0) {
                sm100::mbar_arrive_expect_tx(&sh.bar[q], in_bytes);
                if (!mbar_wait_cluster(&sh.bar[q], (ph >> q) & 1u, da.polls)) {
                    sh.abort = 1;
                    atomicExch(da.err, 1);
                }
            }
        }
        __syncthreads();
        ph ^= 1u << q;
        return sh.abort == 0;
    };
    // Cluster total of one value per thread; bc[1] = num / total (or, with
    // inv, total / num), formed once.
    auto all_sum = [&](double v, int slot, double num, bool inv) -> bool {
        const int q = 2 + slot;
        sh.vals[tid] = v;
        __syncthreads();
        if (warp == 0) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < kDsT / 32; ++k) s += sh.vals[k * 32 + lane];
            s = warp_allsum_d(s);
            const uint32_t bar = sm100::smem_u32(&sh.bar[q]);
            if (lane == (int)rk) sh.red[slot][rk] = s;
            else if (lane < (int)nc)
                st_async_f64(mapa_u32(sm100::smem_u32(&sh.red[slot][rk]), lane), s,
                             mapa_u32(bar, lane));
            if (lane == 0) {
                sm100::mbar_arrive_expect_tx(&sh.bar[q], (nc - 1) * 8u);
                if (!mbar_wait_cluster(&sh.bar[q], (ph >> q) & 1u, da.polls)) {
                    sh.abort = 1;
                    atomicExch(da.err, 1);
                }
            }
            __syncwarp();
            double c = lane < (int)nc ? sh.red[slot][lane] : 0.0;
            c = warp_allsum_d(c);
            if (lane == 0) {
                sh.bc[0] = c;
                sh.bc[1] = inv ? c / num : num / c;
            }
        }
        __syncthreads();
        ph ^= 1u << q;
        return sh.abort == 0;
    };

    bool ok = true;
    for (int i = r0 + tid; i < r1; i += kDsT) {
        const double di = 1.0 / (a.h1[i] + mu);
        a.dinv[i] = di;
        put_slot<MIXED>(Ts, i, a.w[i] * di);
    }
    ok = exchange(Ts, r0, rs.bytes(n, rk), t_in, 0);
    double part = 0.0;
    if (ok) {
        for (int j = c0 + tid; j < c1; j += kDsT) {
            const double zy = a.z[j] - list_sum_s<MIXED>(a.colptr, a.rowidx, j, Ts);
            a.x[j] = 0.0;
            a.r[j] = zy;
            a.p[j] = zy;
            put_slot<MIXED>(Ps, j, zy);
            part += zy * zy;
        }
        ok = all_sum(part, 1, 1.0, false);
    }
    double rr = sh.bc[0];
    if (ok) ok = exchange(Ps, c0, cs.bytes(m, rk), p_in, 1);
    const double thresh2 = fmax(a.tol * a.tol * rr, 2.2250738585072014e-308);
    bool done = rr == 0.0 || rr < thresh2;
    int it = 0;
    while (ok && !done) {
        for (int i = r0 + tid; i < r1; i += kDsT)
            put_slot<MIXED>(Ts, i, list_sum_s<MIXED>(a.rowptr, a.colidx, i, Ps) * a.dinv[i]);
        if (!(ok = exchange(Ts, r0, rs.bytes(n, rk), t_in, 0))) break;
        part = 0.0;
        for (int j = c0 + tid; j < c1; j += kDsT) {
            const double u = list_sum_s<MIXED>(a.colptr, a.rowidx, j, Ts);
            const double pj = a.p[j];
            const double yj = a.h2[j] * pj + mu * pj - u;
            a.y[j] = yj;
            part += pj * yj;
        }
        if (!(ok = all_sum(part, 0, rr, false))) break;
        const double alpha = sh.bc[1];
        part = 0.0;
        for (int j = c0 + tid; j < c1; j += kDsT) {
            a.x[j] += alpha * a.p[j];
            const double rj = a.r[j] - alpha * a.y[j];
            a.r[j] = rj;
            part += rj * rj;
        }
        if (!(ok = all_sum(part, 1, rr, true))) break;
        const double rn = sh.bc[0];
        ++it;
        if (rn < thresh2 || it >= a.cg_max || !(rn == rn)) {
            done = true;
        } else {
            const double beta = sh.bc[1];  // rn / rr
            rr = rn;
            for (int j = c0 + tid; j < c1; j += kDsT) {
                const double pj = a.r[j] + beta * a.p[j];
                a.p[j] = pj;
                put_slot<MIXED>(Ps, j, pj);
            }
            ok = exchange(Ps, c0, cs.bytes(m, rk), p_in, 1);
        }
    }
    if (ok) {
        // r1 = (w - sigma x) / (h1 + mu)
        for (int j = c0 + tid; j < c1; j += kDsT) put_slot<MIXED>(Ps, j, a.x[j]);
        ok = exchange(Ps, c0, cs.bytes(m, rk), p_in, 1);
        if (ok)
            for (int i = r0 + tid; i < r1; i += kDsT)
                a.r1[i] = (a.w[i] - list_sum_s<MIXED>(a.rowptr, a.colidx, i, Ps)) * a.dinv[i];
    }
    if (rk == 0 && tid == 0) *a.it_out = it;
    // no CTA leaves while another may still write to or read its shared memory
    cluster_barrier();
}

// ---- the mixed engine's cluster CG in double-word FP32 ----
// On this part an FP64 add or FMA has a latency of about 63 cycles, a
// division about 550 and an FP64 <-> FP32 conversion about 64 (measured),
// and every CG step is a chain of them: the reductions, alpha and beta, the
// splits the products read. The mixed engine therefore runs the CG itself in
// double-word FP32 (hi + lo, about 48 bits): x, r, p, y, the reductions,
// alpha and beta. FP64 is left to the per-solve setup and the results. The
// right-hand side is scaled by a power of two that brings ||zy|| near 1
// (exact, so the iterates are the same numbers scaled), which keeps every
// quantity far inside FP32's exponent range. Same exchange scheme as
// k_schur_cg_dsm.
struct DwCgArgs {
    DsmCgArgs d;
    int idx_cap;  // ints of dynamic shared memory after the vectors for the
                  // CTA's index-list slices (each slice fits when >= nnz)
};

struct DwShared {
    float2 vals[kDsT];
    float2 red[2][16];
    float2 bc[2];
    double vals_d[kDsT / 32];
    double red_d[16];
    double bc_d;
    uint64_t bar[4];
    int abort;
};

__device__ __forceinline__ float2 shfl_xor_f2(float2 v, int o) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ float2 warp_allsum_dw(float2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dw_add(v, shfl_xor_f2(v, o));
    return v;
}
// Compensated sum of v[idx[k]], k in [b, e) (idx and v in shared memory, or
// idx in global memory when the CTA's slice did not fit).
__device__ __forceinline__ float2 gather_sum(const int* idx, int b, int e, const float2* v) {
    float s = 0.f, er = 0.f;
    int k = b;
    for (; k + 2 <= e; k += 2) {
        const float2 u0 = v[idx[k]], u1 = v[idx[k + 1]];
        cadd(s, er, u0);
        cadd(s, er, u1);
    }
    if (k < e) cadd(s, er, v[idx[k]]);
    return dw_norm(s, er);
}

// K: rows and columns per thread (the CTA's slices hold at most K * kDsT).
// Each thread keeps its rows' and columns' CG state in registers and the
// CTA's slices of the index lists sit in shared memory: after a
// cluster-scope acquire, global loads no longer hit L1, and the L2 round
// trips of re-reading them every step (about 700 cycles per dependent load)
// had made each phase cost 1-2 thousand cycles.
template <int K>
__global__ void __launch_bounds__(kDsT, 1) k_schur_cg_dw(DwCgArgs wa) {
    extern __shared__ __align__(16) unsigned char ds_dyn[];
    __shared__ DwShared sh;
    const ClusterCgArgs& a = wa.d.c;
    const unsigned nc = cluster_nctarank(), rk = cluster_ctarank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n = a.n, m = a.m;
    const double mu = a.mu;
    float2* Ts = reinterpret_cast<float2*>(ds_dyn);
    float2* Ps = reinterpret_cast<float2*>(ds_dyn + (size_t)((n + 1) & ~1) * 8);
    int* sidx = reinterpret_cast<int*>(ds_dyn + (size_t)(((n + 1) & ~1) + ((m + 1) & ~1)) * 8);
    const DsSlices rs(n, nc), cs(m, nc);
    const int r0 = rs.begin(n, rk), r1 = rs.end(n, rk);
    const int c0 = cs.begin(m, rk), c1 = cs.end(m, rk);
    uint32_t t_in = 0, p_in = 0;
    for (unsigned k = 0; k < nc; ++k)
        if (k != rk) {
            t_in += rs.bytes(n, k);
            p_in += cs.bytes(m, k);
        }
    if (tid == 0) {
        for (int q = 0; q < 4; ++q) sm100::mbar_init(&sh.bar[q], 1);
        sm100::fence_mbar_init();
        sh.abort = 0;
    }
    // this CTA's slices of the index lists, in shared memory when they fit
    const int rbase = __ldg(a.rowptr + r0), rcount = __ldg(a.rowptr + r1) - rbase;
    const int cbase = __ldg(a.colptr + c0), ccount = __ldg(a.colptr + c1) - cbase;
    const bool fit = rcount + ccount <= wa.idx_cap;
    const int* ridx = fit ? sidx : a.colidx + rbase;
    const int* cidx = fit ? sidx + rcount : a.rowidx + cbase;
    if (fit) {
        for (int k = tid; k < rcount; k += kDsT) sidx[k] = __ldg(a.colidx + rbase + k);
        for (int k = tid; k < ccount; k += kDsT) sidx[rcount + k] = __ldg(a.rowidx + cbase + k);
    }
    // per-thread rows i = r0 + tid + u kDsT and columns j = c0 + tid + u kDsT
    int rb[K], re[K], cb[K], ce[K];
    float2 dinv[K], hm[K], x[K], r[K], p[K], y[K];
#pragma unroll
    for (int u = 0; u < K; ++u) {
        const int i = r0 + tid + u * kDsT, j = c0 + tid + u * kDsT;
        rb[u] = re[u] = cb[u] = ce[u] = 0;
        if (i < r1) {
            rb[u] = __ldg(a.rowptr + i) - rbase;
            re[u] = __ldg(a.rowptr + i + 1) - rbase;
        }
        if (j < c1) {
            cb[u] = __ldg(a.colptr + j) - cbase;
            ce[u] = __ldg(a.colptr + j + 1) - cbase;
        }
        dinv[u] = hm[u] = x[u] = r[u] = p[u] = y[u] = make_float2(0.f, 0.f);
    }
    uint32_t ph = 0u;  // bit q: the parity barrier q waits for next
    // barriers initialised, slices staged, every CTA running
    cluster_barrier();

    auto wait_bar = [&](int q) {
        if (!mbar_wait_cluster(&sh.bar[q], (ph >> q) & 1u, wa.d.polls)) {
            sh.abort = 1;
            atomicExch(wa.d.err, 1);
        }
    };
    auto exchange = [&](float2* vs, int b, uint32_t bytes, uint32_t in_bytes, int q) -> bool {
        sm100::fence_proxy_async_smem();
        __syncthreads();
        if (warp == 0) {
            const uint32_t src = sm100::smem_u32(vs) + (uint32_t)b * 8u;
            const uint32_t bar = sm100::smem_u32(&sh.bar[q]);
            if (bytes > 0 && lane < (int)nc && lane != (int)rk)
                bulk_s2cluster(mapa_u32(src, lane), src, bytes, mapa_u32(bar, lane));
            if (lane == 0) {
                sm100::mbar_arrive_expect_tx(&sh.bar[q], in_bytes);
                wait_bar(q);
            }
        }
        __syncthreads();
        ph ^= 1u << q;
        return sh.abort == 0;
    };
    // Cluster total of one double-word value per thread (slot 0: p'q,
    // slot 1: r'r); bc[1] = num / total, or total / num with inv.
    auto all_sum = [&](float2 v, int slot, float2 num, bool inv) -> bool {
        const int q = 2 + slot;
        sh.vals[tid] = v;
        __syncthreads();
        if (warp == 0) {
            float2 u[kDsT / 32];
#pragma unroll
            for (int k = 0; k < kDsT / 32; ++k) u[k] = sh.vals[k * 32 + lane];
#pragma unroll
            for (int w = kDsT / 64; w > 0; w >>= 1)
#pragma unroll
                for (int k = 0; k < w; ++k) u[k] = dw_add(u[k], u[k + w]);
            const float2 s = warp_allsum_dw(u[0]);
            const uint32_t bar = sm100::smem_u32(&sh.bar[q]);
            if (lane == (int)rk) sh.red[slot][rk] = s;
            else if (lane < (int)nc)
                st_async_f2(mapa_u32(sm100::smem_u32(&sh.red[slot][rk]), lane), s,
                            mapa_u32(bar, lane));
            if (lane == 0) {
                sm100::mbar_arrive_expect_tx(&sh.bar[q], (nc - 1) * 8u);
                wait_bar(q);
            }
            __syncwarp();
            float2 c = lane < (int)nc ? sh.red[slot][lane] : make_float2(0.f, 0.f);
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) c = dw_add(c, shfl_xor_f2(c, o));
            if (lane == 0) {
                sh.bc[0] = c;
                sh.bc[1] = inv ? dw_div(c, num) : dw_div(num, c);
            }
        }
        __syncthreads();
        ph ^= 1u << q;
        return sh.abort == 0;
    };
    // exchange and all_sum (slot 1, total / num) in one round: the slice's
    // bulk copies and the CTA total's st.async complete on barrier 1.
    auto exchange_sum = [&](float2* vs, int b, uint32_t bytes, uint32_t in_bytes, float2 v,
                            float2 num) -> bool {
        sh.vals[tid] = v;
        sm100::fence_proxy_async_smem();
        __syncthreads();
        if (warp == 0) {
            float2 u[kDsT / 32];
#pragma unroll
            for (int k = 0; k < kDsT / 32; ++k) u[k] = sh.vals[k * 32 + lane];
#pragma unroll
            for (int w = kDsT / 64; w > 0; w >>= 1)
#pragma unroll
                for (int k = 0; k < w; ++k) u[k] = dw_add(u[k], u[k + w]);
            const float2 t = warp_allsum_dw(u[0]);
            const uint32_t src = sm100::smem_u32(vs) + (uint32_t)b * 8u;
            const uint32_t bar = sm100::smem_u32(&sh.bar[1]);
            if (lane == (int)rk) {
                sh.red[1][rk] = t;
            } else if (lane < (int)nc) {
                const uint32_t rbar = mapa_u32(bar, lane);
                if (bytes > 0) bulk_s2cluster(mapa_u32(src, lane), src, bytes, rbar);
                st_async_f2(mapa_u32(sm100::smem_u32(&sh.red[1][rk]), lane), t, rbar);
            }
            if (lane == 0) {
                sm100::mbar_arrive_expect_tx(&sh.bar[1], in_bytes + (nc - 1) * 8u);
                wait_bar(1);
            }
            __syncwarp();
            float2 c = lane < (int)nc ? sh.red[1][lane] : make_float2(0.f, 0.f);
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) c = dw_add(c, shfl_xor_f2(c, o));
            if (lane == 0) {
                sh.bc[0] = c;
                sh.bc[1] = dw_div(c, num);
            }
        }
        __syncthreads();
        ph ^= 1u << 1;
        return sh.abort == 0;
    };

    // ---- setup in FP64: v = w / (h1 + mu), zy = z - sigma' v, ||zy||^2 ----
#pragma unroll
    for (int u = 0; u < K; ++u) {
        const int i = r0 + tid + u * kDsT;
        if (i < r1) {
            const double di = 1.0 / (a.h1[i] + mu);
            a.dinv[i] = di;
            dinv[u] = dw_from(di);
            Ts[i] = dw_from(a.w[i] * di);
        }
    }
    bool ok = exchange(Ts, r0, rs.bytes(n, rk), t_in, 0);
    double zy[K];
    double part_d = 0.0;
#pragma unroll
    for (int u = 0; u < K; ++u) {
        const int j = c0 + tid + u * kDsT;
        zy[u] = 0.0;
        if (ok && j < c1) {
            zy[u] = a.z[j] - dw_to(gather_sum(cidx, cb[u], ce[u], Ts));
            part_d += zy[u] * zy[u];
        }
    }
    // FP64 total of ||zy||^2 (once per solve), by the same exchange of CTA totals
    double rr0 = 0.0;
    if (ok) {
        const double ws = warp_allsum_d(part_d);
        if (lane == 0) sh.vals_d[warp] = ws;
        __syncthreads();
        if (warp == 0) {
            double s0 = lane < kDsT / 32 ? sh.vals_d[lane] : 0.0;
            s0 = warp_allsum_d(s0);
            const uint32_t bar = sm100::smem_u32(&sh.bar[3]);
            if (lane == (int)rk) sh.red_d[rk] = s0;
            else if (lane < (int)nc)
                st_async_f64(mapa_u32(sm100::smem_u32(&sh.red_d[rk]), lane), s0,
                             mapa_u32(bar, lane));
            if (lane == 0) {
                sm100::mbar_arrive_expect_tx(&sh.bar[3], (nc - 1) * 8u);
                wait_bar(3);
            }
            __syncwarp();
            double c = lane < (int)nc ? sh.red_d[lane] : 0.0;
            c = warp_allsum_d(c);
            if (lane == 0) sh.bc_d = c;
        }
        __syncthreads();
        ph ^= 1u << 3;
        ok = sh.abort == 0;
        rr0 = sh.bc_d;
    }
    // scale 2^-e with ||zy|| = f 2^e, f in [0.5, 1)
    int ex = 0;
    if (rr0 > 0.0) frexp(sqrt(rr0), &ex);
    const double scale = ldexp(1.0, -ex);
    const double thr = fmax(a.tol * a.tol * rr0, 2.2250738585072014e-308);
    const float2 thresh = dw_from(thr * scale * scale);
    float2 rr = dw_from(rr0 * scale * scale);
    bool done = !(rr0 > 0.0) || rr0 < thr;
#pragma unroll
    for (int u = 0; u < K; ++u) {
        const int j = c0 + tid + u * kDsT;
        if (ok && j < c1) {
            r[u] = p[u] = dw_from(zy[u] * scale);
            hm[u] = dw_from(a.h2[j] + mu);
            Ps[j] = p[u];
        }
    }
    // Ps carries r: the rows' products are sigma p = sigma r + beta sigma p_prev
    // (s, per row; p_0 = r_0), which lets r travel with the r'r totals
    if (ok) ok = exchange(Ps, c0, cs.bytes(m, rk), p_in, 1);
    float2 sp[K], beta = make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < K; ++u) sp[u] = make_float2(0.f, 0.f);
    int it = 0;
    while (ok && !done) {
#pragma unroll
        for (int u = 0; u < K; ++u) {
            const int i = r0 + tid + u * kDsT;
            if (i < r1) {
                sp[u] = dw_add(gather_sum(ridx, rb[u], re[u], Ps), dw_mul(beta, sp[u]));
                Ts[i] = dw_mul(sp[u], dinv[u]);
            }
        }
        if (!(ok = exchange(Ts, r0, rs.bytes(n, rk), t_in, 0))) break;
        float2 part = make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < K; ++u) {
            const int j = c0 + tid + u * kDsT;
            if (j < c1) {
                p[u] = dw_add(r[u], dw_mul(beta, p[u]));
                y[u] = dw_sub(dw_mul(hm[u], p[u]), gather_sum(cidx, cb[u], ce[u], Ts));
                part = dw_add(part, dw_mul(p[u], y[u]));
            }
        }
        if (!(ok = all_sum(part, 0, rr, false))) break;
        const float2 alpha = sh.bc[1];
        part = make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < K; ++u) {
            const int j = c0 + tid + u * kDsT;
            if (j < c1) {
                x[u] = dw_add(x[u], dw_mul(alpha, p[u]));
                r[u] = dw_sub(r[u], dw_mul(alpha, y[u]));
                Ps[j] = r[u];
                part = dw_add(part, dw_mul(r[u], r[u]));
            }
        }
        if (!(ok = exchange_sum(Ps, c0, cs.bytes(m, rk), p_in, part, rr))) break;
        const float2 rn = sh.bc[0];
        ++it;
        if (dw_lt(rn, thresh) || it >= a.cg_max || !(rn.x == rn.x)) {
            done = true;
        } else {
            beta = sh.bc[1];  // rn / rr
            rr = rn;
        }
    }
    if (ok) {
        // x (unscaled, FP64) and r1 = (w - sigma x) / (h1 + mu)
        const double inv_scale = ldexp(1.0, ex);
#pragma unroll
        for (int u = 0; u < K; ++u) {
            const int j = c0 + tid + u * kDsT;
            if (j < c1) {
                a.x[j] = dw_to(x[u]) * inv_scale;
                Ps[j] = x[u];
            }
        }
        ok = exchange(Ps, c0, cs.bytes(m, rk), p_in, 1);
        if (ok) {
#pragma unroll
            for (int u = 0; u < K; ++u) {
                const int i = r0 + tid + u * kDsT;
                if (i < r1)
                    a.r1[i] = (a.w[i] - dw_to(gather_sum(ridx, rb[u], re[u], Ps)) * inv_scale) *
                              a.dinv[i];
            }
        }
    }
    if (rk == 0 && tid == 0) *a.it_out = it;
    // no CTA leaves while another may still read its shared memory
    cluster_barrier();
}

__global__ void k_time(unsigned long long t0, unsigned long long* out) {
    *out = globaltimer_ns() - t0;
}

}  // namespace

// --------------------------------------------------------------- engine --
// Scalars of a primal value: the two P3 totals and the merged primal
// scalars of the state.
struct PrimRaw {
    double tot[2];
    double prim[5];
};

class QrotEngine {
public:
    QrotEngine(regot_dproblem* P, double reg, double tau, cudaStream_t st)
        : P_(P), st_(st), ops_(P, reg, st), n_(P->n), m_(P->m), reg_(reg), tau_(tau),
          mixed_(P->prec == REGOT_PREC_MIXED) {
        const int N = n_ + m_;
        gamma_.alloc(N, st);
        grad_.alloc(N, st);
        h_.alloc(N, st);
        vec_.alloc(6 * (size_t)std::max(n_, m_), st);
        // block partials of the merge kernels: up to 6 per 64-thread block,
        // 3 per (32, 8) block of 32 rows or columns
        parts_.alloc(std::max(6 * (size_t)cdiv(N, kVT), 3 * (size_t)(cdiv(n_, 32) + cdiv(m_, 32))),
                     st);
        state_.alloc(1, st);
        QState z{};
        h2d(state_.get(), &z, sizeof(z), st);
        scal_.alloc(8, st);
        const PassShape sh = ops_.buf().shape;
        bm_words_ = (size_t)n_ * sh.nslabs * (mixed_ ? Geo<float>::LC : Geo<double>::LC);
        sum_a_ = P->sum_a;
    }

    int n() const { return n_; }
    int m() const { return m_; }
    ErotOps& ops() { return ops_; }
    cudaStream_t stream() const { return st_; }
    double* gamma() { return gamma_.get(); }
    double* grad() { return grad_.get(); }
    QState* state() { return state_.get(); }

    // obj and grad at the device vector gamma (n + m). With `mask`, also the
    // sigma bitmask and h = (h1, h2) of compute_D_hess.
    double eval(const double* gamma, double* grad, bool mask) {
        const PassShape sh = ops_.buf().shape;
        if (mask && !bm_.get()) bm_.alloc(bm_words_, st_);
        ops_.maxabs(gamma, n_ + m_, nullptr, 0, &state_.get()->maxabs);
        PassParams p = ops_.base_params();
        p.ra = gamma;
        p.cb = gamma + n_;
        p.grid = &state_.get()->maxabs;
        p.bitmask = mask ? bm_.get() : nullptr;
        ops_.pass(mask ? OP_Q_GRADMASK : OP_Q_GRAD, p);
        const int blocks = pass_blocks(mask ? OP_Q_GRADMASK : OP_Q_GRAD, mixed_, n_, m_);
        k_sum_totals<<<1, 256, 0, st_>>>(ops_.buf().totpart.get(), blocks, scal_.get());
        const int g = cdiv(n_, 32) + cdiv(m_, 32);
        if (mixed_)
            k_q_grad<float><<<g, dim3(32, 8), 0, st_>>>(
                (const float*)ops_.buf().rowpart.get(), sh.nslabs,
                (const float*)ops_.buf().colpart.get(), sh.nrb, n_, m_, mask ? 1 : 0, gamma,
                P_->a, P_->b, reg_, grad, h_.get(), h_.get() + n_, parts_.get(), state_.get());
        else
            k_q_grad<double><<<g, dim3(32, 8), 0, st_>>>(
                (const double*)ops_.buf().rowpart.get(), sh.nslabs,
                (const double*)ops_.buf().colpart.get(), sh.nrb, n_, m_, mask ? 1 : 0, gamma,
                P_->a, P_->b, reg_, grad, h_.get(), h_.get() + n_, parts_.get(), state_.get());
        count_launch(2);
        REGOT_CHECK_LAUNCH();
        double sq = 0.0;
        QState hs;
        d2h(&sq, scal_.get(), sizeof(double), st_);
        d2h(&hs, state_.get(), sizeof(hs), st_);
        sync(st_);
        ++passes_;
        // qrot_problem.cpp:226-253 (tau terms: 342-351)
        double obj = 0.5 * sq - reg_ * hs.dot_ab;
        if (tau_ > 0.0) {
            const double d = hs.sum_a - hs.sum_b;
            obj += 0.5 * tau_ * d * d;
            tau_grad_ = tau_ * d;
        }
        return obj;
    }
    double tau_grad() const { return tau_grad_; }

    // Line-search trial at x = xp + step d: writes grad f(x) (without the tau
    // term) to grad() and returns f(x) - f(xp) without the tau and linear
    // terms' cancellation: with w_ij = d_i + d_j (row and column parts of d),
    // 0.5 sum (D(x)^2 - D(xp)^2) = step sum w D(xp) + sum rem, where
    // rem = 0.5 (Dn^2 - D^2) - step w D >= 0 is accumulated per entry by
    // the pass. sum w D(xp) is the quadratic part of grad f(xp)' d, so the
    // change is step * (grad f(xp)' d) + sum rem (+ the exact tau term, added
    // by the caller). Also returns sum D(x)^2 in *sq.
    double eval_step(const double* xp, const double* d, double step, double* sq) {
        const PassShape sh = ops_.buf().shape;
        ops_.maxabs(xp, n_ + m_, nullptr, 0, &state_.get()->maxabs);
        PassParams p = ops_.base_params();
        p.ra = xp;
        p.cb = xp + n_;
        p.rd = d;
        p.cd = d + n_;
        p.steps[0] = step;
        p.nsteps = 1;
        p.grid = &state_.get()->maxabs;
        ops_.pass(OP_Q_GRADLS, p);
        const int blocks = pass_blocks(OP_Q_GRADLS, mixed_, n_, m_);
        k_sum_totals<<<1, 256, 0, st_>>>(ops_.buf().totpart.get(), blocks, scal_.get());
        k_sum_totals<<<1, 256, 0, st_>>>(ops_.buf().totpart.get() + blocks, blocks,
                                          scal_.get() + 1);
        const int g = cdiv(n_, 32) + cdiv(m_, 32);
        if (mixed_)
            k_q_grad<float><<<g, dim3(32, 8), 0, st_>>>(
                (const float*)ops_.buf().rowpart.get(), sh.nslabs,
                (const float*)ops_.buf().colpart.get(), sh.nrb, n_, m_, 0, gamma_.get(), P_->a,
                P_->b, reg_, grad_.get(), h_.get(), h_.get() + n_, parts_.get(), state_.get());
        else
            k_q_grad<double><<<g, dim3(32, 8), 0, st_>>>(
                (const double*)ops_.buf().rowpart.get(), sh.nslabs,
                (const double*)ops_.buf().colpart.get(), sh.nrb, n_, m_, 0, gamma_.get(), P_->a,
                P_->b, reg_, grad_.get(), h_.get(), h_.get() + n_, parts_.get(), state_.get());
        count_launch(3);
        REGOT_CHECK_LAUNCH();
        double tot[2];
        d2h(tot, scal_.get(), 2 * sizeof(double), st_);
        sync(st_);
        ++passes_;
        *sq = tot[0];
        return tot[1];
    }

    // primal_val (qrot_problem.cpp:10-24)
    // Primal value (primal_val with approx_proj, qrot_problem.cpp): three
    // passes and their merges, enqueued; the scalars land in *raw when the
    // stream gets there. The three passes share one split of gamma (grid:
    // max |gamma|, from `grid` when the caller has it); the merge kernels
    // write the next passes' row and column operands into the split arrays
    // in place.
    void primal_launch(const double* gamma, const double* grid, PrimRaw* raw) {
        const PassShape sh = ops_.buf().shape;
        double* xr = vec_.get();
        double* yc = xr + std::max(n_, m_);
        double* fc = yc + std::max(n_, m_);
        if (!grid) {
            ops_.maxabs(gamma, n_ + m_, nullptr, 0, &state_.get()->maxabs);
            grid = &state_.get()->maxabs;
        }
        PassParams p = ops_.base_params();
        p.ra = gamma;
        p.cb = gamma + n_;
        p.grid = grid;
        const int gn = cdiv(n_, kVT), gm = cdiv(m_, kVT);
        float4* rs = mixed_ ? ops_.rsplit_mut() : nullptr;
        float4* cs = mixed_ ? ops_.csplit_mut() : nullptr;
        ops_.pass(OP_Q_P1, p);
        if (mixed_)
            k_prim1<float><<<gn, kVT, 0, st_>>>((const float*)ops_.buf().rowpart.get(), sh.nslabs,
                                                 n_, P_->a, reg_, xr, rs);
        else
            k_prim1<double><<<gn, kVT, 0, st_>>>((const double*)ops_.buf().rowpart.get(),
                                                  sh.nslabs, n_, P_->a, reg_, xr, nullptr);
        p.rx = xr;
        ops_.pass_presplit(OP_Q_P2, p);
        if (mixed_)
            k_prim2<float><<<gm, kVT, 0, st_>>>((const float*)ops_.buf().colpart.get(), sh.nrb,
                                                 m_, P_->b, reg_, yc, fc, parts_.get(),
                                                 state_.get(), cs);
        else
            k_prim2<double><<<gm, kVT, 0, st_>>>((const double*)ops_.buf().colpart.get(), sh.nrb,
                                                  m_, P_->b, reg_, yc, fc, parts_.get(),
                                                  state_.get(), nullptr);
        p.cx = yc;
        p.cx2 = fc;
        ops_.pass_presplit(OP_Q_P3, p);
        const int blocks = pass_blocks(OP_Q_P3, mixed_, n_, m_);
        k_sum_totals<<<1, 256, 0, st_>>>(ops_.buf().totpart.get(), blocks, scal_.get());
        k_sum_totals<<<1, 256, 0, st_>>>(ops_.buf().totpart.get() + blocks, blocks,
                                          scal_.get() + 1);
        if (mixed_)
            k_prim3<float><<<gn, kVT, 0, st_>>>((const float*)ops_.buf().rowpart.get(), sh.nslabs,
                                                 n_, P_->a, xr, reg_, parts_.get(), state_.get());
        else
            k_prim3<double><<<gn, kVT, 0, st_>>>((const double*)ops_.buf().rowpart.get(),
                                                  sh.nslabs, n_, P_->a, xr, reg_, parts_.get(),
                                                  state_.get());
        count_launch(5);
        REGOT_CHECK_LAUNCH();
        passes_ += 3;
        // the scalars the value is formed from, copied to *raw (page-locked:
        // the copies are asynchronous)
        d2h(raw->tot, scal_.get(), 2 * sizeof(double), st_);
        d2h(raw->prim, state_.get()->prim, 5 * sizeof(double), st_);
    }
    // The primal value from the scalars of primal_launch (once they landed).
    double primal_value(const PrimRaw& r) const {
        const double RM = r.tot[0] / reg_;            // <R, M>, R_ij = P_ij x_i y_j
        const double RR = r.tot[1] / (reg_ * reg_);  // ||R||^2
        const double f2 = r.prim[0], S = r.prim[1], eCc = r.prim[2], xeB = r.prim[3],
                     e2 = r.prim[4];
        // res = R + e f' / S (approx_proj.h:22-24)
        const double val_M = RM + eCc / S;
        const double sqn = RR + 2.0 * xeB / S + e2 * f2 / (S * S);
        return val_M + 0.5 * reg_ * sqn;
    }
    double primal(const double* gamma, const double* grid = nullptr) {
        PrimRaw raw;
        primal_launch(gamma, grid, &raw);
        sync(st_);
        return primal_value(raw);
    }

    // beta = optimal_beta(alpha) (qrot_problem.cpp:397-404), into beta (device).
    void optimal_beta(const double* alpha, double* beta) { root_solve(false, alpha, beta); }

    // alpha = optimal_alpha(beta) (qrot_problem.cpp:409-419), into alpha
    // (device): Newton's method from above on each row's piecewise-linear
    // equation, one OP_Q_ROWROOT pass per round, as optimal_beta for columns.
    void optimal_alpha(const double* beta, double* alpha) { root_solve(true, beta, alpha); }

    // The Newton rounds run as a device-side loop: a graph whose only node
    // is a conditional WHILE node, its body one root pass, the update of
    // the roots and k_root_loop (cached per pair of vectors). One launch and
    // one read of the state per call, where a round trip per round made the
    // solvers that call these every iteration latency-bound.
    void root_solve(bool rows, const double* other, double* x) {
        const int len = rows ? n_ : m_;
        k_root_init<<<cdiv(len, kVT), kVT, 0, st_>>>(len, x, vec_.get());
        k_root_begin<<<1, 1, 0, st_>>>(state_.get());
        count_launch(2);
        RootGraph& g = root_graph(rows, other, x);
        REGOT_CUDA(cudaGraphLaunch(g.exec, st_));
        QState hs;
        d2h(&hs, state_.get(), sizeof(hs), st_);
        sync(st_);
        count_launch(g.kernels * hs.root_rounds);
        passes_ += hs.root_rounds;
        if (hs.root_unconverged)
            throw Error(REGOT_ERR_NUMERIC,
                        rows ? "optimal_alpha did not converge" : "optimal_beta did not converge");
    }
    // sigma x (n) with optional division by (h1 + mu); mu from *mu_dev when
    // given. With x2 (the FP32 pairs of x; mixed engine) the compensated
    // FP32 kernel runs and out2, if given, receives the pairs of the result.
    void sigma_rows(const double* x, const float2* x2, double mu, bool divide, double* out,
                    float2* out2, const int* done, const double* mu_dev = nullptr) {
        const int warps = 8;
        if (mixed_ && x2)
            k_sigma_rows_f<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<cdiv(n_, warps), warps * 32, 0, st_>>>(bm_.get(), n_, m_, nslabs(), x2,
                                                          h_.get(), mu, mu_dev, divide ? 1 : 0,
                                                          out, out2, done);
        else if (mixed_)
            k_sigma_rows<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<cdiv(n_, warps), warps * 32, 0, st_>>>(bm_.get(), n_, m_, nslabs(), x, h_.get(),
                                                          mu, mu_dev, divide ? 1 : 0, out, done);
        else
            k_sigma_rows<Geo<double>::CW, Geo<double>::VW, Geo<double>::LC>
                <<<cdiv(n_, warps), warps * 32, 0, st_>>>(bm_.get(), n_, m_, nslabs(), x, h_.get(),
                                                          mu, mu_dev, divide ? 1 : 0, out, done);
        count_launch();
    }
    // partial sums of sigma' y over kColChunks row chunks (y2 as for x2 above)
    void sigma_cols(const double* y, const float2* y2, double* partial, const int* done) {
        dim3 grid(cdiv(m_, 128), kColChunks);
        if (mixed_ && y2)
            k_sigma_cols_f<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<grid, 128, 0, st_>>>(bm_.get(), n_, m_, nslabs(), y2, partial, done);
        else if (mixed_)
            k_sigma_cols<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<grid, 128, 0, st_>>>(bm_.get(), n_, m_, nslabs(), y, partial, done);
        else
            k_sigma_cols<Geo<double>::CW, Geo<double>::VW, Geo<double>::LC>
                <<<grid, 128, 0, st_>>>(bm_.get(), n_, m_, nslabs(), y, partial, done);
        count_launch();
    }
    bool mixed() const { return mixed_; }
    // the sigma bitmask of the last eval(..., mask = true) and its slabs per row
    const uint32_t* bitmask() const { return bm_.get(); }
    int slabs() { return nslabs(); }
    const double* h1() const { return h_.get(); }
    const double* h2() const { return h_.get() + n_; }
    double* parts() { return parts_.get(); }
    long long passes() const { return passes_; }
    void add_passes(long long k) { passes_ += k; }

    void plan(const double* gamma, double* out) {
        ops_.maxabs(gamma, n_ + m_, nullptr, 0, &state_.get()->maxabs);
        PassParams p = ops_.base_params();
        p.ra = gamma;
        p.cb = gamma + n_;
        p.grid = &state_.get()->maxabs;
        p.out = out;
        ops_.pass(OP_Q_PLAN, p);
    }

private:
    int nslabs() { return ops_.buf().shape.nslabs; }
    regot_dproblem* P_;
    cudaStream_t st_;
    ErotOps ops_;
    int n_, m_;
    double reg_, tau_;
    bool mixed_;
    DBuf<double> gamma_, grad_, h_, vec_, parts_, scal_;
    DBuf<QState> state_;
    DBuf<uint32_t> bm_;
    size_t bm_words_ = 0;
    double sum_a_ = 0.0;
    double tau_grad_ = 0.0;
    long long passes_ = 0;

    struct RootGraph {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        long long kernels = 0;
    };
    std::map<std::tuple<bool, const double*, double*>, RootGraph> root_graphs_;

    RootGraph& root_graph(bool rows, const double* other, double* x) {
        RootGraph& g = root_graphs_[std::make_tuple(rows, other, x)];
        if (g.exec) return g;
        const int len = rows ? n_ : m_;
        REGOT_CUDA(cudaGraphCreate(&g.graph, 0));
        cudaGraphConditionalHandle h;
        REGOT_CUDA(cudaGraphConditionalHandleCreate(&h, g.graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        REGOT_CUDA(cudaGraphAddNode(&node, g.graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        long long* saved = g_launch_counter;
        g.kernels = 0;
        g_launch_counter = &g.kernels;
        REGOT_CUDA(cudaStreamBeginCaptureToGraph(st_, body, nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal));
        try {
            PassParams p = ops_.base_params();
            p.ra = rows ? x : other;
            p.cb = rows ? other : x;
            const PassShape sh = ops_.buf().shape;
            // the root passes read ra and cb in FP64: no split of them
            ops_.pass_presplit(rows ? OP_Q_ROWROOT : OP_Q_COLROOT, p);
            if (rows)
                k_rowroot_update<<<cdiv(n_, kVT), kVT, 0, st_>>>(
                    (const double*)ops_.buf().rowpart.get(), sh.nslabs, n_, P_->a, reg_, x,
                    vec_.get(), state_.get());
            else
                k_root_update<<<cdiv(m_, 32), dim3(32, 8), 0, st_>>>(
                    (const double*)ops_.buf().colpart.get(), sh.nrb, m_, P_->b, reg_, x,
                    vec_.get(), state_.get());
            k_root_loop<<<1, 1, 0, st_>>>(state_.get(), len + 2, h);
            count_launch(2);
        } catch (...) {
            cudaGraph_t tmp = nullptr;
            cudaStreamEndCapture(st_, &tmp);
            g_launch_counter = saved;
            throw;
        }
        REGOT_CUDA(cudaStreamEndCapture(st_, &body));
        g_launch_counter = saved;
        REGOT_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
        return g;
    }

public:
    ~QrotEngine() {
        for (auto& kv : root_graphs_) {
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
            if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
        }
    }
};

namespace {

// Result from the device dual d_gamma and host histories; the plan is made by
// plan_fn(dst) into an n x m FP64 destination (device or host view).
template <typename F>
void finish_qrot_with(QrotEngine& E, const double* d_gamma, const std::vector<double>& hobj,
                      const std::vector<double>& hmar, const std::vector<double>& htime,
                      const std::vector<double>& hprim, int niter, const regot_opts& o,
                      regot_result* res, F&& plan_fn) {
    cudaStream_t st = E.stream();
    const int n = E.n(), m = E.m();
    const int L = (int)hobj.size();
    res->niter = niter;
    res->hist_len = L;
    res->passes = E.passes();
    d2h(res->dual, d_gamma, (size_t)(n + m) * sizeof(double), st);
    sync(st);
    if (res->obj_vals) std::memcpy(res->obj_vals, hobj.data(), L * sizeof(double));
    if (res->mar_errs) std::memcpy(res->mar_errs, hmar.data(), L * sizeof(double));
    if (res->run_times) std::memcpy(res->run_times, htime.data(), L * sizeof(double));
    if (res->prim_vals) std::memcpy(res->prim_vals, hprim.data(), L * sizeof(double));
    if (o.plan && res->plan) emit_plan(res->plan, o.plan_mem, (size_t)n * m, st, plan_fn);
    E.ops().check_err();
}

void finish_qrot(QrotEngine& E, const double* d_gamma, const std::vector<double>& hobj,
                 const std::vector<double>& hmar, const std::vector<double>& htime,
                 const std::vector<double>& hprim, int niter, const regot_opts& o,
                 regot_result* res) {
    finish_qrot_with(E, d_gamma, hobj, hmar, htime, hprim, niter, o, res,
                     [&](double* dst) { E.plan(d_gamma, dst); });
}

// Wall clock in milliseconds on the device (globaltimer), like the
// reference's std::chrono Timer (timer.h:9-54).
class DevClock {
public:
    explicit DevClock(cudaStream_t st) : st_(st), buf_(1, st) {}
    double now_ms() {
        unsigned long long t = 0;
        k_time<<<1, 1, 0, st_>>>(0ULL, buf_.get());
        count_launch();
        d2h(&t, buf_.get(), sizeof(t), st_);
        sync(st_);
        return (double)t * 1e-6;
    }

private:
    cudaStream_t st_;
    DBuf<unsigned long long> buf_;
};

void init_gamma(QrotEngine& E, const regot_opts& o, std::vector<double>& gamma) {
    const int n = E.n(), m = E.m();
    gamma.assign(n + m, 0.0);
    if (o.x0 && o.x0_len == n + m) {
        std::copy(o.x0, o.x0 + n + m, gamma.begin());
        h2d(E.gamma(), gamma.data(), (n + m) * sizeof(double), E.stream());
        return;
    }
    // alpha = 0, beta = optimal_beta(0) (qrot_lbfgs_dual.cpp:111-117)
    DBuf<double> zero(n, E.stream());
    zero.zero();
    E.optimal_beta(zero.get(), E.gamma() + n);
    REGOT_CUDA(cudaMemsetAsync(E.gamma(), 0, n * sizeof(double), E.stream()));
    d2h(gamma.data(), E.gamma(), (n + m) * sizeof(double), E.stream());
    sync(E.stream());
}

}  // namespace

namespace {

// ---- L-BFGS with device vectors (qrot_lbfgs_dual) ----
// LBFGS++'s minimize and Nocedal-Wright line search (restated in lbfgs.h)
// keep their control flow on the host, and every vector of the algorithm
// stays on the device: the iterates x, the gradients, the direction, and the
// ring of m = 6 correction pairs (s, y). A line-search trial is the trial
// point, one dense pass and one merge kernel. The merge's last block writes
// every scalar the host needs into one record: the objective terms, g'd,
// |g|^2, |x|^2 and the 34 products of the trial's correction pair
// (s = x - xp, y = g - gp, staged on the device) with the stored pairs and
// with g. One small copy and one synchronisation per trial. The two-loop
// recursion (BFGSMat::apply_Hv, src/LBFGSpp/LBFGSpp/BFGSMat.h:276-302) then
// runs on the host on scalars: with the Gram matrices S'Y and Y'Y of the
// stored pairs, kept up to date as pairs are added, every alpha_j and beta_j
// follows from scalar recurrences, and the next direction is one linear
// combination of g and the pairs, formed by one kernel from coefficients
// the host copies to the device. (A single device thread ran this scalar
// chain an order of magnitude slower: FP64 latency on this part.)
constexpr int kLbM = 6;          // LBFGSParam m (Param.h:168-182)
// Blocks of two warps: the vector kernels are FP64 work on n + m entries,
// which this part issues at a small fraction of its FP32 rate per SM, so
// they are spread over as many SMs as the vector length allows.
constexpr int kLbBlock = 64;
constexpr int kLbPairSums = 5 * kLbM + 4;
constexpr int kLbBufs = 3;       // rotating iterate / gradient buffers

struct LbScal {
    double sq;   // sum D^2 at the trial point
    double rem;  // sum of the second-order remainders of the change from xp
    double dab;  // x'(a, b)
    double dg;   // grad(x)' drt
    double gg;   // |grad(x)|^2
    double xx;   // |x|^2
    double dg0;  // grad' drt of a new direction
    double pad;
    // products of the trial's pair (s, y) with the stored pairs (s_k, y_k)
    // and the trial gradient g: [5k..5k+4] = s'y_k, s_k'y, y'y_k, s_k'g,
    // y_k'g for ring slot k; then s'y, y'y, s'g, y'g
    double prod[kLbPairSums];
};

// Direction coefficients and buffer maps, written by the host.
struct LbCoef {
    double cv, cy[kLbM], cs[kLbM];  // direction = cv g + sum_k cy[k] y_k + cs[k] s_k
    int ncorr;
    int phys[kLbM];      // ring slot -> physical pair buffer
    int stage[kLbBufs];  // iterate buffer -> physical staging pair buffer
};

// Warp sums of K values per lane with about 1.1 K FP64 adds per lane instead
// of 5 K: three halving exchanges (at lane distances 16, 8, 4 each lane
// keeps half of its values and adds the partner's copy of that half), then
// two plain exchanges on the K8 = ceil(K / 8) values left. Lane l then holds
// the totals of values off(l) .. off(l) + K8 - 1 (off from lane bits 4, 3,
// 2); put(k, total) is called once per value, from the lanes with bits 1
// and 0 clear.
template <int K, typename Put>
__device__ __forceinline__ void warp_sums_multi(const double (&v)[K], int lane, Put put) {
    constexpr int K8 = (K + 7) / 8;
    constexpr int KP = 8 * K8;
    double a[KP];
#pragma unroll
    for (int k = 0; k < KP; ++k) a[k] = k < K ? v[k] : 0.0;
    int off = 0;
#pragma unroll
    for (int lev = 0; lev < 3; ++lev) {
        const int o = 16 >> lev;
        const int H = KP >> (lev + 1);  // values kept after this level
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < H; ++i) {
            const double mine = upper ? a[i + H] : a[i];
            const double send = upper ? a[i] : a[i + H];
            a[i] = mine + __shfl_xor_sync(0xffffffffu, send, o);
        }
        off += upper ? H : 0;
    }
#pragma unroll
    for (int i = 0; i < K8; ++i) {
        a[i] += __shfl_xor_sync(0xffffffffu, a[i], 2);
        a[i] += __shfl_xor_sync(0xffffffffu, a[i], 1);
    }
    if ((lane & 3) == 0) {
#pragma unroll
        for (int i = 0; i < K8; ++i)
            if (off + i < K) put(off + i, a[i]);
    }
}

// Block sums of K values, then the last block to arrive adds the block sums
// in block order: true in every thread of that block, with the totals in
// s_out (shared, K entries). The last block's sums are spread over its
// warps (value k to warp k mod warps, blocks to lanes) with every load of a
// lane issued before its adds, so that they take a few memory latencies
// instead of one per block.
template <int K>
__device__ bool lb_reduce(const double (&v)[K], double* parts, unsigned* counter, double* s_out) {
    constexpr int NW = kLbBlock / 32;
    constexpr int PER = (K + NW - 1) / NW;
    __shared__ double s_red[K][NW];
    __shared__ int s_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    warp_sums_multi<K>(v, lane, [&](int k, double x) { s_red[k][warp] = x; });
    __syncthreads();
    if (tid < K) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += s_red[tid][w];
        parts[(size_t)blockIdx.x * K + tid] = s;
        __threadfence();
    }
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double acc[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) acc[q] = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) {
        double x[PER];
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int k = warp + q * NW;
            x[q] = k < K ? __ldcg(&parts[(size_t)b * K + k]) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < PER; ++q) acc[q] += x[q];
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int k = warp + q * NW;
        const double t = warp_sum_d(acc[q]);
        if (lane == 0 && k < K) s_out[k] = t;
    }
    if (tid == 0) *counter = 0u;
    __syncthreads();
    return true;
}

__global__ void k_lb_axpy(const double* __restrict__ xp, const double* __restrict__ d,
                          double step, int N, double* __restrict__ x) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < N) x[t] = xp[t] + step * d[t];
}

// Gradient of the last dense pass at the trial point x (rows, then
// columns: D1 - reg a, D'1 - reg b), the trial's correction pair s = x - xp,
// y = g - gp into the staging buffer of x's buffer, the record's dot
// products (with the pair products), the pass totals (sum D^2 and, with
// nt == 2, the remainder sum) and max |x| beside x's buffer. Without gp
// (the first evaluation) no pair is formed.
template <typename Acc>
__global__ void __launch_bounds__(kLbBlock) k_lb_merge(
    const Acc* __restrict__ rp, int nslabs, const Acc* __restrict__ cp, int nrb, int n, int m,
    const double* __restrict__ totpart, int nblocks, int nt, const double* __restrict__ x,
    const double* __restrict__ drt, const double* __restrict__ a, const double* __restrict__ b,
    double reg, double* __restrict__ grad, const double* __restrict__ xp,
    const double* __restrict__ gp, double* __restrict__ pairs, const LbCoef* __restrict__ cf,
    int xbuf, double* parts, unsigned* counter, LbScal* out,
    unsigned long long* __restrict__ mxparts, double* __restrict__ xmax) {
    constexpr int K = 4 + kLbPairSums;
    const int N = n + m;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = 0.0;
    unsigned long long xbits = 0ULL;
    if (t < N) {
        double g, w;
        if (t < n) {
            g = merge_strided(rp + t, nslabs, (size_t)n) - reg * a[t];
            w = a[t];
        } else {
            const int j = t - n;
            g = merge_strided(cp + j, nrb, (size_t)m) - reg * b[j];
            w = b[j];
        }
        grad[t] = g;
        const double xt = x[t];
        xbits = abs_bits(xt);
        v[0] = xt * w;
        v[1] = g * drt[t];
        v[2] = g * g;
        v[3] = xt * xt;
        if (gp) {
        const double sn = xt - xp[t], yn = g - gp[t];
        const int stg = cf->stage[xbuf];
        pairs[(size_t)(2 * stg) * N + t] = sn;
        pairs[(size_t)(2 * stg + 1) * N + t] = yn;
        int ph[kLbM];
#pragma unroll
        for (int k = 0; k < kLbM; ++k) ph[k] = cf->phys[k];
#pragma unroll
        for (int k = 0; k < kLbM; ++k) {
            const double sk = pairs[(size_t)(2 * ph[k]) * N + t];
            const double yk = pairs[(size_t)(2 * ph[k] + 1) * N + t];
            v[4 + 5 * k + 0] = sn * yk;
            v[4 + 5 * k + 1] = sk * yn;
            v[4 + 5 * k + 2] = yn * yk;
            v[4 + 5 * k + 3] = sk * g;
            v[4 + 5 * k + 4] = yk * g;
        }
        v[4 + 5 * kLbM + 0] = sn * yn;
        v[4 + 5 * kLbM + 1] = yn * yn;
        v[4 + 5 * kLbM + 2] = sn * g;
        v[4 + 5 * kLbM + 3] = yn * g;
        }
    }
    // max |x| of this block (bit patterns of non-negative doubles order like
    // the values), for the split grid of a line search from x
    {
        __shared__ unsigned long long s_wmax[kLbBlock / 32];
        const unsigned long long wm = warp_max_u64(xbits);
        if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = wm;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long bm = 0ULL;
            for (int w = 0; w < kLbBlock / 32; ++w) bm = s_wmax[w] > bm ? s_wmax[w] : bm;
            mxparts[blockIdx.x] = bm;
        }
    }
    __shared__ double s_sum[K];
    if (!lb_reduce<K>(v, parts, counter, s_sum)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        unsigned long long bm = 0ULL;
        for (unsigned b = lane; b < gridDim.x; b += 32) {
            const unsigned long long q = __ldcg(&mxparts[b]);
            bm = q > bm ? q : bm;
        }
        bm = warp_max_u64(bm);
        if (lane == 0) *xmax = __longlong_as_double((long long)bm);
    }
    __shared__ double s_tot[2];
    if (warp < 2) {
        double s = 0.0;
        if (warp < nt) {
#pragma unroll 4
            for (int k = lane; k < nblocks; k += 32) s += totpart[(size_t)warp * nblocks + k];
        }
        s = warp_sum_d(s);
        if (lane == 0) s_tot[warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        out->sq = s_tot[0];
        out->rem = nt > 1 ? s_tot[1] : 0.0;
        out->dab = s_sum[0];
        out->dg = s_sum[1];
        out->gg = s_sum[2];
        out->xx = s_sum[3];
    }
    if (threadIdx.x < kLbPairSums) out->prod[threadIdx.x] = s_sum[4 + threadIdx.x];
}

// drt = cv g + sum_k cy[k] y_k + cs[k] s_k over the stored pairs, and g'drt.
// With xt given, also the first trial point xt = xp + step drt.
__global__ void __launch_bounds__(kLbBlock) k_lb_dir(const double* __restrict__ g,
                                                     const double* __restrict__ pairs, int N,
                                                     double* __restrict__ drt, double* parts,
                                                     unsigned* counter,
                                                     const LbCoef* __restrict__ cf, LbScal* out,
                                                     const double* __restrict__ xp, double step,
                                                     double* __restrict__ xt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (t < N) {
        const double gt = g[t];
        double d = cf->cv * gt;
        const int ncorr = cf->ncorr;
        int ph[kLbM];
        double cy[kLbM], cs[kLbM];
#pragma unroll
        for (int k = 0; k < kLbM; ++k) {
            ph[k] = cf->phys[k];
            cy[k] = cf->cy[k];
            cs[k] = cf->cs[k];
        }
#pragma unroll
        for (int k = 0; k < kLbM; ++k) {
            if (k < ncorr) {
                d += cy[k] * pairs[(size_t)(2 * ph[k] + 1) * N + t];
                d += cs[k] * pairs[(size_t)(2 * ph[k]) * N + t];
            }
        }
        drt[t] = d;
        if (xt) xt[t] = xp[t] + step * d;
        v[0] = gt * d;
    }
    __shared__ double r[1];
    if (!lb_reduce<1>(v, parts, counter, r)) return;
    if (threadIdx.x == 0) out->dg0 = r[0];
}

// Page-locked host copy of one T (the per-trial record, the coefficients).
template <typename T>
struct Pinned {
    T* p = nullptr;
    Pinned() { REGOT_CUDA(cudaHostAlloc((void**)&p, sizeof(T), cudaHostAllocDefault)); }
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
    Pinned(const Pinned&) = delete;
    Pinned& operator=(const Pinned&) = delete;
};

// The host side of the pair ring: Gram matrices of the stored pairs in ring
// slots (logical order of BFGSMat), s'y of each, theta, and the maps of the
// device buffers.
struct LbHost {
    int ncorr = 0;
    int ptr = kLbM;  // BFGSMat::reset: m_ptr = m
    int phys[kLbM];
    int stage[kLbBufs];
    double theta = 1.0;
    double ys[kLbM] = {};
    double SY[kLbM][kLbM] = {};  // s_i' y_j
    double YY[kLbM][kLbM] = {};
    LbHost() {
        for (int k = 0; k < kLbM; ++k) phys[k] = k;
        for (int b = 0; b < kLbBufs; ++b) stage[b] = kLbM + b;
    }
};

// BFGSMat::add_correction (BFGSMat.h:81-100, as LBFGS.h:160-161 calls it:
// the pair is stored when s'y > eps y'y) for the pair staged with iterate
// buffer xb, whose products with the ring and the new gradient are r (the
// record's prod), then the coefficients of apply_Hv(g, -1)
// (BFGSMat.h:276-302) by the scalar two-loop recursion: newest to oldest
// alpha_j = s_j'res / ys_j, res -= alpha_j y_j; res /= theta; oldest to
// newest beta_j = y_j'res / ys_j, res += (alpha_j - beta_j) s_j, with res
// kept as coefficients of g and the pairs.
void lb_host_step(LbHost& H, const double* r, int xb, LbCoef& c) {
    constexpr int M = kLbM;
    double SV[M], YV[M];
    for (int k = 0; k < M; ++k) {
        SV[k] = r[5 * k + 3];
        YV[k] = r[5 * k + 4];
    }
    const double ys = r[5 * M + 0], yy = r[5 * M + 1];
    if (ys > DBL_EPSILON * yy) {
        const int loc = H.ptr % M;
        for (int k = 0; k < M; ++k) {
            if (k == loc) continue;
            H.SY[loc][k] = r[5 * k + 0];
            H.SY[k][loc] = r[5 * k + 1];
            H.YY[loc][k] = r[5 * k + 2];
            H.YY[k][loc] = r[5 * k + 2];
        }
        H.SY[loc][loc] = ys;
        H.YY[loc][loc] = yy;
        H.ys[loc] = ys;
        H.theta = yy / ys;
        std::swap(H.phys[loc], H.stage[xb]);
        SV[loc] = r[5 * M + 2];
        YV[loc] = r[5 * M + 3];
        if (H.ncorr < M) H.ncorr++;
        H.ptr = loc + 1;
    }
    const double av = -1.0, theta = H.theta;
    const int ncorr = H.ncorr;
    double alpha[M] = {}, beta[M] = {};
    int order[M];
    int j = H.ptr % M;
    for (int i = 0; i < ncorr; ++i) {
        j = (j + M - 1) % M;
        double sres = av * SV[j];
        for (int q = 0; q < i; ++q) sres -= alpha[order[q]] * H.SY[j][order[q]];
        alpha[j] = sres / H.ys[j];
        order[i] = j;
    }
    for (int i = 0; i < ncorr; ++i) {
        // j is the oldest pair here, then moves to newer ones
        double yres = av * YV[j];
        for (int q = 0; q < ncorr; ++q) yres -= alpha[order[q]] * H.YY[j][order[q]];
        yres /= theta;
        for (int q = 0; q < i; ++q) {
            const int k = (j + M - 1 - q) % M;  // the pairs already added, newest first
            yres += (alpha[k] - beta[k]) * H.SY[k][j];
        }
        beta[j] = yres / H.ys[j];
        j = (j + 1) % M;
    }
    c.cv = av / theta;
    for (int k = 0; k < M; ++k) {
        c.cy[k] = 0.0;
        c.cs[k] = 0.0;
    }
    for (int q = 0; q < ncorr; ++q) {
        const int k = order[q];
        c.cy[k] = -alpha[k] / theta;
        c.cs[k] = alpha[k] - beta[k];
    }
    c.ncorr = ncorr;
    for (int k = 0; k < M; ++k) c.phys[k] = H.phys[k];
    for (int b = 0; b < kLbBufs; ++b) c.stage[b] = H.stage[b];
}

__global__ void k_lb_stamp(unsigned long long* out) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *out = t;
}

}  // namespace

// qrot_lbfgs_dual_internal (qrot_lbfgs_dual.cpp:81-126) with LBFGSSolver::
// minimize (LBFGS.h:79-175) and LineSearchNocedalWright::LineSearch
// (LineSearchNocedalWright.h:85-280) on device vectors; tau = 0.
void qrot_lbfgs_dual_device(regot_ctx* ctx, regot_dproblem* P, double reg, double tol,
                            int max_iter, const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    QrotEngine E(P, reg, 0.0, st);
    ErotOps& ops = E.ops();
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    const PassShape sh = ops.buf().shape;
    constexpr int M = kLbM;
    const int gN = cdiv(N, kLbBlock);

    DBuf<double> X(kLbBufs * (size_t)N, st), G(kLbBufs * (size_t)N, st), drt(N, st);
    // pair buffers: the ring's M plus one staging pair per iterate buffer
    DBuf<double> pairs((size_t)(M + kLbBufs) * 2 * N, st);
    DBuf<double> parts((size_t)gN * (4 + kLbPairSums), st);
    DBuf<unsigned> counter(1, st);
    DBuf<LbCoef> dcoef(1, st);
    DBuf<LbScal> dscal(1, st);
    DBuf<double> grid(1, st);
    // max |x| of each iterate buffer, written by the merge of the pass at x
    // (the split grid of a line search from x)
    DBuf<double> xmax(kLbBufs, st);
    DBuf<unsigned long long> mxparts(gN, st);
    pairs.zero();
    counter.zero();
    LbHost ring;
    Pinned<LbCoef> pcoef;
    LbCoef* coef = pcoef.p;
    std::memset(coef, 0, sizeof(LbCoef));
    coef->cv = -1.0;  // the first direction is -g (LBFGS.h:104)
    for (int k = 0; k < M; ++k) coef->phys[k] = ring.phys[k];
    for (int b = 0; b < kLbBufs; ++b) coef->stage[b] = ring.stage[b];
    Pinned<LbScal> pin;
    LbScal* hs = pin.p;
    // the pair products of the last trial written into each iterate buffer
    double hprod[kLbBufs][kLbPairSums] = {};
    auto xbuf = [&](int i) { return X.get() + (size_t)i * N; };
    auto gbuf = [&](int i) { return G.get() + (size_t)i * N; };

    const int cap = max_iter + 2;
    DBuf<unsigned long long> stamps(2 * (size_t)cap + 2, st);
    std::vector<double> hobj, hmar, hprim;
    int nstamp = 0;
    auto stamp = [&]() {
        k_lb_stamp<<<1, 1, 0, st>>>(stamps.get() + nstamp++);
        count_launch();
    };

    // Initial point: alpha = 0, beta = optimal_beta(0), or x0.
    std::vector<double> gamma0;
    stamp();  // the reference's timer starts before the first evaluation
    init_gamma(E, o, gamma0);
    d2d(xbuf(0), E.gamma(), (size_t)N * sizeof(double), st);

    // Merge of the last pass at x into grad, plus the record; returns after
    // the record has reached the host.
    // Merge of the last pass at x (buffer xi) into grad (buffer gi) and the
    // record, and its copy to the host (not waited for). With xpi >= 0 the
    // trial's correction pair from (xpi, gpi) is staged and its products
    // enter the record.
    auto merge_launch = [&](int op, int nt, int xi, int gi, int xpi, int gpi) {
        const int blocks = pass_blocks(op, mixed, n, m);
        const double* xp = xpi >= 0 ? xbuf(xpi) : xbuf(xi);
        const double* gp = gpi >= 0 ? gbuf(gpi) : nullptr;
        if (mixed)
            k_lb_merge<float><<<gN, kLbBlock, 0, st>>>(
                (const float*)ops.buf().rowpart.get(), sh.nslabs,
                (const float*)ops.buf().colpart.get(), sh.nrb, n, m, ops.buf().totpart.get(),
                blocks, nt, xbuf(xi), drt.get(), P->a, P->b, reg, gbuf(gi), xp, gp, pairs.get(),
                dcoef.get(), xi, parts.get(), counter.get(), dscal.get(), mxparts.get(),
                xmax.get() + xi);
        else
            k_lb_merge<double><<<gN, kLbBlock, 0, st>>>(
                (const double*)ops.buf().rowpart.get(), sh.nslabs,
                (const double*)ops.buf().colpart.get(), sh.nrb, n, m, ops.buf().totpart.get(),
                blocks, nt, xbuf(xi), drt.get(), P->a, P->b, reg, gbuf(gi), xp, gp, pairs.get(),
                dcoef.get(), xi, parts.get(), counter.get(), dscal.get(), mxparts.get(),
                xmax.get() + xi);
        count_launch();
        REGOT_CHECK_LAUNCH();
        d2h(hs, dscal.get(), sizeof(LbScal), st);
    };
    // f and grad at x in buffer xi (the Q_GRAD pass), as
    // Problem::dual_obj_grad: enqueued. Only a mixed pass splits x, on the
    // grid of max |x|.
    auto eval_launch = [&](int xi, int gi) {
        const double* x = xbuf(xi);
        if (mixed) ops.maxabs(x, N, nullptr, 0, grid.get());
        PassParams p = ops.base_params();
        p.ra = x;
        p.cb = x + n;
        p.grid = grid.get();
        ops.pass(OP_Q_GRAD, p);
        merge_launch(OP_Q_GRAD, 1, xi, gi, -1, -1);
    };
    auto eval_at = [&](int xi, int gi) {
        eval_launch(xi, gi);
        sync(st);
        E.add_passes(1);
        return 0.5 * hs->sq - reg * hs->dab;
    };
    // Trial at xp + s drt into buffers (xt, gt) from the line search's base
    // (xp, gp): the axpy (unless the direction kernel wrote the point), the
    // trial pass OP_Q_GRADLS (the gradient at the trial point and the
    // objective change from xp without cancellation; mixed: from the split
    // of xp and drt, made here when `split` is set, on the grid of max |xp|
    // from xp's merge) and the merge; enqueued, not waited for.
    auto trial_launch = [&](int xpi, int gpi, int xti, int gti, double s, bool split,
                            bool have_x) {
        if (!have_x) {
            k_lb_axpy<<<gN, kLbBlock, 0, st>>>(xbuf(xpi), drt.get(), s, N, xbuf(xti));
            count_launch();
        }
        PassParams p = ops.base_params();
        p.ra = xbuf(xpi);
        p.cb = xbuf(xpi) + n;
        p.rd = drt.get();
        p.cd = drt.get() + n;
        p.steps[0] = s;
        p.nsteps = 1;
        p.grid = xmax.get() + xpi;
        if (split) ops.pass(OP_Q_GRADLS, p);
        else ops.pass_presplit(OP_Q_GRADLS, p);
        merge_launch(OP_Q_GRADLS, 2, xti, gti, xpi, gpi);
    };
    // From the second iteration on, the copy of the coefficients, the new
    // direction and the first trial of the next line search (step 1, base =
    // the accepted point) are the same operations every iteration: one CUDA
    // graph per assignment of the rotating buffers, captured on first use.
    // The coefficient copy reads the page-locked block at each replay.
    std::map<int, cudaGraphExec_t> iter_graphs;
    long long iter_graph_kernels = 0;
    struct GraphSet {
        std::map<int, cudaGraphExec_t>& g;
        ~GraphSet() {
            for (auto& kv : g) cudaGraphExecDestroy(kv.second);
        }
    } graph_set{iter_graphs};
    auto iter_graph = [&](int xi, int gi) {
        const int key = xi * kLbBufs + gi;
        auto it = iter_graphs.find(key);
        if (it != iter_graphs.end()) return it->second;
        long long* saved = g_launch_counter;
        long long kernels = 0;
        g_launch_counter = &kernels;
        cudaGraph_t graph = nullptr;
        REGOT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            REGOT_CUDA(cudaMemcpyAsync(dcoef.get(), coef, sizeof(LbCoef),
                                       cudaMemcpyHostToDevice, st));
            k_lb_dir<<<gN, kLbBlock, 0, st>>>(gbuf(gi), pairs.get(), N, drt.get(), parts.get(),
                                              counter.get(), dcoef.get(), dscal.get(), xbuf(xi),
                                              1.0, xbuf((xi + 1) % kLbBufs));
            count_launch();
            trial_launch(xi, gi, (xi + 1) % kLbBufs, (gi + 1) % kLbBufs, 1.0, true, true);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
            g_launch_counter = saved;
            throw;
        }
        REGOT_CUDA(cudaStreamEndCapture(st, &graph));
        g_launch_counter = saved;
        cudaGraphExec_t exec = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        REGOT_CUDA(e);
        iter_graph_kernels = kernels;
        iter_graphs[key] = exec;
        return exec;
    };

    int ix = 0, ig = 0;
    double fx = eval_at(ix, ig);
    double last_obj = fx;
    double gg = hs->gg, xx = hs->xx;
    int it = 0;
    // Primal values (prim_vals) are enqueued with their copy into a
    // page-locked slot and read after the next synchronisation, which the
    // line search makes anyway: no synchronisation of their own.
    struct PrimSlots {
        PrimRaw s[2];
    };
    Pinned<PrimSlots> pslots;
    int prim_pending = -1;  // history index of the value in flight
    auto prim_finish = [&]() {
        if (prim_pending >= 0) {
            hprim[prim_pending] = E.primal_value(pslots.p->s[prim_pending & 1]);
            prim_pending = -1;
        }
    };
    auto iterate = [&](int xi, double gnorm) {
        stamp();
        prim_finish();  // the previous iteration's trials synchronised after it
        if (o.prim_vals) {
            E.primal_launch(xbuf(xi), xmax.get() + xi, &pslots.p->s[it & 1]);
            prim_pending = it;
        }
        hobj.push_back(last_obj);
        hmar.push_back(gnorm / reg);
        hprim.push_back(0.0);
        if (o.verbose >= 1)
            std::printf("iter = %d, objval = %g, ||grad|| = %g\n", it, last_obj, gnorm);
        it++;
        stamp();
    };

    lbfgs::Param param;
    param.epsilon = tol;
    param.epsilon_rel = tol;
    param.max_iterations = max_iter;
    int niter = 0;
    double gnorm = std::sqrt(gg);
    iterate(ix, gnorm);
    if (gnorm <= param.epsilon || gnorm <= param.epsilon_rel * std::sqrt(xx)) {
        niter = 1;
    } else {
        // drt = -g (LBFGS.h:104), its g'drt; step = 1 / |drt|
        h2d(dcoef.get(), coef, sizeof(LbCoef), st);
        k_lb_dir<<<gN, kLbBlock, 0, st>>>(gbuf(ig), pairs.get(), N, drt.get(), parts.get(),
                                          counter.get(), dcoef.get(), dscal.get(), nullptr, 0.0,
                                          nullptr);
        count_launch();
        REGOT_CHECK_LAUNCH();
        double step = 1.0 / gnorm;
        bool dg_known = true;  // the first g'drt is -|g|^2
        bool pre_launched = false;
        double dg = -gg;
        int k = 1;
        for (;;) {
            const int ixp = ix, igp = ig;
            // ---- line search (LineSearchNocedalWright.h:85-280) ----
            if (step <= 0.0) throw Error(REGOT_ERR_INVALID_ARG, "'step' must be positive");
            const double fx_init = fx;
            bool split_done = false;
            int ixl = ixp, igl = igp;  // x_lo, grad_lo (start as xp, gradp)
            int ixt = (ixp + 1) % 3, igt = (igp + 1) % 3;  // trial targets
            double dg_init = dg, test_decr = 0.0, test_curv = 0.0;
            auto free_of = [](int a, int b) { return 3 - a - b; };
            // One trial at step: x = xp + step drt into buffer ixt, grad into
            // igt; returns f and sets dgt, ggt, xxt.
            double dgt = 0.0, ggt = 0.0, xxt = 0.0;
            auto trial = [&](double s) {
                if (pre_launched) {
                    // the first trial (step 1) ran in the iteration's graph
                    pre_launched = false;
                } else {
                    trial_launch(ixp, igp, ixt, igt, s, !split_done, false);
                }
                split_done = true;
                sync(st);
                E.add_passes(1);
                std::memcpy(hprod[ixt], hs->prod, sizeof(hprod[ixt]));
                // The decrease tests use the exact change f(xp + s d) - f(xp)
                // = s g'd + rem: near the solution the change falls below the
                // rounding of f itself, where a difference of two evaluated
                // objectives is noise and the line search fails by chance.
                // The reported objective is the evaluated one.
                if (!dg_known) dg_init = hs->dg0;
                last_obj = 0.5 * hs->sq - reg * hs->dab;
                const double f = fx_init + s * dg_init + hs->rem;
                if (!dg_known) {
                    dg_known = true;
                    if (dg_init > 0.0)
                        throw Error(REGOT_ERR_LINESEARCH,
                                    "the moving direction increases the objective function value");
                }
                test_decr = param.ftol * dg_init;
                test_curv = -param.wolfe * dg_init;
                dgt = hs->dg;
                ggt = hs->gg;
                xxt = hs->xx;
                return f;
            };
            double step_hi = 0.0, fx_hi = 0.0, step_lo = 0.0, fx_lo = fx_init, dg_lo = 0.0;
            double gg_lo = gg, xx_lo = xx;
            bool lo_is_init = true;
            int lsit = 0;
            bool done = false;
            // expansion phase
            for (;;) {
                fx = trial(step);
                dg = dgt;
                if (lo_is_init) dg_lo = dg_init;
                if (fx - fx_init > step * test_decr || (0.0 < step_lo && fx >= fx_lo)) {
                    step_hi = step;
                    fx_hi = fx;
                    break;
                }
                if (std::abs(dg) <= test_curv) {
                    done = true;
                    break;
                }
                step_hi = step_lo;
                fx_hi = fx_lo;
                step_lo = step;
                fx_lo = fx;
                dg_lo = dg;
                lo_is_init = false;
                std::swap(ixl, ixt);  // x_lo.swap(x)
                std::swap(igl, igt);
                gg_lo = ggt;
                xx_lo = xxt;
                if (ixt == ixp) ixt = free_of(ixp, ixl);
                if (igt == igp) igt = free_of(igp, igl);
                if (dg >= 0.0) break;
                lsit++;
                if (lsit >= param.max_linesearch) {
                    // x.swap(x_lo): the accepted point is x_lo
                    std::swap(ixl, ixt);
                    std::swap(igl, igt);
                    ggt = gg_lo;
                    xxt = xx_lo;
                    done = true;
                    break;
                }
                step *= 2.0;
            }
            if (!done) {
                // zoom phase
                for (;;) {
                    step = lbfgs::quad_interp(step_lo, step_hi, fx_lo, fx_hi,
                                              lo_is_init ? dg_init : dg_lo);
                    fx = trial(step);
                    dg = dgt;
                    if (lo_is_init) dg_lo = dg_init;
                    if (fx - fx_init > step * test_decr || fx >= fx_lo) {
                        if (step == step_hi)
                            throw Error(REGOT_ERR_LINESEARCH,
                                        "the line search routine failed, possibly due to "
                                        "insufficient numeric precision");
                        step_hi = step;
                        fx_hi = fx;
                    } else {
                        if (std::abs(dg) <= test_curv) break;
                        if (dg * (step_hi - step_lo) >= 0.0) {
                            step_hi = step_lo;
                            fx_hi = fx_lo;
                        }
                        if (step == step_lo)
                            throw Error(REGOT_ERR_LINESEARCH,
                                        "the line search routine failed, possibly due to "
                                        "insufficient numeric precision");
                        step_lo = step;
                        fx_lo = fx;
                        dg_lo = dg;
                        lo_is_init = false;
                        std::swap(ixl, ixt);
                        std::swap(igl, igt);
                        gg_lo = ggt;
                        xx_lo = xxt;
                        if (ixt == ixp) ixt = free_of(ixp, ixl);
                        if (igt == igp) igt = free_of(igp, igl);
                    }
                    lsit++;
                    if (lsit >= param.max_linesearch) {
                        if (step_lo <= 0.0)
                            throw Error(REGOT_ERR_LINESEARCH,
                                        "the line search routine failed, unable to sufficiently "
                                        "decrease the function value");
                        step = step_lo;
                        fx = fx_lo;
                        dg = dg_lo;
                        std::swap(ixl, ixt);
                        std::swap(igl, igt);
                        ggt = gg_lo;
                        xxt = xx_lo;
                        break;
                    }
                }
            }
            // the accepted point is in (ixt, igt)
            ix = ixt;
            ig = igt;
            gg = ggt;
            xx = xxt;
            gnorm = std::sqrt(gg);
            iterate(ix, gnorm);
            if (gnorm <= param.epsilon || gnorm <= param.epsilon_rel * std::sqrt(xx)) break;
            if (param.max_iterations != 0 && k >= param.max_iterations) break;
            // correction pair and direction coefficients (host), then the
            // next direction and the next line search's first trial at
            // step 1 (the graph of this buffer assignment)
            lb_host_step(ring, hprod[ix], ix, *coef);
            REGOT_CUDA(cudaGraphLaunch(iter_graph(ix, ig), st));
            count_launch(iter_graph_kernels);
            pre_launched = true;
            dg_known = false;  // read with the first trial's record
            step = 1.0;
            k++;
        }
        niter = k;
    }
    // run_times from the device stamps (each iteration: from the end of the
    // previous iterate call, or the start, to the start of this one)
    std::vector<unsigned long long> hst(nstamp);
    d2h(hst.data(), stamps.get(), nstamp * sizeof(unsigned long long), st);
    sync(st);
    prim_finish();
    std::vector<double> htime(hobj.size());
    double cum = 0.0;
    for (size_t q = 0; q < hobj.size(); ++q) {
        cum += (double)(hst[2 * q + 1] - hst[2 * q]) * 1e-6;
        htime[q] = cum;
    }
    finish_qrot(E, xbuf(ix), hobj, hmar, htime, hprim, niter, o, res);
}

// qrot_lbfgs_dual_internal (qrot_lbfgs_dual.cpp:81-126, QROTDual 18-79).
void qrot_lbfgs_dual_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                         const regot_opts& o, regot_result* res) {
    if (o.tau == 0.0) {
        qrot_lbfgs_dual_device(ctx, P, reg, tol, max_iter, o, res);
        return;
    }
    // tau > 0 (only reachable through the C ABI: the reference's Python
    // layer never sets it): the host-vector driver with the exact tau terms.
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    QrotEngine E(P, reg, o.tau, st);
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    DevClock clock(st);
    lbfgs::Param param;
    param.epsilon = tol;
    param.epsilon_rel = tol;
    param.max_iterations = max_iter;
    std::vector<double> gamma;
    init_gamma(E, o, gamma);

    std::vector<double> hobj, hmar, htime, hprim;
    double last_obj = std::numeric_limits<double>::infinity();
    int it = 0;
    lbfgs::FunGrad fg = [&](const lbfgs::Vec& x, lbfgs::Vec& g) {
        h2d(E.gamma(), x.data(), N * sizeof(double), st);
        last_obj = E.eval(E.gamma(), E.grad(), false);
        d2h(g.data(), E.grad(), N * sizeof(double), st);
        sync(st);
        if (E.tau_grad() != 0.0) {
            for (int i = 0; i < n; ++i) g[i] += E.tau_grad();
            for (int j = 0; j < m; ++j) g[n + j] -= E.tau_grad();
        }
        return last_obj;
    };
    double t_prev = clock.now_ms();
    auto iterate = [&](const lbfgs::Vec& x, double gnorm) {
        const double t = clock.now_ms();
        const double d = t - t_prev;
        // prim_vals are outside the timed region, as in QROTDual::iterate.
        double prim = 0.0;
        if (o.prim_vals) {
            h2d(E.gamma(), x.data(), N * sizeof(double), st);
            prim = E.primal(E.gamma());
        }
        hobj.push_back(last_obj);
        hmar.push_back(gnorm / reg);
        htime.push_back((htime.empty() ? 0.0 : htime.back()) + d);
        hprim.push_back(prim);
        if (o.verbose >= 1)
            std::printf("iter = %d, objval = %g, ||grad|| = %g\n", it, last_obj, gnorm);
        it++;
        t_prev = clock.now_ms();
    };
    // In mixed precision, f(x) - f(xp) is far below the FP32 rounding of f
    // itself near convergence, and the line search compares such values: the
    // trial evaluates the change directly (eval_step) and returns
    // f(xp) + change. FP64 evaluates f(x) as the reference does.
    DBuf<double> xp_d(N, st), d_d(N, st);
    const std::vector<double>& ha = P->ha;
    const std::vector<double>& hb = P->hb;
    lbfgs::TrialFn trial = [&](const lbfgs::Vec& xp, const lbfgs::Vec& drt, double step,
                               double fx_init, double dg_init, lbfgs::Vec& x, lbfgs::Vec& g) {
        for (int k = 0; k < N; ++k) x[k] = xp[k] + step * drt[k];
        if (!mixed) return fg(x, g);
        h2d(E.gamma(), x.data(), N * sizeof(double), st);
        h2d(xp_d.get(), xp.data(), N * sizeof(double), st);
        h2d(d_d.get(), drt.data(), N * sizeof(double), st);
        double sq = 0.0;
        const double rem = E.eval_step(xp_d.get(), d_d.get(), step, &sq);
        d2h(g.data(), E.grad(), N * sizeof(double), st);
        sync(st);
        double change = step * dg_init + rem;
        double dab = 0.0;
        for (int i = 0; i < n; ++i) dab += x[i] * ha[i];
        for (int j = 0; j < m; ++j) dab += x[n + j] * hb[j];
        // History records f(x) evaluated directly; the line search gets the
        // accumulated value.
        last_obj = 0.5 * sq - reg * dab;
        if (o.tau > 0.0) {
            double sa = 0.0, sb = 0.0, ea = 0.0, eb = 0.0;
            for (int i = 0; i < n; ++i) {
                sa += x[i];
                ea += drt[i];
            }
            for (int j = 0; j < m; ++j) {
                sb += x[n + j];
                eb += drt[n + j];
            }
            const double dn = sa - sb, e = ea - eb;
            last_obj += 0.5 * o.tau * dn * dn;
            change += 0.5 * o.tau * step * step * e * e;
            for (int i = 0; i < n; ++i) g[i] += o.tau * dn;
            for (int j = 0; j < m; ++j) g[n + j] -= o.tau * dn;
        }
        return fx_init + change;
    };
    double fx;
    const int niter = lbfgs::minimize(fg, trial, iterate, param, gamma, fx);
    h2d(E.gamma(), gamma.data(), N * sizeof(double), st);
    finish_qrot(E, E.gamma(), hobj, hmar, htime, hprim, niter, o, res);
}

namespace {

// (H + mu I)^{-1} rhs for the generalized Hessian H of the last masked
// evaluation (sigma bitmask, h1, h2): hess_cg (qrot_cg.cpp:9-50) with the
// Schur complement on the column block, identity preconditioner, relative
// tolerance cg_tol and at most 2m steps, run on the device; the CG steps
// are launched in batches between convergence checks.
class QrotSchurCG {
public:
    // verbose >= 2 prints each solve's CG step count, as hess_cg does
    QrotSchurCG(QrotEngine& E, double cg_tol, int verbose = 0)
        : E_(E), st_(E.stream()), n_(E.n()), m_(E.m()), cg_tol_(cg_tol), verbose_(verbose),
          dvec_(8 * (size_t)std::max(n_, m_), st_), partial_((size_t)kColChunks * m_, st_),
          rhs_d_(n_ + m_, st_) {
        if (E.mixed()) {
            const size_t k2 = std::max(n_, m_);
            f2vec_.alloc(3 * k2, st_);
            p2_ = f2vec_.get();
            t2_ = p2_ + k2;
            x2_ = t2_ + k2;
        }
        const size_t k = std::max(n_, m_);
        t_d_ = dvec_.get() + k;
        zy_ = t_d_ + k;
        xs_ = zy_ + k;
        rs_ = xs_ + k;
        ps_ = rs_ + k;
        ys_ = ps_ + k;
        r1_ = ys_ + k;
        QState hs;
        d2h(&hs, E.state(), sizeof(hs), st_);
        sync(st_);
        hs.cg_max = 2 * m_;
        h2d(E.state(), &hs, sizeof(hs), st_);
    }

    void solve(const std::vector<double>& rhs, double mu, std::vector<double>& out) {
        QState* S = E_.state();
        const int n = n_, m = m_, N = n + m;
        const int gn = cdiv(n, kVT), gm = cdiv(m, kVT);
        h2d(rhs_d_.get(), rhs.data(), N * sizeof(double), st_);
        if (solve_compact(mu, out)) return;
        // v = w / (h1 + mu); zy = z - sigma' v
        k_div_h1<<<gn, kVT, 0, st_>>>(n, rhs_d_.get(), E_.h1(), mu, t_d_, t2_);
        count_launch();
        E_.sigma_cols(t_d_, t2_, partial_.get(), nullptr);
        k_sub_partial<<<gm, kVT, 0, st_>>>(m, rhs_d_.get() + n, partial_.get(), kColChunks, zy_);
        k_acg_init<<<gm, kVT, 0, st_>>>(m, zy_, cg_tol_, xs_, rs_, ps_, E_.parts(), S, x2_, p2_);
        count_launch(2);
        h2d(&S->mu, &mu, sizeof(double), st_);
        if (!exec_) build_graph();
        // kGraphSteps CG steps per graph launch; every kernel returns at once
        // after convergence (cg_done)
        int batch = 2;
        for (;;) {
            for (int q = 0; q < batch; ++q) REGOT_CUDA(cudaGraphLaunch(exec_, st_));
            count_launch(graph_kernels_ * batch);
            int done = 0;
            d2h(&done, &S->cg_done, sizeof(int), st_);
            sync(st_);
            if (done) break;
            batch = std::min(batch * 2, 32);
        }
        // r1 = (w - sigma r2) / (h1 + mu)
        E_.sigma_rows(xs_, x2_, mu, false, t_d_, nullptr, nullptr);
        k_backsub<<<gn, kVT, 0, st_>>>(n, rhs_d_.get(), t_d_, E_.h1(), mu, r1_);
        count_launch();
        out.resize(N);
        d2h(out.data(), r1_, n * sizeof(double), st_);
        d2h(out.data() + n, xs_, m * sizeof(double), st_);
        int it = 0;
        if (verbose_ >= 2) d2h(&it, &S->cg_it, sizeof(int), st_);
        sync(st_);
        if (verbose_ >= 2) std::printf("[cg] bitmask products, niter = %d\n", it);
    }

    ~QrotSchurCG() {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
    }

private:
    static constexpr int kGraphSteps = 8;
    // sigma is taken as index lists when it holds at most n m / kDenseRatio
    // entries: the list products then cost less than testing every bit.
    static constexpr long long kDenseRatio = 64;

    // The compact path: count the set bits of every row and of every
    // (row chunk, column), scan them into row and column pointers, fill the
    // index lists, and run the whole CG in one cluster launch. Returns false
    // (nothing solved) when sigma is too dense for it or no cluster fits.
    bool solve_compact(double mu, std::vector<double>& out) {
        const int mode = g_qrot_cg_path.load(std::memory_order_relaxed);
        const int C = cluster_ctas(E_.mixed());
        if (mode == 1 || C == 0) return false;
        const int n = n_, m = m_;
        if (!rcnt_.get()) {
            rcnt_.alloc(n, st_);
            rowptr_.alloc(n + 1, st_);
            ccnt_.alloc((size_t)kColChunks * m, st_);
            ccol_.alloc(m, st_);
            colptr_.alloc(m + 1, st_);
            nnz_d_.alloc(2, st_);
            it_d_.alloc(2, st_);
            dinv_.alloc(n, st_);
        }
        const uint32_t* bm = E_.bitmask();
        const int ns = E_.slabs();
        const int warps = 8;
        const dim3 cgrid(cdiv(m, 128), kColChunks);
        if (E_.mixed()) {
            k_cs_row_counts<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<cdiv(n, warps), warps * 32, 0, st_>>>(bm, n, ns, rcnt_.get());
            k_cs_col_counts<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<cgrid, 128, 0, st_>>>(bm, n, m, ns, ccnt_.get());
        } else {
            k_cs_row_counts<Geo<double>::CW, Geo<double>::VW, Geo<double>::LC>
                <<<cdiv(n, warps), warps * 32, 0, st_>>>(bm, n, ns, rcnt_.get());
            k_cs_col_counts<Geo<double>::CW, Geo<double>::VW, Geo<double>::LC>
                <<<cgrid, 128, 0, st_>>>(bm, n, m, ns, ccnt_.get());
        }
        k_cs_col_offsets<<<cdiv(m, 128), 128, 0, st_>>>(m, kColChunks, ccnt_.get(), ccol_.get());
        k_cs_scan<<<1, 1024, 0, st_>>>(rcnt_.get(), n, rowptr_.get(), ccol_.get(), m,
                                       colptr_.get(), nnz_d_.get());
        count_launch(5);
        long long nnz[2] = {0, 0};
        d2h(nnz, nnz_d_.get(), sizeof(nnz), st_);
        sync(st_);
        if (nnz[0] != nnz[1])
            throw Error(REGOT_ERR_NUMERIC, "qrot Schur CG: row and column counts of sigma differ");
        if (nnz[0] > (long long)INT32_MAX / 2) return false;
        if (mode == 0 && nnz[0] * kDenseRatio > (long long)n * m) return false;
        if ((size_t)nnz[0] > idx_cap_) {
            idx_cap_ = std::max<size_t>((size_t)nnz[0] + nnz[0] / 2, 1024);
            colidx_.alloc(idx_cap_, st_);
            rowidx_.alloc(idx_cap_, st_);
        }
        if (E_.mixed()) {
            k_cs_row_fill<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<cdiv(n, warps), warps * 32, 0, st_>>>(bm, n, ns, rowptr_.get(), colidx_.get());
            k_cs_col_fill<Geo<float>::CW, Geo<float>::VW, Geo<float>::LC>
                <<<cgrid, 128, 0, st_>>>(bm, n, m, ns, colptr_.get(), ccnt_.get(), rowidx_.get());
        } else {
            k_cs_row_fill<Geo<double>::CW, Geo<double>::VW, Geo<double>::LC>
                <<<cdiv(n, warps), warps * 32, 0, st_>>>(bm, n, ns, rowptr_.get(), colidx_.get());
            k_cs_col_fill<Geo<double>::CW, Geo<double>::VW, Geo<double>::LC>
                <<<cgrid, 128, 0, st_>>>(bm, n, m, ns, colptr_.get(), ccnt_.get(), rowidx_.get());
        }
        ClusterCgArgs a;
        a.n = n;
        a.m = m;
        a.cg_max = 2 * m;
        a.mu = mu;
        a.tol = cg_tol_;
        a.rowptr = rowptr_.get();
        a.colidx = colidx_.get();
        a.colptr = colptr_.get();
        a.rowidx = rowidx_.get();
        a.h1 = E_.h1();
        a.h2 = E_.h2();
        a.w = rhs_d_.get();
        a.z = rhs_d_.get() + n;
        a.dinv = dinv_.get();
        a.t = t_d_;
        a.p = ps_;
        a.r = rs_;
        a.y = ys_;
        a.x = xs_;
        a.r1 = r1_;
        a.t2 = t2_;
        a.p2 = p2_;
        a.it_out = it_d_.get();
        // both vectors' copies in every CTA's shared memory when they fit
        const size_t ds_bytes = (size_t)(((n + 1) & ~1) + ((m + 1) & ~1)) * 8;
        int Cd = ds_bytes <= (size_t)kDsMaxBytes && mode != 3 ? dsm_ctas(E_.mixed()) : 0;
        // mixed engine: rows and columns per thread of the double-word kernel
        int K = 0;
        if (Cd && E_.mixed()) {
            const int per = std::max(((n + 2 * Cd - 1) / (2 * Cd)) * 2,
                                     ((m + 2 * Cd - 1) / (2 * Cd)) * 2);
            K = cdiv(per, kDsT);
            K = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : 0;
            if (!K) Cd = 0;
        }
        // the CTAs' index-list slices in the shared memory left over
        const int idx_cap =
            (int)std::min<long long>(2 * nnz[0], (long long)(kDsMaxBytes - ds_bytes) / 4) & ~3;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(Cd ? Cd : C);
        cfg.blockDim = dim3(Cd ? kDsT : kCgT);
        cfg.dynamicSmemBytes = Cd ? ds_bytes + (K ? (size_t)idx_cap * 4 : 0) : 0;
        cfg.stream = st_;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = Cd ? Cd : C;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        REGOT_CUDA(cudaMemsetAsync(it_d_.get(), 0, 2 * sizeof(int), st_));
        if (Cd) {
            DsmCgArgs da;
            da.c = a;
            da.polls = wait_limit();
            da.err = it_d_.get() + 1;
            if (E_.mixed()) {
                DwCgArgs wa;
                wa.d = da;
                wa.idx_cap = idx_cap;
                if (K == 1) REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_schur_cg_dw<1>, wa));
                else if (K == 2) REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_schur_cg_dw<2>, wa));
                else if (K == 4) REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_schur_cg_dw<4>, wa));
                else REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_schur_cg_dw<8>, wa));
            } else {
                REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_schur_cg_dsm<false>, da));
            }
        } else if (E_.mixed()) {
            REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_schur_cg_cluster<true>, a));
        } else {
            REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_schur_cg_cluster<false>, a));
        }
        count_launch(3);
        out.resize(n + m);
        int it[2] = {0, 0};
        d2h(out.data(), r1_, n * sizeof(double), st_);
        d2h(out.data() + n, xs_, m * sizeof(double), st_);
        d2h(it, it_d_.get(), 2 * sizeof(int), st_);
        sync(st_);
        if (it[1])
            throw Error(REGOT_ERR_TIMEOUT,
                        "qrot Schur CG: a cluster exchange did not complete within the wait limit");
        if (verbose_ >= 2)
            std::printf("[cg] index lists (nnz = %lld%s), niter = %d\n", nnz[0],
                        Cd ? ", shared-memory exchange" : "", it[0]);
        return true;
    }

    // CTAs per cluster of the compact CG: 16 where the device takes such a
    // cluster (a non-portable size), else the largest smaller power of two;
    // 0 if none fits.
    static int cluster_ctas(bool mixed) {
        static const int sizes[2] = {probe_cluster(false), probe_cluster(true)};
        return sizes[mixed ? 1 : 0];
    }
    static int probe_cluster(bool mixed) {
        auto kern = mixed ? k_schur_cg_cluster<true> : k_schur_cg_cluster<false>;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
            cudaSuccess) {
            cudaGetLastError();
        }
        for (int c = 16; c >= 1; c >>= 1) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(kCgT);
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int num = 0;
            if (cudaOccupancyMaxActiveClusters(&num, kern, &cfg) == cudaSuccess && num > 0)
                return c;
            cudaGetLastError();
        }
        return 0;
    }

    // CTAs per cluster of the shared-memory-exchange CG (the largest
    // dynamic shared memory it may use set once), as cluster_ctas.
    static int dsm_ctas(bool mixed) {
        static const int sizes[2] = {probe_dsm(k_schur_cg_dsm<false>), probe_dw()};
        return sizes[mixed ? 1 : 0];
    }
    // every instance of the double-word kernel takes the same cluster and
    // shared-memory attributes; the cluster size is probed on the first
    static int probe_dw() {
        const int c = probe_dsm(k_schur_cg_dw<1>);
        if (c && (set_dsm_attrs(k_schur_cg_dw<2>) && set_dsm_attrs(k_schur_cg_dw<4>) &&
                  set_dsm_attrs(k_schur_cg_dw<8>)))
            return c;
        return 0;
    }
    template <typename Kern>
    static bool set_dsm_attrs(Kern kern) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess ||
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kDsMaxBytes) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return true;
    }
    template <typename Kern>
    static int probe_dsm(Kern kern) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess ||
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kDsMaxBytes) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        for (int c = 16; c >= 1; c >>= 1) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(kDsT);
            cfg.dynamicSmemBytes = kDsMaxBytes;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int num = 0;
            if (cudaOccupancyMaxActiveClusters(&num, kern, &cfg) == cudaSuccess && num > 0)
                return c;
            cudaGetLastError();
        }
        return 0;
    }

    DBuf<int> rcnt_, rowptr_, ccnt_, ccol_, colptr_, colidx_, rowidx_, it_d_;
    DBuf<long long> nnz_d_;
    DBuf<double> dinv_;
    size_t idx_cap_ = 0;

    // One CG step on Delta = h2 o x + mu x - sigma' ((sigma x) / (h1 + mu)),
    // mu from the state; a no-op once the device flag cg_done is set.
    void step() {
        QState* S = E_.state();
        const int gm = cdiv(m_, kVT);
        E_.sigma_rows(ps_, p2_, 0.0, true, t_d_, t2_, &S->cg_done, &S->mu);
        E_.sigma_cols(t_d_, t2_, partial_.get(), &S->cg_done);
        k_acg_a<<<cdiv(m_, 32), dim3(32, 8), 0, st_>>>(m_, partial_.get(), kColChunks,
                                                       E_.h2(), ps_, ys_, E_.parts(), S);
        k_acg_b<<<gm, kVT, 0, st_>>>(m_, ps_, ys_, xs_, rs_, E_.parts(), S, x2_);
        k_acg_c<<<gm, kVT, 0, st_>>>(m_, rs_, ps_, S, p2_);
        count_launch(3);
    }

    // kGraphSteps steps captured once per solver call: the shift is read
    // from the state, so the graph serves every solve.
    void build_graph() {
        long long* saved = g_launch_counter;
        graph_kernels_ = 0;
        g_launch_counter = &graph_kernels_;
        REGOT_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        try {
            for (int q = 0; q < kGraphSteps; ++q) step();
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st_, &g);
            if (g) cudaGraphDestroy(g);
            g_launch_counter = saved;
            throw;
        }
        REGOT_CUDA(cudaStreamEndCapture(st_, &graph_));
        g_launch_counter = saved;
        REGOT_CUDA(cudaGraphInstantiate(&exec_, graph_, 0));
    }

    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    long long graph_kernels_ = 0;

    QrotEngine& E_;
    cudaStream_t st_;
    int n_, m_;
    double cg_tol_;
    int verbose_;
    DBuf<double> dvec_, partial_, rhs_d_;
    double *t_d_, *zy_, *xs_, *rs_, *ps_, *ys_, *r1_;
    // mixed engine: FP32 (hi, lo) copies of p, sigma p / (h1 + mu) and x
    DBuf<float2> f2vec_;
    float2 *p2_ = nullptr, *t2_ = nullptr, *x2_ = nullptr;
};

}  // namespace

// qrot_lbfgs_semi_dual_internal: qrot_lbfgs_semi_dual.cpp:84-126
// (QROTSemiDual 18-82). L-BFGS on alpha (epsilon = epsilon_rel = tol) of the
// semi-dual f(alpha) = 0.5 ||D||^2 - reg (a'alpha + b'beta(alpha)),
// beta(alpha) = optimal_beta(alpha) (semi_dual_obj_grad,
// qrot_problem.cpp:420-442): every evaluation is the optimal_beta root
// passes plus one gradient pass. In mixed precision a line-search trial
// forms f(x) - f(xp) without cancellation: with d = (x - xp, beta(x) -
// beta(xp)) and the full dual gradient (g_alpha, g_beta) at (xp, beta(xp)),
// the change is g_alpha'd_alpha + g_beta'd_beta + sum rem (OP_Q_GRADLS at
// the base point along d); g_beta vanishes up to rounding at an exact beta.
void qrot_lbfgs_semi_dual_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol,
                              int max_iter, const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    QrotEngine E(P, reg, 0.0, st);
    DevClock clock(st);
    lbfgs::Param param;
    param.epsilon = tol;
    param.epsilon_rel = tol;
    param.max_iterations = max_iter;
    std::vector<double> alpha(n, 0.0);
    if (o.x0 && o.x0_len == n + m) std::copy(o.x0, o.x0 + n, alpha.begin());

    // The last few evaluations: alpha, beta(alpha) and the beta block of the
    // full gradient there (the base points of later line searches).
    struct Rec {
        std::vector<double> alpha, beta, gbeta;
    };
    std::vector<Rec> recs;
    auto find = [&](const std::vector<double>& x) -> const Rec* {
        for (auto it = recs.rbegin(); it != recs.rend(); ++it)
            if (it->alpha == x) return &*it;
        return nullptr;
    };
    std::vector<double> gfull(N), beta(m);
    auto record = [&](const std::vector<double>& x) {
        if (recs.size() >= 4) recs.erase(recs.begin());
        recs.push_back(Rec{x, beta, std::vector<double>(gfull.begin() + n, gfull.end())});
    };
    // f and g at x: beta = optimal_beta(x) on the device, then one pass
    double last_obj = std::numeric_limits<double>::infinity();
    lbfgs::FunGrad fg = [&](const lbfgs::Vec& x, lbfgs::Vec& g) {
        h2d(E.gamma(), x.data(), n * sizeof(double), st);
        E.optimal_beta(E.gamma(), E.gamma() + n);
        last_obj = E.eval(E.gamma(), E.grad(), false);
        d2h(gfull.data(), E.grad(), N * sizeof(double), st);
        d2h(beta.data(), E.gamma() + n, m * sizeof(double), st);
        sync(st);
        std::copy(gfull.begin(), gfull.begin() + n, g.begin());
        record(x);
        return last_obj;
    };
    DBuf<double> xp_d(N, st), d_d(N, st);
    std::vector<double> xpf(N), dv(N), gtmp(n);
    const std::vector<double>& ha = P->ha;
    const std::vector<double>& hb = P->hb;
    lbfgs::TrialFn trial = [&](const lbfgs::Vec& xp, const lbfgs::Vec& drt, double step,
                               double fx_init, double dg_init, lbfgs::Vec& x, lbfgs::Vec& g) {
        for (int k = 0; k < n; ++k) x[k] = xp[k] + step * drt[k];
        if (!mixed) return fg(x, g);
        if (!find(xp)) fg(xp, gtmp);  // not expected: the base point is an evaluated one
        const Rec base = *find(xp);
        h2d(E.gamma(), x.data(), n * sizeof(double), st);
        E.optimal_beta(E.gamma(), E.gamma() + n);
        d2h(beta.data(), E.gamma() + n, m * sizeof(double), st);
        sync(st);
        double gb = 0.0;
        for (int k = 0; k < n; ++k) {
            xpf[k] = xp[k];
            dv[k] = x[k] - xp[k];
        }
        for (int j = 0; j < m; ++j) {
            xpf[n + j] = base.beta[j];
            dv[n + j] = beta[j] - base.beta[j];
            gb += base.gbeta[j] * dv[n + j];
        }
        h2d(xp_d.get(), xpf.data(), N * sizeof(double), st);
        h2d(d_d.get(), dv.data(), N * sizeof(double), st);
        double sq = 0.0;
        const double rem = E.eval_step(xp_d.get(), d_d.get(), 1.0, &sq);
        d2h(gfull.data(), E.grad(), N * sizeof(double), st);
        sync(st);
        std::copy(gfull.begin(), gfull.begin() + n, g.begin());
        double dab = 0.0;
        for (int i = 0; i < n; ++i) dab += x[i] * ha[i];
        for (int j = 0; j < m; ++j) dab += beta[j] * hb[j];
        last_obj = 0.5 * sq - reg * dab;  // history: f(x) evaluated directly
        record(x);
        return fx_init + (step * dg_init + gb + rem);
    };
    std::vector<double> hobj, hmar, htime, hprim;
    int it = 0;
    double t_prev = clock.now_ms();
    // gamma = (alpha, optimal_beta(alpha)) on the device
    auto full_dual = [&](const std::vector<double>& x) {
        h2d(E.gamma(), x.data(), n * sizeof(double), st);
        if (const Rec* r = find(x)) h2d(E.gamma() + n, r->beta.data(), m * sizeof(double), st);
        else E.optimal_beta(E.gamma(), E.gamma() + n);
    };
    auto iterate = [&](const lbfgs::Vec& x, double gnorm) {
        const double d = clock.now_ms() - t_prev;
        double prim = 0.0;
        if (o.prim_vals) {
            full_dual(x);
            prim = E.primal(E.gamma());
        }
        hobj.push_back(last_obj);
        hmar.push_back(gnorm / reg);
        htime.push_back((htime.empty() ? 0.0 : htime.back()) + d);
        hprim.push_back(prim);
        if (o.verbose >= 1)
            std::printf("iter = %d, objval = %g, ||grad|| = %g\n", it, last_obj, gnorm);
        it++;
        t_prev = clock.now_ms();
    };
    double fx;
    const int niter = lbfgs::minimize(fg, trial, iterate, param, alpha, fx);
    full_dual(alpha);
    finish_qrot(E, E.gamma(), hobj, hmar, htime, hprim, niter, o, res);
}

// qrot_assn_internal (qrot_assn.cpp:16-170) with the CG solve of
// QROTLinearSolver (method 0, qrot_linsolve.cpp:72-105; qrot_cg.cpp:9-50).
void qrot_assn_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                   const regot_opts& o, regot_result* res) {
    require(o.tau == 0.0, "qrot_assn: tau > 0 is not supported");
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    QrotEngine E(P, reg, 0.0, st);
    DevClock clock(st);
    constexpr double nu = 0.99, eta1 = 0.25, eta2 = 0.75, gamma1 = 2.0, gamma2 = 4.0,
                     lam_min = 0.01, beta_ = 0.5, cg_tol = 1e-8;
    double xi = 0.0, lam = 1.0;

    std::vector<double> gamma, g(N), u(N), gu(N), v(N), gv(N), direc(N);
    init_gamma(E, o, gamma);
    QrotSchurCG cg(E, cg_tol, o.verbose);
    auto solve = [&](const std::vector<double>& rhs, double mu, std::vector<double>& out) {
        cg.solve(rhs, mu, out);
    };
    auto grad_at = [&](const std::vector<double>& x, std::vector<double>& gr, bool mask) {
        h2d(E.gamma(), x.data(), N * sizeof(double), st);
        const double f = E.eval(E.gamma(), E.grad(), mask);
        d2h(gr.data(), E.grad(), N * sizeof(double), st);
        sync(st);
        return f;
    };
    auto primal = [&](const std::vector<double>& x) {
        if (!o.prim_vals) return 0.0;
        h2d(E.gamma(), x.data(), N * sizeof(double), st);
        return E.primal(E.gamma());
    };
    std::vector<double> hobj, hmar, htime, hprim;
    double t0 = clock.now_ms();
    double f = grad_at(gamma, g, true);
    double gnorm = lbfgs::norm(g);
    double dur = clock.now_ms() - t0;
    hobj.push_back(f);
    hmar.push_back(gnorm / reg);
    htime.push_back(dur);
    hprim.push_back(primal(gamma));
    int i;
    for (i = 0; i < max_iter; i++) {
        if (o.verbose >= 1)
            std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
        t0 = clock.now_ms();
        if (gnorm < tol) break;
        if (i == 0) xi = gnorm;
        const double mu = lam * gnorm;
        std::vector<double> rhs(N);
        for (int q = 0; q < N; ++q) rhs[q] = -g[q];
        solve(rhs, mu, direc);
        for (int q = 0; q < N; ++q) u[q] = gamma[q] + direc[q];
        grad_at(u, gu, false);
        const double gunorm = lbfgs::norm(gu);
        if (gunorm <= nu * xi) {
            gamma.swap(u);
            xi = gunorm;
        } else {
            const double numer = -lbfgs::dot(gu, direc);
            const double denom = lbfgs::dot(direc, direc);
            const double rho = numer / denom;
            for (int q = 0; q < N; ++q) v[q] = gamma[q] + (-numer) / (gunorm * gunorm) * gu[q];
            grad_at(v, gv, false);
            const double gvnorm = lbfgs::norm(gv);
            if (rho >= eta1 && gvnorm <= gnorm) {
                gamma.swap(v);
            } else {
                for (int q = 0; q < N; ++q) gamma[q] -= beta_ * g[q];
            }
            if (rho >= eta2) {
                lam = 0.5 * (lam_min + lam);
            } else if (rho >= eta1) {
                lam *= gamma1;
            } else {
                lam *= gamma2;
            }
        }
        f = grad_at(gamma, g, true);
        gnorm = lbfgs::norm(g);
        dur = clock.now_ms() - t0;
        hobj.push_back(f);
        hmar.push_back(gnorm / reg);
        htime.push_back(htime.back() + dur);
        hprim.push_back(primal(gamma));
    }
    h2d(E.gamma(), gamma.data(), N * sizeof(double), st);
    finish_qrot(E, E.gamma(), hobj, hmar, htime, hprim, i, o, res);
}

// qrot_grssn_internal: qrot_grssn.cpp:16-133. Regularized semi-smooth Newton:
// direction (H + shift I)^{-1} (-g) by the Schur CG of hess_cg (CG tolerance
// 1e-8; the reference's sparse direct factorizations, methods 1-3, solve
// the same system), then Armijo backtracking (theta = kappa = 0.5, <= 20
// trials, the last trial kept if none passes). Mixed precision tests
// f(x + s d) - f(x) <= s theta g'd on the exact change s g'd + sum rem of
// the trial pass OP_Q_GRADLS; FP64 evaluates the objective directly, as
// the reference does.
void qrot_grssn_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                    const regot_opts& o, regot_result* res) {
    require(o.tau == 0.0, "qrot_grssn: tau > 0 is not supported");
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    constexpr double theta = 0.5, kappa = 0.5, cg_tol = 1e-8;
    constexpr int nlinesearch = 20;
    const double shift = o.shift;
    QrotEngine E(P, reg, 0.0, st);
    DevClock clock(st);
    std::vector<double> gamma, newgamma(N), g(N), direc(N), rhs(N);
    init_gamma(E, o, gamma);
    QrotSchurCG cg(E, cg_tol, o.verbose);
    DBuf<double> xp_d(N, st), d_d(N, st);
    // f, g and the generalized Hessian (sigma bitmask, h1, h2) at gamma
    auto grad_hess = [&]() {
        h2d(E.gamma(), gamma.data(), N * sizeof(double), st);
        const double f = E.eval(E.gamma(), E.grad(), true);
        d2h(g.data(), E.grad(), N * sizeof(double), st);
        sync(st);
        return f;
    };
    auto primal = [&]() { return o.prim_vals ? E.primal(E.gamma()) : 0.0; };

    std::vector<double> hobj, hmar, htime, hprim;
    double t0 = clock.now_ms();
    double f = grad_hess();
    double gnorm = lbfgs::norm(g);
    hobj.push_back(f);
    hmar.push_back(gnorm / reg);
    htime.push_back(clock.now_ms() - t0);
    hprim.push_back(primal());
    int i;
    for (i = 0; i < max_iter; i++) {
        if (o.verbose >= 1) std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
        t0 = clock.now_ms();
        if (gnorm < tol) break;
        for (int q = 0; q < N; ++q) rhs[q] = -g[q];
        cg.solve(rhs, shift, direc);
        double step = 1.0;
        double gd = 0.0;
        for (int q = 0; q < N; ++q) gd += g[q] * direc[q];
        const double thresh = theta * gd;
        if (mixed) {
            h2d(xp_d.get(), gamma.data(), N * sizeof(double), st);
            h2d(d_d.get(), direc.data(), N * sizeof(double), st);
        }
        for (int k = 0; k < nlinesearch; k++) {
            for (int q = 0; q < N; ++q) newgamma[q] = gamma[q] + step * direc[q];
            bool ok;
            if (mixed) {
                double sq = 0.0;
                const double rem = E.eval_step(xp_d.get(), d_d.get(), step, &sq);
                ok = step * gd + rem <= step * thresh;
            } else {
                h2d(E.gamma(), newgamma.data(), N * sizeof(double), st);
                const double newf = E.eval(E.gamma(), E.grad(), false);
                ok = newf <= f + step * thresh;
            }
            if (ok) break;
            step *= kappa;
        }
        gamma.swap(newgamma);
        f = grad_hess();
        gnorm = lbfgs::norm(g);
        const double dur = clock.now_ms() - t0;
        hobj.push_back(f);
        hmar.push_back(gnorm / reg);
        htime.push_back(htime.back() + dur);
        hprim.push_back(primal());
    }
    finish_qrot(E, E.gamma(), hobj, hmar, htime, hprim, i, o, res);
}

namespace {

// Initial value shared by qrot_bcd and qrot_gd: x0, or (0, optimal_beta(0)).
void qrot_initial(QrotEngine& E, const regot_opts& o, int n, int m) {
    cudaStream_t st = E.stream();
    if (o.x0 && o.x0_len == n + m) {
        h2d(E.gamma(), o.x0, (n + m) * sizeof(double), st);
        return;
    }
    REGOT_CUDA(cudaMemsetAsync(E.gamma(), 0, n * sizeof(double), st));
    E.optimal_beta(E.gamma(), E.gamma() + n);
}

double host_norm(const std::vector<double>& g) {
    double s = 0.0;
    for (double v : g) s += v * v;
    return std::sqrt(s);
}

}  // namespace

// qrot_bcd_internal: qrot_bcd.cpp:14-103. alpha = optimal_alpha(beta), then
// beta = optimal_beta(alpha), each by Newton's method from above on the
// device (OP_Q_ROWROOT / OP_Q_COLROOT passes); the problem has tau = 0.
void qrot_bcd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                  const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    QrotEngine E(P, reg, 0.0, st);
    DevClock clock(st);
    qrot_initial(E, o, n, m);
    std::vector<double> g(N), hobj, hmar, htime, hprim;
    auto grad = [&]() {
        const double f = E.eval(E.gamma(), E.grad(), false);
        d2h(g.data(), E.grad(), N * sizeof(double), st);
        sync(st);
        return f;
    };
    double t0 = clock.now_ms();
    double f = grad();
    double gnorm = host_norm(g);
    hobj.push_back(f);
    hmar.push_back(gnorm / reg);
    htime.push_back(clock.now_ms() - t0);
    hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
    int i;
    for (i = 0; i < max_iter; i++) {
        if (o.verbose >= 1) std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
        t0 = clock.now_ms();
        if (gnorm < tol) break;
        E.optimal_alpha(E.gamma() + n, E.gamma());
        E.optimal_beta(E.gamma(), E.gamma() + n);
        f = grad();
        gnorm = host_norm(g);
        const double dur = clock.now_ms() - t0;
        hobj.push_back(f);
        hmar.push_back(gnorm / reg);
        htime.push_back(htime.back() + dur);
        hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
    }
    finish_qrot(E, E.gamma(), hobj, hmar, htime, hprim, i, o, res);
}

// qrot_gd_internal: qrot_gd.cpp:14-120. Armijo backtracking along -g
// (theta = kappa = 0.5, <= 20 trials, the last trial kept if none passes).
// Mixed precision tests newf - f <= -step theta |g|^2 on the exact change
// step g'd + sum rem (+ tau term) of the trial pass OP_Q_GRADLS; FP64
// evaluates newf directly, as the reference does.
void qrot_gd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                 const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    constexpr double theta = 0.5, kappa = 0.5;
    constexpr int nlinesearch = 20;
    QrotEngine E(P, reg, o.tau, st);
    DevClock clock(st);
    qrot_initial(E, o, n, m);
    std::vector<double> gamma(N), newgamma(N), g(N), d(N), hobj, hmar, htime, hprim;
    d2h(gamma.data(), E.gamma(), N * sizeof(double), st);
    sync(st);
    DBuf<double> xp_d(N, st), d_d(N, st);
    // f and the full gradient (tau term included) at the device gamma
    auto grad = [&]() {
        const double f = E.eval(E.gamma(), E.grad(), false);
        d2h(g.data(), E.grad(), N * sizeof(double), st);
        sync(st);
        if (E.tau_grad() != 0.0) {
            for (int q = 0; q < n; ++q) g[q] += E.tau_grad();
            for (int q = 0; q < m; ++q) g[n + q] -= E.tau_grad();
        }
        return f;
    };
    double t0 = clock.now_ms();
    double f = grad();
    double gnorm = host_norm(g);
    hobj.push_back(f);
    hmar.push_back(gnorm / reg);
    htime.push_back(clock.now_ms() - t0);
    hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
    int i;
    for (i = 0; i < max_iter; i++) {
        if (o.verbose >= 1) std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
        t0 = clock.now_ms();
        if (gnorm < tol) break;
        double step = 1.0;
        const double g2 = gnorm * gnorm, thresh = theta * g2;
        if (mixed) {
            for (int q = 0; q < N; ++q) d[q] = -g[q];
            h2d(xp_d.get(), gamma.data(), N * sizeof(double), st);
            h2d(d_d.get(), d.data(), N * sizeof(double), st);
        }
        for (int k = 0; k < nlinesearch; k++) {
            for (int q = 0; q < N; ++q) newgamma[q] = gamma[q] - step * g[q];
            bool ok;
            if (mixed) {
                double sq = 0.0;
                double change = -step * g2 + E.eval_step(xp_d.get(), d_d.get(), step, &sq);
                if (o.tau > 0.0) {
                    double e = 0.0;
                    for (int q = 0; q < n; ++q) e += d[q];
                    for (int q = 0; q < m; ++q) e -= d[n + q];
                    change += 0.5 * o.tau * step * step * e * e;
                }
                ok = change <= -step * thresh;
            } else {
                h2d(E.gamma(), newgamma.data(), N * sizeof(double), st);
                const double newf = E.eval(E.gamma(), E.grad(), false);
                ok = newf <= f - step * thresh;
            }
            if (ok) break;
            step *= kappa;
        }
        gamma.swap(newgamma);
        h2d(E.gamma(), gamma.data(), N * sizeof(double), st);
        f = grad();
        gnorm = host_norm(g);
        const double dur = clock.now_ms() - t0;
        hobj.push_back(f);
        hmar.push_back(gnorm / reg);
        htime.push_back(htime.back() + dur);
        hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
    }
    finish_qrot(E, E.gamma(), hobj, hmar, htime, hprim, i, o, res);
}

namespace {

using HVec = std::vector<double>;

// Averaged plan of qrot_apdagd / qrot_pdaam, kept on the device in the pass's
// element type: X <- c_old X + c_new D(gamma) / reg (X <- D / reg at the
// start), with the primal objective <M, X> + reg/2 ||X||^2 and the marginal
// error of X (qrot_apdagd.cpp:133-146, qrot_pdaam.cpp:142-155), one pass
// (OP_Q_AVG).
class QrotAvgPlan {
public:
    QrotAvgPlan(regot_ctx* ctx, QrotEngine& E, regot_dproblem* P)
        : ctx_(ctx), E_(E), P_(P), n_(P->n), m_(P->m), st_(E.stream()),
          mixed_(P->prec == REGOT_PREC_MIXED),
          X_((size_t)n_ * m_ * (mixed_ ? sizeof(float) : sizeof(double)), st_),
          sums_(n_ + m_ + 2, st_), mx_(1, st_) {}

    void update(const double* gamma, double c_old, double c_new, bool init, double* primal,
                double* mar_err) {
        ErotOps& ops = E_.ops();
        PassParams p = ops.base_params();
        p.ra = gamma;
        p.cb = gamma + n_;
        p.xavg = X_.get();
        p.steps[0] = c_old;
        p.steps[1] = c_new;
        p.nsteps = init ? 0 : 2;
        ops.maxabs(gamma, n_ + m_, nullptr, 0, mx_.get());
        p.grid = mx_.get();
        ops.pass(OP_Q_AVG, p);
        ops.merge_rows(1, sums_.get());
        ops.merge_cols(1, sums_.get() + n_);
        ops.merge_totals(OP_Q_AVG, 2, sums_.get() + n_ + m_);
        E_.add_passes(1);
        const int cnt = n_ + m_ + 2;
        const double* h = static_cast<const double*>(ctx_stage(ctx_, cnt * sizeof(double)));
        d2h(const_cast<double*>(h), sums_.get(), cnt * sizeof(double), st_);
        sync(st_);
        double r2 = 0.0;
        for (int i = 0; i < n_; ++i) r2 += (h[i] - P_->ha[i]) * (h[i] - P_->ha[i]);
        for (int j = 0; j < m_; ++j) r2 += (h[n_ + j] - P_->hb[j]) * (h[n_ + j] - P_->hb[j]);
        *mar_err = std::sqrt(r2);
        *primal = h[n_ + m_] + 0.5 * E_.ops().reg() * h[n_ + m_ + 1];
    }

    // X to an n x m FP64 destination (device or mapped host).
    void emit(double* dst) {
        const long long count = (long long)n_ * m_;
        if (mixed_) {
            k_widen<float><<<1024, 256, 0, st_>>>(reinterpret_cast<const float*>(X_.get()),
                                                  count, dst);
            count_launch();
            REGOT_CHECK_LAUNCH();
        } else {
            REGOT_CUDA(cudaMemcpyAsync(dst, X_.get(), (size_t)count * sizeof(double),
                                       cudaMemcpyDefault, st_));
        }
    }

private:
    regot_ctx* ctx_;
    QrotEngine& E_;
    regot_dproblem* P_;
    int n_, m_;
    cudaStream_t st_;
    bool mixed_;
    DBuf<char> X_;
    DBuf<double> sums_, mx_;
};

// obj and gradient at the host point x (uploaded to the engine's gamma).
double qrot_grad_at(QrotEngine& E, const HVec& x, HVec& g) {
    cudaStream_t st = E.stream();
    const size_t bytes = x.size() * sizeof(double);
    h2d(E.gamma(), x.data(), bytes, st);
    const double f = E.eval(E.gamma(), E.grad(), false);
    d2h(g.data(), E.grad(), bytes, st);
    sync(st);
    return f;
}

// f(xp + d) - f(xp) - g'd (>= 0) at the device points xp, d, from the
// trial pass; the caller adds g'd. Uploads both host vectors.
double qrot_change_rem(QrotEngine& E, DBuf<double>& xp_d, DBuf<double>& d_d, const HVec& xp,
                       const HVec& d) {
    cudaStream_t st = E.stream();
    h2d(xp_d.get(), xp.data(), xp.size() * sizeof(double), st);
    h2d(d_d.get(), d.data(), d.size() * sizeof(double), st);
    double sq = 0.0;
    return E.eval_step(xp_d.get(), d_d.get(), 1.0, &sq);
}

}  // namespace

// qrot_apdagd_internal: qrot_apdagd.cpp:14-179. dual = -gamma, phi = -f / reg;
// the averaged plan lives on the device. The line-search test
// phi_new >= phit + g'diff / reg - L/2 |diff|^2 (diff = dual_new - dualt) is,
// with f_new - f_t = -g'diff + rem, the test rem <= reg L/2 |diff|^2: mixed
// precision takes rem from the trial pass (no cancellation); FP64 evaluates
// f_new directly, as the reference does.
void qrot_apdagd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                     const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    constexpr double L0 = 1.0;
    constexpr int max_inner = 20;
    QrotEngine E(P, reg, 0.0, st);
    QrotAvgPlan X(ctx, E, P);
    DevClock clock(st);
    qrot_initial(E, o, n, m);
    HVec gamma(N), g(N), dual(N), dual_new(N), dualp(N), dualp_new(N), dualt(N), d(N);
    d2h(gamma.data(), E.gamma(), N * sizeof(double), st);
    sync(st);
    for (int q = 0; q < N; ++q) dual[q] = -gamma[q];
    dualp = dual;
    dualt = dual;
    double primal_obj = 0.0, mar_err = 0.0;
    X.update(E.gamma(), 0.0, 1.0, true, &primal_obj, &mar_err);
    DBuf<double> xp_d(N, st), d_d(N, st);
    HVec hobj, hmar, htime, hprim;

    double t0 = clock.now_ms();
    double f = qrot_grad_at(E, gamma, g);
    hobj.push_back(f);
    hmar.push_back(host_norm(g) / reg);
    htime.push_back(clock.now_ms() - t0);
    hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
    int i;
    double L = L0, pbeta = 0.0;
    for (i = 0; i < max_iter; i++) {
        t0 = clock.now_ms();
        L *= 0.5;
        double ptau = 0.0, phi_new = 0.0;
        for (int j = 0; j < max_inner; j++) {
            const double palpha = (1.0 + std::sqrt(4.0 * L * pbeta + 1.0)) / (2.0 * L);
            const double pbeta_new = pbeta + palpha;
            ptau = palpha / pbeta_new;
            for (int q = 0; q < N; ++q) {
                dualt[q] = (1.0 - ptau) * dual[q] + ptau * dualp[q];
                gamma[q] = -dualt[q];
            }
            const double ft = qrot_grad_at(E, gamma, g);
            const double phit = -ft / reg;
            double gd = 0.0, dd = 0.0;
            for (int q = 0; q < N; ++q) {
                dualp_new[q] = dualp[q] + (palpha / reg) * g[q];
                dual_new[q] = (1.0 - ptau) * dual[q] + ptau * dualp_new[q];
                const double df = dual_new[q] - dualt[q];
                gd += g[q] * df;
                dd += df * df;
            }
            bool accept;
            if (mixed) {
                for (int q = 0; q < N; ++q) d[q] = -(dual_new[q] - dualt[q]);
                const double rem = qrot_change_rem(E, xp_d, d_d, gamma, d);
                f = ft - gd + rem;
                phi_new = -f / reg;
                accept = rem <= 0.5 * L * reg * dd;
            } else {
                for (int q = 0; q < N; ++q) d[q] = -dual_new[q];
                h2d(E.gamma(), d.data(), N * sizeof(double), st);
                f = E.eval(E.gamma(), E.grad(), false);
                phi_new = -f / reg;
                accept = phi_new >= phit + gd / reg - 0.5 * L * dd;
            }
            if (o.verbose >= 2)
                std::printf("j = %d, palpha = %g, pbeta = %g, phit = %g, phi_new = %g\n", j,
                            palpha, pbeta_new, phit, phi_new);
            if (accept || j >= max_inner - 1) {
                pbeta = pbeta_new;
                dualp.swap(dualp_new);
                dual.swap(dual_new);
                break;
            }
            L *= 2.0;
        }
        // plan = (1 - ptau) plan + ptau plan(-dualt) and its statistics
        for (int q = 0; q < N; ++q) gamma[q] = -dualt[q];
        h2d(E.gamma(), gamma.data(), N * sizeof(double), st);
        X.update(E.gamma(), 1.0 - ptau, ptau, false, &primal_obj, &mar_err);
        hobj.push_back(f);
        hmar.push_back(mar_err);
        htime.push_back(htime.back() + (clock.now_ms() - t0));
        hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
        if (o.verbose >= 1)
            std::printf("iter = %d, primal_obj = %g, phi_new = %g, mar_err = %g\n", i,
                        primal_obj, phi_new, mar_err);
        if (primal_obj - phi_new <= tol && mar_err <= tol) break;
    }
    finish_qrot_with(E, E.gamma(), hobj, hmar, htime, hprim, i, o, res,
                     [&](double* dst) { X.emit(dst); });
}

// qrot_pdaam_internal: qrot_pdaam.cpp:14-188. At the extrapolated point
// dualt, the block (alpha or beta) with the larger gradient norm is
// minimised exactly on the device (optimal_alpha / optimal_beta passes);
// the test phi_new >= phit + |g|^2 / (2 L reg^2) is, with
// f_new - f_t = g'd + rem (d = gamma_new - gamma_t), the test
// g'd + rem <= -|g|^2 / (2 L reg): mixed precision takes rem from the
// trial pass, FP64 evaluates f_new directly, as the reference does.
void qrot_pdaam_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                    const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    constexpr double L0 = 1.0;
    constexpr int max_inner = 20;
    QrotEngine E(P, reg, 0.0, st);
    QrotAvgPlan X(ctx, E, P);
    DevClock clock(st);
    qrot_initial(E, o, n, m);
    HVec gamma(N), gt(N), g(N), dual(N), dualp(N), dualt(N), d(N);
    d2h(gamma.data(), E.gamma(), N * sizeof(double), st);
    sync(st);
    for (int q = 0; q < N; ++q) dual[q] = -gamma[q];
    dualp = dual;
    dualt = dual;
    double primal_obj = 0.0, mar_err = 0.0;
    X.update(E.gamma(), 0.0, 1.0, true, &primal_obj, &mar_err);
    DBuf<double> xp_d(N, st), d_d(N, st);
    HVec hobj, hmar, htime, hprim;

    double t0 = clock.now_ms();
    double f = qrot_grad_at(E, gamma, g);
    hobj.push_back(f);
    hmar.push_back(host_norm(g) / reg);
    htime.push_back(clock.now_ms() - t0);
    hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
    int i;
    double L = L0, palpha = 0.0;
    for (i = 0; i < max_iter; i++) {
        t0 = clock.now_ms();
        double L_new = 0.5 * L, phi_new = 0.0, tau_old = 0.0, tau_new = 0.0;
        for (int j = 0; j < max_inner; j++) {
            const double palpha_new =
                (1.0 + std::sqrt(4.0 * palpha * palpha * L * L_new + 1.0)) / (2.0 * L_new);
            const double ptau = 1.0 / (palpha_new * L_new);
            for (int q = 0; q < N; ++q) {
                dualt[q] = (1.0 - ptau) * dual[q] + ptau * dualp[q];
                gt[q] = -dualt[q];
            }
            const double ft = qrot_grad_at(E, gt, g);  // E.gamma() = gamma_t
            const double phit = -ft / reg;
            double lam = 0.0, mu = 0.0;
            for (int q = 0; q < n; ++q) lam += g[q] * g[q];
            for (int q = 0; q < m; ++q) mu += g[n + q] * g[n + q];
            if (lam > mu) E.optimal_alpha(E.gamma() + n, E.gamma());
            else E.optimal_beta(E.gamma(), E.gamma() + n);
            d2h(gamma.data(), E.gamma(), N * sizeof(double), st);
            sync(st);
            bool accept;
            if (mixed) {
                double gd = 0.0;
                for (int q = 0; q < N; ++q) {
                    d[q] = gamma[q] - gt[q];
                    gd += g[q] * d[q];
                }
                const double rem = qrot_change_rem(E, xp_d, d_d, gt, d);
                f = ft + (gd + rem);
                phi_new = -f / reg;
                accept = gd + rem <= -(lam + mu) / (2.0 * L_new * reg);
            } else {
                f = E.eval(E.gamma(), E.grad(), false);
                phi_new = -f / reg;
                accept = phi_new >= phit + (lam + mu) / (2.0 * L_new * reg * reg);
            }
            if (o.verbose >= 2)
                std::printf("j = %d, L = %g, palpha = %g, phit = %g, phi_new = %g\n", j, L_new,
                            palpha, phit, phi_new);
            if (accept || j >= max_inner - 1) {
                const double ar = palpha / palpha_new, lr = L / L_new;
                tau_old = ar * ar * lr;
                tau_new = ptau;
                palpha = palpha_new;
                L = L_new;
                for (int q = 0; q < N; ++q) dual[q] = -gamma[q];
                break;
            }
            L_new *= 2.0;
        }
        for (int q = 0; q < N; ++q) dualp[q] += (palpha / reg) * g[q];
        // plan = tau_old plan + tau_new plan(-dualt) and its statistics
        for (int q = 0; q < N; ++q) gamma[q] = -dualt[q];
        h2d(E.gamma(), gamma.data(), N * sizeof(double), st);
        X.update(E.gamma(), tau_old, tau_new, false, &primal_obj, &mar_err);
        hobj.push_back(f);
        hmar.push_back(mar_err);
        htime.push_back(htime.back() + (clock.now_ms() - t0));
        hprim.push_back(o.prim_vals ? E.primal(E.gamma()) : 0.0);
        if (o.verbose >= 1)
            std::printf("iter = %d, primal_obj = %g, phi_new = %g, mar_err = %g\n", i,
                        primal_obj, phi_new, mar_err);
        if (primal_obj - phi_new <= tol && mar_err <= tol) break;
    }
    finish_qrot_with(E, E.gamma(), hobj, hmar, htime, hprim, i, o, res,
                     [&](double* dst) { X.emit(dst); });
}

int force_qrot_cg_path(int mode) {
    return g_qrot_cg_path.exchange(mode >= 1 && mode <= 3 ? mode : 0);
}

}  // namespace regot

// ------------------------------------------------------- pass-level C ABI --
using namespace regot;

namespace {
template <typename F>
int qguard(regot_ctx* ctx, F&& f) {
    if (!ctx) return REGOT_ERR_INVALID_ARG;
    long long* saved = g_launch_counter;
    g_launch_counter = &ctx->launches;
    int rc = REGOT_OK;
    try {
        REGOT_CUDA(cudaSetDevice(ctx->device));
        f();
        ctx->last_error.clear();
    } catch (const Error& e) {
        ctx->last_error = e.what();
        rc = e.code;
    } catch (const std::exception& e) {
        ctx->last_error = e.what();
        rc = REGOT_ERR_NUMERIC;
    }
    g_launch_counter = saved;
    return rc;
}
}  // namespace

extern "C" {

int regot_qrot_dual_obj_grad(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                             double* obj, double* grad) {
    return qguard(ctx, [&] {
        require(P && gamma && obj && grad, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        QrotEngine E(P, reg, 0.0, ctx->stream);
        const int N = P->n + P->m;
        h2d(E.gamma(), gamma, N * sizeof(double), ctx->stream);
        *obj = E.eval(E.gamma(), E.grad(), false);
        d2h(grad, E.grad(), N * sizeof(double), ctx->stream);
        E.ops().check_err();
    });
}

int regot_qrot_optimal_beta(regot_ctx* ctx, regot_dproblem* P, double reg, const double* alpha,
                            double* beta) {
    return qguard(ctx, [&] {
        require(P && alpha && beta, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        QrotEngine E(P, reg, 0.0, ctx->stream);
        h2d(E.gamma(), alpha, P->n * sizeof(double), ctx->stream);
        E.optimal_beta(E.gamma(), E.gamma() + P->n);
        d2h(beta, E.gamma() + P->n, P->m * sizeof(double), ctx->stream);
        E.ops().check_err();
    });
}

int regot_qrot_optimal_alpha(regot_ctx* ctx, regot_dproblem* P, double reg, const double* beta,
                             double* alpha) {
    return qguard(ctx, [&] {
        require(P && alpha && beta, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        QrotEngine E(P, reg, 0.0, ctx->stream);
        h2d(E.gamma() + P->n, beta, P->m * sizeof(double), ctx->stream);
        E.optimal_alpha(E.gamma() + P->n, E.gamma());
        d2h(alpha, E.gamma(), P->n * sizeof(double), ctx->stream);
        E.ops().check_err();
    });
}

int regot_qrot_primal_val(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                          double* value) {
    return qguard(ctx, [&] {
        require(P && gamma && value, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        QrotEngine E(P, reg, 0.0, ctx->stream);
        h2d(E.gamma(), gamma, (P->n + P->m) * sizeof(double), ctx->stream);
        *value = E.primal(E.gamma());
        E.ops().check_err();
    });
}

int regot_qrot_plan(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                    double* plan, int plan_mem) {
    return qguard(ctx, [&] {
        require(P && gamma && plan, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        QrotEngine E(P, reg, 0.0, ctx->stream);
        const int n = P->n, m = P->m;
        h2d(E.gamma(), gamma, (n + m) * sizeof(double), ctx->stream);
        emit_plan(plan, plan_mem, (size_t)n * m, ctx->stream,
                  [&](double* dst) { E.plan(E.gamma(), dst); });
        E.ops().check_err();
    });
}

}  // extern "C"
