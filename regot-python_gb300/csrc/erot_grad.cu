// Backward building blocks for differentiating EROT solves: contractions of
// the weighted plan with a dense matrix, without ever forming an n x m array:
//   G_ij = T_ij                               (no adjoint given), or
//   G_ij = T_ij (u_i + u_{n+j} - W_ij) / reg  (implicit adjoint u, optional W)
//   rows:    sums_i = sum_j G_ij,  Z_ik = sum_j G_ij Y_jk   (Z = G Y)
//   columns: sums_j = sum_i G_ij,  Z_jk = sum_i G_ij X_ik   (Z = G'X)
// with T_ij = exp((alpha_i + beta_j - M_ij)/reg) recomputed from the stored
// M. With G = T the row contraction gives dL/dx = 2 (sums o x - Z) / scale of
// a squared-Euclidean cost and the column contraction dL/dy; with the
// adjoint they are the same contractions of dL/dM for a loss on the plan.
// There is no reference counterpart (the reference has no derivatives).
//
// FP32 storage (mixed precision) runs on the tensor cores (erot_tc.cu).
// FP64 storage runs k_tyy64 on the CUDA cores in FP64: a CTA owns 64 rows
// (columns) and walks the other dimension 32 at a time; the G tile is built
// in shared memory by threads laid out along the contiguous dimension of M,
// the matching 32 x d block of Y (X) is staged beside it, and each thread
// accumulates 16 of the 64 x d outputs. d <= 64 per launch; wider Y is done
// in 64-column slices.
#include <cmath>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "solvers.h"

namespace regot {

namespace {

constexpr int kTyyOwners = 64;
constexpr int kTyyK = 32;
constexpr int kTyyD = 64;

template <bool COLS>
__global__ void __launch_bounds__(256) k_tyy64(const double* __restrict__ M, long long ldm, int n,
                                               int m, const double* __restrict__ gamma,
                                               double inv_reg, const double* __restrict__ u,
                                               const double* __restrict__ W,
                                               const double* __restrict__ Y, int ldy, int d,
                                               double* __restrict__ sums, double* __restrict__ Z,
                                               int ldz) {
    __shared__ double s_g[kTyyOwners][kTyyK + 1];
    __shared__ double s_y[kTyyK][kTyyD];
    const int nown = COLS ? m : n, K = COLS ? n : m;
    const int o0 = blockIdx.x * kTyyOwners;
    // contraction layout: owner r, output quarter qd
    const int r = threadIdx.x >> 2, qd = threadIdx.x & 3;
    double acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = 0.0;
    double rsum = 0.0;
    for (int k0 = 0; k0 < K; k0 += kTyyK) {
        // G tile, built along the contiguous dimension of M: rows mode has
        // 4 threads per owner row (8 columns each), columns mode 64
        // consecutive owner columns per row of M
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            int rr, kk;
            if constexpr (COLS) {
                rr = threadIdx.x & 63;
                kk = (threadIdx.x >> 6) * 8 + c;
            } else {
                rr = threadIdx.x >> 2;
                kk = (threadIdx.x & 3) * 8 + c;
            }
            const int o = o0 + rr, k = k0 + kk;
            const int i = COLS ? k : o, j = COLS ? o : k;
            double g = 0.0;
            if (o < nown && k < K) {
                const double T = exp(((gamma[i] + gamma[n + j]) - M[(long long)i * ldm + j]) * inv_reg);
                if (u) {
                    const double w = W ? W[(long long)i * m + j] : 0.0;
                    g = T * (u[i] + u[n + j] - w) * inv_reg;
                } else {
                    g = T;
                }
            }
            s_g[rr][kk] = g;
        }
        for (int e = threadIdx.x; e < kTyyK * kTyyD; e += 256) {
            const int kk = e / kTyyD, k = e % kTyyD, row = k0 + kk;
            s_y[kk][k] = (row < K && k < d) ? Y[(long long)row * ldy + k] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 8; ++c) rsum += s_g[r][qd * 8 + c];
#pragma unroll 4
        for (int kk = 0; kk < kTyyK; ++kk) {
            const double g = s_g[r][kk];
#pragma unroll
            for (int k = 0; k < 16; ++k) acc[k] = fma(g, s_y[kk][qd * 16 + k], acc[k]);
        }
        __syncthreads();
    }
    // the four threads of an owner are adjacent lanes
    rsum += __shfl_xor_sync(0xffffffffu, rsum, 1);
    rsum += __shfl_xor_sync(0xffffffffu, rsum, 2);
    const int o = o0 + r;
    if (o >= nown) return;
    if (qd == 0 && sums) sums[o] = rsum;
    if (!Z) return;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int kk = qd * 16 + k;
        if (kk < d) Z[(long long)o * ldz + kk] = acc[k];
    }
}

// M_ij = scale sum_k (x_ik - y_jk)^2 by direct differences (no cancellation
// of |x|^2 + |y|^2 - 2 x.y), in the element type of the output. A CTA
// computes a 64 x 64 tile of M, staging 64 x 32 blocks of x and y in shared
// memory; each thread owns a 4 x 4 block of outputs.
template <typename TO>
__global__ void __launch_bounds__(256) k_sqeuclid(const TO* __restrict__ x, const TO* __restrict__ y,
                                                  int n, int m, int d, TO scale, TO* __restrict__ M,
                                                  long long ldm) {
    __shared__ TO sx[32][65];
    __shared__ TO sy[32][65];
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    TO acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = (TO)0;
    for (int k0 = 0; k0 < d; k0 += 32) {
        for (int e = threadIdx.x; e < 64 * 32; e += 256) {
            const int r = e >> 5, k = e & 31;
            sx[k][r] = (i0 + r < n && k0 + k < d) ? x[(long long)(i0 + r) * d + k0 + k] : (TO)0;
            sy[k][r] = (j0 + r < m && k0 + k < d) ? y[(long long)(j0 + r) * d + k0 + k] : (TO)0;
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
            TO xv[4], yv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) xv[a] = sx[k][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) yv[b] = sy[k][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const TO t = xv[a] - yv[b];
                    acc[a][b] = fma(t, t, acc[a][b]);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int i = i0 + ty + 16 * a;
        if (i >= n) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int j = j0 + tx + 16 * b;
            if (j < m) M[(long long)i * ldm + j] = acc[a][b] * scale;
        }
    }
}

}  // namespace

void sqeuclid_gpu(const void* x, const void* y, int n, int m, int d, double scale, bool fp64,
                  void* M, long long ldm, cudaStream_t st) {
    const dim3 grid(cdiv(m, 64), cdiv(n, 64));
    if (fp64)
        k_sqeuclid<double><<<grid, 256, 0, st>>>(static_cast<const double*>(x),
                                                 static_cast<const double*>(y), n, m, d, scale,
                                                 static_cast<double*>(M), ldm);
    else
        k_sqeuclid<float><<<grid, 256, 0, st>>>(static_cast<const float*>(x),
                                                static_cast<const float*>(y), n, m, d,
                                                (float)scale, static_cast<float*>(M), ldm);
    count_launch();
    REGOT_CHECK_LAUNCH();
}

void erot_contract_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, const double* d_gamma,
                       const double* d_u, const double* d_W, const double* d_Y, int d, bool cols,
                       double* d_sums, double* d_Z) {
    if (P->prec == REGOT_PREC_MIXED) {
        erot_contract_tc(ctx, P, reg, d_gamma, d_u, d_W, d_Y, d, cols, d_sums, d_Z);
        return;
    }
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m;
    const int blocks = cdiv(cols ? m : n, kTyyOwners);
    for (int k0 = 0; k0 < d || (d == 0 && k0 == 0); k0 += kTyyD) {
        const int dk = std::min(kTyyD, d - k0);
        double* sums = k0 == 0 ? d_sums : nullptr;  // the sums once
        double* Z = d_Z ? d_Z + k0 : nullptr;
        const double* Y = d_Y ? d_Y + k0 : nullptr;
        if (cols)
            k_tyy64<true><<<blocks, 256, 0, st>>>(static_cast<const double*>(P->M), P->ldm, n, m,
                                                  d_gamma, 1.0 / reg, d_u, d_W, Y, d, dk, sums, Z,
                                                  d);
        else
            k_tyy64<false><<<blocks, 256, 0, st>>>(static_cast<const double*>(P->M), P->ldm, n, m,
                                                   d_gamma, 1.0 / reg, d_u, d_W, Y, d, dk, sums,
                                                   Z, d);
        count_launch();
        REGOT_CHECK_LAUNCH();
        if (d == 0) break;
    }
}

}  // namespace regot
