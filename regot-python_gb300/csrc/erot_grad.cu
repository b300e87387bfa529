// Backward building blocks for differentiating EROT solves.
//
// k_tyy contracts the weighted plan with a dense m x d matrix without ever
// forming an n x m array:
//   G_ij = T_ij                               (no adjoint given), or
//   G_ij = T_ij (u_i + u_{n+j} - W_ij) / reg  (implicit adjoint u, optional W)
//   rows_i = sum_j G_ij,  Z_ik = sum_j G_ij Y_jk,
// with T_ij = exp((alpha_i + beta_j - M_ij)/reg) recomputed from the stored M
// exactly as the dense passes form it (mixed: FP32 hi/lo split of the duals,
// ex2.approx; FP64: exp). With G = T this is dL/dx of a squared-Euclidean
// cost, 2 (rows o x - T y) / scale; with the adjoint it is the same
// contraction of dL/dM for a loss on the plan. There is no reference
// counterpart (the reference has no derivatives).
//
// A CTA owns 64 rows and loops over the columns 32 at a time: the G tile is
// built in shared memory (each thread 8 entries of one row), the matching
// 32 x d block of Y is staged beside it, and each thread accumulates 16 of
// the 64 x d outputs. d <= 64 per launch; wider Y is done in 64-column
// slices. 2 n m d FMAs in the pass's element type: 2.1 GFLOP at n = m = 4096,
// d = 64, well under the time of the solve it differentiates.
#include <cmath>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "solvers.h"

namespace regot {

namespace {

constexpr int kTyyRows = 64;
constexpr int kTyyCols = 32;
constexpr int kTyyD = 64;

__device__ __forceinline__ float ex2_approx_f32(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

template <typename TM>
__global__ void __launch_bounds__(256) k_tyy(const TM* __restrict__ M, long long ldm, int n, int m,
                                             const float4* __restrict__ rs,
                                             const float4* __restrict__ cs,
                                             const double* __restrict__ gamma, float kexp_f,
                                             double inv_reg, const double* __restrict__ u,
                                             const double* __restrict__ W,
                                             const double* __restrict__ Y, int ldy, int d,
                                             double* __restrict__ rows, double* __restrict__ Z,
                                             int ldz) {
    constexpr bool MIXED = std::is_same<TM, float>::value;
    __shared__ TM s_g[kTyyRows][kTyyCols + 1];
    __shared__ TM s_y[kTyyCols][kTyyD];
    const int r = threadIdx.x >> 2, qd = threadIdx.x & 3;
    const int i = blockIdx.x * kTyyRows + r;
    const bool row_ok = i < n;
    float4 ri = make_float4(0.f, 0.f, 0.f, 0.f);
    double ai = 0.0, ui = 0.0;
    if (row_ok) {
        if constexpr (MIXED) ri = rs[i];
        else ai = gamma[i];
        if (u) ui = u[i];
    }
    const float rlk = __fmul_rn(ri.y, kexp_f);
    TM acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = (TM)0;
    double rsum = 0.0;
    for (int j0 = 0; j0 < m; j0 += kTyyCols) {
        // G tile: row r, columns qd*8 .. qd*8+7 of this chunk
        TM part = (TM)0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int jj = qd * 8 + c, j = j0 + jj;
            TM g = (TM)0;
            if (row_ok && j < m) {
                const TM mv = M[(long long)i * ldm + j];
                TM T;
                if constexpr (MIXED) {
                    const float4 cj = cs[j];
                    const float s = (ri.x + cj.x) - mv;
                    T = ex2_approx_f32(fmaf(s, kexp_f, __fadd_rn(rlk, __fmul_rn(cj.y, kexp_f))));
                } else {
                    T = exp(((ai + gamma[n + j]) - mv) * inv_reg);
                }
                if (u) {
                    const double w = W ? W[(long long)i * m + j] : 0.0;
                    g = (TM)((double)T * (ui + u[n + j] - w) * inv_reg);
                } else {
                    g = T;
                }
            }
            s_g[r][jj] = g;
            part += g;
        }
        rsum += (double)part;
        for (int e = threadIdx.x; e < kTyyCols * kTyyD; e += 256) {
            const int jj = e / kTyyD, k = e % kTyyD, j = j0 + jj;
            s_y[jj][k] = (j < m && k < d) ? (TM)Y[(long long)j * ldy + k] : (TM)0;
        }
        __syncthreads();
#pragma unroll 4
        for (int jj = 0; jj < kTyyCols; ++jj) {
            const TM g = s_g[r][jj];
#pragma unroll
            for (int k = 0; k < 16; ++k) acc[k] = fma(g, s_y[jj][qd * 16 + k], acc[k]);
        }
        __syncthreads();
    }
    // the four threads of a row are adjacent lanes
    rsum += __shfl_xor_sync(0xffffffffu, rsum, 1);
    rsum += __shfl_xor_sync(0xffffffffu, rsum, 2);
    if (!row_ok) return;
    if (qd == 0 && rows) rows[i] = rsum;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int kk = qd * 16 + k;
        if (kk < d) Z[(long long)i * ldz + kk] = (double)acc[k];
    }
}

}  // namespace

void erot_tyy_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, const double* d_gamma,
                  const double* d_u, const double* d_W, const double* d_Y, int d, double* d_rows,
                  double* d_Z) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    ErotOps ops(P, reg, st);
    DBuf<float4> rs, cs;
    DBuf<double> mx(1, st);
    if (mixed) {
        rs.alloc(n, st);
        cs.alloc(m, st);
        ops.maxabs(d_gamma, n + m, nullptr, 0, mx.get());
        PassParams p = ops.base_params();
        p.ra = d_gamma;
        p.cb = d_gamma + n;
        p.grid = mx.get();
        launch_split(p, rs.get(), cs.get(), nullptr, st);
    }
    const float kexp_f = (float)(1.4426950408889634 / reg);
    const int blocks = cdiv(n, kTyyRows);
    for (int k0 = 0; k0 < d || (d == 0 && k0 == 0); k0 += kTyyD) {
        const int dk = std::min(kTyyD, d - k0);
        double* rows = k0 == 0 ? d_rows : nullptr;  // the row sums once
        if (mixed)
            k_tyy<float><<<blocks, 256, 0, st>>>(
                static_cast<const float*>(P->M), P->ldm, n, m, rs.get(), cs.get(), d_gamma,
                kexp_f, 1.0 / reg, d_u, d_W, d_Y + k0, d, dk, rows, d_Z + k0, d);
        else
            k_tyy<double><<<blocks, 256, 0, st>>>(
                static_cast<const double*>(P->M), P->ldm, n, m, nullptr, nullptr, d_gamma,
                kexp_f, 1.0 / reg, d_u, d_W, d_Y + k0, d, dk, rows, d_Z + k0, d);
        count_launch();
        REGOT_CHECK_LAUNCH();
        if (d == 0) break;
    }
}

}  // namespace regot
