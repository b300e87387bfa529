// Batched sinkhorn_bcd: many independent EROT problems with squared-
// Euclidean costs computed on the fly, solved together (the reference solves
// one problem per call; its BCD is src/sinkhorn_bcd.cpp:14-124).
//
// Layout: the problems' points, marginals and duals are concatenated; per-
// problem offsets locate them. A problem is assigned a dimension class
// DP in {4, 8, 16} (d rounded up), its points are zero-padded to DP in
// registers and shared memory, and each class has its own row and column
// kernels, so a 3-D problem does not pay for 16 dimensions.
//
// One sweep = row kernels (one CTA per 32 rows of a problem: every CTA sees
// whole rows, so the new alpha and the row sums of the iterate come out of
// it directly), a finalize kernel (one warp per problem: marginal error,
// stopping test, per-problem done mask), and column kernels (one CTA per 32
// columns, new beta in place). Each element costs DP subtractions and FMAs
// for the distance, one FMA for the exponent and one ex2: the sweep is bound
// by FP32 issue and the SFU, not by memory (nothing n x m is stored).
//
// Log-sum-exp: each lane keeps a running (max, scaled sum) in base 2, so no
// anchor has to be right in advance (the first sweep starts from alpha = 0,
// where a row far from every column would underflow a fixed anchor); the
// exponent is ((hi_i + hi_j) - M_ij) k + (lo_i + lo_j) k with the duals split
// on a common FP32 grid as in the dense passes, so hi_i + hi_j is exact.
//
// The sweeps run as a device-side loop (a conditional WHILE graph node whose
// body is two sweeps and a loop kernel): it continues while a problem is
// running, no dual has left the split grid, and fewer than max_iter / 2 + 3
// bodies have run. Once few problems are left, the rest of their sweeps run
// in one launch of the tail kernel (k_btail: a thread-block cluster per
// problem, cluster barriers in place of kernel boundaries).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "device_util.cuh"
#include "sm100_util.cuh"
#include "solvers.h"

namespace regot {

namespace {

constexpr int kBWarps = 8;
constexpr int kBPer = 4;                    // rows (columns) per warp
constexpr int kBItems = kBWarps * kBPer;    // rows (columns) per CTA
constexpr int kBTile = 256;                 // columns (rows) staged per tile
constexpr int kBClasses = 3;
constexpr int kBClassDim[kBClasses] = {4, 8, 16};

struct BatchDev {
    const int* n;
    const int* m;
    const int* d;
    const float* scale;
    const long long* xo;  // offsets of the points of problem p (floats)
    const long long* yo;
    const int* ro;        // offsets into the concatenated row / column vectors
    const int* co;
    const int* rbo;       // offsets of the problem's row blocks (partials)
    const float* X;
    const float* Y;
    const double* a;
    const double* loga;
    const double* logb;
};

struct BatchState {
    int active;     // problems still running
    int regrid;     // a dual reached the bound of the split grid
    int loops;
    int loop_cap;
    int stop_below;  // leave the device loop when this few problems still run
    int err;         // a bounded wait of a tensor-core sweep gave up
    double maxabs;  // max |dual| for the grid
    double g, inv_g, bound;
};

__device__ __forceinline__ float bex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Running log-sum-exp in base 2: sum 2^z = 2^mx * s. The reference point mx
// only moves when a term exceeds it by 2^16, so terms stay below 2^16 and
// the rescaling branch is rare after the first term (mx starts at -inf).
constexpr float kLseSlack = 16.f;

__device__ __forceinline__ void lse_add(float& mx, float& s, float z) {
    if (z > mx + kLseSlack) {
        s = fmaf(s, bex2(mx - z), 1.f);
        mx = z;
    } else {
        s += bex2(z - mx);
    }
}

// Four terms (one per row or column of the lane): the common case adds
// without a branch per term.
__device__ __forceinline__ void lse_add4(float (&mx)[4], float (&s)[4], const float (&z)[4]) {
    const bool slow = (z[0] > mx[0] + kLseSlack) | (z[1] > mx[1] + kLseSlack) |
                      (z[2] > mx[2] + kLseSlack) | (z[3] > mx[3] + kLseSlack);
    if (slow) {
#pragma unroll
        for (int r = 0; r < 4; ++r) lse_add(mx[r], s[r], z[r]);
    } else {
#pragma unroll
        for (int r = 0; r < 4; ++r) s[r] += bex2(z[r] - mx[r]);
    }
}

__device__ __forceinline__ void lse_merge(float& mx, float& s, float m2, float s2) {
    const float m = fmaxf(mx, m2);
    s = (m == -INFINITY) ? 0.f : s * bex2(mx - m) + s2 * bex2(m2 - m);
    mx = m;
}

// Costs of two pairs at once, u = x and v = -y per dimension (the row
// kernel pairs two rows with one column, the column kernel one row with two
// columns). The packed FP32x2 instructions round each half exactly as the
// scalar fadd / ffma / fmul would, so both kernels produce the same M_ij.
// Four partial sums over the dimensions (k mod 4) keep the FMA chains short:
// with one running sum the kernels were bound by its latency.
template <int DP>
__device__ __forceinline__ float2 bcost2(const float2 (&u)[DP], const float2 (&v)[DP],
                                         float2 sc2) {
    float2 s[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) s[q] = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < DP; ++k) {
        const float2 t = __fadd2_rn(u[k], v[k]);
        s[k & 3] = __ffma2_rn(t, t, s[k & 3]);
    }
    return __fmul2_rn(__fadd2_rn(__fadd2_rn(s[0], s[1]), __fadd2_rn(s[2], s[3])), sc2);
}

// Exponent of T in base 2 for two pairs: ((hi_i + hi_j) - M) k + (lo_i k + lo_j k).
__device__ __forceinline__ float2 bexpo2(float2 hi_i, float2 hi_j, float2 lok_i, float2 lok_j,
                                         float2 M, float2 k2) {
    const float2 e = __fadd2_rn(__fadd2_rn(hi_i, hi_j), make_float2(-M.x, -M.y));
    return __ffma2_rn(e, k2, __fadd2_rn(lok_i, lok_j));
}

// The row and column results are formed with FP32 transcendentals (log2f,
// exp2f of the fractional part, the power of two applied in FP64): FP64
// arithmetic issues at a small fraction of the FP32 rate on this part, and
// the FP64 log / exp of the epilogues took as long as the element loop of a
// small problem. log2f is accurate to about 1e-7 relative, which moves a
// dual by ~1e-7 reg, far below what the 1e-6 marginal tolerance resolves.
__device__ __forceinline__ double row_sum(float mx, float s) {
    const float fl = floorf(mx);
    return ldexp((double)(s * exp2f(mx - fl)), (int)fl);
}

__device__ __forceinline__ float2 bsplit(double v, const BatchState* st, int* regrid) {
    if (!(fabs(v) < st->bound)) atomicOr(regrid, 1);
    const double h = rint(v * st->inv_g) * st->g;
    return make_float2((float)h, (float)(v - h));
}

// Loads of vectors that other CTAs write during the same launch (the tail
// kernel below): COH = true reads them at L2 (ld.global.cg), past any copy
// in L1 or the read-only path; the per-sweep kernels read them plainly.
template <bool COH, typename T>
__device__ __forceinline__ T bld(const T* p) {
    if constexpr (COH) return __ldcg(p);
    else return *p;
}

// Row half-sweep of iterate k for the row blocks `items` (problem, block):
// S_i = sum_j exp((alpha_i + beta_j - M_ij)/reg) at (alpha_k, beta_k), the
// new alpha_i = alpha_i + reg (log a_i - log S_i) (sinkhorn_problem_bcd.cpp:
// 177-201 with the current alpha as shift) with its split, and the block's
// sum of (S_i - a_i)^2 for the marginal error. A dual leaving the split
// grid sets *rgf. The column tile is staged in the caller's shared memory:
// spts holds kBTile x (DP + 1) pairs, spar kBTile pairs.
template <int DP, bool COH = false>
__device__ __forceinline__ void row_item(const BatchDev& B, int2 it, const float2* __restrict__ as_cur,
                                         const float2* __restrict__ bs,
                                         const double* __restrict__ alpha_cur, double* alpha_next,
                                         float2* as_next, double* part, BatchState* st, int* rgf,
                                         float k2, double reg, float2* spts, float2* spar) {
    const int p = it.x;
    const int n = B.n[p], m = B.m[p], d = B.d[p];
    const float sc = B.scale[p];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = it.y * kBItems + warp * kBPer;
    const float* X = B.X + B.xo[p];
    const float* Y = B.Y + B.yo[p];
    const int ro = B.ro[p], co = B.co[p];

    // rows in pairs: xp[h][k] = (x_{2h}[k], x_{2h+1}[k])
    float2 xp[kBPer / 2][DP], ah[kBPer / 2], al[kBPer / 2];
    float mx[kBPer], sm[kBPer];
#pragma unroll
    for (int r = 0; r < kBPer; ++r) {
        const int i = i0 + r;
        const bool ok = i < n;
#pragma unroll
        for (int k = 0; k < DP; ++k) {
            const float v = (ok && k < d) ? X[(long long)i * d + k] : 0.f;
            if (r & 1) xp[r >> 1][k].y = v;
            else xp[r >> 1][k].x = v;
        }
        const float2 s = ok ? bld<COH>(as_cur + ro + i) : make_float2(0.f, 0.f);
        const float lk = __fmul_rn(s.y, k2);
        if (r & 1) {
            ah[r >> 1].y = s.x;
            al[r >> 1].y = lk;
        } else {
            ah[r >> 1].x = s.x;
            al[r >> 1].x = lk;
        }
        mx[r] = -INFINITY;
        sm[r] = 0.f;
    }
    const float2 sc2 = make_float2(sc, sc), k22 = make_float2(k2, k2);
    // columns staged negated and duplicated, (-y, -y), ready for the packed
    // instructions (rows padded by one entry against bank conflicts)
    float2 (*sy)[DP + 1] = reinterpret_cast<float2 (*)[DP + 1]>(spts);
    float2* sb = spar;
    for (int j0 = 0; j0 < m; j0 += kBTile) {
        const int cnt = min(kBTile, m - j0);
        for (int e = threadIdx.x; e < kBTile * DP; e += kBWarps * 32) {
            const int jj = e / DP, k = e % DP;
            const float v = (jj < cnt && k < d) ? -Y[(long long)(j0 + jj) * d + k] : 0.f;
            sy[jj][k] = make_float2(v, v);
        }
        for (int jj = threadIdx.x; jj < kBTile; jj += kBWarps * 32)
            sb[jj] = jj < cnt ? bld<COH>(bs + co + j0 + jj) : make_float2(0.f, 0.f);
        __syncthreads();
        for (int jj = lane; jj < cnt; jj += 32) {
            float2 ny[DP];
#pragma unroll
            for (int k = 0; k < DP; ++k) ny[k] = sy[jj][k];
            const float2 bj = sb[jj];
            const float blk = __fmul_rn(bj.y, k2);
            float z[kBPer];
#pragma unroll
            for (int h = 0; h < kBPer / 2; ++h) {
                const float2 Mv = bcost2<DP>(xp[h], ny, sc2);
                const float2 zz = bexpo2(ah[h], make_float2(bj.x, bj.x), al[h],
                                         make_float2(blk, blk), Mv, k22);
                z[2 * h] = zz.x;
                z[2 * h + 1] = zz.y;
            }
            lse_add4(mx, sm, z);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < kBPer; ++r)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float m2 = __shfl_xor_sync(0xffffffffu, mx[r], o);
            const float s2 = __shfl_xor_sync(0xffffffffu, sm[r], o);
            lse_merge(mx[r], sm[r], m2, s2);
        }
    // lane r < kBPer finishes row i0 + r in FP64
    double g2 = 0.0;
    float mxr = mx[0], smr = sm[0];
#pragma unroll
    for (int r = 1; r < kBPer; ++r)
        if (lane == r) {
            mxr = mx[r];
            smr = sm[r];
        }
    const int i = i0 + lane;
    if (lane < kBPer && i < n) {
        const double lg2 = (double)mxr + (double)log2f(smr);  // log2 S_i
        const double S = row_sum(mxr, smr);
        const double gi = S - B.a[ro + i];
        g2 = gi * gi;
        const double an =
            bld<COH>(alpha_cur + ro + i) + reg * (B.loga[ro + i] - 0.69314718055994531 * lg2);
        alpha_next[ro + i] = an;
        as_next[ro + i] = bsplit(an, st, rgf);
    }
    // block partial of sum (S_i - a_i)^2 in a fixed order
    __shared__ double s_g2[kBWarps];
    g2 += __shfl_xor_sync(0xffffffffu, g2, 1);
    g2 += __shfl_xor_sync(0xffffffffu, g2, 2);
    if (lane == 0) s_g2[warp] = g2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kBWarps; ++w) t += s_g2[w];
        part[B.rbo[p] + it.y] = t;
    }
}

// One CTA per work item; the CTAs of finished problems return at once.
// (Persistent CTAs fetching items from a counter measured 1.8x slower on the
// batched workload: the hardware block scheduler balances these short
// CTAs better.)
template <int DP>
__global__ void __launch_bounds__(kBWarps * 32) k_brow(
    const BatchDev B, const int2* __restrict__ items, const float2* __restrict__ as_cur,
    const float2* __restrict__ bs, const double* __restrict__ alpha_cur, double* alpha_next,
    float2* as_next, double* part, const int* __restrict__ done, BatchState* st, float k2,
    double reg) {
    const int2 it = items[blockIdx.x];
    if (done[it.x]) return;
    __shared__ float2 sy[kBTile][DP + 1];
    __shared__ float2 sb[kBTile];
    row_item<DP>(B, it, as_cur, bs, alpha_cur, alpha_next, as_next, part, st, &st->regrid, k2, reg,
                 &sy[0][0], sb);
}


// Column half-sweep for the column blocks `items`: with the new alpha,
// S_j = sum_i exp((alpha_i + beta_j - M_ij)/reg) and beta_j += reg (log b_j -
// log S_j) in place (sinkhorn_problem_bcd.cpp:149-174, current beta as
// shift). write_split = 0 skips the split (first half-sweep, before the grid
// is known).
template <int DP, bool COH = false>
__device__ __forceinline__ void col_item(const BatchDev& B, int2 it, const float2* __restrict__ as,
                                         float2* bs, double* beta, BatchState* st, int* rgf,
                                         float k2, double reg, int write_split, float2* spts,
                                         float2* spar) {
    const int p = it.x;
    const int n = B.n[p], m = B.m[p], d = B.d[p];
    const float sc = B.scale[p];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j0c = it.y * kBItems + warp * kBPer;
    const float* X = B.X + B.xo[p];
    const float* Y = B.Y + B.yo[p];
    const int ro = B.ro[p], co = B.co[p];

    // columns in pairs, negated: ny[h][k] = (-y_{2h}[k], -y_{2h+1}[k])
    float2 ny[kBPer / 2][DP], bh[kBPer / 2], bl[kBPer / 2];
    float mx[kBPer], sm[kBPer];
#pragma unroll
    for (int r = 0; r < kBPer; ++r) {
        const int j = j0c + r;
        const bool ok = j < m;
#pragma unroll
        for (int k = 0; k < DP; ++k) {
            const float v = (ok && k < d) ? -Y[(long long)j * d + k] : 0.f;
            if (r & 1) ny[r >> 1][k].y = v;
            else ny[r >> 1][k].x = v;
        }
        const float2 s = ok ? bld<COH>(bs + co + j) : make_float2(0.f, 0.f);
        const float lk = __fmul_rn(s.y, k2);
        if (r & 1) {
            bh[r >> 1].y = s.x;
            bl[r >> 1].y = lk;
        } else {
            bh[r >> 1].x = s.x;
            bl[r >> 1].x = lk;
        }
        mx[r] = -INFINITY;
        sm[r] = 0.f;
    }
    const float2 sc2 = make_float2(sc, sc), k22 = make_float2(k2, k2);
    // rows staged duplicated, (x, x), for the packed instructions
    float2 (*sx)[DP + 1] = reinterpret_cast<float2 (*)[DP + 1]>(spts);
    float2* sa = spar;
    for (int i0 = 0; i0 < n; i0 += kBTile) {
        const int cnt = min(kBTile, n - i0);
        for (int e = threadIdx.x; e < kBTile * DP; e += kBWarps * 32) {
            const int ii = e / DP, k = e % DP;
            const float v = (ii < cnt && k < d) ? X[(long long)(i0 + ii) * d + k] : 0.f;
            sx[ii][k] = make_float2(v, v);
        }
        for (int ii = threadIdx.x; ii < kBTile; ii += kBWarps * 32)
            sa[ii] = ii < cnt ? bld<COH>(as + ro + i0 + ii) : make_float2(0.f, 0.f);
        __syncthreads();
        for (int ii = lane; ii < cnt; ii += 32) {
            float2 xv[DP];
#pragma unroll
            for (int k = 0; k < DP; ++k) xv[k] = sx[ii][k];
            const float2 ai = sa[ii];
            const float alk = __fmul_rn(ai.y, k2);
            float z[kBPer];
#pragma unroll
            for (int h = 0; h < kBPer / 2; ++h) {
                // the same operations, in the same order, as the row kernel
                const float2 Mv = bcost2<DP>(xv, ny[h], sc2);
                const float2 zz = bexpo2(make_float2(ai.x, ai.x), bh[h], make_float2(alk, alk),
                                         bl[h], Mv, k22);
                z[2 * h] = zz.x;
                z[2 * h + 1] = zz.y;
            }
            lse_add4(mx, sm, z);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < kBPer; ++r)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float m2 = __shfl_xor_sync(0xffffffffu, mx[r], o);
            const float s2 = __shfl_xor_sync(0xffffffffu, sm[r], o);
            lse_merge(mx[r], sm[r], m2, s2);
        }
    float mxr = mx[0], smr = sm[0];
#pragma unroll
    for (int r = 1; r < kBPer; ++r)
        if (lane == r) {
            mxr = mx[r];
            smr = sm[r];
        }
    const int j = j0c + lane;
    if (lane < kBPer && j < m) {
        const double lg2 = (double)mxr + (double)log2f(smr);
        const double bn =
            bld<COH>(beta + co + j) + reg * (B.logb[co + j] - 0.69314718055994531 * lg2);
        beta[co + j] = bn;
        if (write_split) bs[co + j] = bsplit(bn, st, rgf);
    }
}

template <int DP>
__global__ void __launch_bounds__(kBWarps * 32) k_bcol(
    const BatchDev B, const int2* __restrict__ items, const float2* __restrict__ as, float2* bs,
    double* beta, const int* __restrict__ done, BatchState* st, float k2, double reg,
    int write_split) {
    const int2 it = items[blockIdx.x];
    if (done[it.x]) return;
    __shared__ float2 sx[kBTile][DP + 1];
    __shared__ float2 sa[kBTile];
    col_item<DP>(B, it, as, bs, beta, st, &st->regrid, k2, reg, write_split, &sx[0][0], sa);
}

// ---- tensor-core variant of the half-sweeps ----
// The cost tile x y' on the fifth-generation tensor cores: a CTA owns 128
// points of one side of a problem (the MMA's M = 128 rows, one TMEM lane
// each) and walks the other side in tiles of 256 points (N = 256). Both
// sides' points, zero-padded to 16 dimensions, are split into TF32 hi + lo
// parts (hi = x rounded to TF32, lo = the rest rounded to TF32: x = hi + lo
// to about 2^-22 relative) and stored K-major in shared memory; one thread
// issues, per 8-wide K step, hi*hi + hi*lo + lo*hi (TF32x3) into an FP32
// accumulator of 128 lanes x 256 columns in tensor memory. The epilogue
// reads each thread's row of the tile (tcgen05.ld) and forms
// M_ij = s (|x_i|^2 + |y_j|^2 - 2 x_i.y_j) before the same split exponent
// and running log-sum-exp as the CUDA-core kernels. The expansion loses the
// direct difference's relative accuracy on small distances: M carries an
// absolute error of about 2^-21 s (|x_i|^2 + |y_j|^2), which the batched
// tests measure against the direct difference. Which variant a dimension
// class uses is chosen by timing (see the host code).
constexpr int kTcOwn = 128;
constexpr int kTcTile = 256;
constexpr int kTcK = 16;
constexpr uint32_t kTcLbo = 128, kTcSbo = 512;  // K-major TF32 core matrices (8 rows x 16 B)
constexpr uint32_t kTcABytes = (kTcOwn / 8) * kTcSbo;
constexpr uint32_t kTcBBytes = (kTcTile / 8) * kTcSbo;
// Dynamic shared memory per CTA: the tiles and the per-point parameters;
// requested at 100 KB so that at most two CTAs share an SM, whose tensor
// memory (512 columns) then holds both accumulators.
constexpr size_t kTcSmem = 100 * 1024;
static_assert(2 * (size_t)kTcABytes + 2 * (size_t)kTcBBytes + kTcTile * 16 + 1024 <= kTcSmem,
              "tensor-core sweep tiles exceed the requested shared memory");
constexpr uint32_t kTcTmemCols = 256;
constexpr long long kTcPolls = 1LL << 14;

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Point row r (16 values) into the hi / lo tiles.
__device__ __forceinline__ void tc_put_point(unsigned char* hi, unsigned char* lo, int r,
                                             const float (&v)[kTcK]) {
#pragma unroll
    for (int kg = 0; kg < kTcK / 4; ++kg) {
        float h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            h[e] = tf32_rna(v[4 * kg + e]);
            l[e] = tf32_rna(v[4 * kg + e] - h[e]);
        }
        const uint32_t off = (uint32_t)(r >> 3) * kTcSbo + (uint32_t)kg * kTcLbo + (uint32_t)(r & 7) * 16;
        *reinterpret_cast<float4*>(hi + off) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(lo + off) = make_float4(l[0], l[1], l[2], l[3]);
    }
}

// Half-sweep with the cost tile on the tensor cores. COLS = false: the row
// half-sweep of row_item (items are blocks of 128 rows; each warp of the
// first four writes the marginal-error partial of its 32 rows, the layout
// k_bfin reads); COLS = true: the column half-sweep of col_item.
template <bool COLS>
__global__ void __launch_bounds__(256, 1) k_bsweep_tc(
    const BatchDev B, const int2* __restrict__ items, const float2* __restrict__ own_split,
    const float2* __restrict__ oth_split, const double* __restrict__ own_cur, double* own_next,
    float2* own_split_next, double* part, const int* __restrict__ done, BatchState* st, float k2,
    double reg, int write_split) {
    const int2 it = items[blockIdx.x];
    const int p = it.x;
    if (done[p]) return;
    extern __shared__ unsigned char tc_raw[];
    unsigned char* smem = tc_raw + ((1024 - (sm100::smem_u32(tc_raw) & 1023)) & 1023);
    unsigned char* Ahi = smem;
    unsigned char* Alo = Ahi + kTcABytes;
    unsigned char* Bhi = Alo + kTcABytes;
    unsigned char* Blo = Bhi + kTcBBytes;
    float4* sp = reinterpret_cast<float4*>(Blo + kTcBBytes);  // other point: |y|^2, hi, lo k
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_tmem;
    __shared__ float s_mx[kTcOwn], s_sm[kTcOwn];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r = tid & (kTcOwn - 1), half = tid >> 7;
    const int n = B.n[p], m = B.m[p], d = B.d[p];
    const int n_own = COLS ? m : n, n_oth = COLS ? n : m;
    const float* Po = COLS ? B.Y + B.yo[p] : B.X + B.xo[p];
    const float* Pt = COLS ? B.X + B.xo[p] : B.Y + B.yo[p];
    const int oo = COLS ? B.co[p] : B.ro[p], ot = COLS ? B.ro[p] : B.co[p];
    const float sc = B.scale[p];
    const int o = it.y * kTcOwn + r;
    const bool own_ok = o < n_own;

    // own point: row r of A (written by the first 128 threads), its squared
    // norm and split dual (both halves keep them)
    float v[kTcK];
    float own_sq = 0.f;
#pragma unroll
    for (int k = 0; k < kTcK; ++k) {
        v[k] = (own_ok && k < d) ? Po[(long long)o * d + k] : 0.f;
        own_sq = __fmaf_rn(v[k], v[k], own_sq);
    }
    if (half == 0) tc_put_point(Ahi, Alo, r, v);
    const float2 osp = own_ok ? own_split[oo + o] : make_float2(0.f, 0.f);
    const float oh = osp.x, olk = __fmul_rn(osp.y, k2);

    if (tid == 0) {
        sm100::mbar_init(&s_bar, 1);
        sm100::fence_mbar_init();
    }
    if (warp == 0) {
        sm100::tmem_alloc(&s_tmem, kTcTmemCols);
        sm100::tmem_relinquish();
    }
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = s_tmem;
    constexpr uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcTile >> 3) << 17) |
                               ((uint32_t)(kTcOwn >> 4) << 24);
    const uint32_t ah = sm100::smem_u32(Ahi), al = sm100::smem_u32(Alo);
    const uint32_t bh = sm100::smem_u32(Bhi), bl = sm100::smem_u32(Blo);

    // running log-sum-exp: one reference point, four partial sums (four
    // independent add chains per thread)
    float mx = -INFINITY, sm4[4] = {0.f, 0.f, 0.f, 0.f};
    bool failed = false;
    int tile = 0;
    for (int j0 = 0; j0 < n_oth; j0 += kTcTile, ++tile) {
        // other points of the tile: row tid of B and its parameters
        {
            const int j = j0 + tid;
            const bool ok = j < n_oth;
            float w[kTcK];
            float sq = 0.f;
#pragma unroll
            for (int k = 0; k < kTcK; ++k) {
                w[k] = (ok && k < d) ? Pt[(long long)j * d + k] : 0.f;
                sq = __fmaf_rn(w[k], w[k], sq);
            }
            tc_put_point(Bhi, Blo, tid, w);
            const float2 s2 = ok ? oth_split[ot + j] : make_float2(0.f, 0.f);
            sp[tid] = make_float4(sq, s2.x, __fmul_rn(s2.y, k2), 0.f);
        }
        sm100::fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kTcK / 8; ++ks) {
                const uint64_t dah = sm100::smem_desc(ah + ks * 2 * kTcLbo, kTcLbo, kTcSbo);
                const uint64_t dal = sm100::smem_desc(al + ks * 2 * kTcLbo, kTcLbo, kTcSbo);
                const uint64_t dbh = sm100::smem_desc(bh + ks * 2 * kTcLbo, kTcLbo, kTcSbo);
                const uint64_t dbl = sm100::smem_desc(bl + ks * 2 * kTcLbo, kTcLbo, kTcSbo);
                sm100::mma_tf32(tmem, dah, dbh, idesc, ks != 0 ? 1u : 0u);
                sm100::mma_tf32(tmem, dah, dbl, idesc, 1u);
                sm100::mma_tf32(tmem, dal, dbh, idesc, 1u);
            }
            sm100::mma_commit(&s_bar);
        }
        const bool ok = sm100::mbar_wait(&s_bar, (uint32_t)(tile & 1), kTcPolls);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        sm100::tc_fence_after();
        const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
        const int cnt = min(kTcTile, n_oth - j0);  // valid columns of the tile
#pragma unroll 1
        for (int x = 0; x < 8; ++x) {
            const int c0 = half * 128 + 16 * x;
            float dv[16];
            sm100::tmem_ld16(trow + (uint32_t)c0, dv);
            if (!own_ok || c0 >= cnt) continue;
            float z[16];
            float zmax = -INFINITY;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const float4 q = sp[c0 + e];
                const float Mij = __fmul_rn(__fmaf_rn(-2.f, dv[e], __fadd_rn(own_sq, q.x)), sc);
                const float ex = __fadd_rn(__fadd_rn(oh, q.y), -Mij);
                z[e] = (c0 + e < cnt) ? __fmaf_rn(ex, k2, __fadd_rn(olk, q.z)) : -INFINITY;
                zmax = fmaxf(zmax, z[e]);
            }
            if (zmax > mx + kLseSlack) {  // move the reference point (rare after the first)
                const float f = bex2(mx - zmax);
#pragma unroll
                for (int h = 0; h < 4; ++h) sm4[h] *= f;
                mx = zmax;
            }
#pragma unroll
            for (int e = 0; e < 16; ++e) sm4[e & 3] += bex2(z[e] - mx);
        }
        sm100::tc_fence_before();
        __syncthreads();
    }
    if (failed) {
        // the commit covers every MMA this CTA issued; wait for it (bounded)
        // before the tensor memory is freed
        if (tid == 0) {
            atomicOr(&st->err, 1);
            sm100::mbar_wait(&s_bar, (uint32_t)(tile & 1), kTcPolls);
        }
        sm100::tc_fence_before();
        __syncthreads();
        if (warp == 0) sm100::tmem_dealloc(tmem, kTcTmemCols);
        return;
    }
    if (warp == 0) sm100::tmem_dealloc(tmem, kTcTmemCols);
    float sm = (sm4[0] + sm4[1]) + (sm4[2] + sm4[3]);
    // merge the two column halves of each owner
    if (half == 1) {
        s_mx[r] = mx;
        s_sm[r] = sm;
    }
    __syncthreads();
    if (half == 1) return;
    lse_merge(mx, sm, s_mx[r], s_sm[r]);
    double g2 = 0.0;
    if (own_ok) {
        const double lg2 = (double)mx + (double)log2f(sm);
        if constexpr (!COLS) {
            const double S = row_sum(mx, sm);
            const double gi = S - B.a[oo + o];
            g2 = gi * gi;
            const double an = own_cur[oo + o] + reg * (B.loga[oo + o] - 0.69314718055994531 * lg2);
            own_next[oo + o] = an;
            own_split_next[oo + o] = bsplit(an, st, &st->regrid);
        } else {
            const double bn = own_cur[oo + o] + reg * (B.logb[oo + o] - 0.69314718055994531 * lg2);
            own_next[oo + o] = bn;
            if (write_split) own_split_next[oo + o] = bsplit(bn, st, &st->regrid);
        }
    }
    if constexpr (!COLS) {
        // partial of sum (S_i - a_i)^2 per 32 rows, in the 32-row layout
        g2 = warp_sum_d(g2);
        const int blk = it.y * (kTcOwn / kBItems) + warp;
        if (lane == 0 && blk * kBItems < n) part[B.rbo[p] + blk] = g2;
    }
}

// Marginal error and stopping test of iterate k for every running problem
// (one warp each): mar = sqrt(sum over the problem's row blocks), stop when
// mar < tol or k >= max_iter (sinkhorn_bcd.cpp), the iterate's alpha being in
// the buffers of `parity`.
__global__ void k_bfin(const BatchDev B, int count, const double* part, int* done, int* iter,
                       int* fpar, double* mar, int max_iter, double tol, BatchState* st,
                       int parity) {
    const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= count || done[p]) return;
    const int nb = (B.n[p] + kBItems - 1) / kBItems;
    double s = 0.0;
    for (int k = lane; k < nb; k += 32) s += part[B.rbo[p] + k];
    s = warp_sum_d(s);
    if (lane == 0) {
        const double g = sqrt(s);
        const int k = iter[p];
        mar[p] = g;
        if (g < tol || k >= max_iter) {
            done[p] = 1;
            fpar[p] = parity;
            atomicSub(&st->active, 1);
        } else {
            iter[p] = k + 1;
        }
    }
}

// Condition of the device-side loop, run once per body.
__global__ void k_bloop(BatchState* st, cudaGraphConditionalHandle h) {
    const int loops = ++st->loops;
    const bool go = st->active > st->stop_below && !st->regrid && loops < st->loop_cap;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

// ---- the tail of the batch: one thread-block cluster per running problem ----
// When few problems are left, a sweep of the graph loop is a handful of short
// kernels whose launches cost more than their work. The tail kernel instead
// gives each running problem one cluster of C CTAs (16, or 8 where a device
// cannot hold clusters of 16), which runs that problem's sweeps to its stop in
// one launch: CTA r takes the row blocks and the column blocks r, r + C, ...
// of the problem (the same row_item /
// col_item arithmetic as the sweep kernels), and a cluster barrier stands
// where a kernel boundary stood. The problems' clusters are independent and
// nothing waits across them.
//
// Uniform control flow: every decision (stop, regrid) is taken by every CTA
// of the cluster from the same data read after a barrier (the row blocks'
// partials, the problem's own regrid flag) and the same local iteration
// count, so all CTAs leave the sweep loop at the same point and pass the
// same barriers. Rank 0 alone writes the problem's iteration count, error,
// done flag and final parity.
constexpr int kTailCta = 16;  // CTAs per cluster where the device holds such clusters, else 8
constexpr size_t kTailSmem = (size_t)kBTile * (kBClassDim[kBClasses - 1] + 1) * sizeof(float2) +
                             (size_t)kBTile * sizeof(float2);

struct TailArgs {
    BatchDev B;
    const int* plist;  // the running problems, one per cluster
    const int* pcls;   // dimension class of each problem
    float2* as[2];
    double* a[2];
    float2* bs;
    double* beta;
    double* part;
    int* done;
    int* iter;
    int* fpar;
    double* mar;
    int* pflag;        // per problem: a dual left the split grid
    BatchState* st;
    int max_iter;
    int body_cap;
    int loops0;        // loop bodies run before this launch (for the sweep count)
    double tol;
    float k2;
    double reg;
};

__device__ __forceinline__ void tail_barrier() {
    __threadfence();
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n\t"
        "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

template <int DP>
__device__ void tail_solve(const TailArgs& a, int p, int rank, int ncta, float2* spts,
                           float2* spar) {
    const BatchDev& B = a.B;
    const int nb = (B.n[p] + kBItems - 1) / kBItems, mb = (B.m[p] + kBItems - 1) / kBItems;
    int* rgf = a.pflag + p;
    __shared__ double s_g;
    int k = __ldcg(a.iter + p);  // written by rank 0 only, after this read
    for (int body = 0; body < a.body_cap; ++body) {
        // alpha of the current iterate in buffers 0 at the start of a body,
        // as in the graph loop
        for (int q = 0; q < 2; ++q) {
            for (int rb = rank; rb < nb; rb += ncta)
                row_item<DP, true>(B, make_int2(p, rb), a.as[q], a.bs, a.a[q], a.a[1 - q],
                                   a.as[1 - q], a.part, a.st, rgf, a.k2, a.reg, spts, spar);
            tail_barrier();
            // marginal error and stopping test of the iterate (k_bfin)
            if (threadIdx.x < 32) {
                double s = 0.0;
                for (int j = threadIdx.x; j < nb; j += 32) s += __ldcg(a.part + B.rbo[p] + j);
                s = warp_sum_d(s);
                if (threadIdx.x == 0) s_g = sqrt(s);
            }
            __syncthreads();
            const double g = s_g;
            const bool stop = g < a.tol || k >= a.max_iter;
            if (rank == 0 && threadIdx.x == 0) {
                a.mar[p] = g;
                if (stop) {
                    a.done[p] = 1;
                    a.fpar[p] = q;
                    atomicSub(&a.st->active, 1);
                    atomicMax(&a.st->loops, a.loops0 + body + 1);
                } else {
                    a.iter[p] = k + 1;
                }
            }
            if (stop) return;
            ++k;
            for (int cb = rank; cb < mb; cb += ncta)
                col_item<DP, true>(B, make_int2(p, cb), a.as[1 - q], a.bs, a.beta, a.st, rgf,
                                   a.k2, a.reg, 1, spts, spar);
            tail_barrier();
        }
        // a dual of this problem left the split grid: stop at the body's end
        // (alpha in buffers 0) for the host to re-split on a new grid. Every
        // CTA reads the flag before the barrier, and none can set it again
        // (in the next row half-sweep) before all have passed the barrier,
        // so all CTAs see the same value.
        const int rg = __ldcg(rgf);
        tail_barrier();
        if (rg) {
            if (rank == 0 && threadIdx.x == 0) {
                atomicOr(&a.st->regrid, 1);
                atomicMax(&a.st->loops, a.loops0 + body + 1);
            }
            return;
        }
    }
    if (rank == 0 && threadIdx.x == 0) atomicMax(&a.st->loops, a.loops0 + a.body_cap);
}

__global__ void __launch_bounds__(kBWarps * 32) k_btail(const TailArgs a) {
    extern __shared__ __align__(16) float2 tail_smem[];
    unsigned rank, ncta, cid;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(ncta));
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(cid));
    const int p = a.plist[cid];
    float2* spts = tail_smem;
    float2* spar = tail_smem + kBTile * (kBClassDim[kBClasses - 1] + 1);
    switch (a.pcls[p]) {
        case 0: tail_solve<4>(a, p, (int)rank, (int)ncta, spts, spar); break;
        case 1: tail_solve<8>(a, p, (int)rank, (int)ncta, spts, spar); break;
        default: tail_solve<16>(a, p, (int)rank, (int)ncta, spts, spar); break;
    }
}

// Backward of the batch: for each problem, the gradient of its regularised
// OT cost L = a'alpha + b'beta - reg sum T at the returned duals with respect
// to the points. By the envelope theorem dL/dM = T, and M_ij = s |x_i - y_j|^2
// gives dL/dx_i = 2 s sum_j T_ij (x_i - y_j) and dL/dy_j = 2 s sum_i T_ij
// (y_j - x_i). One warp per own point (a row for dL/dx, a column for dL/dy),
// lanes over the other side's points staged in shared memory. T_ij comes out
// as in the sweeps (the same FP32 cost, the split exponent) and the weighted
// differences are summed against a running base-2 reference like the
// log-sum-exp, so no term overflows whatever the duals. Summing T (x_i - y_j)
// instead of forming r_i x_i - (T y)_i avoids cancelling the two terms.
// The gradients are accumulated in FP32 and stored as FP32, the type of the
// points. side 0 also writes the row sums of T (for the cost).
constexpr int kGWarps = 8;  // own points per CTA

template <int DP>
__global__ void __launch_bounds__(kGWarps * 32) k_bgrad(
    const BatchDev B, const int2* __restrict__ items, int side, const float2* __restrict__ as,
    const float2* __restrict__ bs, float k2, float* __restrict__ grad,
    double* __restrict__ tsum) {
    const int2 it = items[blockIdx.x];
    const int p = it.x;
    const int d = B.d[p];
    const int n_own = side ? B.m[p] : B.n[p];
    const int n_oth = side ? B.n[p] : B.m[p];
    const float* Po = side ? B.Y + B.yo[p] : B.X + B.xo[p];
    const float* Pt = side ? B.X + B.xo[p] : B.Y + B.yo[p];
    const float2* so = side ? bs + B.co[p] : as + B.ro[p];
    const float2* sx = side ? as + B.ro[p] : bs + B.co[p];
    const float sc = B.scale[p];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = it.y * kGWarps + warp;
    const bool ok = i < n_own;  // the same for the whole warp
    float u[DP], acc[DP];
#pragma unroll
    for (int k = 0; k < DP; ++k) {
        u[k] = (ok && k < d) ? Po[(long long)i * d + k] : 0.f;
        acc[k] = 0.f;
    }
    const float2 s_own = ok ? so[i] : make_float2(0.f, 0.f);
    const float lk_own = __fmul_rn(s_own.y, k2);
    float mx = -INFINITY, ts = 0.f;
    __shared__ float sv[kBTile][DP + 1];
    __shared__ float2 sd[kBTile];
    for (int j0 = 0; j0 < n_oth; j0 += kBTile) {
        const int cnt = min(kBTile, n_oth - j0);
        for (int e = threadIdx.x; e < kBTile * DP; e += kGWarps * 32) {
            const int jj = e / DP, k = e % DP;
            sv[jj][k] = (jj < cnt && k < d) ? Pt[(long long)(j0 + jj) * d + k] : 0.f;
        }
        for (int jj = threadIdx.x; jj < kBTile; jj += kGWarps * 32)
            sd[jj] = jj < cnt ? sx[j0 + jj] : make_float2(0.f, 0.f);
        __syncthreads();
        if (ok) {
            for (int jj = lane; jj < cnt; jj += 32) {
                float t[DP], q[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int k = 0; k < DP; ++k) {
                    t[k] = __fsub_rn(u[k], sv[jj][k]);
                    q[k & 3] = __fmaf_rn(t[k], t[k], q[k & 3]);
                }
                const float M = __fmul_rn(__fadd_rn(__fadd_rn(q[0], q[1]), __fadd_rn(q[2], q[3])), sc);
                const float2 sj = sd[jj];
                const float e = __fadd_rn(__fadd_rn(s_own.x, sj.x), -M);
                const float z = __fmaf_rn(e, k2, __fadd_rn(lk_own, __fmul_rn(sj.y, k2)));
                if (z > mx + kLseSlack) {
                    const float f = bex2(mx - z);
#pragma unroll
                    for (int k = 0; k < DP; ++k) acc[k] *= f;
                    ts *= f;
                    mx = z;
                }
                const float w = bex2(z - mx);
#pragma unroll
                for (int k = 0; k < DP; ++k) acc[k] = __fmaf_rn(w, t[k], acc[k]);
                ts += w;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float m2 = __shfl_xor_sync(0xffffffffu, mx, o);
        const float t2 = __shfl_xor_sync(0xffffffffu, ts, o);
        float a2[DP];
#pragma unroll
        for (int k = 0; k < DP; ++k) a2[k] = __shfl_xor_sync(0xffffffffu, acc[k], o);
        const float m = fmaxf(mx, m2);
        if (m != -INFINITY) {
            const float f1 = bex2(mx - m), f2 = bex2(m2 - m);
#pragma unroll
            for (int k = 0; k < DP; ++k) acc[k] = acc[k] * f1 + a2[k] * f2;
            ts = ts * f1 + t2 * f2;
        }
        mx = m;
    }
    if (!ok) return;
    const float fl = floorf(mx);
    const float fr = exp2f(mx - fl);
    float v = 0.f;
#pragma unroll
    for (int k = 0; k < DP; ++k)
        if (lane == k) v = acc[k];
    if (grad && lane < d) {
        const long long off = side ? B.yo[p] : B.xo[p];
        grad[off + (long long)i * d + lane] =
            (float)(2.0 * (double)sc * ldexp((double)(v * fr), (int)fl));
    }
    if (side == 0 && lane == 0) tsum[B.ro[p] + i] = ldexp((double)(ts * fr), (int)fl);
}

// Each problem's alpha from the buffer of its last iterate.
__global__ void k_bfinal(const BatchDev B, const int* __restrict__ fpar,
                         const double* __restrict__ a0, const double* __restrict__ a1, double* af) {
    const int p = blockIdx.x;
    const int ro = B.ro[p], n = B.n[p];
    const double* src = fpar[p] ? a1 : a0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) af[ro + i] = src[ro + i];
}

// L_p = sum a_i (alpha_i + c) + sum b_j (beta_j - c) - reg sum T, with the
// gauge c = beta_m of the returned duals (one block of 256 per problem).
__global__ void k_bcost(const BatchDev B, const double* __restrict__ b,
                        const double* __restrict__ af, const double* __restrict__ beta,
                        const double* __restrict__ tsum, double reg, double* cost) {
    const int p = blockIdx.x;
    const int ro = B.ro[p], co = B.co[p], n = B.n[p], m = B.m[p];
    const double c = beta[co + m - 1];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        s += B.a[ro + i] * (af[ro + i] + c) - reg * tsum[ro + i];
    for (int j = threadIdx.x; j < m; j += blockDim.x) s += b[co + j] * (beta[co + j] - c);
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) cost[p] = red[0];
}

__global__ void k_blog(const double* x, int len, double* y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < len) y[t] = log(x[t]);
}

// st->maxabs = max |x|, |y| (zeroed by the caller), then the grid.
__global__ void k_bmax(const double* x, int nx, const double* y, int ny, BatchState* st) {
    unsigned long long v = 0ULL;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nx + ny; t += gridDim.x * blockDim.x) {
        const unsigned long long q = abs_bits(t < nx ? x[t] : y[t - nx]);
        v = q > v ? q : v;
    }
    block_atomic_max_bits(&st->maxabs, v);
}

// Grid of the split from max |dual|: g = 2^(e + 3 - 21), bound 2^(e + 4)
// (8x headroom, as in the single-problem BCD).
__global__ void k_bgrid(BatchState* st) {
    const double m0 = st->maxabs;
    const int e = (m0 > 0.0 && isfinite(m0)) ? ilogb(m0) : 0;
    st->g = ldexp(1.0, e + 3 - 21);
    st->inv_g = ldexp(1.0, -(e + 3 - 21));
    st->bound = ldexp(1.0, e + 4);
    st->regrid = 0;
}

__global__ void k_bsplit_all(const double* v, int len, float2* out, BatchState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < len) out[t] = bsplit(v[t], st, &st->regrid);
}


struct BatchGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~BatchGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

template <typename T>
void upload_vec(DBuf<T>& buf, const std::vector<T>& v, cudaStream_t st) {
    buf.alloc(v.size(), st);
    h2d(buf.get(), v.data(), v.size() * sizeof(T), st);
}

// Which half-sweep kernels a dimension class uses: 0 = CUDA-core direct
// differences (k_brow / k_bcol), 1 = tensor-core cost tile (k_bsweep_tc).
// Chosen per device and class by timing one row half-sweep of each on the
// first batch that has problems of the class; a forced choice overrides.
std::mutex g_bvar_mutex;
std::map<std::pair<std::string, int>, int> g_bvar;
std::atomic<int> g_bvar_force{-1};
std::atomic<int> g_btail{REGOT_BATCH_TAIL_DEFAULT};

std::string bdevice_name() {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return "unknown";
    return std::string(prop.name) + " sm" + std::to_string(prop.multiProcessorCount);
}

template <bool COLS>
void configure_tc_sweep() {
    static std::atomic<unsigned long long> configured{0};
    int dev = 0;
    REGOT_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(configured.load() & (1ULL << dev))) {
        REGOT_CUDA(cudaFuncSetAttribute(k_bsweep_tc<COLS>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kTcSmem));
        if (dev < 64) configured.fetch_or(1ULL << dev);
    }
}

// CTAs per tail cluster on the current device: 16 (a non-portable size) when
// the device can hold a cluster of 16 of these CTAs, else the portable 8.
int tail_cluster_size() {
    static std::atomic<int> cached[64] = {};
    int dev = 0;
    REGOT_CUDA(cudaGetDevice(&dev));
    if (dev < 64 && cached[dev].load() > 0) return cached[dev].load();
    int size = 8;
    if (cudaFuncSetAttribute(k_btail, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
        cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kTailCta);
        cfg.blockDim = dim3(kBWarps * 32);
        cfg.dynamicSmemBytes = kTailSmem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = kTailCta;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, k_btail, &cfg) == cudaSuccess && clusters > 0)
            size = kTailCta;
    }
    cudaGetLastError();  // a refused query leaves no error behind
    if (dev < 64) cached[dev].store(size);
    return size;
}

}  // namespace

int force_batch_variant(int v) { return g_bvar_force.exchange(v == 0 || v == 1 ? v : -1); }

int set_batch_tail(int max_active) { return g_btail.exchange(std::max(0, max_active)); }

std::vector<int> batch_variants() {
    std::vector<int> out(kBClasses, -1);
    const std::string dev = bdevice_name();
    std::lock_guard<std::mutex> lock(g_bvar_mutex);
    for (int c = 0; c < kBClasses; ++c) {
        auto it = g_bvar.find({dev, c});
        if (it != g_bvar.end()) out[c] = it->second;
    }
    return out;
}

void erot_solve_batched_gpu(regot_ctx* ctx, const regot_batch_desc* D, double reg, double tol,
                            int max_iter, regot_batch_result* res, double* cost, float* grad_x,
                            float* grad_y) {
    cudaStream_t st = ctx->stream;
    const int P = D->count;
    std::vector<int> hn(P), hm(P), hd(P), ro(P), co(P), rbo(P + 1), cls(P);
    std::vector<long long> xo(P), yo(P);
    std::vector<float> hsc(P);
    long long NX = 0, NY = 0, NR = 0, NC = 0, NRB = 0;
    for (int p = 0; p < P; ++p) {
        const int n = D->n[p], m = D->m[p], d = D->d[p];
        require(n > 0 && m > 0, "every problem needs at least one row and one column");
        require(d >= 1 && d <= REGOT_BATCH_MAX_DIM, "point dimension must be in 1..16");
        const double sc = D->cost_scale ? D->cost_scale[p] : 1.0;
        require(std::isfinite(sc) && sc > 0.0, "cost scales must be positive and finite");
        hn[p] = n;
        hm[p] = m;
        hd[p] = d;
        hsc[p] = (float)sc;
        ro[p] = (int)NR;
        co[p] = (int)NC;
        xo[p] = NX;
        yo[p] = NY;
        rbo[p] = (int)NRB;
        NR += n;
        NC += m;
        NX += (long long)n * d;
        NY += (long long)m * d;
        NRB += cdiv(n, kBItems);
        cls[p] = d <= kBClassDim[0] ? 0 : d <= kBClassDim[1] ? 1 : 2;
    }
    require(NR < (1LL << 31) && NC < (1LL << 31), "batch too large");
    rbo[P] = (int)NRB;

    // Work items per dimension class, the longest first (rows: by m, columns:
    // by n) so that the large problems do not finish last.
    // The lists hold the running problems only: they are rebuilt, and the
    // sweep graph captured again, each time the number of running problems
    // has halved (or, below 17, each time one has finished), so that the
    // last sweeps of a few slow problems do not launch a CTA for every block
    // of every problem.
    std::vector<int2> ritems[kBClasses], citems[kBClasses];
    std::vector<int2> rtc[kBClasses], ctc[kBClasses];  // blocks of 128 (tensor-core sweeps)
    auto build_items = [&](const std::vector<int>& running) {
        std::vector<int> order(running);
        for (int c = 0; c < kBClasses; ++c) {
            ritems[c].clear();
            citems[c].clear();
            rtc[c].clear();
            ctc[c].clear();
        }
        std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return hm[u] > hm[v]; });
        for (int p : order) {
            for (int k = 0; k < cdiv(hn[p], kBItems); ++k)
                ritems[cls[p]].push_back(make_int2(p, k));
            for (int k = 0; k < cdiv(hn[p], kTcOwn); ++k) rtc[cls[p]].push_back(make_int2(p, k));
        }
        std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return hn[u] > hn[v]; });
        for (int p : order) {
            for (int k = 0; k < cdiv(hm[p], kBItems); ++k)
                citems[cls[p]].push_back(make_int2(p, k));
            for (int k = 0; k < cdiv(hm[p], kTcOwn); ++k) ctc[cls[p]].push_back(make_int2(p, k));
        }
    };
    {
        std::vector<int> all(P);
        for (int p = 0; p < P; ++p) all[p] = p;
        build_items(all);
    }

    DBuf<int> dn, dm, dd, dro, dco, drbo;
    DBuf<long long> dxo, dyo;
    DBuf<float> dsc;
    upload_vec(dn, hn, st);
    upload_vec(dm, hm, st);
    upload_vec(dd, hd, st);
    upload_vec(dro, ro, st);
    upload_vec(dco, co, st);
    upload_vec(drbo, rbo, st);
    upload_vec(dxo, xo, st);
    upload_vec(dyo, yo, st);
    upload_vec(dsc, hsc, st);
    DBuf<int2> dri[kBClasses], dci[kBClasses], drt[kBClasses], dct[kBClasses];
    auto upload_items = [&]() {
        for (int c = 0; c < kBClasses; ++c) {
            if (!ritems[c].empty()) upload_vec(dri[c], ritems[c], st);
            if (!citems[c].empty()) upload_vec(dci[c], citems[c], st);
            if (!rtc[c].empty()) upload_vec(drt[c], rtc[c], st);
            if (!ctc[c].empty()) upload_vec(dct[c], ctc[c], st);
        }
    };
    upload_items();

    // points and marginals on the device
    DBuf<float> hX, hY;
    DBuf<double> ha, hb, loga(NR, st), logb(NC, st);
    const float* X = D->x;
    const float* Y = D->y;
    const double* a = D->a;
    const double* b = D->b;
    if (D->mem == REGOT_MEM_HOST) {
        hX.alloc(NX, st);
        hY.alloc(NY, st);
        ha.alloc(NR, st);
        hb.alloc(NC, st);
        h2d(hX.get(), D->x, NX * sizeof(float), st);
        h2d(hY.get(), D->y, NY * sizeof(float), st);
        h2d(ha.get(), D->a, NR * sizeof(double), st);
        h2d(hb.get(), D->b, NC * sizeof(double), st);
        X = hX.get();
        Y = hY.get();
        a = ha.get();
        b = hb.get();
    }
    k_blog<<<cdiv(NR, 256), 256, 0, st>>>(a, (int)NR, loga.get());
    k_blog<<<cdiv(NC, 256), 256, 0, st>>>(b, (int)NC, logb.get());
    count_launch(2);

    DBuf<double> A[2] = {DBuf<double>(NR, st), DBuf<double>(NR, st)}, beta(NC, st);
    DBuf<float2> AS[2] = {DBuf<float2>(NR, st), DBuf<float2>(NR, st)}, BS(NC, st);
    DBuf<int> done(P, st), iter(P, st), fpar(P, st);
    DBuf<double> mar(P, st), part(std::max<long long>(NRB, 1), st);
    DBuf<BatchState> dstate(1, st);
    for (int q = 0; q < 2; ++q) {
        A[q].zero();
        AS[q].zero();
    }
    beta.zero();
    BS.zero();
    done.zero();
    iter.zero();
    fpar.zero();
    BatchState h0{};
    h0.active = P;
    h0.loop_cap = max_iter / 2 + 3;
    h2d(dstate.get(), &h0, sizeof(h0), st);
    BatchState* S = dstate.get();

    BatchDev B{dn.get(), dm.get(), dd.get(), dsc.get(), dxo.get(), dyo.get(), dro.get(),
               dco.get(), drbo.get(), X, Y, a, loga.get(), logb.get()};
    const float k2 = (float)(1.4426950408889634 / reg);
    int use_tc[kBClasses] = {0, 0, 0};
    configure_tc_sweep<false>();
    configure_tc_sweep<true>();
    auto launch_rows_class = [&](int q, int c, int tc) {
        if (tc) {
            k_bsweep_tc<false><<<(int)rtc[c].size(), 256, kTcSmem, st>>>(
                B, drt[c].get(), AS[q].get(), BS.get(), A[q].get(), A[1 - q].get(),
                AS[1 - q].get(), part.get(), done.get(), S, k2, reg, 1);
            count_launch();
            return true;
        }
        return false;
    };
    auto launch_rows = [&](int q) {
        for (int c = 0; c < kBClasses; ++c) {
            const int ni = (int)ritems[c].size();
            if (!ni) continue;
            if (use_tc[c] < -1) continue;
            if (launch_rows_class(q, c, use_tc[c] == 1)) continue;
            const dim3 grid(ni), block(kBWarps * 32);
            if (c == 0)
                k_brow<4><<<grid, block, 0, st>>>(B, dri[c].get(), AS[q].get(), BS.get(),
                                                  A[q].get(), A[1 - q].get(), AS[1 - q].get(),
                                                  part.get(), done.get(), S, k2, reg);
            else if (c == 1)
                k_brow<8><<<grid, block, 0, st>>>(B, dri[c].get(), AS[q].get(), BS.get(),
                                                  A[q].get(), A[1 - q].get(), AS[1 - q].get(),
                                                  part.get(), done.get(), S, k2, reg);
            else
                k_brow<16><<<grid, block, 0, st>>>(B, dri[c].get(), AS[q].get(),
                                                   BS.get(), A[q].get(), A[1 - q].get(),
                                                   AS[1 - q].get(), part.get(), done.get(), S, k2,
                                                   reg);
            count_launch();
        }
    };
    auto launch_cols = [&](int q, int write_split) {
        for (int c = 0; c < kBClasses; ++c) {
            const int ni = (int)citems[c].size();
            if (!ni) continue;
            if (use_tc[c] == 1) {
                k_bsweep_tc<true><<<(int)ctc[c].size(), 256, kTcSmem, st>>>(
                    B, dct[c].get(), BS.get(), AS[q].get(), beta.get(), beta.get(), BS.get(),
                    part.get(), done.get(), S, k2, reg, write_split);
                count_launch();
                continue;
            }
            const dim3 grid(ni), block(kBWarps * 32);
            if (c == 0)
                k_bcol<4><<<grid, block, 0, st>>>(B, dci[c].get(), AS[q].get(), BS.get(),
                                                  beta.get(), done.get(), S, k2, reg, write_split);
            else if (c == 1)
                k_bcol<8><<<grid, block, 0, st>>>(B, dci[c].get(), AS[q].get(), BS.get(),
                                                  beta.get(), done.get(), S, k2, reg, write_split);
            else
                k_bcol<16><<<grid, block, 0, st>>>(B, dci[c].get(), AS[q].get(),
                                                   BS.get(), beta.get(), done.get(), S, k2, reg,
                                                   write_split);
            count_launch();
        }
    };
    // split of alpha (buffers q) and beta on a fresh grid from their max
    auto regrid = [&](int q) {
        REGOT_CUDA(cudaMemsetAsync(&S->maxabs, 0, sizeof(double), st));
        k_bmax<<<64, 256, 0, st>>>(A[q].get(), (int)NR, beta.get(), (int)NC, S);
        k_bgrid<<<1, 1, 0, st>>>(S);
        k_bsplit_all<<<cdiv(NR, 256), 256, 0, st>>>(A[q].get(), (int)NR, AS[q].get(), S);
        k_bsplit_all<<<cdiv(NC, 256), 256, 0, st>>>(beta.get(), (int)NC, BS.get(), S);
        count_launch(4);
        REGOT_CHECK_LAUNCH();
    };

    cudaEvent_t e0 = nullptr, e1 = nullptr;
    REGOT_CUDA(cudaEventCreate(&e0));
    REGOT_CUDA(cudaEventCreate(&e1));
    struct Events {
        cudaEvent_t a, b;
        ~Events() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } events{e0, e1};
    REGOT_CUDA(cudaEventRecord(e0, st));

    // beta = optimal_beta(alpha = 0) (sinkhorn_bcd.cpp:38-47): one column
    // half-sweep from zero duals, then the split grid from |beta|.
    // Variant per class: forced, known for this device, or timed now (a row
    // and a column half-sweep of each variant from the current iterate: the
    // row sweeps write only the next-iterate buffers and the column sweeps a
    // scratch copy of beta, so the solve is unaffected).
    const int forced = g_bvar_force.load();
    const std::string devname = bdevice_name();
    for (int c = 0; c < kBClasses; ++c) {
        if (forced >= 0) {
            use_tc[c] = forced;
            continue;
        }
        std::lock_guard<std::mutex> lock(g_bvar_mutex);
        auto it = g_bvar.find({devname, c});
        use_tc[c] = it != g_bvar.end() ? it->second : -1;
    }
    launch_cols(0, 0);  // the untuned classes run the CUDA-core kernels here
    regrid(0);
    for (int c = 0; c < kBClasses; ++c) {
        if (use_tc[c] >= 0) continue;
        if (ritems[c].empty()) {
            use_tc[c] = 0;
            continue;
        }
        float ms[2] = {0.f, 0.f};
        cudaEvent_t t0, t1;
        REGOT_CUDA(cudaEventCreate(&t0));
        REGOT_CUDA(cudaEventCreate(&t1));
        // the column half-sweeps update a scratch copy of beta (write_split
        // 0), so the timing leaves the solve's state as it was
        DBuf<double> beta_t(NC, st);
        const int nr = (int)ritems[c].size(), nc = (int)citems[c].size();
        for (int v = 0; v < 2; ++v) {
            for (int rep = 0; rep < 2; ++rep) {  // warm, then timed
                d2d(beta_t.get(), beta.get(), NC * sizeof(double), st);
                REGOT_CUDA(cudaEventRecord(t0, st));
                if (v == 1) {
                    launch_rows_class(0, c, 1);
                    k_bsweep_tc<true><<<(int)ctc[c].size(), 256, kTcSmem, st>>>(
                        B, dct[c].get(), BS.get(), AS[1].get(), beta_t.get(), beta_t.get(),
                        BS.get(), part.get(), done.get(), S, k2, reg, 0);
                } else if (c == 0) {
                    k_brow<4><<<nr, kBWarps * 32, 0, st>>>(B, dri[c].get(), AS[0].get(), BS.get(),
                                                            A[0].get(), A[1].get(), AS[1].get(),
                                                            part.get(), done.get(), S, k2, reg);
                    k_bcol<4><<<nc, kBWarps * 32, 0, st>>>(B, dci[c].get(), AS[1].get(), BS.get(),
                                                            beta_t.get(), done.get(), S, k2, reg, 0);
                } else if (c == 1) {
                    k_brow<8><<<nr, kBWarps * 32, 0, st>>>(B, dri[c].get(), AS[0].get(), BS.get(),
                                                            A[0].get(), A[1].get(), AS[1].get(),
                                                            part.get(), done.get(), S, k2, reg);
                    k_bcol<8><<<nc, kBWarps * 32, 0, st>>>(B, dci[c].get(), AS[1].get(), BS.get(),
                                                            beta_t.get(), done.get(), S, k2, reg, 0);
                } else {
                    k_brow<16><<<nr, kBWarps * 32, 0, st>>>(B, dri[c].get(), AS[0].get(),
                                                             BS.get(), A[0].get(), A[1].get(),
                                                             AS[1].get(), part.get(), done.get(), S,
                                                             k2, reg);
                    k_bcol<16><<<nc, kBWarps * 32, 0, st>>>(B, dci[c].get(), AS[1].get(),
                                                             BS.get(), beta_t.get(), done.get(), S,
                                                             k2, reg, 0);
                }
                count_launch(2);
                REGOT_CUDA(cudaEventRecord(t1, st));
            }
            REGOT_CUDA(cudaEventSynchronize(t1));
            REGOT_CUDA(cudaEventElapsedTime(&ms[v], t0, t1));
        }
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        use_tc[c] = ms[1] < ms[0] ? 1 : 0;
        std::lock_guard<std::mutex> lock(g_bvar_mutex);
        g_bvar[{devname, c}] = use_tc[c];
    }

    // The sweeps: a graph whose only node is a conditional WHILE node; its
    // body is two sweeps (alpha ping-pongs between A[0] and A[1]) and k_bloop.
    long long body_kernels = 0;
    const int fin_blocks = cdiv(P, 8);
    auto make_graph = [&](BatchGraph& lg) {
        REGOT_CUDA(cudaGraphCreate(&lg.graph, 0));
        cudaGraphConditionalHandle loop_h;
        REGOT_CUDA(cudaGraphConditionalHandleCreate(&loop_h, lg.graph, 1,
                                                    cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = loop_h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop_node;
        REGOT_CUDA(cudaGraphAddNode(&loop_node, lg.graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        long long* saved_counter = g_launch_counter;
        body_kernels = 0;
        g_launch_counter = &body_kernels;
        REGOT_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal));
        try {
            for (int q = 0; q < 2; ++q) {
                launch_rows(q);
                k_bfin<<<fin_blocks, 256, 0, st>>>(B, P, part.get(), done.get(), iter.get(),
                                                   fpar.get(), mar.get(), max_iter, tol, S, q);
                count_launch();
                launch_cols(1 - q, 1);
            }
            k_bloop<<<1, 1, 0, st>>>(S, loop_h);
            count_launch();
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            g_launch_counter = saved_counter;
            throw;
        }
        REGOT_CUDA(cudaStreamEndCapture(st, &body));
        g_launch_counter = saved_counter;
        REGOT_CUDA(cudaGraphInstantiate(&lg.exec, lg.graph, 0));
    };
    auto set_stop_below = [&](int v) {
        h2d(&S->stop_below, &v, sizeof(int), st);
    };
    // the graph loop hands over to the tail kernel once at most tail_max
    // problems run, and rebuilds its items each time the number has halved
    const int tail_max = g_btail.load();
    // where the graph loop stops next: after this body when the tail may take
    // over, else when the running problems have halved (above 16) or one more
    // has finished
    auto next_stop = [&](int active, bool try_tail) {
        if (try_tail && active <= tail_max) return active;
        return active > 16 ? active / 2 : std::max(active - 1, 0);
    };
    std::vector<int> stop_host(1, next_stop(P, true));
    set_stop_below(stop_host[0]);
    std::unique_ptr<BatchGraph> lg(new BatchGraph());
    make_graph(*lg);

    BatchState hs{};
    int prev_loops = 0;
    for (;;) {
        REGOT_CUDA(cudaGraphLaunch(lg->exec, st));
        read_small(ctx, &hs, S, sizeof(hs), st);
        count_launch(body_kernels * (hs.loops - prev_loops));
        prev_loops = hs.loops;
        if (hs.err)
            throw Error(REGOT_ERR_TIMEOUT, "a tensor-core half-sweep gave up waiting for its MMAs");
        if (hs.active == 0) break;
        if (hs.loops >= hs.loop_cap) throw Error(REGOT_ERR_NUMERIC, "batched BCD did not terminate");
        bool acted = false;
        if (hs.regrid) {
            regrid(0);  // at a body boundary the running problems' alpha is in A[0]
            acted = true;
        }
        if (hs.active <= stop_host[0]) {
            std::vector<int> hdone(P), running;
            read_small(ctx, hdone.data(), done.get(), P * sizeof(int), st);
            for (int p = 0; p < P; ++p)
                if (!hdone[p]) running.push_back(p);
            if (hs.active <= tail_max) break;
            build_items(running);
            upload_items();
            stop_host[0] = next_stop(hs.active, false);
            set_stop_below(stop_host[0]);
            lg.reset(new BatchGraph());
            make_graph(*lg);
            acted = true;
        }
        if (!acted) throw Error(REGOT_ERR_NUMERIC, "batched BCD did not terminate");
    }

    // The tail: one cluster per running problem, each to its stop. A launch
    // ends early only for problems whose duals left the split grid; those
    // continue, after a re-split, in the next launch.
    if (hs.active > 0) {
        DBuf<int> dcls, plist(P, st), pflag(P, st);
        upload_vec(dcls, cls, st);
        const int tail_cta = tail_cluster_size();
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = tail_cta;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        for (;;) {
            std::vector<int> hdone(P), running;
            read_small(ctx, hdone.data(), done.get(), P * sizeof(int), st);
            for (int p = 0; p < P; ++p)
                if (!hdone[p]) running.push_back(p);
            if (running.empty()) break;
            h2d(plist.get(), running.data(), running.size() * sizeof(int), st);
            pflag.zero();
            TailArgs ta{};
            ta.B = B;
            ta.plist = plist.get();
            ta.pcls = dcls.get();
            for (int q = 0; q < 2; ++q) {
                ta.as[q] = AS[q].get();
                ta.a[q] = A[q].get();
            }
            ta.bs = BS.get();
            ta.beta = beta.get();
            ta.part = part.get();
            ta.done = done.get();
            ta.iter = iter.get();
            ta.fpar = fpar.get();
            ta.mar = mar.get();
            ta.pflag = pflag.get();
            ta.st = S;
            ta.max_iter = max_iter;
            ta.body_cap = std::max(1, hs.loop_cap - hs.loops);
            ta.loops0 = hs.loops;
            ta.tol = tol;
            ta.k2 = k2;
            ta.reg = reg;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)running.size() * tail_cta);
            cfg.blockDim = dim3(kBWarps * 32);
            cfg.dynamicSmemBytes = kTailSmem;
            cfg.stream = st;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            REGOT_CUDA(cudaLaunchKernelEx(&cfg, k_btail, ta));
            count_launch();
            read_small(ctx, &hs, S, sizeof(hs), st);
            if (hs.active == 0) break;
            if (!hs.regrid || hs.loops >= hs.loop_cap)
                throw Error(REGOT_ERR_NUMERIC, "batched BCD did not terminate");
            regrid(0);
        }
    }

    // Backward: costs and point gradients at every problem's last iterate,
    // its alpha gathered into one buffer and both duals split on a common
    // grid from their max.
    DBuf<double> Af, tsum, dcost;
    DBuf<float> gxd, gyd;
    if (cost || grad_x || grad_y) {
        Af.alloc(NR, st);
        tsum.alloc(NR, st);
        k_bfinal<<<P, 256, 0, st>>>(B, fpar.get(), A[0].get(), A[1].get(), Af.get());
        REGOT_CUDA(cudaMemsetAsync(&S->maxabs, 0, sizeof(double), st));
        k_bmax<<<64, 256, 0, st>>>(Af.get(), (int)NR, beta.get(), (int)NC, S);
        k_bgrid<<<1, 1, 0, st>>>(S);
        k_bsplit_all<<<cdiv(NR, 256), 256, 0, st>>>(Af.get(), (int)NR, AS[0].get(), S);
        k_bsplit_all<<<cdiv(NC, 256), 256, 0, st>>>(beta.get(), (int)NC, BS.get(), S);
        count_launch(5);
        if (grad_x) gxd.alloc(NX, st);
        if (grad_y) gyd.alloc(NY, st);
        std::vector<int> order(P);
        for (int p = 0; p < P; ++p) order[p] = p;
        for (int side = 0; side < 2; ++side) {
            float* out = side ? gyd.get() : gxd.get();
            if (side == 1 && !grad_y) break;
            // side 0 gives grad_x and the row sums of T that the cost needs
            if (side == 0 && !cost && !grad_x) continue;
            std::stable_sort(order.begin(), order.end(), [&](int u, int v) {
                return side ? hn[u] > hn[v] : hm[u] > hm[v];
            });
            std::vector<int2> gi[kBClasses];
            for (int p : order)
                for (int k = 0; k < cdiv(side ? hm[p] : hn[p], kGWarps); ++k)
                    gi[cls[p]].push_back(make_int2(p, k));
            for (int c = 0; c < kBClasses; ++c) {
                const int ni = (int)gi[c].size();
                if (!ni) continue;
                DBuf<int2> items;
                upload_vec(items, gi[c], st);
                const dim3 grid(ni), block(kGWarps * 32);
                if (c == 0)
                    k_bgrad<4><<<grid, block, 0, st>>>(B, items.get(), side, AS[0].get(), BS.get(),
                                                       k2, out, tsum.get());
                else if (c == 1)
                    k_bgrad<8><<<grid, block, 0, st>>>(B, items.get(), side, AS[0].get(), BS.get(),
                                                       k2, out, tsum.get());
                else
                    k_bgrad<16><<<grid, block, 0, st>>>(B, items.get(), side, AS[0].get(),
                                                        BS.get(), k2, out, tsum.get());
                count_launch();
                REGOT_CHECK_LAUNCH();  // the item list is freed in stream order
            }
        }
        if (cost) {
            dcost.alloc(P, st);
            k_bcost<<<P, 256, 0, st>>>(B, b, Af.get(), beta.get(), tsum.get(), reg, dcost.get());
            count_launch();
        }
        REGOT_CHECK_LAUNCH();
    }
    REGOT_CUDA(cudaEventRecord(e1, st));

    // results: each problem's alpha from the buffers of its last iterate,
    // gauge-fixed with its last beta
    std::vector<double> h0a(NR), h1a(NR), hbeta(NC), hmar(P);
    std::vector<int> hfpar(P), hiter(P);
    d2h(h0a.data(), A[0].get(), NR * sizeof(double), st);
    d2h(h1a.data(), A[1].get(), NR * sizeof(double), st);
    d2h(hbeta.data(), beta.get(), NC * sizeof(double), st);
    d2h(hmar.data(), mar.get(), P * sizeof(double), st);
    d2h(hfpar.data(), fpar.get(), P * sizeof(int), st);
    d2h(hiter.data(), iter.get(), P * sizeof(int), st);
    if (grad_x) d2h(grad_x, gxd.get(), NX * sizeof(float), st);
    if (grad_y) d2h(grad_y, gyd.get(), NY * sizeof(float), st);
    if (cost) d2h(cost, dcost.get(), P * sizeof(double), st);
    sync(st);
    float ms = 0.f;
    REGOT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    for (int p = 0; p < P; ++p) {
        const std::vector<double>& ap = hfpar[p] ? h1a : h0a;
        const double bl = hbeta[co[p] + hm[p] - 1];
        if (res->alpha)
            for (int i = 0; i < hn[p]; ++i) res->alpha[ro[p] + i] = ap[ro[p] + i] + bl;
        if (res->beta)
            for (int j = 0; j < hm[p]; ++j) res->beta[co[p] + j] = hbeta[co[p] + j] - bl;
        if (res->niter) res->niter[p] = hiter[p];
        if (res->mar_err) res->mar_err[p] = hmar[p];
    }
    res->sweeps = 2LL * hs.loops;
    res->solve_ms = ms;
}

}  // namespace regot
