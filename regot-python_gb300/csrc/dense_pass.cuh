// The dense streaming pass over the cost matrix M (the n x m hot path of
// the EROT and QROT solvers) as a kernel template over the pass operation
// and a launch configuration; included by one translation unit per
// (element type, configuration), which instantiates the launchers. The
// runtime choice of the configuration (passes.cu) is the autotuner's.
//
// Every pass reads M exactly once with 16-byte coalesced loads and reduces
// in registers/shared memory; row results leave as per-(row, column-slab)
// partials, column results as per-(row-block, column) partials, scalars as
// per-CTA partials. The finalize kernels of the solvers merge those
// partials in FP64 in a fixed order (deterministic; no floating-point
// atomics).
//
// Element formulas (reference: src/sinkhorn_problem_obj.cpp:16-136 for
// T = exp((alpha_i + beta_j - M_ij)/reg), src/qrot_problem.cpp:36-94 for
// D = (alpha_i + beta_j - M_ij)+):
//   FP64 storage:  arg = (ra_i + cb_j) - M_ij in FP64, T = exp(arg / reg).
//   FP32 storage:  ra and cb are split on a common power-of-two grid G into
//                  hi (multiple of G, exact in FP32, |hi| <= 2^22 G) and lo
//                  (FP32 rounding of the remainder), so that
//                  arg = ((rh + ch) - M_ij) + (rl + cl) has a hi sum that is
//                  exact and an error relative to |arg| instead of |ra|+|cb|;
//                  T = 2^(arg * log2(e)/reg) by ex2.approx.
//
// Launch configurations (PassCfg): the row-copy ring depth and the number
// of CTAs per SM, which sets the register budget of a thread. Both keep the
// tile shape (kRB x CW) and so the partial layouts, which the solvers'
// finalize kernels read.
#pragma once

#include <atomic>
#include <cfloat>
#include <cmath>
#include <type_traits>

#include "internal.h"

namespace regot {

namespace {

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---- bulk asynchronous copies (TMA engine) completing on an mbarrier ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
// try_wait with a suspend-time hint: a waiting warp sleeps until the phase
// completes (or the hint elapses) instead of spinning on issue slots that the
// computing warps need.
constexpr uint32_t kSuspendHintNs = 200000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendHintNs)
        : "memory");
    return ok != 0;
}
// Global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Bounded wait: gives up after `limit` suspended polls (kDefaultWaitSpins:
// a few seconds at most) and reports it through *err. A wait that gave up
// still drains the copy under the default limit before returning, so that
// the buffer is not refilled, and the CTA does not exit, while the copy is
// in flight; the caller treats the data as missing either way.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err,
                                                  long long limit) {
    for (long long s = 0; s < limit; ++s)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicOr(err, 1);
    for (long long s = 0; s < kDefaultWaitSpins; ++s)
        if (mbar_try_wait(bar, parity)) break;
    return false;
}

// e^x - 1 - x without cancellation: for |x| < 1/2 the Taylor series
// x^2 (1/2! + x/3! + x^2/4! + ...) by Horner's rule with the coefficients
// 1/k! as constants (no divisions), FP32 up to x^9 (truncation below 2e-9
// relative), FP64 up to x^17 (below 1e-20); expm1(x) - x beyond, where no
// cancellation occurs.
// Root passes' FP32 filter: the bound on |d - (y - c)| (d its FP32 value)
// relative to the magnitudes involved, and an absolute floor below FP32's
// normal range.
constexpr float kRootSlack = 4.76837158203125e-07f;  // 2^-21
constexpr float kRootFloor = 1e-37f;

template <typename T>
__device__ __forceinline__ T expm1_minus_x(T x);
template <>
__device__ __forceinline__ float expm1_minus_x<float>(float x) {
    if (fabsf(x) < 0.5f) {
        float p = 2.7557319e-06f;           // 1/9!
        p = fmaf(p, x, 2.4801587e-05f);     // 1/8!
        p = fmaf(p, x, 1.9841270e-04f);     // 1/7!
        p = fmaf(p, x, 1.3888889e-03f);     // 1/6!
        p = fmaf(p, x, 8.3333333e-03f);     // 1/5!
        p = fmaf(p, x, 4.1666667e-02f);     // 1/4!
        p = fmaf(p, x, 1.6666667e-01f);     // 1/3!
        p = fmaf(p, x, 0.5f);               // 1/2!
        return (x * x) * p;
    }
    // no cancellation here: e^x - 1 - x >= 0.106, so the relative error of
    // ex2.approx (about 2^-22) grows at most elevenfold
    return (ex2_approx(x * 1.44269504f) - 1.0f) - x;
}
template <>
__device__ __forceinline__ double expm1_minus_x<double>(double x) {
    if (fabs(x) < 0.5) {
        double p = 2.8114572543455206e-15;  // 1/17!
        p = fma(p, x, 4.7794773323873853e-14);  // 1/16!
        p = fma(p, x, 7.6471637318198164e-13);  // 1/15!
        p = fma(p, x, 1.1470745597729725e-11);  // 1/14!
        p = fma(p, x, 1.6059043836821613e-10);  // 1/13!
        p = fma(p, x, 2.0876756987868099e-09);  // 1/12!
        p = fma(p, x, 2.5052108385441720e-08);  // 1/11!
        p = fma(p, x, 2.7557319223985888e-07);  // 1/10!
        p = fma(p, x, 2.7557319223985893e-06);  // 1/9!
        p = fma(p, x, 2.4801587301587302e-05);  // 1/8!
        p = fma(p, x, 1.9841269841269841e-04);  // 1/7!
        p = fma(p, x, 1.3888888888888889e-03);  // 1/6!
        p = fma(p, x, 8.3333333333333333e-03);  // 1/5!
        p = fma(p, x, 4.1666666666666667e-02);  // 1/4!
        p = fma(p, x, 1.6666666666666667e-01);  // 1/3!
        p = fma(p, x, 0.5);                     // 1/2!
        return (x * x) * p;
    }
    return expm1(x) - x;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <typename TM> struct Vec;
template <> struct Vec<float> {
    using type = float4;
    __device__ static float4 zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ static float get(const float4& v, int e) {
        return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
    }
};
template <> struct Vec<double> {
    using type = double2;
    __device__ static double2 zero() { return make_double2(0.0, 0.0); }
    __device__ static double get(const double2& v, int e) { return e == 0 ? v.x : v.y; }
};

// Accumulator / reduction arity of each operation.
__host__ __device__ constexpr int op_nr(int op) {
    return op == OP_E_ROW ? 1 : op == OP_E_ROWCOL ? 1 : op == OP_E_HVP ? 1 : op == OP_E_ROWMAX ? 1
         : op == OP_Q_GRAD ? 1 : op == OP_Q_GRADMASK ? 2 : op == OP_Q_P1 ? 1 : op == OP_Q_P3 ? 3
         : op == OP_Q_GRADLS ? 1 : op == OP_E_GRADLS ? 1 : op == OP_E_AVG ? 1
         : op == OP_Q_ROWROOT ? 2 : op == OP_Q_AVG ? 1 : 0;
}
__host__ __device__ constexpr int op_nc(int op) {
    return op == OP_E_COL ? 1 : op == OP_E_ROWCOL ? 1 : op == OP_E_HVP ? 1 : op == OP_E_COLMAX ? 1
         : op == OP_Q_GRAD ? 1 : op == OP_Q_GRADMASK ? 2 : op == OP_Q_P2 ? 1 : op == OP_Q_COLROOT ? 2
         : op == OP_Q_GRADLS ? 1 : op == OP_E_GRADLS ? 1 : op == OP_E_AVG ? 1
         : op == OP_Q_AVG ? 1 : 0;
}
__host__ __device__ constexpr int op_nt(int op) {
    return op == OP_E_LS ? 4 : op == OP_Q_GRAD ? 1 : op == OP_Q_GRADMASK ? 1 : op == OP_Q_OBJ ? 1
         : op == OP_Q_P3 ? 2 : op == OP_Q_GRADLS ? 2 : op == OP_E_GRADLS ? 1 : op == OP_E_AVG ? 2
         : op == OP_Q_AVG ? 2 : 0;
}
// Root-finding passes accumulate in FP64 in both storage modes.
__host__ __device__ constexpr bool op_fp64_acc(int op) {
    return op == OP_Q_COLROOT || op == OP_Q_ROWROOT;
}
__host__ __device__ constexpr bool op_is_erot(int op) {
    return op <= OP_E_COLMAX || op == OP_E_GRADLS || op == OP_E_AVG;
}
__host__ __device__ constexpr bool op_is_max(int op) {
    return op == OP_E_ROWMAX || op == OP_E_COLMAX;
}
__host__ __device__ constexpr bool op_needs_ra(int op) {
    return op != OP_E_ROWMAX;
}
__host__ __device__ constexpr bool op_needs_cb(int op) {
    return op != OP_E_COLMAX;
}

__device__ __forceinline__ void split(double v, double g, double inv_g, float& hi, float& lo) {
    if (!isfinite(v)) {
        hi = (float)v;
        lo = 0.f;
        return;
    }
    const double h = rint(v * inv_g) * g;
    hi = (float)h;
    lo = (float)(v - h);
}

__host__ __device__ constexpr bool op_uses_cx(int op) {
    return op == OP_E_HVP || op == OP_Q_P3;
}
__host__ __device__ constexpr bool op_uses_cx2(int op) { return op == OP_Q_P3; }
__host__ __device__ constexpr bool op_uses_cd(int op) {
    return op == OP_E_LS || op == OP_Q_GRADLS || op == OP_E_GRADLS;
}
__host__ __device__ constexpr bool op_uses_rx(int op) {
    return op == OP_E_HVP || op == OP_Q_P2 || op == OP_Q_P3;
}
__host__ __device__ constexpr bool op_uses_rd(int op) {
    return op == OP_E_LS || op == OP_Q_GRADLS || op == OP_E_GRADLS;
}

// Sum (or max) of the per-lane partials of a warp's N rows (N a power of
// two <= 32): a transposed butterfly whose first log2(N) exchange levels
// halve the number of values per lane, then plain levels; N - 1 + 5 - log2(N)
// shuffles instead of 5 N. Afterwards lane L holds the total of row
// L >> (5 - log2 N).
template <bool ISMAX, int N, typename T>
__device__ __forceinline__ T warp_reduce_rows(T (&v)[N], int lane) {
    constexpr int L = N >= 32 ? 5 : N >= 16 ? 4 : N >= 8 ? 3 : N >= 4 ? 2 : N >= 2 ? 1 : 0;
#pragma unroll
    for (int lvl = 0; lvl < L; ++lvl) {
        const int o = 16 >> lvl;
        const int K = N >> lvl;
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < K / 2; ++k) {
            const T send = upper ? v[k] : v[k + K / 2];
            const T keep = upper ? v[k + K / 2] : v[k];
            const T got = __shfl_xor_sync(0xffffffffu, send, o);
            v[k] = ISMAX ? fmax(keep, got) : keep + got;
        }
    }
    T r = v[0];
#pragma unroll
    for (int o = 16 >> L; o > 0; o >>= 1) {
        const T got = __shfl_xor_sync(0xffffffffu, r, o);
        r = ISMAX ? fmax(r, got) : r + got;
    }
    return r;
}

// Plan output: the VW values of one lane vector are collected in pv and
// stored together once the vector is complete. The plan may be host memory
// written across the host link, where only whole, contiguous lines per warp
// store run at the link's rate, so with FP32 M (VW = 4: a lane owns 32 bytes
// of every 1 KB block of the row) the values are first exchanged between
// lanes so that each store instruction of the warp covers 512 contiguous
// bytes. Partial blocks and rows that do not start on 16 bytes are stored
// lane by lane. With FP64 M (VW = 2) a lane's 16 bytes are already
// contiguous across the warp. The control flow around the call is uniform
// across the warp (one row per warp), as the shuffles require.
template <int VW>
__device__ __forceinline__ void plan_put(double (&pv)[VW], int q, double val, double* out, int i,
                                         int m, int c0, int lane) {
    const int e = q % VW;
    pv[e] = val;
    if (e != VW - 1) return;
    double* row = out + (long long)i * m;
    const int j0 = c0 + ((q / VW) * 32 + lane) * VW;
    if constexpr (VW == 4) {
        const int jb = c0 + (q / VW) * 128;  // first column of the warp's 1 KB block
        if (jb + 128 <= m && (reinterpret_cast<uintptr_t>(row + jb) & 15) == 0) {
            const int s1 = lane >> 1, s2 = 16 + (lane >> 1);
            const bool odd = lane & 1;
            const double a0 = __shfl_sync(0xffffffffu, pv[0], s1);
            const double a1 = __shfl_sync(0xffffffffu, pv[1], s1);
            const double a2 = __shfl_sync(0xffffffffu, pv[2], s1);
            const double a3 = __shfl_sync(0xffffffffu, pv[3], s1);
            const double b0 = __shfl_sync(0xffffffffu, pv[0], s2);
            const double b1 = __shfl_sync(0xffffffffu, pv[1], s2);
            const double b2 = __shfl_sync(0xffffffffu, pv[2], s2);
            const double b3 = __shfl_sync(0xffffffffu, pv[3], s2);
            *reinterpret_cast<double2*>(row + jb + 2 * lane) =
                odd ? make_double2(a2, a3) : make_double2(a0, a1);
            *reinterpret_cast<double2*>(row + jb + 64 + 2 * lane) =
                odd ? make_double2(b2, b3) : make_double2(b0, b1);
            return;
        }
    }
    double* dst = row + j0;
    if (j0 + VW <= m && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
#pragma unroll
        for (int h = 0; h < VW; h += 2)
            *reinterpret_cast<double2*>(dst + h) = make_double2(pv[h], pv[h + 1]);
    } else {
#pragma unroll
        for (int h = 0; h < VW; ++h)
            if (j0 + h < m) dst[h] = pv[h];
    }
}

// Persistent dense pass. The grid holds as many CTAs as fit on the SMs; CTA
// b processes tiles b, b + G, b + 2G, ... (tile t = row block t / nslabs,
// column slab t % nslabs; RB rows x CW columns). Each warp streams RB/8 rows
// of every tile through its own ring of NS shared-memory row buffers, NS rows
// ahead of the row it is reducing and across tile boundaries, so HBM never
// idles between waves of CTAs. Every lane copies the 16-byte vectors of a row
// that it will itself read (cp.async.cg, one commit group per row), so a
// row is ready once the lane's own group has landed (cp.async.wait_group):
// no barrier between lanes and no proxy fence. Issuing each 2 KB row as one
// bulk copy from lane 0 (cp.async.bulk on an mbarrier) streamed about 10 %
// slower at n = m = 8192 (0.71 against 0.79 of the measured HBM bandwidth).
// The per-tile column / row parameters do go through bulk copies.
template <typename TM, int OP, int CFG>
__global__ void __launch_bounds__(kThreads, PassCfg<CFG>::kMinBlocks) dense_pass(const PassParams p) {
    if (p.done && *p.done) return;
    using G = Geo<TM>;
    constexpr int VW = G::VW, LC = G::LC, CW = G::CW, NV = LC / VW;
    constexpr bool MIXED = std::is_same<TM, float>::value;
    constexpr bool COLROOT = (OP == OP_Q_COLROOT);
    constexpr bool ROWROOT = (OP == OP_Q_ROWROOT);
    constexpr bool ROOT = COLROOT || ROWROOT;
    using Acc = typename std::conditional<ROOT, double, TM>::type;
    using VT = typename Vec<TM>::type;
    constexpr int NR = op_nr(OP), NC = op_nc(OP), NT = op_nt(OP);
    constexpr int NRa = NR > 0 ? NR : 1, NCa = NC > 0 ? NC : 1, NTa = NT > 0 ? NT : 1;
    constexpr bool ISMAX = op_is_max(OP);
    constexpr bool EROT = op_is_erot(OP);
    constexpr int RPW = kRB / kWarps;  // rows per warp per tile (4)
    constexpr int LOGR = RPW >= 8 ? 3 : RPW >= 4 ? 2 : RPW >= 2 ? 1 : 0;
    constexpr int NS = PassCfg<CFG>::kStages;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = p.n, m = p.m;
    const long long ldm = p.ldm;
    const int nslabs = (m + CW - 1) / CW;
    const int nrb = (n + kRB - 1) / kRB;
    const int ntiles = nslabs * nrb;
    const int my_tiles =
        (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int rw0 = warp * RPW;
    const TM* Mb = reinterpret_cast<const TM*>(p.M);

    extern __shared__ __align__(128) unsigned char dyn_smem[];
    TM* ring = reinterpret_cast<TM*>(dyn_smem) + (size_t)warp * NS * CW;
    Acc* s_cred = reinterpret_cast<Acc*>(dyn_smem + (size_t)kWarps * NS * CW * sizeof(TM));
    // Mixed mode: per-tile column and row parameters (FP32 splits), double
    // buffered and prefetched one tile ahead with bulk copies.
    constexpr size_t kCredBytes = (size_t)NCa * (kWarps / 2) * CW * sizeof(Acc);
    float4* s_colp = reinterpret_cast<float4*>(dyn_smem + (size_t)kWarps * NS * CW * sizeof(TM) +
                                               (NC > 0 ? kCredBytes : 0));  // [2][CW]
    float4* s_rowp = s_colp + 2 * CW;                                      // [2][kRB]
    float* s_cdp = reinterpret_cast<float*>(s_rowp + 2 * kRB);             // [2][CW] (LS only)
    __shared__ __align__(8) uint64_t s_pbar[2];
    constexpr bool STAGE_PARAMS = MIXED && !ROOT;

    if (STAGE_PARAMS && threadIdx.x == 0) {
        mbar_init(&s_pbar[0], 1);
        mbar_init(&s_pbar[1], 1);
    }
    __syncthreads();
    // Issue the parameter copies of tile number kk (of this CTA) into buffer kk % 2.
    auto issue_params = [&](int kk) {
        const int t = (int)blockIdx.x + kk * (int)gridDim.x;
        const int slab = t % nslabs, rb = t / nslabs;
        const int c0 = slab * CW, r0 = rb * kRB;
        const int ncol = (m - c0) < CW ? (m - c0) : CW;
        const int nrow = (n - r0) < kRB ? (n - r0) : kRB;
        uint64_t* bar = &s_pbar[kk & 1];
        const bool want_cd = op_uses_cd(OP) && p.cdsplit != nullptr;
        // 16-byte multiples: float4 entries always; cd floats in groups of 4
        const int ncd = want_cd ? (ncol / 4) * 4 : 0;
        const uint32_t bytes = (p.csplit ? (uint32_t)ncol * 16u : 0u) +
                               (p.rsplit ? (uint32_t)nrow * 16u : 0u) + (uint32_t)ncd * 4u;
        mbar_arrive_expect_tx(bar, bytes);
        if (p.csplit) bulk_g2s(s_colp + (kk & 1) * CW, p.csplit + c0, (uint32_t)ncol * 16u, bar);
        if (p.rsplit) bulk_g2s(s_rowp + (kk & 1) * kRB, p.rsplit + r0, (uint32_t)nrow * 16u, bar);
        if (ncd) bulk_g2s(s_cdp + (kk & 1) * CW, p.cdsplit + c0, (uint32_t)ncd * 4u, bar);
    };
    if (STAGE_PARAMS && threadIdx.x == 0) {
        if (my_tiles > 0) issue_params(0);
        if (my_tiles > 1) issue_params(1);
    }

    // Producer cursor (lane 0): the next row to issue, advanced in order.
    const int total = my_tiles * RPW;  // rows this warp streams
    int pk = 0, pu = 0;                // tile counter, row within the tile
    long long prow = 0;                // first row of this warp in the current tile
    const TM* psrc = nullptr;          // &M[prow, c0]
    uint32_t pseg = 0;                 // row segment bytes of the tile's slab
    auto cursor_tile = [&]() {
        const int t = (int)blockIdx.x + pk * (int)gridDim.x;
        const int slab = t % nslabs, rb = t / nslabs;
        const long long c0 = (long long)slab * CW;
        prow = (long long)rb * kRB + rw0;
        psrc = Mb + prow * ldm + c0;
        pseg = (uint32_t)((ldm - c0) < CW ? (ldm - c0) : CW) * (uint32_t)sizeof(TM);
    };
    auto issue = [&](int q) {  // row q of this warp == (pk, pu): each lane copies its own vectors
        const bool valid = prow + pu < n;
        if (valid) {
            TM* dst = ring + (size_t)(q % NS) * CW;
            const TM* src = psrc + (long long)pu * ldm;
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const int off = (v * 32 + lane) * VW;
                if ((uint32_t)(off * (int)sizeof(TM)) < pseg)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst + off)), "l"(src + off) : "memory");
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (++pu == RPW) {
            pu = 0;
            if (++pk < my_tiles) cursor_tile();
        }
    };
    if (total > 0) cursor_tile();
    for (int q = 0; q < NS; ++q) {
        if (q < total) issue(q);
        else asm volatile("cp.async.commit_group;" ::: "memory");
    }

    // Constants prepared on the host (no FP64 arithmetic in this kernel:
    // FP64 throughput on this part is a small fraction of FP32).
    const TM kexp = MIXED ? (TM)p.kexp_f : (TM)p.kexp_d;
    const TM inv_reg = MIXED ? (TM)p.inv_reg_f : (TM)p.inv_reg_d;
    const TM init = ISMAX ? (TM)(-INFINITY) : (TM)0;
    TM steps[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) steps[t] = (TM)p.steps[t];
    const int nsteps = p.nsteps;

    // The averaged-plan totals are accumulated per row in the pass's type and
    // added into FP64 here (the duality-gap test needs them to ~1e-9).
    constexpr bool AVG = OP == OP_E_AVG || OP == OP_Q_AVG;
    using TotT = typename std::conditional<AVG, double, Acc>::type;
    TotT tot[NTa];
#pragma unroll
    for (int t = 0; t < NTa; ++t) tot[t] = 0;
    bool ok_wait = true;

#pragma unroll 1
    for (int k = 0; k < my_tiles; ++k) {
        const int t = (int)blockIdx.x + k * (int)gridDim.x;
        const int slab = t % nslabs, rb = t / nslabs;
        const int c0 = slab * CW, r0 = rb * kRB;
        const int seg = (int)((ldm - c0) < CW ? (ldm - c0) : CW);

        if constexpr (STAGE_PARAMS) {
            const bool got = mbar_wait_bounded(&s_pbar[k & 1], (uint32_t)((k >> 1) & 1), p.err,
                                               p.wait_limit);
            ok_wait = ok_wait && got;
        }
        // ---- per-column parameters of this slab (only what OP uses) ----
        // Per-column vectors stay in registers, loaded once per tile. Reading
        // them from the staged parameters in the element loop instead (no
        // spills at 128 registers) was measured slower: a lane's columns are
        // 16 bytes apart in the staged arrays, so those reads conflict on
        // the shared-memory banks (HVP 0.64 -> 0.26 of peak).
        TM ch[LC], clk[LC], cxv[op_uses_cx(OP) ? LC : 1], cx2v[op_uses_cx2(OP) ? LC : 1],
            cdv[op_uses_cd(OP) ? LC : 1];
        // root passes: the column values in FP64 (FP64 M), or rounded to FP32
        // for the mixed engine's filter (its exact test reloads them)
        double cbd[(ROOT && !MIXED) ? LC : 1];
        float cbf[(ROOT && MIXED) ? LC : 1];
        bool cvalid[LC];
#pragma unroll
        for (int q = 0; q < LC; ++q) {
            const int v = q / VW, e = q % VW;
            const int j = c0 + (v * 32 + lane) * VW + e;
            const bool ok = j < m;
            cvalid[q] = ok;
            if constexpr (ROOT) {
                if constexpr (MIXED) cbf[q] = ok ? __double2float_rn(p.cb[j]) : -INFINITY;
                else cbd[q] = ok ? p.cb[j] : -INFINITY;
                ch[q] = 0;
                clk[q] = 0;
            } else if constexpr (MIXED) {
                const float4 c = (ok && p.csplit) ? s_colp[(k & 1) * CW + (j - c0)]
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
                ch[q] = ok ? c.x : -INFINITY;
                // EROT folds the exp2 scale into the low part: lo * kexp.
                clk[q] = ok ? (EROT ? __fmul_rn(c.y, kexp) : c.y) : 0.f;
                if constexpr (op_uses_cx(OP)) cxv[q] = c.z;
                if constexpr (op_uses_cx2(OP)) cx2v[q] = c.w;
                if constexpr (op_uses_cd(OP)) {
                    // entries past the last group of four were not staged
                    const int jj = j - c0;
                    const int ncol = (m - c0) < CW ? (m - c0) : CW;
                    cdv[q] = (ok && p.cdsplit)
                                 ? (jj < (ncol / 4) * 4 ? s_cdp[(k & 1) * CW + jj] : p.cdsplit[j])
                                 : 0.f;
                }
            } else {
                ch[q] = ok ? ((p.cb && op_needs_cb(OP)) ? (TM)p.cb[j] : (TM)0) : (TM)(-INFINITY);
                clk[q] = 0;
                if constexpr (op_uses_cx(OP)) cxv[q] = (ok && p.cx) ? (TM)p.cx[j] : (TM)0;
                if constexpr (op_uses_cx2(OP)) cx2v[q] = (ok && p.cx2) ? (TM)p.cx2[j] : (TM)0;
                if constexpr (op_uses_cd(OP)) cdv[q] = (ok && p.cd) ? (TM)p.cd[j] : (TM)0;
            }
        }
        auto cd_at = [&](int q) -> TM { return cdv[q]; };
        Acc cacc[NCa][LC];
#pragma unroll
        for (int c = 0; c < NCa; ++c)
#pragma unroll
            for (int q = 0; q < LC; ++q) cacc[c][q] = (Acc)init;
        // Per-lane partials of the warp's RPW rows of this tile.
        Acc rowv[NRa][RPW];
#pragma unroll
        for (int rr = 0; rr < NRa; ++rr)
#pragma unroll
            for (int u = 0; u < RPW; ++u) rowv[rr][u] = (Acc)init;

        // Rows are processed in pairs: both waits and both shared-memory
        // loads come first, so the two rows' element chains interleave.
#pragma unroll
        for (int u2 = 0; u2 < RPW; u2 += 2) {
            VT mvp[2][NV];
            TM prh[2], prlk[2], prx[2], prd[2];
            double prad[2];
#pragma unroll
            for (int r2 = 0; r2 < 2; ++r2) {
                // groups are committed one per row (empty past the end), so
                // the pair's two rows are complete when at most NS - 2 of the
                // lane's groups are still pending
                if (r2 == 0) asm volatile("cp.async.wait_group %0;" ::"n"(NS - 2) : "memory");
                const int u = u2 + r2;
                const int qs = k * RPW + u;
                const int i = r0 + rw0 + u;
                prh[r2] = 0;
                prlk[r2] = 0;
                prx[r2] = 0;
                prd[r2] = 0;
                prad[r2] = 0.0;
#pragma unroll
                for (int v = 0; v < NV; ++v) mvp[r2][v] = Vec<TM>::zero();
                if (i < n) {
                    if constexpr (ROOT) {
                        prad[r2] = p.ra ? p.ra[i] : 0.0;
                    } else if constexpr (MIXED) {
                        const float4 r = p.rsplit ? s_rowp[(k & 1) * kRB + (i - r0)]
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
                        prh[r2] = r.x;
                        prlk[r2] = EROT ? __fmul_rn(r.y, kexp) : r.y;
                        prx[r2] = r.z;
                        prd[r2] = r.w;
                    } else {
                        prh[r2] = (p.ra && op_needs_ra(OP)) ? (TM)p.ra[i] : (TM)0;
                        if constexpr (op_uses_rx(OP)) prx[r2] = p.rx ? (TM)p.rx[i] : (TM)0;
                        if constexpr (op_uses_rd(OP)) prd[r2] = p.rd ? (TM)p.rd[i] : (TM)0;
                    }
                    const TM* buf = ring + (size_t)(qs % NS) * CW;
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        const int off = (v * 32 + lane) * VW;
                        if (ok_wait && off < seg)
                            mvp[r2][v] = *reinterpret_cast<const VT*>(buf + off);
                    }
                }
            }
            // Both buffers are free once every lane has read them into
            // registers: refill them before the rows are reduced, so that the
            // copies overlap this pair's arithmetic. The warp barrier orders
            // the generic-proxy reads before the async-proxy writes.
#pragma unroll
            for (int r2 = 0; r2 < 2; ++r2) {
                const int qs = k * RPW + u2 + r2;
                if (qs + NS < total) issue(qs + NS);
                else asm volatile("cp.async.commit_group;" ::: "memory");
            }
#pragma unroll
            for (int r2 = 0; r2 < 2; ++r2) {
                const int u = u2 + r2;
                const int i = r0 + rw0 + u;
                if (i >= n) continue;
                const TM rh = prh[r2], rlk = prlk[r2], rxv = prx[r2], rdv = prd[r2];
                const double rad = prad[r2];
                (void)rxv;
                (void)rdv;
                (void)rad;
                // root passes, mixed engine: the row value in FP32 for the filter
                const float radf = (ROOT && MIXED) ? __double2float_rn(rad) : 0.f;
                (void)radf;
                const VT(&mv)[NV] = mvp[r2];
                    Acc racc[NRa];
    #pragma unroll
                    for (int rr = 0; rr < NRa; ++rr) racc[rr] = (Acc)init;
                    uint32_t bits = 0;
                    (void)bits;
                    constexpr bool PAIRED = MIXED && (OP == OP_E_ROW || OP == OP_E_COL ||
                                                      OP == OP_E_ROWCOL || OP == OP_E_HVP);
                    if constexpr (PAIRED) {
                        // Two columns per instruction with the packed FP32x2
                        // arithmetic of sm_100+: same roundings as the scalar path.
                        const float2 rh2 = make_float2(rh, rh), rl2 = make_float2(rlk, rlk);
                        const float2 k2 = make_float2(kexp, kexp), neg1 = make_float2(-1.f, -1.f);
                        float2 racc2 = make_float2(0.f, 0.f);
    #pragma unroll
                        for (int q = 0; q < LC; q += 2) {
                            const float2 mv2 = make_float2(Vec<TM>::get(mv[q / VW], q % VW),
                                                           Vec<TM>::get(mv[q / VW], (q + 1) % VW));
                            float2 sv = __fadd2_rn(rh2, make_float2(ch[q], ch[q + 1]));
                            sv = __ffma2_rn(mv2, neg1, sv);  // (hi_i + hi_j) - M_ij, one rounding
                            const float2 lo = __fadd2_rn(rl2, make_float2(clk[q], clk[q + 1]));
                            const float2 z = __ffma2_rn(sv, k2, lo);
                            const float2 T = make_float2(ex2_approx(z.x), ex2_approx(z.y));
                            if constexpr (OP == OP_E_ROW || OP == OP_E_ROWCOL) {
                                racc2 = __fadd2_rn(racc2, T);
                            }
                            if constexpr (OP == OP_E_COL || OP == OP_E_ROWCOL) {
                                const float2 c = __fadd2_rn(make_float2(cacc[0][q], cacc[0][q + 1]), T);
                                cacc[0][q] = c.x;
                                cacc[0][q + 1] = c.y;
                            }
                            if constexpr (OP == OP_E_HVP) {
                                racc2 = __ffma2_rn(T, make_float2(cxv[q], cxv[q + 1]), racc2);
                                const float2 c = __ffma2_rn(T, make_float2(rxv, rxv),
                                                            make_float2(cacc[0][q], cacc[0][q + 1]));
                                cacc[0][q] = c.x;
                                cacc[0][q + 1] = c.y;
                            }
                        }
                        racc[0] = racc2.x + racc2.y;
                    }
                    // QROT objective / gradient and line-search trial, two
                    // columns per packed FP32x2 instruction: the argument is
                    // formed in the scalar path's order, and the relu, the
                    // trial shift and the second-order remainder of the
                    // objective change follow it per component.
                    constexpr bool QPAIRED = MIXED && (OP == OP_Q_GRAD || OP == OP_Q_GRADLS);
                    if constexpr (QPAIRED) {
                        const float2 rh2 = make_float2(rh, rh), rl2 = make_float2(rlk, rlk);
                        const float2 neg1 = make_float2(-1.f, -1.f), half2 = make_float2(0.5f, 0.5f);
                        const float2 st2 = make_float2(steps[0], steps[0]), rd2 = make_float2(rdv, rdv);
                        float2 racc2 = make_float2(0.f, 0.f), t0 = make_float2(0.f, 0.f),
                               t1 = make_float2(0.f, 0.f);
    #pragma unroll
                        for (int q = 0; q < LC; q += 2) {
                            const float2 mv2 = make_float2(Vec<TM>::get(mv[q / VW], q % VW),
                                                           Vec<TM>::get(mv[q / VW], (q + 1) % VW));
                            float2 sv = __fadd2_rn(rh2, make_float2(ch[q], ch[q + 1]));
                            sv = __ffma2_rn(mv2, neg1, sv);
                            const float2 arg =
                                __fadd2_rn(sv, __fadd2_rn(rl2, make_float2(clk[q], clk[q + 1])));
                            if constexpr (OP == OP_Q_GRAD) {
                                const float2 D = make_float2(fmaxf(arg.x, 0.f), fmaxf(arg.y, 0.f));
                                racc2 = __fadd2_rn(racc2, D);
                                const float2 c = __fadd2_rn(make_float2(cacc[0][q], cacc[0][q + 1]), D);
                                cacc[0][q] = c.x;
                                cacc[0][q + 1] = c.y;
                                t0 = __ffma2_rn(D, D, t0);
                            } else {
                                const float2 sw =
                                    __fmul2_rn(st2, __fadd2_rn(rd2, make_float2(cd_at(q), cd_at(q + 1))));
                                const float2 Cn = __fadd2_rn(arg, sw);
                                const float2 Dn = make_float2(fmaxf(Cn.x, 0.f), fmaxf(Cn.y, 0.f));
                                // 0.5 (Dn^2 - D^2) - s w D >= 0 in every case
                                const float2 ra = __fmul2_rn(half2, __fmul2_rn(sw, sw));
                                const float2 rb = __fmul2_rn(make_float2(-arg.x, -arg.y),
                                                             __ffma2_rn(half2, arg, sw));
                                const float2 rc = __fmul2_rn(half2, __fmul2_rn(Cn, Cn));
                                const float2 rem = make_float2(
                                    arg.x > 0.f ? (Cn.x > 0.f ? ra.x : rb.x) : (Cn.x > 0.f ? rc.x : 0.f),
                                    arg.y > 0.f ? (Cn.y > 0.f ? ra.y : rb.y) : (Cn.y > 0.f ? rc.y : 0.f));
                                racc2 = __fadd2_rn(racc2, Dn);
                                const float2 c = __fadd2_rn(make_float2(cacc[0][q], cacc[0][q + 1]), Dn);
                                cacc[0][q] = c.x;
                                cacc[0][q + 1] = c.y;
                                t0 = __ffma2_rn(Dn, Dn, t0);
                                t1 = __fadd2_rn(t1, rem);
                            }
                        }
                        racc[0] = racc2.x + racc2.y;
                        tot[0] += t0.x + t0.y;
                        if constexpr (OP == OP_Q_GRADLS) tot[1] += t1.x + t1.y;
                    }
                    double pv[VW];  // plan values of one vector (plan passes)
                    (void)pv;
                    Acc rchunk[2] = {(Acc)0, (Acc)0};  // this row's averaged-plan totals
                    (void)rchunk;
    #pragma unroll
                    for (int q = 0; q < ((PAIRED || QPAIRED) ? 0 : LC); ++q) {
                        const TM mval = Vec<TM>::get(mv[q / VW], q % VW);
                        if constexpr (OP == OP_E_ROWMAX) {
                            TM a;
                            if constexpr (MIXED) a = (ch[q] - mval) + clk[q] * (TM)p.inv_kexp_f;
                            else a = ch[q] - mval;
                            racc[0] = fmax(racc[0], a);
                        } else if constexpr (OP == OP_E_COLMAX) {
                            TM a;
                            if constexpr (MIXED) a = (rh - mval) + rlk * (TM)p.inv_kexp_f;
                            else a = rh - mval;
                            if (cvalid[q]) cacc[0][q] = fmax(cacc[0][q], (Acc)a);
                        } else if constexpr (COLROOT) {
                            if constexpr (MIXED) {
                                // y = M - ra_i is below cb_j on a few entries per
                                // column: an FP32 test rules out the rest, and only
                                // entries within its error bound (2^-21 of the
                                // magnitudes, about 8x the worst rounding) take the
                                // exact FP64 test, so the active set and the sums
                                // are those of the FP64 test on every entry
                                const float yf = mval - radf;
                                const float d = yf - cbf[q];
                                const float bnd = fmaf(kRootSlack,
                                                       fabsf(yf) + (fabsf(radf) + fabsf(cbf[q])),
                                                       kRootFloor);
                                if (cvalid[q] && !(d > bnd)) {
                                    const int j = c0 + ((q / VW) * 32 + lane) * VW + (q % VW);
                                    const double y = (double)mval - rad;
                                    if (y < p.cb[j]) {
                                        cacc[0][q] += 1.0;
                                        cacc[1][q] += y;
                                    }
                                }
                            } else {
                                const double y = (double)mval - rad;
                                if (cvalid[q] && y < cbd[q]) {
                                    cacc[0][q] += 1.0;
                                    cacc[1][q] += y;
                                }
                            }
                        } else if constexpr (ROWROOT) {
                            if constexpr (MIXED) {
                                // the same filter for y = M - cb_j below ra_i
                                const float yf = mval - cbf[q];
                                const float d = yf - radf;
                                const float bnd = fmaf(kRootSlack,
                                                       fabsf(yf) + (fabsf(radf) + fabsf(cbf[q])),
                                                       kRootFloor);
                                if (cvalid[q] && !(d > bnd)) {
                                    const int j = c0 + ((q / VW) * 32 + lane) * VW + (q % VW);
                                    const double y = (double)mval - p.cb[j];
                                    if (y < rad) {
                                        racc[0] += 1.0;
                                        racc[1] += y;
                                    }
                                }
                            } else {
                                const double y = (double)mval - cbd[q];
                                if (cvalid[q] && y < rad) {
                                    racc[0] += 1.0;
                                    racc[1] += y;
                                }
                            }
                        } else if constexpr (EROT) {
                            // T = 2^((ra_i + cb_j - M_ij) log2(e) / reg): exact hi sum,
                            // then (hi - M) * k + (lo_i + lo_j) * k in one FMA.
                            TM T;
                            if constexpr (MIXED) {
                                const TM s = (rh + ch[q]) - mval;
                                T = ex2_approx(fmaf(s, kexp, rlk + clk[q]));
                            } else {
                                T = exp(((rh + ch[q]) - mval) * kexp);
                            }
                            if constexpr (OP == OP_E_ROW) {
                                racc[0] += T;
                            } else if constexpr (OP == OP_E_COL) {
                                cacc[0][q] += T;
                            } else if constexpr (OP == OP_E_ROWCOL) {
                                racc[0] += T;
                                cacc[0][q] += T;
                            } else if constexpr (OP == OP_E_HVP) {
                                racc[0] += T * cxv[q];
                                cacc[0][q] += T * rxv;
                            } else if constexpr (OP == OP_E_LS) {
                                const TM w = (rdv + cd_at(q)) * inv_reg;
                                tot[0] += T * expm1_minus_x(steps[0] * w);
                                // a uniform branch: a one-step pass (the full
                                // step tried alone) evaluates one series
                                if (nsteps > 1) {
    #pragma unroll
                                    for (int s2 = 1; s2 < 4; ++s2)
                                        if (s2 < nsteps)
                                            tot[s2] += T * expm1_minus_x(steps[s2] * w);
                                }
                            } else if constexpr (OP == OP_E_PLAN) {
                                plan_put<VW>(pv, q, (double)T, p.out, i, m, c0, lane);
                            } else if constexpr (OP == OP_E_GRADLS) {
                                racc[0] += T;
                                cacc[0][q] += T;
                                if (cvalid[q]) {
                                    // T e^(-s w) is T at the base point
                                    const TM sw = steps[0] * ((rdv + cd_at(q)) * inv_reg);
                                    TM back;
                                    if constexpr (MIXED) back = ex2_approx(-sw * 1.44269504f);
                                    else back = exp(-sw);
                                    tot[0] += (T * back) * expm1_minus_x(sw);
                                }
                            } else if constexpr (OP == OP_E_AVG) {
                                if (cvalid[q]) {
                                    const int j = c0 + ((q / VW) * 32 + lane) * VW + (q % VW);
                                    TM* X = static_cast<TM*>(p.xavg) + (long long)i * m + j;
                                    const TM xo = nsteps > 0 ? *X : (TM)0;
                                    const TM xn = nsteps > 0 ? ((TM)1 - steps[0]) * xo + steps[0] * T : T;
                                    *X = xn;
                                    racc[0] += xn;
                                    cacc[0][q] += xn;
                                    rchunk[0] += mval * xn;
                                    // FP64: 0 (1 - log 0) is NaN, as in the reference's
                                    // array expression; an FP32 zero is an underflow of a
                                    // positive value and contributes its limit 0
                                    if constexpr (MIXED) rchunk[1] += xn > 0.f ? xn * (1.f - logf(xn)) : 0.f;
                                    else rchunk[1] += xn * (1.0 - log(xn));
                                }
                            }
                        } else {
                            TM arg;
                            if constexpr (MIXED) arg = ((rh + ch[q]) - mval) + (rlk + clk[q]);
                            else arg = (rh + ch[q]) - mval;
                            const TM D = arg > (TM)0 ? arg : (TM)0;
                            if constexpr (OP == OP_Q_GRAD) {
                                racc[0] += D;
                                cacc[0][q] += D;
                                tot[0] += D * D;
                            } else if constexpr (OP == OP_Q_GRADMASK) {
                                const bool pos = arg > (TM)0;
                                racc[0] += D;
                                cacc[0][q] += D;
                                tot[0] += D * D;
                                racc[1] += pos ? (TM)1 : (TM)0;
                                cacc[1][q] += pos ? (TM)1 : (TM)0;
                                const uint32_t word = __ballot_sync(0xffffffffu, pos);
                                if (lane == q) bits = word;
                            } else if constexpr (OP == OP_Q_GRADLS) {
                            // objective change along s w without cancellation:
                            // 0.5 (Dn^2 - D^2) - s w D >= 0 in every case
                            const TM sw = steps[0] * (rdv + cd_at(q));
                            const TM Cn = arg + sw;
                            const TM Dn = Cn > (TM)0 ? Cn : (TM)0;
                            TM rem;
                            if (arg > (TM)0) rem = Cn > (TM)0 ? (TM)0.5 * sw * sw
                                                              : -arg * ((TM)0.5 * arg + sw);
                            else rem = Cn > (TM)0 ? (TM)0.5 * Cn * Cn : (TM)0;
                            racc[0] += Dn;
                            cacc[0][q] += Dn;
                            tot[0] += Dn * Dn;
                            tot[1] += rem;
                        } else if constexpr (OP == OP_Q_OBJ) {
                                tot[0] += D * D;
                            } else if constexpr (OP == OP_Q_P1) {
                                racc[0] += D;
                            } else if constexpr (OP == OP_Q_P2) {
                                cacc[0][q] += D * rxv;
                            } else if constexpr (OP == OP_Q_P3) {
                                const TM Dy = D * cxv[q];
                                racc[0] += Dy;
                                racc[1] += Dy * cx2v[q];
                                racc[2] += mval * cx2v[q];
                                const TM R = rxv * Dy;
                                tot[0] += R * mval;
                                tot[1] += R * R;
                            } else if constexpr (OP == OP_Q_PLAN) {
                                plan_put<VW>(pv, q, (double)D * p.inv_reg_d, p.out, i, m, c0, lane);
                            } else if constexpr (OP == OP_Q_AVG) {
                                if (cvalid[q]) {
                                    const int j = c0 + ((q / VW) * 32 + lane) * VW + (q % VW);
                                    TM* X = static_cast<TM*>(p.xavg) + (long long)i * m + j;
                                    const TM xd = D * inv_reg;
                                    const TM xn = nsteps > 0 ? steps[0] * *X + steps[1] * xd : xd;
                                    *X = xn;
                                    racc[0] += xn;
                                    cacc[0][q] += xn;
                                    rchunk[0] += mval * xn;
                                    rchunk[1] += xn * xn;
                                }
                            }
                        }
                    }
                    if constexpr (OP == OP_Q_GRADMASK) {
                        if (lane < LC) p.bitmask[((long long)i * nslabs + slab) * LC + lane] = bits;
                    }
                    if constexpr (AVG) {
                        tot[0] += (double)rchunk[0];
                        tot[1] += (double)rchunk[1];
                    }

#pragma unroll
                for (int rr = 0; rr < NR; ++rr) rowv[rr][u] = racc[rr];
            }
        }

        // ---- row partials of this tile ----
        if constexpr (NR > 0) {
            Acc* rp = reinterpret_cast<Acc*>(p.rowpart);
            const int i = r0 + rw0 + (lane >> (5 - LOGR));
#pragma unroll
            for (int rr = 0; rr < NR; ++rr) {
                const Acc tot_r = warp_reduce_rows<ISMAX, RPW>(rowv[rr], lane);
                if ((lane & ((1 << (5 - LOGR)) - 1)) == 0 && i < n)
                    rp[((long long)rr * nslabs + slab) * n + i] = tot_r;
            }
        }

        // ---- column partials of this tile: reduce the warps through a
        // buffer of half of them (upper half stores, lower half adds) ----
        if constexpr (NC > 0) {
            constexpr int HW = kWarps / 2;
            if (warp >= HW) {
#pragma unroll
                for (int c = 0; c < NC; ++c)
#pragma unroll
                    for (int q = 0; q < LC; ++q) {
                        const int off = (q / VW) * 32 * VW + lane * VW + (q % VW);
                        s_cred[((size_t)c * HW + (warp - HW)) * CW + off] = cacc[c][q];
                    }
            }
            __syncthreads();
            if (warp < HW) {
#pragma unroll
                for (int c = 0; c < NC; ++c)
#pragma unroll
                    for (int q = 0; q < LC; ++q) {
                        const int off = (q / VW) * 32 * VW + lane * VW + (q % VW);
                        Acc& slot = s_cred[((size_t)c * HW + warp) * CW + off];
                        slot = ISMAX ? fmax(slot, cacc[c][q]) : slot + cacc[c][q];
                    }
            }
            __syncthreads();
            Acc* cp = reinterpret_cast<Acc*>(p.colpart);
            for (int tt = threadIdx.x; tt < CW; tt += kThreads) {
                const int j = c0 + tt;
                if (j >= m) continue;
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    Acc s = s_cred[((size_t)c * HW + 0) * CW + tt];
#pragma unroll
                    for (int w = 1; w < HW; ++w) {
                        const Acc x = s_cred[((size_t)c * HW + w) * CW + tt];
                        s = ISMAX ? fmax(s, x) : s + x;
                    }
                    cp[((long long)c * nrb + rb) * m + j] = s;
                }
            }
            __syncthreads();
        }
        if constexpr (STAGE_PARAMS) {
            // Every warp is done with this tile's parameter buffer: refill it.
            if constexpr (NC == 0) __syncthreads();
            if (threadIdx.x == 0 && k + 2 < my_tiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_params(k + 2);
            }
        }
    }

    asm volatile("cp.async.wait_all;" ::: "memory");  // nothing in flight at exit
    // ---- per-CTA totals ----
    if constexpr (NT > 0) {
        __shared__ double s_t[NT][kWarps];
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const double v = warp_sum((double)tot[t]);
            if (lane == 0) s_t[t][warp] = v;
        }
        __syncthreads();
        if (threadIdx.x < NT) {
            double s = 0.0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) s += s_t[threadIdx.x][w];
            p.totpart[(long long)threadIdx.x * gridDim.x + blockIdx.x] = s;
        }
    }
}


template <typename TM, int OP, int CFG>
constexpr size_t pass_smem_bytes() {
    using Acc = typename std::conditional<op_fp64_acc(OP), double, TM>::type;
    constexpr int CW = Geo<TM>::CW;
    constexpr int NS = PassCfg<CFG>::kStages;
    return (size_t)kWarps * NS * CW * sizeof(TM) +
           (size_t)(op_nc(OP) > 0 ? op_nc(OP) : 0) * (kWarps / 2) * CW * sizeof(Acc) +
           2 * ((size_t)CW * 16 + (size_t)kRB * 16 + (op_uses_cd(OP) ? (size_t)CW * 4 : 0));
}

// Opt in to the pass's dynamic shared memory, once per device (host threads
// may race here: the attribute is idempotent).
template <typename TM, int OP, int CFG>
void configure_pass() {
    static std::atomic<unsigned long long> configured{0};
    int dev = 0;
    REGOT_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(configured.load(std::memory_order_acquire) & (1ULL << dev))) {
        REGOT_CUDA(cudaFuncSetAttribute(dense_pass<TM, OP, CFG>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)pass_smem_bytes<TM, OP, CFG>()));
        if (dev < 64) configured.fetch_or(1ULL << dev, std::memory_order_acq_rel);
    }
}

template <typename TM, int OP, int CFG>
void launch_one(const PassParams& p, cudaStream_t st, int blocks) {
    configure_pass<TM, OP, CFG>();
    dense_pass<TM, OP, CFG><<<blocks, kThreads, pass_smem_bytes<TM, OP, CFG>(), st>>>(p);
    REGOT_CHECK_LAUNCH();
    count_launch();
}

template <typename TM, int OP, int CFG>
int occupancy_of() {
    configure_pass<TM, OP, CFG>();
    int occ = 0;
    REGOT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ, dense_pass<TM, OP, CFG>, kThreads, pass_smem_bytes<TM, OP, CFG>()));
    const int cap = PassCfg<CFG>::kMinBlocks;
    return occ > 0 ? (occ < cap ? occ : cap) : 1;
}

template <typename TM, int CFG>
struct Dispatch {
    template <int OP>
    static void go(int op, const PassParams& p, cudaStream_t st, int blocks) {
        if constexpr (OP < OP_COUNT) {
            if (op == OP) launch_one<TM, OP, CFG>(p, st, blocks);
            else go<OP + 1>(op, p, st, blocks);
        } else {
            throw Error(REGOT_ERR_INVALID_ARG, "unknown dense pass");
        }
    }
    template <int OP>
    static int occ(int op) {
        if constexpr (OP < OP_COUNT) return op == OP ? occupancy_of<TM, OP, CFG>() : occ<OP + 1>(op);
        else return 1;
    }
};

}  // namespace

template <typename TM, int CFG>
void launch_pass_cfg(int op, const PassParams& p, cudaStream_t st, int blocks) {
    Dispatch<TM, CFG>::template go<0>(op, p, st, blocks);
}

template <typename TM, int CFG>
int occupancy_cfg(int op) {
    return Dispatch<TM, CFG>::template occ<0>(op);
}

}  // namespace regot
