// sinkhorn_ssns on the GPU (reference: src/sinkhorn_ssns.cpp:16-234).
//
// One iteration:
//  * the direction solves (H_s + shift I) d = -g for the sparsified Hessian
//    H_s = [diag(h1) S; S' diag(h2)], S = sparsify(T) / reg
//    (sinkhorn_hess.h:46-158, sinkhorn_hess.cpp:15-164), by conjugate
//    gradients on the Schur complement of the beta block
//    Delta = diag(h2 + shift) - S' diag(1 / (h1 + shift)) S (sinkhorn_cg.cpp:9-50);
//  * line_selection over {1, .5, .25, .1} (sinkhorn_problem_ls.cpp:13-41)
//    evaluates all four candidates in one dense pass, on exact objective
//    differences f(gamma + s d) - f(gamma) = s g'd + reg sum T phi(s w)
//    (phi(x) = e^x - 1 - x, w_ij = (d_i + d_j) / reg);
//  * rho = (f - f_new) / (-g's - s'H_s s / 2) decides whether gamma moves and
//    how the shift factor mu changes (sinkhorn_ssns.cpp:146-176);
//  * after a move: gradient pass, then the sparsification.
//
// Linear solver. Method 0 is the reference's CG exactly: identity
// preconditioner, relative residual 1e-8, at most 2 (m - 1) iterations.
// Method 1 (the default) factors H_s with SimplicialLDLT in the reference
// (sinkhorn_linsolve.cpp:58-106); here it is the same Schur-complement CG with
// a Jacobi preconditioner run to the relative residual cg_tol (1e-10), so the
// direction equals the factorisation's to that accuracy.
//
// Sparsification (sparsify_mat3, sinkhorn_sparsify3.cpp:276-405):
//  1. k_tt writes T' (column j of T as a contiguous row, j < m - 1);
//  2. k_col_select finds per column the threshold
//       x_j = min{x in column j : sum of the column's values <= x exceeds delta}
//     by a weighted radix select over the bit patterns of T (non-negative
//     floating-point numbers order like their bit patterns). The entries
//     below x_j are the dropped ones: the smallest entries whose sum stays
//     <= delta. find_small (from the small side) and find_large (from the
//     large side, target colsum - delta) both select exactly this set in
//     exact arithmetic. They differ when the column sum is <= delta:
//     find_small then drops every entry (x_j = inf), find_large keeps the
//     largest (x_j = column maximum). density_hint > 0.2 selects find_small
//     (sinkhorn_sparsify3.cpp:303);
//  3. k_row_stage forms per row the dropped values d_ij, their sum R_i and,
//     where R_i > 2 delta, the threshold y_i = min{y : sum of d_ij <= y
//     exceeds 2 delta}; dropped entries >= y_i are kept again
//     (sinkhorn_sparsify3.cpp:333-353). It writes the row's kept entries in
//     column order (CSR rows, fixed stride m - 1);
//  4. k_csc_fill writes the same kept entries per column in row order from T'
//     (CSC columns, fixed stride n).
// The kept entries are those with Delta == 0 (sinkhorn_sparsify3.cpp:378):
// every exact zero of the FP64 T is one. Zeros count towards nnz and the
// density but add nothing to a product, so k_tt counts them and they are not
// stored. In mixed mode T is FP32 with flush-to-zero; the FP64 T is zero when
// its base-2 exponent argument is below -1075.
//
// Threshold sums are exact integer sums of the values in a fixed-point scale
// of about 2^-61 times the column (row) sum, so the selection does not depend
// on the summation order and uses no FP64 arithmetic (slow on this GPU). It
// can differ from the reference's sequential FP64 sums only where a partial
// sum lies within about 1e-15 (relative) of delta.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <limits>
#include <type_traits>
#include <vector>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "solvers.h"
#include "wolfe.h"

namespace regot {

namespace {

constexpr int kVT = 64;            // vector kernels
constexpr int kSelThreads = 256;   // selection / fill kernels
constexpr int kSelWarps = kSelThreads / 32;
constexpr int kSpWarps = 8;        // warp-per-row sparse kernels: 8 warps per block
constexpr unsigned kFull = 0xffffffffu;
constexpr size_t kMaxCacheBytes = 160 * 1024;

struct SsnState {
    unsigned counter;
    int done;
    int it;
    int max_it;
    double shift;
    double absnew;   // r'z of the CG residual
    double alpha;
    double beta;
    double thresh2;
    double rr;
    double f;
    double gnorm;
    double gtd;      // g'd
    double dhd;      // d'H_s d
    double maxabs;
    double nnz;      // stored kept entries
};

__device__ __forceinline__ float ex2_approx_f(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// T_ij exactly as the mixed dense passes form it (hi parts summed exactly,
// lo parts scaled, one FMA, ex2.approx), and whether the FP64 T is zero.
__device__ __forceinline__ float t_mixed(float mv, float4 r, float4 c, float kexp, bool& zero64) {
    const float s = (r.x + c.x) - mv;
    const float z = fmaf(s, kexp, __fadd_rn(__fmul_rn(r.y, kexp), __fmul_rn(c.y, kexp)));
    zero64 = z < -1075.0f;
    return ex2_approx_f(z);
}

__device__ __forceinline__ double t_plain(double mv, double ra, double cb, double kexp,
                                          bool& zero64) {
    const double t = exp(((ra + cb) - mv) * kexp);
    zero64 = (t == 0.0);
    return t;
}

template <typename TM>
struct KeyOf;
template <>
struct KeyOf<float> {
    using U = unsigned;
    __device__ static U key(float v) { return __float_as_uint(v); }
    __device__ static float val(U k) { return __uint_as_float(k); }
};
template <>
struct KeyOf<double> {
    using U = unsigned long long;
    __device__ static U key(double v) { return (U)__double_as_longlong(v); }
    __device__ static double val(U k) { return __longlong_as_double((long long)k); }
};

constexpr int kBins = 2048;  // widest radix digit: 11 bits

struct SelSmem {
    unsigned long long hsum[kBins];
    unsigned hcnt[kBins];
    unsigned long long wscan[kSelWarps];
    double red[kSelWarps];
    double red2[kSelWarps];
    int wcount[kSelWarps];
    unsigned long long base;
    double result;
    int bin;
    unsigned count;
};

// v * 2^k truncated to an integer, from the bit pattern (v >= 0 finite,
// v * 2^k < 2^63): the threshold sums are exact integer sums, so they do not
// depend on the summation order and need no FP64 arithmetic.
__device__ __forceinline__ unsigned long long fix_of(float v, int k) {
    const unsigned bits = __float_as_uint(v);
    const int e = (int)(bits >> 23);
    unsigned long long mant = bits & 0x7fffffu;
    int sh;
    if (e == 0) {
        sh = k - 149;
    } else {
        mant |= 0x800000u;
        sh = e - 150 + k;
    }
    if (sh >= 0) return mant << sh;
    return sh > -64 ? (mant >> -sh) : 0ull;
}
__device__ __forceinline__ unsigned long long fix_of(double v, int k) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int e = (int)(bits >> 52);
    unsigned long long mant = bits & 0xfffffffffffffull;
    int sh;
    if (e == 0) {
        sh = k - 1074;
    } else {
        mant |= 0x10000000000000ull;
        sh = e - 1075 + k;
    }
    if (sh >= 0) return mant << sh;
    return sh > -64 ? (mant >> -sh) : 0ull;
}

// Scale 2^k with est * 2^k < 2^61 (est >= the sum to be formed, up to the
// rounding of its estimate) and target * 2^k as an integer (saturated).
__device__ __forceinline__ int fix_scale(double est) {
    return est > 0.0 ? 60 - ilogb(est) : 0;
}
__device__ __forceinline__ unsigned long long fix_target(double target, int k) {
    const double t = ldexp(target, k);
    return t >= 1.8e19 ? ~0ull : (unsigned long long)floor(t);
}

// Block-wide sum (in TM: an estimate that only sets the fixed-point scale)
// and maximum of v[0, len).
template <typename TM>
__device__ void block_est_max(const TM* v, int len, SelSmem& sh, double& est, double& mx) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    TM s = 0, m = 0;
    for (int k = threadIdx.x; k < len; k += kSelThreads) {
        const TM x = v[k];
        s += x;
        m = x > m ? x : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(kFull, s, o);
        const TM mo = __shfl_xor_sync(kFull, m, o);
        m = mo > m ? mo : m;
    }
    if (lane == 0) {
        sh.red[w] = (double)s;
        sh.red2[w] = (double)m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, mm = 0.0;
        for (int q = 0; q < kSelWarps; ++q) {
            t += sh.red[q];
            mm = fmax(mm, sh.red2[q]);
        }
        sh.result = mm;
        // headroom for the rounding of the estimate
        sh.red[0] = t * (1.0 + 1e-3) + mm;
    }
    __syncthreads();
    est = sh.red[0];
    mx = sh.result;
    __syncthreads();
}

template <typename TM>
struct Digits;
template <>
struct Digits<float> {
    static constexpr int kTop = 30;  // key bits 30..0 (the sign bit is 0)
};
template <>
struct Digits<double> {
    static constexpr int kTop = 62;
};

// Smallest x among v[0, len) (values >= 0) with sum_{v_k <= x} v_k > target,
// in the fixed-point scale 2^k (target already scaled; x > 0), by a radix select
// over the bit patterns: 11-bit then 10/11-bit digits, most significant
// first. Each round histograms the candidates (entries sharing the digits
// chosen so far) into integer bin sums and counts with shared-memory atomics,
// scans the bins and keeps the bin where the running sum first exceeds
// target. Returns false when the total does not exceed target.
template <typename TM>
__device__ bool block_select(const TM* v, int len, unsigned long long target, int k,
                             SelSmem& sh, TM& out) {
    using K = KeyOf<TM>;
    using U = typename K::U;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    U prefix = 0, mask = 0;
    unsigned long long base = 0;
    int hi = Digits<TM>::kTop;
    bool first = true;
    while (hi >= 0) {
        const int width = first ? 11 : ((hi + 1) % 11 == 0 ? 11 : 10);
        const int lo = hi - width + 1 > 0 ? hi - width + 1 : 0;
        const int nb = 1 << (hi - lo + 1);
        for (int b = threadIdx.x; b < nb; b += kSelThreads) {
            sh.hsum[b] = 0ull;
            sh.hcnt[b] = 0u;
        }
        if (threadIdx.x == 0) sh.bin = -1;
        __syncthreads();
        for (int q = threadIdx.x; q < len; q += kSelThreads) {
            const TM val = v[q];
            const U key = K::key(val);
            // zeros add nothing and cannot complete a crossing
            if (key != 0 && (key & mask) == prefix) {
                const int b = (int)((key >> lo) & (U)(nb - 1));
                atomicAdd(&sh.hsum[b], fix_of(val, k));
                atomicAdd(&sh.hcnt[b], 1u);
            }
        }
        __syncthreads();
        // Exclusive scan over the bins: each thread owns nb / 256 consecutive bins.
        const int per = nb / kSelThreads;
        const int b0 = threadIdx.x * per;
        unsigned long long ls = 0;
        for (int q = 0; q < per; ++q) ls += sh.hsum[b0 + q];
        unsigned long long inc = ls;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long o = __shfl_up_sync(kFull, inc, d);
            if (lane >= d) inc += o;
        }
        if (lane == 31) sh.wscan[w] = inc;
        __syncthreads();
        unsigned long long run = base + (inc - ls);
        for (int q = 0; q < w; ++q) run += sh.wscan[q];
        for (int q = 0; q < per; ++q) {
            const unsigned long long nx = run + sh.hsum[b0 + q];
            if (run <= target && nx > target && sh.hcnt[b0 + q] > 0) {
                sh.bin = b0 + q;
                sh.base = run;
                sh.count = sh.hcnt[b0 + q];
            }
            run = nx;
        }
        __syncthreads();
        const int sb = sh.bin;
        const unsigned cnt = sh.count;
        const unsigned long long nbase = sh.base;
        __syncthreads();
        if (sb < 0) return false;
        prefix |= (U)sb << lo;
        mask |= (U)(nb - 1) << lo;
        base = nbase;
        if (cnt == 1 && lo > 0) {
            // a single candidate left: it is the answer
            for (int q = threadIdx.x; q < len; q += kSelThreads) {
                const TM val = v[q];
                if ((K::key(val) & mask) == prefix) sh.result = (double)val;
            }
            __syncthreads();
            out = (TM)sh.result;
            __syncthreads();
            return true;
        }
        hi = lo - 1;
        first = false;
    }
    out = K::val(prefix);
    return true;
}

// Ordered compaction of the indices k in [0, len) with keep(k): emit(k, slot)
// with consecutive slots in index order. Each warp owns a contiguous segment:
// it counts its kept entries, the warps' offsets come from one block-wide
// exchange, and a second sweep writes. Returns the total.
template <typename Keep, typename Emit>
__device__ int block_compact(int len, SelSmem& sh, Keep keep, Emit emit) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int seg = (len + kSelThreads - 1) / kSelThreads * 32;
    const int lo = w * seg;
    const int hi = lo + seg < len ? lo + seg : len;
    int cnt = 0;
    for (int k0 = lo; k0 < hi; k0 += 32) {
        const int k = k0 + lane;
        cnt += __popc(__ballot_sync(kFull, k < hi && keep(k)));
    }
    if (lane == 0) sh.wcount[w] = cnt;
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int q = 0; q < kSelWarps; ++q) {
        const int c = sh.wcount[q];
        off += q < w ? c : 0;
        tot += c;
    }
    for (int k0 = lo; k0 < hi; k0 += 32) {
        const int k = k0 + lane;
        const bool kp = k < hi && keep(k);
        const unsigned bal = __ballot_sync(kFull, kp);
        if (kp) emit(k, off + __popc(bal & ((1u << lane) - 1u)));
        off += __popc(bal);
    }
    __syncthreads();
    return tot;
}

struct DenseArgs {
    const void* M;
    long long ldm;
    int n, m1;
    const float4* rs;  // mixed: row split
    const float4* cs;  // mixed: column split
    float kexp_f;
    const double* gamma;  // plain: duals (beta at gamma + n)
    double kexp_d;
};

template <typename TM>
__device__ __forceinline__ TM t_at(const DenseArgs& a, int i, int j, TM mv, bool& z64);
template <>
__device__ __forceinline__ float t_at<float>(const DenseArgs& a, int i, int j, float mv,
                                             bool& z64) {
    return t_mixed(mv, a.rs[i], a.cs[j], a.kexp_f, z64);
}
template <>
__device__ __forceinline__ double t_at<double>(const DenseArgs& a, int i, int j, double mv,
                                               bool& z64) {
    return t_plain(mv, a.gamma[i], a.gamma[a.n + j], a.kexp_d, z64);
}

// T' (rows j < m - 1 of length n, stride ldt) and the count of FP64 zeros.
template <typename TM>
__global__ void __launch_bounds__(256) k_tt(DenseArgs a, TM* TT, long long ldt,
                                            unsigned long long* zeros) {
    __shared__ TM tile[32][33];
    const TM* M = static_cast<const TM*>(a.M);
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    unsigned zc = 0;
    const int j = j0 + tx;
#pragma unroll
    for (int k = ty; k < 32; k += 8) {
        const int i = i0 + k;
        TM t = 0;
        if (i < a.n && j < a.m1) {
            bool z64;
            t = t_at<TM>(a, i, j, M[(size_t)i * a.ldm + j], z64);
            zc += z64 ? 1u : 0u;
        }
        tile[tx][k] = t;
    }
    __syncthreads();
#pragma unroll
    for (int k = ty; k < 32; k += 8) {
        const int jj = j0 + k, ii = i0 + tx;
        if (jj < a.m1 && ii < a.n) TT[(size_t)jj * ldt + ii] = tile[k][tx];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) zc += __shfl_xor_sync(kFull, zc, o);
    if (tx == 0 && zc) atomicAdd(zeros, (unsigned long long)zc);
}

// T' for FP32 storage with 16-byte rows (M 16-byte aligned, ldm a multiple
// of 4): 32 rows x 128 columns per block. Warp w reads rows w, w + 8, ...
// as float4 per lane (each lane's four columns share their split entries
// across the rows), the tile is transposed through shared memory (row
// stride 33: the column-major reads are conflict-free) and written as float4
// per thread, eight threads per T' row segment.
__global__ void __launch_bounds__(256) k_tt4(DenseArgs a, float* TT, long long ldt,
                                             unsigned long long* zeros) {
    __shared__ float tile[128][33];
    const float* M = static_cast<const float*>(a.M);
    const int j0 = blockIdx.x * 128, i0 = blockIdx.y * 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int jl = 4 * lane, jg = j0 + jl;
    unsigned zc = 0;
    float4 cs4[4];
#pragma unroll
    for (int e = 0; e < 4; ++e)
        cs4[e] = jg + e < a.m1 ? a.cs[jg + e] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int il = w + 8 * r, i = i0 + il;
        float t[4] = {0.f, 0.f, 0.f, 0.f};
        if (i < a.n) {
            const float4 rr = a.rs[i];
            const float* row = M + (size_t)i * a.ldm;
            float mv[4];
            if (jg + 3 < a.m1) {
                const float4 q = __ldg(reinterpret_cast<const float4*>(row + jg));
                mv[0] = q.x;
                mv[1] = q.y;
                mv[2] = q.z;
                mv[3] = q.w;
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) mv[e] = jg + e < a.m1 ? row[jg + e] : 0.f;
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (jg + e < a.m1) {
                    bool z64;
                    t[e] = t_mixed(mv[e], rr, cs4[e], a.kexp_f, z64);
                    zc += z64 ? 1u : 0u;
                }
            }
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) tile[jl + e][il] = t[e];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int jr = (int)threadIdx.x / 8 + 32 * q;  // T' row within the tile
        const int ic = 4 * ((int)threadIdx.x % 8);     // first of its four entries
        const int j = j0 + jr, i = i0 + ic;
        if (j < a.m1 && i < a.n) {
            const float4 v = make_float4(tile[jr][ic], tile[jr][ic + 1], tile[jr][ic + 2],
                                         tile[jr][ic + 3]);
            *reinterpret_cast<float4*>(TT + (size_t)j * ldt + i) = v;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) zc += __shfl_xor_sync(kFull, zc, o);
    if (lane == 0 && zc) atomicAdd(zeros, (unsigned long long)zc);
}

// Column thresholds x_j (see the file comment).
template <typename TM>
__global__ void __launch_bounds__(kSelThreads) k_col_select(const TM* TT, long long ldt, int n,
                                                            int m1, double delta, int from_large,
                                                            int cache, TM* xout) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ SelSmem sh;
    TM* s_col = reinterpret_cast<TM*>(s_dyn);
    for (int j = blockIdx.x; j < m1; j += gridDim.x) {
        const TM* col = TT + (size_t)j * ldt;
        const TM* v = col;
        if (cache) {
            const int nvec = (int)(((size_t)n * sizeof(TM) + 15) / 16);
            const float4* src = reinterpret_cast<const float4*>(col);
            float4* dst = reinterpret_cast<float4*>(s_col);
            for (int k = threadIdx.x; k < nvec; k += kSelThreads) dst[k] = src[k];
            __syncthreads();
            v = s_col;
        }
        double est, mx;
        block_est_max(v, n, sh, est, mx);
        const int k = fix_scale(est);
        TM x;
        if (!block_select(v, n, fix_target(delta, k), k, sh, x))
            x = from_large ? (TM)mx : (TM)INFINITY;  // column sum <= delta
        if (threadIdx.x == 0) xout[j] = x;
        __syncthreads();
    }
}

struct RowStageArgs {
    int ldr;          // CSR row stride (m - 1)
    int cache;        // rows of T and d in shared memory
    long long lds;    // per-block scratch stride (2 rows) when not cached
    int keep_row0;    // keep every entry of row 0 (sparsify_mat_with_density)
};

// Row stage and CSR rows (see the file comment).
template <typename TM>
__global__ void __launch_bounds__(kSelThreads) k_row_stage(DenseArgs a, RowStageArgs r,
                                                           const TM* xcol, double delta2,
                                                           TM* scratch, TM* yout, int* rcount,
                                                           int* rcols, TM* rvals) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ SelSmem sh;
    const TM* M = static_cast<const TM*>(a.M);
    const int m1 = a.m1;
    TM* tbuf = r.cache ? reinterpret_cast<TM*>(s_dyn) : scratch + (size_t)blockIdx.x * r.lds;
    TM* dbuf = tbuf + (r.cache ? (size_t)((m1 + 3) & ~3) : (size_t)(r.lds / 2));
    for (int i = blockIdx.x; i < a.n; i += gridDim.x) {
        const TM* Mi = M + (size_t)i * a.ldm;
        for (int j = threadIdx.x; j < m1; j += kSelThreads) {
            bool z64;
            const TM t = t_at<TM>(a, i, j, Mi[j], z64);
            tbuf[j] = t;
            dbuf[j] = t < xcol[j] ? t : (TM)0;
        }
        __syncthreads();
        double est, mx;
        block_est_max(dbuf, m1, sh, est, mx);
        TM y = (TM)INFINITY;
        if (est > delta2) {  // est bounds the dropped mass from above
            const int k = fix_scale(est);
            TM yy;
            // the dropped mass exceeds 2 delta: re-keep down to y
            if (block_select(dbuf, m1, fix_target(delta2, k), k, sh, yy)) y = yy;
        }
        if (r.keep_row0 && i == 0) y = (TM)0;
        int* cols = rcols + (size_t)i * r.ldr;
        TM* vals = rvals + (size_t)i * r.ldr;
        const int total = block_compact(
            m1, sh,
            [&](int j) {
                const TM t = tbuf[j];
                return t != (TM)0 && (t >= xcol[j] || t >= y);
            },
            [&](int j, int slot) {
                cols[slot] = j;
                vals[slot] = tbuf[j];
            });
        if (threadIdx.x == 0) {
            rcount[i] = total;
            yout[i] = y;
        }
        __syncthreads();
    }
}

// CSC columns from T' with the column and row thresholds.
template <typename TM>
__global__ void __launch_bounds__(kSelThreads) k_csc_fill(const TM* TT, long long ldt, int n,
                                                          int m1, const TM* xcol, const TM* yrow,
                                                          int ldc, int cache, int* ccount,
                                                          int* crows, TM* cvals) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ SelSmem sh;
    TM* s_col = reinterpret_cast<TM*>(s_dyn);
    for (int j = blockIdx.x; j < m1; j += gridDim.x) {
        const TM* col = TT + (size_t)j * ldt;
        if (cache) {
            const int nvec = (int)(((size_t)n * sizeof(TM) + 15) / 16);
            const float4* src = reinterpret_cast<const float4*>(col);
            float4* dst = reinterpret_cast<float4*>(s_col);
            for (int k = threadIdx.x; k < nvec; k += kSelThreads) dst[k] = src[k];
            __syncthreads();
            col = s_col;
        }
        const TM xj = xcol[j];
        int* rows = crows + (size_t)j * ldc;
        TM* vals = cvals + (size_t)j * ldc;
        const int total = block_compact(
            n, sh,
            [&](int i) {
                const TM t = col[i];
                return t != (TM)0 && (t >= xj || t >= __ldg(yrow + i));
            },
            [&](int i, int slot) {
                rows[slot] = i;
                vals[slot] = col[i];
            });
        if (threadIdx.x == 0) ccount[j] = total;
    }
}

// ---- register-resident sparsification (rows and columns up to 256 x VPT) ----
// The same selections as k_col_select / k_row_stage / k_csc_fill, with each
// row (column) held in registers: thread t owns the VPT entries
// W (t + 256 c) + e (c < VPT / W, e < W, W entries per 16-byte vector), all
// loaded up front by vector loads, so that a row's loads are in flight at
// once and the radix rounds, the threshold tests and the ordered compaction
// read registers. The first radix digit has 11 bits (the exponent and the
// leading mantissa bits: 2048 bins), the later ones 8; the answer of the
// select does not depend on the digit widths. Bin sums are exact 64-bit
// integers kept as two 32-bit words and added by 32-bit shared-memory
// atomics with an explicit carry.
// Blocks of 256 threads; the register bounds aim at three blocks per SM
// where the row fits in 32 words per thread without spills (two for the
// row stage, which also keeps the kept mask and the thresholds).
constexpr int kRT = 256;  // threads
constexpr int kRW = kRT / 32;
constexpr int kRBins = 2048;

struct RSmem {
    unsigned hlo[kRBins];
    unsigned hhi[kRBins];
    unsigned hcnt[kRBins];
    unsigned long long wtot[kRW];
    double red[kRW];
    double red2[kRW];
    int wcnt[16][kRW];  // compaction: per chunk and warp (VPT / W <= 16)
    unsigned long long base;
    double result;
    int bin;
    unsigned count;
};

// Exact 64-bit add into (hi, lo) by 32-bit atomics: the carry out of the low
// word is read from the value the atomic returns.
__device__ __forceinline__ void bin_add(unsigned* lo, unsigned* hi, unsigned long long v) {
    const unsigned vl = (unsigned)v, vh = (unsigned)(v >> 32);
    const unsigned old = atomicAdd(lo, vl);
    const unsigned up = vh + ((old + vl < old) ? 1u : 0u);
    if (up) atomicAdd(hi, up);
}

template <typename TM>
struct VecOf;
template <>
struct VecOf<float> {
    static constexpr int W = 4;
    using V = float4;
};
template <>
struct VecOf<double> {
    static constexpr int W = 2;
    using V = double2;
};

template <typename TM, int VPT>
__device__ __forceinline__ int r_index(int k) {
    constexpr int W = VecOf<TM>::W;
    return W * ((int)threadIdx.x + kRT * (k / W)) + (k % W);
}

// v[k] = src[r_index(k)] for indices < len, else 0. `vec`: src is 16-byte
// aligned and readable up to the end of the last vector that holds an index
// < len (rows padded to whole vectors).
template <typename TM, int VPT>
__device__ __forceinline__ void r_load(const TM* __restrict__ src, int len, bool vec,
                                       TM (&v)[VPT]) {
    constexpr int W = VecOf<TM>::W;
    using V = typename VecOf<TM>::V;
#pragma unroll
    for (int c = 0; c < VPT / W; ++c) {
        const int i0 = W * ((int)threadIdx.x + kRT * c);
        if (vec && i0 < len) {
            const V q = __ldg(reinterpret_cast<const V*>(src + i0));
            const TM* e = reinterpret_cast<const TM*>(&q);
#pragma unroll
            for (int w = 0; w < W; ++w) v[c * W + w] = (i0 + w < len) ? e[w] : (TM)0;
        } else {
#pragma unroll
            for (int w = 0; w < W; ++w) v[c * W + w] = (i0 + w < len) ? src[i0 + w] : (TM)0;
        }
    }
}

// The next row (column) of a block is fetched while the current one is
// processed: each thread copies its own vectors of that row into the
// shared-memory row buffer by cp.async (16 bytes each, the positions it
// reads back), so no block synchronisation guards the buffer; r_load_next
// waits for the thread's own copies and moves them into registers, after
// which the thread may start the following fetch into the same buffer.
template <typename TM, int VPT>
__device__ __forceinline__ void r_fetch(const TM* __restrict__ src, int len, TM* sbuf) {
    constexpr int W = VecOf<TM>::W;
#pragma unroll
    for (int c = 0; c < VPT / W; ++c) {
        const int i0 = W * ((int)threadIdx.x + kRT * c);
        if (i0 < len)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                             static_cast<uint32_t>(__cvta_generic_to_shared(sbuf + i0))),
                         "l"(src + i0)
                         : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <typename TM, int VPT>
__device__ __forceinline__ void r_load_next(const TM* sbuf, int len, TM (&v)[VPT]) {
    constexpr int W = VecOf<TM>::W;
    using V = typename VecOf<TM>::V;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
#pragma unroll
    for (int c = 0; c < VPT / W; ++c) {
        const int i0 = W * ((int)threadIdx.x + kRT * c);
        if (i0 < len) {
            const V q = *reinterpret_cast<const V*>(sbuf + i0);
            const TM* e = reinterpret_cast<const TM*>(&q);
#pragma unroll
            for (int w = 0; w < W; ++w) v[c * W + w] = (i0 + w < len) ? e[w] : (TM)0;
        } else {
#pragma unroll
            for (int w = 0; w < W; ++w) v[c * W + w] = (TM)0;
        }
    }
}

// Shared bytes of the row buffer of the register kernels.
template <typename TM, int VPT>
constexpr size_t r_row_bytes() {
    return (size_t)kRT * VPT * sizeof(TM);
}

// Block sum estimate (as block_est_max: TM sums per thread and warp, FP64
// over warps, with headroom for their rounding) and maximum of the entries
// v[k] with bit k of `use` set (the others count as 0).
template <typename TM, int VPT>
__device__ void r_est_max(const TM (&v)[VPT], unsigned long long use, RSmem& sh, double& est,
                          double& mx) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    TM s = 0, m = 0;
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
        const TM x = ((use >> k) & 1ull) ? v[k] : (TM)0;
        s += x;
        m = x > m ? x : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(kFull, s, o);
        const TM mo = __shfl_xor_sync(kFull, m, o);
        m = mo > m ? mo : m;
    }
    if (lane == 0) {
        sh.red[w] = (double)s;
        sh.red2[w] = (double)m;
    }
    __syncthreads();
    double t = 0.0, mm = 0.0;
#pragma unroll
    for (int q = 0; q < kRW; ++q) {
        t += sh.red[q];
        mm = fmax(mm, sh.red2[q]);
    }
    est = t * (1.0 + 1e-3) + mm;
    mx = mm;
    __syncthreads();
}

// Block-wide select of block_select's threshold over the register values
// v[k] with bit k of `use` set (zeros ignored), most significant digit first.
template <typename TM, int VPT>
__device__ bool r_select(const TM (&v)[VPT], unsigned long long use, unsigned long long target,
                         int kscale, RSmem& sh, TM& out) {
    using K = KeyOf<TM>;
    using U = typename K::U;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    U prefix = 0, mask = 0;
    unsigned long long base = 0;
    int hi = Digits<TM>::kTop;
    bool first = true;
    while (hi >= 0) {
        const int width = first ? 11 : 8;
        const int lo = hi - width + 1 > 0 ? hi - width + 1 : 0;
        const int nb = 1 << (hi - lo + 1);
        for (int b = tid; b < nb; b += kRT) {
            sh.hlo[b] = 0u;
            sh.hhi[b] = 0u;
            sh.hcnt[b] = 0u;
        }
        if (tid == 0) sh.bin = -1;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
            const U key = K::key(v[k]);
            if (((use >> k) & 1ull) && key != 0 && (key & mask) == prefix) {
                const int b = (int)((key >> lo) & (U)(nb - 1));
                bin_add(&sh.hlo[b], &sh.hhi[b], fix_of(v[k], kscale));
                atomicAdd(&sh.hcnt[b], 1u);
            }
        }
        __syncthreads();
        // exclusive scan of the bin sums: thread t owns `per` consecutive bins
        const int per = nb > kRT ? nb / kRT : 1;
        const int b0 = tid * per;
        const bool owner = b0 < nb;
        unsigned long long ls = 0;
        if (owner)
            for (int q = 0; q < per; ++q)
                ls += ((unsigned long long)sh.hhi[b0 + q] << 32) | sh.hlo[b0 + q];
        unsigned long long inc = ls;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long o = __shfl_up_sync(kFull, inc, d);
            if (lane >= d) inc += o;
        }
        if (lane == 31) sh.wtot[w] = inc;
        __syncthreads();
        unsigned long long run = base + (inc - ls);
#pragma unroll
        for (int q = 0; q < kRW; ++q) run += q < w ? sh.wtot[q] : 0ull;
        if (owner) {
            for (int q = 0; q < per; ++q) {
                const int b = b0 + q;
                const unsigned long long nx =
                    run + (((unsigned long long)sh.hhi[b] << 32) | sh.hlo[b]);
                if (run <= target && nx > target && sh.hcnt[b] > 0) {
                    sh.bin = b;
                    sh.base = run;
                    sh.count = sh.hcnt[b];
                }
                run = nx;
            }
        }
        __syncthreads();
        const int sb = sh.bin;
        const unsigned cnt = sh.count;
        const unsigned long long nbase = sh.base;
        __syncthreads();
        if (sb < 0) return false;
        prefix |= (U)sb << lo;
        mask |= (U)(nb - 1) << lo;
        base = nbase;
        if (cnt == 1 && lo > 0) {
            // a single candidate left: it is the answer
#pragma unroll
            for (int k = 0; k < VPT; ++k)
                if (((use >> k) & 1ull) && K::key(v[k]) != 0 && (K::key(v[k]) & mask) == prefix)
                    sh.result = (double)v[k];
            __syncthreads();
            out = (TM)sh.result;
            __syncthreads();
            return true;
        }
        hi = lo - 1;
        first = false;
    }
    out = K::val(prefix);
    return true;
}

// Ordered compaction of the register entries with bit k of `keep` set:
// emit(k, slot) with consecutive slots in index order. Returns the total.
template <typename TM, int VPT, typename Emit>
__device__ int r_compact(unsigned long long keep, RSmem& sh, Emit emit) {
    constexpr int W = VecOf<TM>::W;
    constexpr int NC = VPT / W;
    static_assert(NC <= 16, "compaction chunks");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const int cnt = __popcll((keep >> (c * W)) & ((1ull << W) - 1ull));
        int x = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(kFull, x, d);
            if (lane >= d) x += o;
        }
        incl[c] = x - cnt;  // exclusive within the warp
        if (lane == 31) sh.wcnt[c][w] = x;
    }
    __syncthreads();
    int before = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        int woff = 0, ctot = 0;
#pragma unroll
        for (int q = 0; q < kRW; ++q) {
            const int x = sh.wcnt[c][q];
            ctot += x;
            woff += q < w ? x : 0;
        }
        int slot = before + woff + incl[c];
#pragma unroll
        for (int e = 0; e < W; ++e) {
            const int k = c * W + e;
            if ((keep >> k) & 1ull) emit(k, slot++);
        }
        before += ctot;
    }
    __syncthreads();
    return before;
}

// Column thresholds x_j from the rows of T' (k_col_select).
template <typename TM, int VPT>
__global__ void __launch_bounds__(kRT, VPT * sizeof(TM) <= 128 ? 3 : 1) k_col_select_r(const TM* __restrict__ TT, long long ldt,
                                                      int n, int m1, double delta, int from_large,
                                                      TM* __restrict__ xout) {
    __shared__ RSmem sh;
    extern __shared__ __align__(16) unsigned char r_dyn[];
    TM* sbuf = reinterpret_cast<TM*>(r_dyn);
    if ((int)blockIdx.x < m1) r_fetch<TM, VPT>(TT + (size_t)blockIdx.x * ldt, n, sbuf);
    for (int j = blockIdx.x; j < m1; j += gridDim.x) {
        TM v[VPT];
        r_load_next<TM, VPT>(sbuf, n, v);
        if (j + (int)gridDim.x < m1)
            r_fetch<TM, VPT>(TT + (size_t)(j + gridDim.x) * ldt, n, sbuf);
        double est, mx;
        r_est_max<TM, VPT>(v, ~0ull, sh, est, mx);
        const int k = fix_scale(est);
        TM x;
        if (!r_select<TM, VPT>(v, ~0ull, fix_target(delta, k), k, sh, x))
            x = from_large ? (TM)mx : (TM)INFINITY;  // column sum <= delta
        if (threadIdx.x == 0) xout[j] = x;
    }
}

// Row stage and CSR rows (k_row_stage): T of row i from M, its dropped
// entries (below the column thresholds), the row threshold y_i where their
// sum exceeds delta2, and the kept entries in column order.
template <typename TM, int VPT>
__global__ void __launch_bounds__(kRT, VPT * sizeof(TM) <= 64 ? 3 : VPT * sizeof(TM) <= 128 ? 2 : 1) k_row_stage_r(DenseArgs a, int ldr, int keep_row0,
                                                     int vec, const TM* __restrict__ xcol,
                                                     double delta2, TM* __restrict__ yout,
                                                     int* __restrict__ rcount,
                                                     int* __restrict__ rcols,
                                                     TM* __restrict__ rvals) {
    __shared__ RSmem sh;
    extern __shared__ __align__(16) unsigned char r_dyn[];
    TM* sbuf = reinterpret_cast<TM*>(r_dyn);
    const TM* M = static_cast<const TM*>(a.M);
    const int m1 = a.m1;
    if (vec && (int)blockIdx.x < a.n) r_fetch<TM, VPT>(M + (size_t)blockIdx.x * a.ldm, m1, sbuf);
    for (int i = blockIdx.x; i < a.n; i += gridDim.x) {
        TM t[VPT];
        if (vec) {
            r_load_next<TM, VPT>(sbuf, m1, t);
            if (i + (int)gridDim.x < a.n)
                r_fetch<TM, VPT>(M + (size_t)(i + gridDim.x) * a.ldm, m1, sbuf);
        } else {
            r_load<TM, VPT>(M + (size_t)i * a.ldm, m1, false, t);
        }
        unsigned long long drop = 0ull;
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
            const int j = r_index<TM, VPT>(k);
            TM tk = 0;
            if (j < m1) {
                bool z64;
                tk = t_at<TM>(a, i, j, t[k], z64);
                if (tk < __ldg(xcol + j)) drop |= 1ull << k;
            }
            t[k] = tk;
        }
        double est, mx;
        r_est_max<TM, VPT>(t, drop, sh, est, mx);
        TM y = (TM)INFINITY;
        if (est > delta2) {  // est bounds the dropped mass from above
            const int ks = fix_scale(est);
            TM yy;
            if (r_select<TM, VPT>(t, drop, fix_target(delta2, ks), ks, sh, yy)) y = yy;
        }
        if (keep_row0 && i == 0) y = (TM)0;
        unsigned long long keep = 0ull;
#pragma unroll
        for (int k = 0; k < VPT; ++k)
            if (t[k] != (TM)0 && (!((drop >> k) & 1ull) || t[k] >= y)) keep |= 1ull << k;
        int* cols = rcols + (size_t)i * ldr;
        TM* vals = rvals + (size_t)i * ldr;
        const int total = r_compact<TM, VPT>(keep, sh, [&](int k, int slot) {
            cols[slot] = r_index<TM, VPT>(k);
            vals[slot] = t[k];
        });
        if (threadIdx.x == 0) {
            rcount[i] = total;
            yout[i] = y;
        }
    }
}

// CSC columns from T' with the column and row thresholds (k_csc_fill).
template <typename TM, int VPT>
__global__ void __launch_bounds__(kRT, VPT * sizeof(TM) <= 128 ? 3 : 1) k_csc_fill_r(const TM* __restrict__ TT, long long ldt,
                                                    int n, int m1, const TM* __restrict__ xcol,
                                                    const TM* __restrict__ yrow, int ldc,
                                                    int* __restrict__ ccount,
                                                    int* __restrict__ crows,
                                                    TM* __restrict__ cvals) {
    __shared__ RSmem sh;
    extern __shared__ __align__(16) unsigned char r_dyn[];
    TM* sbuf = reinterpret_cast<TM*>(r_dyn);
    if ((int)blockIdx.x < m1) r_fetch<TM, VPT>(TT + (size_t)blockIdx.x * ldt, n, sbuf);
    for (int j = blockIdx.x; j < m1; j += gridDim.x) {
        TM v[VPT];
        r_load_next<TM, VPT>(sbuf, n, v);
        if (j + (int)gridDim.x < m1)
            r_fetch<TM, VPT>(TT + (size_t)(j + gridDim.x) * ldt, n, sbuf);
        const TM xj = xcol[j];
        unsigned long long keep = 0ull;
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
            const int i = r_index<TM, VPT>(k);
            if (i < n && v[k] != (TM)0 && (v[k] >= xj || v[k] >= __ldg(yrow + i)))
                keep |= 1ull << k;
        }
        int* rows = crows + (size_t)j * ldc;
        TM* vals = cvals + (size_t)j * ldc;
        const int total = r_compact<TM, VPT>(keep, sh, [&](int k, int slot) {
            rows[slot] = r_index<TM, VPT>(k);
            vals[slot] = v[k];
        });
        if (threadIdx.x == 0) ccount[j] = total;
    }
}

// Values per thread of the register path for rows of length len (a power
// of two, at least one vector), or 0 when the row is too long for it.
template <typename TM>
int r_vpt(int len) {
    constexpr int W = VecOf<TM>::W;
    constexpr int kMax = sizeof(TM) == 4 ? 64 : 32;
    int v = W;
    while ((long long)v * kRT < len) v *= 2;
    return v <= kMax ? v : 0;
}

template <typename TM, int V>
constexpr bool r_valid() {
    return V >= VecOf<TM>::W && V <= (sizeof(TM) == 4 ? 64 : 32);
}

// f(std::integral_constant<int, vpt>) for a valid vpt of the register path.
template <typename TM, typename F>
void r_dispatch(int vpt, F&& f) {
    auto go = [&](auto c) {
        if constexpr (r_valid<TM, decltype(c)::value>()) f(c);
    };
    switch (vpt) {
        case 2: go(std::integral_constant<int, 2>{}); break;
        case 4: go(std::integral_constant<int, 4>{}); break;
        case 8: go(std::integral_constant<int, 8>{}); break;
        case 16: go(std::integral_constant<int, 16>{}); break;
        case 32: go(std::integral_constant<int, 32>{}); break;
        case 64: go(std::integral_constant<int, 64>{}); break;
        default: break;
    }
}

// Grid of a register-path kernel: every block resident at once (the blocks
// loop over rows or columns), at most one block per row or column.
template <typename Kern>
int r_grid(Kern kern, int count, size_t smem) {
    // the row buffer may exceed the default 48 KB of dynamic shared memory
    // (idempotent; host threads may race here)
    REGOT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kRT, smem) != cudaSuccess ||
        occ < 1)
        occ = 1;
    return std::max(1, std::min(count, device_sm_count() * occ));
}

std::atomic<int> g_sparsify_legacy{0};

// Number of stored entries (sum of the row counts).
__global__ void k_nnz(const int* rcount, int n, double* parts, SsnState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {t < n ? (double)rcount[t] : 0.0};
    double out[1];
    __threadfence();
    if (grid_reduce<1>(v, parts, &st->counter, out)) st->nnz = out[0];
}

// ---- sparse products (one warp per row or column) ----
// FP64 engine: FP64 products and sums. Mixed engine (FP32 values): the
// vector operand comes as FP32 (hi, lo) pairs and every product and sum is
// formed in compensated FP32 (the exact product error by an FMA, TwoSum for
// the running sum), converted to FP64 once per row. FP64 instructions issue
// at a small fraction of the FP32 rate on this part, and one FP64 FMA (plus
// a conversion) per stored entry made the CG products FP64-bound; the
// compensated sums stay within about 2^-44 of sum |v x| per row.
struct Sparse {
    const int* rcount;
    const int* rcols;
    const void* rvals;
    int ldr;
    const int* ccount;
    const int* crows;
    const void* cvals;
    int ldc;
    int n, m1;
    double inv_reg;
    // mixed engine: FP32 (hi, lo) copies of the CG vectors, written by the
    // kernels that produce them, and 1 / (h1 + shift) in FP32 for the
    // preconditioner
    float2* u2;  // rows (n)
    float2* p2;  // columns (m - 1)
    float2* x2;  // columns: the beta part of the direction
    float2* d2;  // rows: the alpha part of the direction
    float* w32;  // rows
};

template <typename TM>
using SpVec = typename std::conditional<std::is_same<TM, float>::value, float2, double>::type;

__device__ __forceinline__ float2 split_df(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}

// The entries of a row are taken four per lane at a time, their loads
// issued before the products, so that a warp keeps several memory latencies
// in flight; the products are added in the order of k either way.
__device__ __forceinline__ double sp_dot(const double* v, const int* c, int cnt,
                                         const double* x) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    int k = lane;
    for (; k + 96 < cnt; k += 128) {
        double vv[4];
        int cc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            vv[u] = v[k + 32 * u];
            cc[u] = c[k + 32 * u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) s += vv[u] * x[cc[u]];
    }
    for (; k < cnt; k += 32) s += v[k] * x[c[k]];
    return warp_sum_d(s);
}

__device__ __forceinline__ void sp_acc(float& s, float& e, float vv, float2 xx) {
    const float p = vv * xx.x;
    const float pe = fmaf(vv, xx.x, -p);  // exact: vv xx.x = p + pe
    float t, te;
    two_sum_f(s, p, t, te);
    s = t;
    e += te + fmaf(vv, xx.y, pe);
}

__device__ __forceinline__ double sp_dot(const float* v, const int* c, int cnt, const float2* x) {
    const int lane = threadIdx.x & 31;
    float s = 0.f, e = 0.f;
    int k = lane;
    for (; k + 96 < cnt; k += 128) {
        float vv[4];
        int cc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            vv[u] = v[k + 32 * u];
            cc[u] = c[k + 32 * u];
        }
        float2 xx[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) xx[u] = x[cc[u]];
#pragma unroll
        for (int u = 0; u < 4; ++u) sp_acc(s, e, vv[u], xx[u]);
    }
    for (; k < cnt; k += 32) sp_acc(s, e, v[k], x[c[k]]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float so = __shfl_xor_sync(kFull, s, o);
        const float eo = __shfl_xor_sync(kFull, e, o);
        float t, te;
        two_sum_f(s, so, t, te);
        s = t;
        e += eo + te;
    }
    return (double)s + (double)e;
}

template <typename TM>
__device__ __forceinline__ double row_dot(const Sparse& S, int i, const SpVec<TM>* x) {
    const int cnt = S.rcount[i];
    const int* c = S.rcols + (size_t)i * S.ldr;
    const TM* v = static_cast<const TM*>(S.rvals) + (size_t)i * S.ldr;
    return sp_dot(v, c, cnt, x) * S.inv_reg;
}

template <typename TM>
__device__ __forceinline__ double col_dot(const Sparse& S, int j, const SpVec<TM>* x) {
    const int cnt = S.ccount[j];
    const int* r = S.crows + (size_t)j * S.ldc;
    const TM* v = static_cast<const TM*>(S.cvals) + (size_t)j * S.ldc;
    return sp_dot(v, r, cnt, x) * S.inv_reg;
}

// The operand of a sparse product: the FP64 vector itself, or (mixed) its
// FP32 (hi, lo) copy.
template <typename TM>
__device__ __forceinline__ const SpVec<TM>* sp_arg(const double* x, const float2* x2) {
    if constexpr (std::is_same<TM, float>::value) return x2;
    else return x;
}

template <typename TM>
__device__ __forceinline__ void put_split(float2* dst, int k, double v) {
    if constexpr (std::is_same<TM, float>::value) dst[k] = split_df(v);
}

// Vectors: h = (h1 [n], h2 [m - 1]) from the gradient pass, g, direction
// dir = (d_alpha [n], d_beta~ [m - 1], 0). The Schur CG works on x = d_beta~.

// Jacobi diagonal of the Schur complement (method 1). It only preconditions,
// so the mixed engine forms it in FP32 from w32 = 1 / (h1 + shift).
template <typename TM>
__global__ void k_schur_diag(Sparse S, const double* h, SsnState* st, double* diag) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (j >= S.m1) return;
    const double shift = st->shift;
    const int cnt = S.ccount[j];
    const int* r = S.crows + (size_t)j * S.ldc;
    const TM* v = static_cast<const TM*>(S.cvals) + (size_t)j * S.ldc;
    double s;
    if constexpr (std::is_same<TM, float>::value) {
        float sf = 0.f;
        for (int k = lane; k < cnt; k += 32) sf = fmaf(v[k] * v[k], S.w32[r[k]], sf);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sf += __shfl_xor_sync(kFull, sf, o);
        s = (double)sf * S.inv_reg * S.inv_reg;
    } else {
        s = 0.0;
        for (int k = lane; k < cnt; k += 32) {
            const double sv = v[k] * S.inv_reg;
            s += sv * sv / (h[r[k]] + shift);
        }
        s = warp_sum_d(s);
    }
    if (lane == 0) {
        const double dj = h[S.n + j] + shift;
        const double dd = dj - s;
        diag[j] = dd > 1e-3 * dj ? dd : dj;
    }
}

// u_i = rhs_alpha_i / (h1_i + shift) with rhs = -g; with u2 / w32 given (the
// mixed engine) also u's FP32 pair and 1 / (h1_i + shift) in FP32.
__global__ void k_schur_rhs_rows(int n, const double* g, const double* h, SsnState* st,
                                 double* u, float2* u2, float* w32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double w = 1.0 / (h[i] + st->shift);
        const double ui = -g[i] * w;
        u[i] = ui;
        if (u2) u2[i] = split_df(ui);
        if (w32) w32[i] = (float)w;
    }
}

// CG set-up on Delta x = rhs_beta - S' u: x = 0, r = that, z = r / diag, p = z.
template <typename TM>
__global__ void k_schur_init(Sparse S, const double* g, const double* u, const double* diag,
                             double tol, double* x, double* rv, double* z, double* p,
                             double* parts, SsnState* st) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double v[2] = {0.0, 0.0};
    if (j < S.m1) {
        const double w = col_dot<TM>(S, j, sp_arg<TM>(u, S.u2));
        if (lane == 0) {
            const double rj = -g[S.n + j] - w;
            const double zj = diag ? rj / diag[j] : rj;
            x[j] = 0.0;
            put_split<TM>(S.x2, j, 0.0);
            rv[j] = rj;
            z[j] = zj;
            p[j] = zj;
            put_split<TM>(S.p2, j, zj);
            v[0] = rj * rj;
            v[1] = rj * zj;
        }
    }
    double out[2];
    __threadfence();
    if (grid_reduce<2, true>(v, parts, &st->counter, out)) {
        st->thresh2 = fmax(tol * tol * out[0], 2.2250738585072014e-308);
        st->rr = out[0];
        st->absnew = out[1];
        st->it = 0;
        st->done = (out[0] == 0.0 || out[0] < st->thresh2) ? 1 : 0;
    }
}

// u_i = (S p)_i / (h1_i + shift).
template <typename TM>
__global__ void k_schur_rows(Sparse S, const double* p, const double* h, double* u,
                             SsnState* st) {
    if (st->done) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= S.n) return;
    const double s = row_dot<TM>(S, i, sp_arg<TM>(p, S.p2));
    if ((threadIdx.x & 31) == 0) {
        const double ui = s / (h[i] + st->shift);
        u[i] = ui;
        put_split<TM>(S.u2, i, ui);
    }
}

// q_j = (h2_j + shift) p_j - (S' u)_j and pq_j = p_j q_j. The warps of a
// block finish their columns independently (no block-wide reduction here:
// with a warp per column of uneven length, a block barrier kept the early
// warps waiting); k_schur_alpha adds the pq_j.
template <typename TM>
__global__ void k_schur_cols(Sparse S, const double* p, const double* u, const double* h,
                             double* q, double* pq, SsnState* st) {
    if (st->done) return;
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j < S.m1) {
        const double w = col_dot<TM>(S, j, sp_arg<TM>(u, S.u2));
        if ((threadIdx.x & 31) == 0) {
            const double qj = (h[S.n + j] + st->shift) * p[j] - w;
            q[j] = qj;
            pq[j] = p[j] * qj;
        }
    }
}

// alpha = r'z / p'q, p'q summed by one block in a fixed order.
__global__ void __launch_bounds__(1024) k_schur_alpha(int m1, const double* pq, SsnState* st) {
    if (st->done) return;
    __shared__ double s_w[32];
    double s = 0.0;
    for (int j = threadIdx.x; j < m1; j += 1024) s += pq[j];
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = s_w[threadIdx.x];
        t = warp_sum_d(t);
        if (threadIdx.x == 0) st->alpha = st->absnew / t;
    }
}

// x += alpha p, r -= alpha q, z = r / diag; stop on ||r||^2 < thresh2 or
// at the iteration limit (Eigen's ConjugateGradient loop). x2 (mixed): x's
// FP32 pair.
__global__ void k_schur_b(int m1, const double* p, const double* q, const double* diag,
                          double* x, double* rv, double* z, double* parts, SsnState* st,
                          float2* x2) {
    if (st->done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const double al = st->alpha;
    double v[2] = {0.0, 0.0};
    if (j < m1) {
        const double xj = x[j] + al * p[j];
        x[j] = xj;
        if (x2) x2[j] = split_df(xj);
        const double rj = rv[j] - al * q[j];
        rv[j] = rj;
        const double zj = diag ? rj / diag[j] : rj;
        z[j] = zj;
        v[0] = rj * rj;
        v[1] = rj * zj;
    }
    double out[2];
    __threadfence();
    if (grid_reduce<2>(v, parts, &st->counter, out)) {
        st->rr = out[0];
        st->it += 1;
        if (out[0] < st->thresh2 || st->it >= st->max_it || !(out[0] == out[0])) {
            st->done = 1;
        } else {
            st->beta = out[1] / st->absnew;
            st->absnew = out[1];
        }
    }
}

__global__ void k_schur_c(int m1, const double* z, double* p, SsnState* st, float2* p2) {
    if (st->done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m1) {
        const double pj = z[j] + st->beta * p[j];
        p[j] = pj;
        if (p2) p2[j] = split_df(pj);
    }
}

// d_alpha_i = (rhs_alpha_i - (S d_beta)_i) / (h1_i + shift).
template <typename TM>
__global__ void k_schur_back(Sparse S, const double* g, const double* h, double* dir,
                             SsnState* st) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= S.n) return;
    const double s = row_dot<TM>(S, i, sp_arg<TM>(dir + S.n, S.x2));
    if ((threadIdx.x & 31) == 0) {
        const double di = (-g[i] - s) / (h[i] + st->shift);
        dir[i] = di;
        put_split<TM>(S.d2, i, di);
    }
}

// d'H_s d and g'd: rows give d_a (h1 d_a + S d_b), cols d_b (h2 d_b + S' d_a).
template <typename TM>
__global__ void k_dhd_rows(Sparse S, const double* dir, const double* g, const double* h,
                           double* parts, SsnState* st) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    double v[2] = {0.0, 0.0};
    if (i < S.n) {
        const double s = row_dot<TM>(S, i, sp_arg<TM>(dir + S.n, S.x2));
        if ((threadIdx.x & 31) == 0) {
            const double di = dir[i];
            v[0] = di * (h[i] * di + s);
            v[1] = g[i] * di;
        }
    }
    double out[2];
    __threadfence();
    if (grid_reduce<2, true>(v, parts, &st->counter, out)) {
        st->dhd = out[0];
        st->gtd = out[1];
    }
}

template <typename TM>
__global__ void k_dhd_cols(Sparse S, const double* dir, const double* g, const double* h,
                           double* parts, SsnState* st) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    double v[2] = {0.0, 0.0};
    if (j < S.m1) {
        const double s = col_dot<TM>(S, j, sp_arg<TM>(dir, S.d2));
        if ((threadIdx.x & 31) == 0) {
            const double dj = dir[S.n + j];
            v[0] = dj * (h[S.n + j] * dj + s);
            v[1] = g[S.n + j] * dj;
        }
    }
    double out[2];
    __threadfence();
    if (grid_reduce<2, true>(v, parts, &st->counter, out)) {
        st->dhd += out[0];
        st->gtd += out[1];
    }
}

// f, g and h = (r / reg, c~ / reg) from the row/column sums of T.
template <typename Acc>
__global__ void k_ssns_grad(const Acc* rp, int nslabs, const Acc* cp, int nrb, int n, int m,
                            const double* gamma, const double* a, const double* b, double reg,
                            double* g, double* h, double* parts, SsnState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (t < n) {
        const double r = merge_strided(rp + t, nslabs, (size_t)n);
        const double gi = r - a[t];
        g[t] = gi;
        h[t] = r / reg;
        v[0] = gi * gi;
        v[1] = r;
        v[2] = gamma[t] * a[t];
    } else if (t < n + m) {
        const int j = t - n;
        if (j < m - 1) {
            const double c = merge_strided(cp + j, nrb, (size_t)m);
            const double gj = c - b[j];
            g[t] = gj;
            h[t] = c / reg;
            v[0] = gj * gj;
            v[3] = gamma[t] * b[j];
        } else {
            g[t] = 0.0;
            h[t] = 1.0;
        }
    }
    double out[4];
    __threadfence();
    if (grid_reduce<4>(v, parts, &st->counter, out)) {
        st->gnorm = sqrt(out[0]);
        st->f = reg * out[1] - out[2] - out[3];  // sinkhorn_problem_obj.cpp:389-390
    }
}

__global__ void k_ssns_move(int N, double s, const double* d, double* gamma) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < N) gamma[t] += s * d[t];
}

__global__ void k_ls_sum(const double* totpart, int nblocks, int nsteps, double* out) {
    const int s = threadIdx.x;
    if (s >= nsteps) return;
    double acc = 0.0;
    for (int k = 0; k < nblocks; ++k) acc += totpart[(size_t)s * nblocks + k];
    out[s] = acc;
}

// ---- global top-k threshold of T[:, :m-1] (sparsify_mat_with_density) ----
// The k-th largest value is found by a radix select over the bit patterns of
// T' (non-negative values order like their patterns): per digit, a grid-wide
// histogram of the candidates (entries whose higher digits match the prefix
// chosen so far), then one block picks the bin holding the k-th largest.
struct TopK {
    unsigned long long prefix, mask;
    unsigned long long rank;  // position of the threshold among the candidates, from the top
    int empty;                // k == 0: nothing but the preserved row and column
};

template <typename TM>
__global__ void __launch_bounds__(256) k_topk_hist(const TM* TT, long long ldt, int n, int m1,
                                                   const TopK* tk, int lo, int nb,
                                                   unsigned* ghist) {
    using K = KeyOf<TM>;
    using U = typename K::U;
    __shared__ unsigned s_h[kBins];
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s_h[b] = 0u;
    __syncthreads();
    const U prefix = (U)tk->prefix, mask = (U)tk->mask;
    constexpr int VW = 16 / (int)sizeof(TM);
    const long long vpr = ldt / VW;  // ldt is a multiple of VW
    const long long total = vpr * m1;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        const long long j = v / vpr;
        const int i0 = (int)(v - j * vpr) * VW;
        const float4 raw = *reinterpret_cast<const float4*>(TT + j * ldt + i0);
        const TM* e = reinterpret_cast<const TM*>(&raw);
#pragma unroll
        for (int q = 0; q < VW; ++q) {
            const U key = K::key(e[q]);
            if (i0 + q < n && (key & mask) == prefix)
                atomicAdd(&s_h[(int)((key >> lo) & (U)(nb - 1))], 1u);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        if (s_h[b]) atomicAdd(&ghist[b], s_h[b]);
}

// One block of 256 threads: thread t owns nb / 256 consecutive bins counted
// from the top; a scan over the threads gives the count above each bin.
__global__ void __launch_bounds__(256) k_topk_pick(TopK* tk, const unsigned* ghist, int lo,
                                                   int nb) {
    __shared__ unsigned long long s_w[8];
    __shared__ int s_bin;
    __shared__ unsigned long long s_above;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = nb / 256;
    const int btop = nb - t * per;  // this thread's bins: btop - 1 down to btop - per
    unsigned long long loc = 0;
    for (int q = 0; q < per; ++q) loc += ghist[btop - 1 - q];
    unsigned long long inc = loc;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long o = __shfl_up_sync(kFull, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) s_w[w] = inc;
    if (t == 0) s_bin = -1;
    __syncthreads();
    unsigned long long run = inc - loc;
    for (int q = 0; q < w; ++q) run += s_w[q];
    const unsigned long long r = tk->rank;
    for (int q = 0; q < per; ++q) {
        const int b = btop - 1 - q;
        const unsigned long long c = ghist[b];
        if (run < r && run + c >= r) {
            s_bin = b;
            s_above = run;
        }
        run += c;
    }
    __syncthreads();
    if (t == 0 && !tk->empty && s_bin >= 0) {
        tk->prefix |= (unsigned long long)s_bin << lo;
        tk->mask |= (unsigned long long)(nb - 1) << lo;
        tk->rank -= s_above;
    }
}

// Column thresholds of the density sparsification: column 0 keeps every
// entry, the others keep T >= the k-th largest value (all of its ties).
template <typename TM>
__global__ void k_topk_finish(const TopK* tk, int m1, TM* xcol) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m1) return;
    using K = KeyOf<TM>;
    const TM thr = tk->empty ? (TM)INFINITY : K::val((typename K::U)tk->prefix);
    xcol[j] = j == 0 ? (TM)0 : thr;
}

template <typename TM>
class SsnsEngine {
public:
    SsnsEngine(regot_ctx* ctx, regot_dproblem* P, double reg, const regot_opts& o)
        : P_(P), st_(ctx->stream), ops_(P, reg, st_), n_(P->n), m_(P->m), m1_(P->m - 1),
          reg_(reg), mixed_(P->prec == REGOT_PREC_MIXED) {
        const int N = n_ + m_;
        const int method = o.method < 0 ? 1 : o.method;
        jacobi_ = method != 0;
        tol_direct_ = o.cg_tol > 0.0 ? o.cg_tol : 1e-10;
        max_cg_ = o.cg_max_iter > 0 ? o.cg_max_iter : 2 * std::max(m1_, 1);
        max_direct_ = o.cg_max_iter > 0 ? o.cg_max_iter : 10 * std::max(m1_, 1);
        cg_max_ = jacobi_ ? max_direct_ : max_cg_;
        gamma_.alloc(N, st_);
        g_.alloc(N, st_);
        h_.alloc(N, st_);
        dir_.alloc(N, st_);
        u_.alloc(n_, st_);
        const int mm = std::max(m1_, 1);
        rv_.alloc(mm, st_);
        z_.alloc(mm, st_);
        p_.alloc(mm, st_);
        q_.alloc(mm, st_);
        pq_.alloc(mm, st_);
        diag_.alloc(mm, st_);
        parts_.alloc(4 * (size_t)std::max(cdiv(N, kVT), cdiv((long long)std::max(n_, m1_) * 32, 256)),
                     st_);
        state_.alloc(1, st_);
        SsnState z{};
        z.max_it = cg_max_;
        h2d(state_.get(), &z, sizeof(z), st_);
        lsout_.alloc(4, st_);
        zeros_.alloc(1, st_);
        // T' rows padded to 16 bytes; CSR / CSC with full-width strides.
        const int vec = 16 / (int)sizeof(TM);
        ldt_ = ((long long)n_ + vec - 1) / vec * vec;
        tt_.alloc((size_t)m1_ * ldt_, st_);
        xcol_.alloc(mm, st_);
        yrow_.alloc(n_, st_);
        rcount_.alloc(n_, st_);
        rcols_.alloc((size_t)n_ * m1_, st_);
        rvals_.alloc((size_t)n_ * m1_, st_);
        ccount_.alloc(mm, st_);
        crows_.alloc((size_t)m1_ * n_, st_);
        cvals_.alloc((size_t)m1_ * n_, st_);
        const int sms = device_sm_count();
        col_cache_ = (size_t)ldt_ * sizeof(TM) <= kMaxCacheBytes;
        const size_t col_smem = col_cache_ ? (size_t)ldt_ * sizeof(TM) : 0;
        REGOT_CUDA(cudaFuncSetAttribute(k_col_select<TM>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)col_smem));
        REGOT_CUDA(cudaFuncSetAttribute(k_csc_fill<TM>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)col_smem));
        col_smem_ = col_smem;
        const long long rowpad = ((long long)m1_ + 3) & ~3LL;
        row_cache_ = 2 * (size_t)rowpad * sizeof(TM) <= kMaxCacheBytes;
        row_smem_ = row_cache_ ? 2 * (size_t)rowpad * sizeof(TM) : 0;
        REGOT_CUDA(cudaFuncSetAttribute(k_row_stage<TM>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)row_smem_));
        col_grid_ = std::max(1, std::min(m1_, sms * 4));
        row_grid_ = std::max(1, std::min(n_, sms * 4));
        if (!row_cache_) row_scratch_.alloc((size_t)row_grid_ * 2 * rowpad, st_);
        lds_ = 2 * rowpad;
        S_.rcount = rcount_.get();
        S_.rcols = rcols_.get();
        S_.rvals = rvals_.get();
        S_.ldr = m1_;
        S_.ccount = ccount_.get();
        S_.crows = crows_.get();
        S_.cvals = cvals_.get();
        S_.ldc = n_;
        S_.n = n_;
        S_.m1 = m1_;
        S_.inv_reg = 1.0 / reg;
        S_.u2 = S_.p2 = S_.x2 = S_.d2 = nullptr;
        S_.w32 = nullptr;
        if (mixed_) {
            u2_.alloc(n_, st_);
            d2_.alloc(n_, st_);
            w32_.alloc(n_, st_);
            p2_.alloc(mm, st_);
            x2_.alloc(mm, st_);
            S_.u2 = u2_.get();
            S_.d2 = d2_.get();
            S_.w32 = w32_.get();
            S_.p2 = p2_.get();
            S_.x2 = x2_.get();
        }
    }

    double* gamma() { return gamma_.get(); }
    ErotOps& ops() { return ops_; }
    SsnState* state() { return state_.get(); }
    long long passes() const { return passes_; }

    SsnState read_state() {
        SsnState hs;
        read_small(P_->ctx, &hs, state_.get(), sizeof(hs), st_);
        return hs;
    }

    // f, g, h at gamma; leaves the FP32 split of gamma in the ops (mixed).
    void grad() {
        const PassShape sh = ops_.buf().shape;
        ops_.maxabs(gamma_.get(), n_ + m_, nullptr, 0, &state_.get()->maxabs);
        PassParams p = ops_.base_params();
        p.ra = gamma_.get();
        p.cb = gamma_.get() + n_;
        p.grid = &state_.get()->maxabs;
        ops_.pass(OP_E_ROWCOL, p);
        const int gv = cdiv(n_ + m_, kVT);
        if (mixed_)
            k_ssns_grad<float><<<gv, kVT, 0, st_>>>(
                (const float*)ops_.buf().rowpart.get(), sh.nslabs,
                (const float*)ops_.buf().colpart.get(), sh.nrb, n_, m_, gamma_.get(), P_->a,
                P_->b, reg_, g_.get(), h_.get(), parts_.get(), state_.get());
        else
            k_ssns_grad<double><<<gv, kVT, 0, st_>>>(
                (const double*)ops_.buf().rowpart.get(), sh.nslabs,
                (const double*)ops_.buf().colpart.get(), sh.nrb, n_, m_, gamma_.get(), P_->a,
                P_->b, reg_, g_.get(), h_.get(), parts_.get(), state_.get());
        count_launch();
        REGOT_CHECK_LAUNCH();
        ++passes_;
    }

    DenseArgs dense_args() const {
        DenseArgs a;
        a.M = P_->M;
        a.ldm = P_->ldm;
        a.n = n_;
        a.m1 = m1_;
        a.rs = ops_.rsplit();
        a.cs = ops_.csplit();
        a.kexp_f = (float)(1.4426950408889634 / reg_);
        a.gamma = gamma_.get();
        a.kexp_d = 1.0 / reg_;
        return a;
    }

    // sparsify_mat3 of T(gamma) (right after grad()); returns the density
    // (2 nnz + n + m - 1) / (n + m - 1)^2 (sinkhorn_hess.h:75-80).
    double sparsify(double delta, double density_hint) {
        if (m1_ <= 0) return 1.0;
        const DenseArgs a = dense_args();
        zeros_.zero();
        transpose(a);
        col_select(delta, density_hint > 0.2 ? 0 : 1);
        row_stage(a, 2.0 * delta, 0);
        csc_fill();
        k_nnz<<<cdiv(n_, kVT), kVT, 0, st_>>>(rcount_.get(), n_, parts_.get(), state_.get());
        count_launch();
        REGOT_CHECK_LAUNCH();
        passes_ += 4;
        unsigned long long zc = 0;
        d2h(&zc, zeros_.get(), sizeof(zc), st_);
        const SsnState hs = read_state();
        const double nnz = hs.nnz + (double)zc;
        const double dim = (double)(n_ + m_ - 1);
        return (2.0 * nnz + dim) / dim / dim;
    }

    // T' and the count of FP64 zeros of T.
    void transpose(const DenseArgs& a) {
        if constexpr (std::is_same<TM, float>::value) {
            if (reinterpret_cast<uintptr_t>(P_->M) % 16 == 0 && P_->ldm % 4 == 0) {
                dim3 grid(cdiv(m1_, 128), cdiv(n_, 32));
                k_tt4<<<grid, 256, 0, st_>>>(a, tt_.get(), ldt_, zeros_.get());
                count_launch();
                return;
            }
        }
        dim3 tgrid(cdiv(m1_, 32), cdiv(n_, 32));
        k_tt<TM><<<tgrid, dim3(32, 8), 0, st_>>>(a, tt_.get(), ldt_, zeros_.get());
        count_launch();
    }

    // The selection stages of a sparsification: the register path when the
    // rows and the columns fit it, else the shared-memory path.
    bool rpath() const {
        return g_sparsify_legacy.load(std::memory_order_relaxed) == 0 && r_vpt<TM>(n_) > 0 &&
               r_vpt<TM>(m1_) > 0;
    }
    void col_select(double delta, int from_large) {
        if (rpath()) {
            r_dispatch<TM>(r_vpt<TM>(n_), [&](auto c) {
                constexpr int V = decltype(c)::value;
                constexpr size_t sm = r_row_bytes<TM, V>();
                k_col_select_r<TM, V><<<r_grid(k_col_select_r<TM, V>, m1_, sm), kRT, sm, st_>>>(
                    tt_.get(), ldt_, n_, m1_, delta, from_large, xcol_.get());
            });
        } else {
            k_col_select<TM><<<col_grid_, kSelThreads, col_smem_, st_>>>(
                tt_.get(), ldt_, n_, m1_, delta, from_large, col_cache_ ? 1 : 0, xcol_.get());
        }
        count_launch();
    }
    void row_stage(const DenseArgs& a, double delta2, int keep_row0) {
        if (rpath()) {
            constexpr int W = VecOf<TM>::W;
            const int vec = (reinterpret_cast<uintptr_t>(P_->M) % 16 == 0 && P_->ldm % W == 0)
                                ? 1 : 0;
            r_dispatch<TM>(r_vpt<TM>(m1_), [&](auto c) {
                constexpr int V = decltype(c)::value;
                constexpr size_t sm = r_row_bytes<TM, V>();
                k_row_stage_r<TM, V><<<r_grid(k_row_stage_r<TM, V>, n_, sm), kRT, sm, st_>>>(
                    a, m1_, keep_row0, vec, xcol_.get(), delta2, yrow_.get(), rcount_.get(),
                    rcols_.get(), rvals_.get());
            });
        } else {
            RowStageArgs r;
            r.ldr = m1_;
            r.cache = row_cache_ ? 1 : 0;
            r.lds = lds_;
            r.keep_row0 = keep_row0;
            k_row_stage<TM><<<row_grid_, kSelThreads, row_smem_, st_>>>(
                a, r, xcol_.get(), delta2, row_scratch_.get(), yrow_.get(), rcount_.get(),
                rcols_.get(), rvals_.get());
        }
        count_launch();
    }
    void csc_fill() {
        if (rpath()) {
            r_dispatch<TM>(r_vpt<TM>(n_), [&](auto c) {
                constexpr int V = decltype(c)::value;
                constexpr size_t sm = r_row_bytes<TM, V>();
                k_csc_fill_r<TM, V><<<r_grid(k_csc_fill_r<TM, V>, m1_, sm), kRT, sm, st_>>>(
                    tt_.get(), ldt_, n_, m1_, xcol_.get(), yrow_.get(), n_, ccount_.get(),
                    crows_.get(), cvals_.get());
            });
        } else {
            k_csc_fill<TM><<<col_grid_, kSelThreads, col_smem_, st_>>>(
                tt_.get(), ldt_, n_, m1_, xcol_.get(), yrow_.get(), n_, col_cache_ ? 1 : 0,
                ccount_.get(), crows_.get(), cvals_.get());
        }
        count_launch();
    }

    // direction = -(H_s + shift I)^{-1} gv into dir (sinkhorn_ssns.cpp:118-140);
    // gv = g unless given. mode -1 follows the method (0: CG with relative
    // tolerance 1e-8; otherwise the direct-solve stand-in, Jacobi PCG to
    // tol_direct_), mode 0 / 1 forces one of them.
    void direction(double shift, const double* gv = nullptr, int mode = -1) {
        SsnState* S = state_.get();
        const bool jac = mode < 0 ? jacobi_ : mode == 1;
        const double* gsrc = gv ? gv : g_.get();
        cg_tol_ = jac ? tol_direct_ : 1e-8;
        const int maxit = jac ? max_direct_ : max_cg_;
        if (maxit != cg_max_) {
            cg_max_ = maxit;
            REGOT_CUDA(cudaMemcpyAsync(&S->max_it, &cg_max_, sizeof(int), cudaMemcpyHostToDevice,
                                       st_));
        }
        REGOT_CUDA(cudaMemcpyAsync(&S->shift, &shift, sizeof(double), cudaMemcpyHostToDevice,
                                   st_));
        REGOT_CUDA(cudaMemsetAsync(dir_.get(), 0, (size_t)(n_ + m_) * sizeof(double), st_));
        if (m1_ <= 0) {
            k_schur_rhs_rows<<<cdiv(n_, kVT), kVT, 0, st_>>>(n_, gsrc, h_.get(), S, dir_.get(),
                                                             nullptr, nullptr);
            count_launch();
            return;
        }
        const int gr = cdiv((long long)n_ * 32, 32 * kSpWarps);
        const int gc = cdiv((long long)m1_ * 32, 32 * kSpWarps);
        const int bt = 32 * kSpWarps;
        const double* diag = nullptr;
        k_schur_rhs_rows<<<cdiv(n_, kVT), kVT, 0, st_>>>(n_, gsrc, h_.get(), S, u_.get(), S_.u2,
                                                         S_.w32);
        if (jac) {
            k_schur_diag<TM><<<gc, bt, 0, st_>>>(S_, h_.get(), S, diag_.get());
            count_launch();
            diag = diag_.get();
        }
        double* x = dir_.get() + n_;
        k_schur_init<TM><<<gc, bt, 0, st_>>>(S_, gsrc, u_.get(), diag, cg_tol_, x, rv_.get(),
                                             z_.get(), p_.get(), parts_.get(), S);
        count_launch(2);
        REGOT_CHECK_LAUNCH();
        if (!exec_ || graph_jacobi_ != jac) build_graph(diag, jac);
        int batch = 8;
        for (;;) {
            for (int q = 0; q < batch; ++q) REGOT_CUDA(cudaGraphLaunch(exec_, st_));
            count_launch(graph_kernels_ * batch);
            int done = 0;
            d2h(&done, &S->done, sizeof(int), st_);
            sync(st_);
            if (done) break;
            batch = std::min(batch * 2, 64);
        }
        k_schur_back<TM><<<gr, bt, 0, st_>>>(S_, gsrc, h_.get(), dir_.get(), S);
        count_launch();
        REGOT_CHECK_LAUNCH();
    }

    // g'd and d'H_s d into the state.
    void dir_dots() {
        const int bt = 32 * kSpWarps;
        const int gr = cdiv((long long)n_ * 32, bt);
        const int gc = cdiv((long long)std::max(m1_, 1) * 32, bt);
        k_dhd_rows<TM><<<gr, bt, 0, st_>>>(S_, dir_.get(), g_.get(), h_.get(), parts_.get(),
                                           state_.get());
        k_dhd_cols<TM><<<gc, bt, 0, st_>>>(S_, dir_.get(), g_.get(), h_.get(), parts_.get(),
                                           state_.get());
        count_launch(2);
        REGOT_CHECK_LAUNCH();
    }

    // reg * sum T phi(s w) for up to four steps s (one dense pass).
    void ls_pass(const double* steps, int ns, double* tots) {
        ops_.maxabs(gamma_.get(), n_ + m_, dir_.get(), n_ + m_, &state_.get()->maxabs);
        PassParams p = ops_.base_params();
        p.ra = gamma_.get();
        p.cb = gamma_.get() + n_;
        p.rd = dir_.get();
        p.cd = dir_.get() + n_;
        p.grid = &state_.get()->maxabs;
        for (int s = 0; s < 4; ++s) p.steps[s] = s < ns ? steps[s] : 0.0;
        p.nsteps = ns;
        ops_.pass(OP_E_LS, p);
        ++passes_;
        const int blocks = pass_blocks(OP_E_LS, mixed_, n_, m_);
        k_ls_sum<<<1, 32, 0, st_>>>(ops_.buf().totpart.get(), blocks, ns, lsout_.get());
        count_launch();
        d2h(tots, lsout_.get(), ns * sizeof(double), st_);
        sync(st_);
    }

    void move(double s) {
        k_ssns_move<<<cdiv(n_ + m_, kVT), kVT, 0, st_>>>(n_ + m_, s, dir_.get(), gamma_.get());
        count_launch();
        REGOT_CHECK_LAUNCH();
    }

    // Kept pattern of the last sparsify(): mask[i * (m - 1) + j] = 1 for the
    // stored entries (row-major), from the CSR rows.
    void kept_mask(int* mask) {
        std::vector<int> cnt(n_);
        std::vector<int> cols((size_t)n_ * m1_);
        d2h(cnt.data(), rcount_.get(), n_ * sizeof(int), st_);
        d2h(cols.data(), rcols_.get(), cols.size() * sizeof(int), st_);
        sync(st_);
        std::fill(mask, mask + (size_t)n_ * m1_, 0);
        for (int i = 0; i < n_; ++i)
            for (int k = 0; k < cnt[i]; ++k) mask[(size_t)i * m1_ + cols[(size_t)i * m1_ + k]] = 1;
    }
    // Stored entries of the CSC copy (equal to the CSR's when both are built
    // from the same thresholds).
    long long csc_nnz() {
        std::vector<int> cnt(std::max(m1_, 1));
        d2h(cnt.data(), ccount_.get(), m1_ * sizeof(int), st_);
        sync(st_);
        long long s = 0;
        for (int j = 0; j < m1_; ++j) s += cnt[j];
        return s;
    }
    long long zero_count() {
        unsigned long long zc = 0;
        d2h(&zc, zeros_.get(), sizeof(zc), st_);
        sync(st_);
        return (long long)zc;
    }

    // ---- sinkhorn_sparse_newton / sinkhorn_splr pieces ----
    double* g() { return g_.get(); }
    double* dir() { return dir_.get(); }

    // sparsify_mat_with_density of T(gamma) with preserve = true
    // (sinkhorn_sparsify4.cpp:77-174), right after grad(): the largest
    // k = floor(n (m-1) density) entries of T[:, :m-1] (every entry tied with
    // the k-th largest value is kept too; the reference's nth_element keeps
    // an arbitrary subset of such ties), the first column and the first row.
    void sparsify_density(double density) {
        if (m1_ <= 0) return;
        const DenseArgs a = dense_args();
        if (!topk_.get()) {
            topk_.alloc(1, st_);
            hist_.alloc(kBins, st_);
        }
        zeros_.zero();
        transpose(a);
        const double dd = std::min(std::max(density, 0.0), 1.0);
        const unsigned long long len = (unsigned long long)n_ * (unsigned long long)m1_;
        const unsigned long long k = (unsigned long long)((double)len * dd);
        TopK t0{0ull, 0ull, k, k == 0 ? 1 : 0};
        h2d(topk_.get(), &t0, sizeof(TopK), st_);
        if (k > 0) {
            const int grid = std::max(1, device_sm_count() * 4);
            int hi = Digits<TM>::kTop;
            bool first = true;
            while (hi >= 0) {
                const int width = first ? 11 : ((hi + 1) % 11 == 0 ? 11 : 10);
                const int lo = hi - width + 1 > 0 ? hi - width + 1 : 0;
                const int nb = 1 << (hi - lo + 1);
                REGOT_CUDA(cudaMemsetAsync(hist_.get(), 0, (size_t)nb * sizeof(unsigned), st_));
                k_topk_hist<TM><<<grid, 256, 0, st_>>>(tt_.get(), ldt_, n_, m1_, topk_.get(), lo,
                                                       nb, hist_.get());
                k_topk_pick<<<1, 256, 0, st_>>>(topk_.get(), hist_.get(), lo, nb);
                count_launch(2);
                passes_ += 1;
                hi = lo - 1;
                first = false;
            }
        }
        k_topk_finish<TM><<<cdiv(m1_, kVT), kVT, 0, st_>>>(topk_.get(), m1_, xcol_.get());
        row_stage(a, (double)INFINITY, 1);
        csc_fill();
        k_nnz<<<cdiv(n_, kVT), kVT, 0, st_>>>(rcount_.get(), n_, parts_.get(), state_.get());
        count_launch(2);
        REGOT_CHECK_LAUNCH();
        passes_ += 3;
    }

    // Objective and gradient (host, n + m - 1 entries) at the host point x
    // (n + m entries, beta_m = 0), one pass. FP64 forms f directly; mixed
    // precision returns f0 + step g0'd + reg sum T(x) e^(-s w) phi(s w)
    // (OP_E_GRADLS at x along dir with step s), the change from the base
    // point without cancellation.
    double trial(const std::vector<double>& x, double step, double f0, double g0d,
                 std::vector<double>& gx) {
        const int N = n_ + m_;
        if (!xt_.get()) {
            xt_.alloc(N, st_);
            tsum_.alloc(N + 1, st_);
            tmx_.alloc(1, st_);
        }
        h2d(xt_.get(), x.data(), N * sizeof(double), st_);
        double* r = tsum_.get();
        double* c = r + n_;
        if (mixed_)
            ops_.grad_ls(xt_.get(), xt_.get() + n_, dir_.get(), dir_.get() + n_, step, r, c,
                         r + N, tmx_.get());
        else
            ops_.row_col_sums(xt_.get(), xt_.get() + n_, r, c, tmx_.get());
        ++passes_;
        const int cnt = mixed_ ? N + 1 : N;
        double* h = static_cast<double*>(ctx_stage(P_->ctx, (size_t)cnt * sizeof(double)));
        d2h(h, r, (size_t)cnt * sizeof(double), st_);
        sync(st_);
        double tsum = 0.0, lin = 0.0;
        for (int i = 0; i < n_; ++i) {
            gx[i] = h[i] - P_->ha[i];
            tsum += h[i];
            lin += x[i] * P_->ha[i];
        }
        for (int j = 0; j < m1_; ++j) {
            gx[n_ + j] = h[n_ + j] - P_->hb[j];
            lin += x[n_ + j] * P_->hb[j];
        }
        if (mixed_) return f0 + (step * g0d + reg_ * h[N]);
        return reg_ * tsum - lin;
    }

    // gamma <- the host point x (n + m entries)
    void set_gamma(const std::vector<double>& x) {
        h2d(gamma_.get(), x.data(), (size_t)(n_ + m_) * sizeof(double), st_);
    }

    ~SsnsEngine() {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
    }

private:
    void build_graph(const double* diag, bool jac) {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
        exec_ = nullptr;
        graph_ = nullptr;
        SsnState* S = state_.get();
        const int bt = 32 * kSpWarps;
        const int gr = cdiv((long long)n_ * 32, bt);
        const int gc = cdiv((long long)m1_ * 32, bt);
        const int gv = cdiv(m1_, kVT);
        double* x = dir_.get() + n_;
        long long* saved = g_launch_counter;
        graph_kernels_ = 0;
        g_launch_counter = &graph_kernels_;
        REGOT_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        k_schur_rows<TM><<<gr, bt, 0, st_>>>(S_, p_.get(), h_.get(), u_.get(), S);
        k_schur_cols<TM><<<gc, bt, 0, st_>>>(S_, p_.get(), u_.get(), h_.get(), q_.get(),
                                             pq_.get(), S);
        k_schur_alpha<<<1, 1024, 0, st_>>>(m1_, pq_.get(), S);
        k_schur_b<<<gv, kVT, 0, st_>>>(m1_, p_.get(), q_.get(), diag, x, rv_.get(), z_.get(),
                                       parts_.get(), S, S_.x2);
        k_schur_c<<<gv, kVT, 0, st_>>>(m1_, z_.get(), p_.get(), S, S_.p2);
        count_launch(5);
        REGOT_CUDA(cudaStreamEndCapture(st_, &graph_));
        g_launch_counter = saved;
        REGOT_CUDA(cudaGraphInstantiate(&exec_, graph_, 0));
        graph_jacobi_ = jac;
    }

    regot_dproblem* P_;
    cudaStream_t st_;
    ErotOps ops_;
    int n_, m_, m1_;
    double reg_;
    bool mixed_;
    bool jacobi_ = true;
    double cg_tol_ = 1e-10, tol_direct_ = 1e-10;
    int cg_max_ = 0, max_cg_ = 0, max_direct_ = 0;
    DBuf<double> gamma_, g_, h_, dir_, u_, rv_, z_, p_, q_, pq_, diag_, parts_, lsout_;
    DBuf<double> xt_, tsum_, tmx_;
    DBuf<float2> u2_, d2_, p2_, x2_;  // mixed: FP32 (hi, lo) copies of the CG vectors
    DBuf<float> w32_;
    DBuf<TopK> topk_;
    DBuf<unsigned> hist_;
    DBuf<SsnState> state_;
    DBuf<unsigned long long> zeros_;
    long long ldt_ = 0, lds_ = 0;
    DBuf<TM> tt_, xcol_, yrow_, rvals_, cvals_, row_scratch_;
    DBuf<int> rcount_, rcols_, ccount_, crows_;
    bool col_cache_ = false, row_cache_ = false;
    size_t col_smem_ = 0, row_smem_ = 0;
    int col_grid_ = 1, row_grid_ = 1;
    Sparse S_{};
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    bool graph_jacobi_ = false;
    long long graph_kernels_ = 0;
    long long passes_ = 0;
};

template <typename TM>
void run_ssns(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
              const regot_opts& o, regot_result* res) {
    using clock = std::chrono::steady_clock;
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    // sinkhorn_ssns.cpp:32-35, 94
    constexpr double rho_t1 = 0.25, rho_t2 = 0.75, mu_s1 = 4.0, mu_s2 = 0.5, kappa = 0.001,
                     nu0 = 0.01;
    double mu = o.mu0 > 0.0 ? o.mu0 : 1.0;
    require(o.method < 0 || o.method == 0 || o.method == 1,
            "sinkhorn_ssns: method must be 0 (CG) or 1 (direct)");
    SsnsEngine<TM> E(ctx, P, reg, o);
    ErotOps& ops = E.ops();

    // Initial value (sinkhorn_ssns.cpp:48-62): x0, or (0 + beta_m, beta~ - beta_m)
    // with beta = optimal_beta(alpha = 0).
    {
        std::vector<double> h(N, 0.0);
        if (o.x0 && o.x0_len == n + m - 1) {
            std::copy(o.x0, o.x0 + n + m - 1, h.begin());
        } else {
            DBuf<double> beta(m, st), zero(n, st), mx(1, st);
            zero.zero();
            ops.optimal_beta(zero.get(), beta.get(), mx.get());
            std::vector<double> hb(m);
            d2h(hb.data(), beta.get(), m * sizeof(double), st);
            sync(st);
            for (int i = 0; i < n; ++i) h[i] = hb[m - 1];
            for (int j = 0; j < m - 1; ++j) h[n + j] = hb[j] - hb[m - 1];
        }
        h2d(E.gamma(), h.data(), N * sizeof(double), st);
    }
    std::vector<double> hobj, hmar, htime, hdens;
    auto t0 = clock::now();
    E.grad();
    SsnState hs = E.read_state();
    double f = hs.f, gnorm = hs.gnorm;
    double density = E.sparsify(nu0 * gnorm, 0.001);
    sync(st);
    auto ms_since = [](clock::time_point t) {
        return std::chrono::duration<double, std::milli>(clock::now() - t).count();
    };
    hobj.push_back(f);
    hmar.push_back(gnorm);
    htime.push_back(ms_since(t0));
    hdens.push_back(density);
    const double cands[4] = {1.0, 0.5, 0.25, 0.1};
    int i;
    for (i = 0; i < max_iter; i++) {
        if (o.verbose >= 1) std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
        const auto t_it = clock::now();
        if (gnorm < tol || !std::isfinite(f)) break;
        const double shift = mu * gnorm;
        E.direction(shift);
        E.dir_dots();
        hs = E.read_state();
        const double gtd = hs.gtd, dhd = hs.dhd;
        // line_selection: first candidate below f, else the best. The full
        // step is evaluated alone first (one series per entry instead of
        // four); the other three only when it does not decrease f. The
        // per-step totals of a pass do not depend on which steps share it.
        double tots[4];
        E.ls_pass(cands, 1, tots);
        double best = 1.0, best_df = std::numeric_limits<double>::infinity();
        for (int s = 0; s < 4; ++s) {
            if (s == 1) E.ls_pass(cands + 1, 3, tots + 1);
            const double df = cands[s] * gtd + reg * tots[s];
            if (df < best_df) {
                best = cands[s];
                best_df = df;
            }
            if (best_df < 0.0) break;
        }
        const double numer = -best_df;  // f - newf
        const double denom = -best * gtd - 0.5 * best * best * dhd;
        const double rho = numer / denom;
        if (rho > 0.0) E.move(best);
        if (rho < rho_t1) {
            mu = mu_s1 * mu;
        } else if (rho > rho_t2) {
            mu = std::max(mu_s2 * mu, kappa);
        }
        if (rho > 0.0) {
            E.grad();
            hs = E.read_state();
            f = hs.f;
            gnorm = hs.gnorm;
            density = E.sparsify(nu0 * gnorm, density);
        }
        sync(st);
        hobj.push_back(f);
        hmar.push_back(gnorm);
        htime.push_back(htime.back() + ms_since(t_it));
        hdens.push_back(density);
    }
    const int L = (int)hobj.size();
    DBuf<double> hist(4 * (size_t)std::max(L, 1), st);
    h2d(hist.get(), hobj.data(), L * sizeof(double), st);
    h2d(hist.get() + L, hmar.data(), L * sizeof(double), st);
    h2d(hist.get() + 2 * L, htime.data(), L * sizeof(double), st);
    h2d(hist.get() + 3 * L, hdens.data(), L * sizeof(double), st);
    finish_erot_result(ops, E.gamma(), hist.get(), hist.get() + L, hist.get() + 2 * L,
                       hist.get() + 3 * L, L, L, i, E.passes(), o, res);
}

// sinkhorn_sparse_newton_internal (sinkhorn_sparse_newton.cpp:24-171) and
// sinkhorn_splr_internal (sinkhorn_splr.cpp:24-200). Each iteration: the
// direction from the density-sparsified Hessian with shift
// min(gnorm, shift) (SPLR: plus the BFGS correction of solve_low_rank,
// sinkhorn_linsolve.cpp:160-225, when y's > 1e-6 y'y), the More-Thuente
// line search from min(1, 1.5 alpha) with one dense pass per trial, the
// gradient pass at the new point, the density update and the
// sparsification. The driver keeps gamma, g and the direction on the host
// in FP64 (n + m entries each).
template <typename TM>
void run_sparse_newton(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                       const regot_opts& o, regot_result* res, bool splr) {
    using clock = std::chrono::steady_clock;
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m, N1 = n + m - 1;
    const double density_max = o.density > 0.0 ? o.density : 0.01;
    const double density_min = 0.01 * density_max;
    double density = 0.1 * density_max;
    const double shift_max = o.shift;
    constexpr double eps = 1e-6;
    SsnsEngine<TM> E(ctx, P, reg, o);
    ErotOps& ops = E.ops();
    auto density_T2H = [&](double d) {  // sinkhorn_sparse_newton.cpp:17-22
        const double nnz = 2.0 * d * n * (m - 1) + n + m - 1;
        return nnz / double(n + m - 1) / double(n + m - 1);
    };
    std::vector<double> gamma(N, 0.0), gamma_pre(N, 0.0), g(N, 0.0), g_pre(N, 0.0),
        dir(N, 0.0), x(N, 0.0), gx(N, 0.0), y(N, 0.0), sv(N, 0.0), ir(N, 0.0), iy(N, 0.0);
    // Initial value (sinkhorn_sparse_newton.cpp:56-65)
    if (o.x0 && o.x0_len == N1) {
        std::copy(o.x0, o.x0 + N1, gamma.begin());
    } else {
        DBuf<double> beta(m, st), zero(n, st), mx(1, st);
        zero.zero();
        ops.optimal_beta(zero.get(), beta.get(), mx.get());
        std::vector<double> hb(m);
        read_small(ctx, hb.data(), beta.get(), m * sizeof(double), st);
        for (int i = 0; i < n; ++i) gamma[i] = hb[m - 1];
        for (int j = 0; j < m - 1; ++j) gamma[n + j] = hb[j] - hb[m - 1];
    }
    E.set_gamma(gamma);
    auto lin = [&](const std::vector<double>& v) {  // alpha'a + beta~'b~
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += v[i] * P->ha[i];
        for (int j = 0; j < m - 1; ++j) s += v[n + j] * P->hb[j];
        return s;
    };
    auto read_g = [&]() {
        d2h(g.data(), E.g(), (size_t)N * sizeof(double), st);
        sync(st);
    };
    auto dot = [&](const std::vector<double>& u, const std::vector<double>& v) {
        double s = 0.0;
        for (int q = 0; q < N1; ++q) s += u[q] * v[q];
        return s;
    };
    auto ms_since = [](clock::time_point t) {
        return std::chrono::duration<double, std::milli>(clock::now() - t).count();
    };

    std::vector<double> hobj, hmar, htime, hdens;
    auto t0 = clock::now();
    E.grad();
    SsnState hs = E.read_state();
    double f = hs.f, gnorm = hs.gnorm;
    const double gnorm_init = gnorm;
    read_g();
    E.sparsify_density(density);
    sync(st);
    hobj.push_back(f);
    hmar.push_back(gnorm);
    htime.push_back(ms_since(t0));
    hdens.push_back(density_T2H(density));
    double alpha = 1.0;
    DBuf<double> ny(N, st);
    int i;
    for (i = 0; i < max_iter; i++) {
        if (o.verbose >= 1) std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, f, gnorm);
        const auto t_it = clock::now();
        if (gnorm < tol || !std::isfinite(f)) break;
        const double shift = std::min(gnorm, shift_max);
        bool low_rank = false;
        double ys = 0.0;
        if (splr) {
            double yy = 0.0;
            for (int q = 0; q < N1; ++q) {
                y[q] = g[q] - g_pre[q];
                sv[q] = gamma[q] - gamma_pre[q];
                ys += y[q] * sv[q];
                yy += y[q] * y[q];
            }
            low_rank = i > 0 && ys > eps * yy;
        }
        if (low_rank) {
            // res = A^-1 r + ((1 + y'A^-1 y / y's) r's / y's - y'A^-1 r / y's) s
            //       - (r's / y's) A^-1 y, r = -g, A = H_s + shift I, both
            // solves by the direct-solve stand-in (the reference factors A)
            std::vector<double> negy(N, 0.0);
            for (int q = 0; q < N1; ++q) negy[q] = -y[q];
            h2d(ny.get(), negy.data(), (size_t)N * sizeof(double), st);
            E.direction(shift, ny.get(), 1);
            d2h(iy.data(), E.dir(), (size_t)N * sizeof(double), st);
            E.direction(shift, nullptr, 1);
            d2h(ir.data(), E.dir(), (size_t)N * sizeof(double), st);
            sync(st);
            double rs = 0.0, yiy = 0.0, yir = 0.0;
            for (int q = 0; q < N1; ++q) {
                rs -= sv[q] * g[q];
                yiy += y[q] * iy[q];
                yir += y[q] * ir[q];
            }
            const double rs_ys = rs / ys;
            const double cs = (1.0 + yiy / ys) * rs_ys - yir / ys;
            for (int q = 0; q < N1; ++q) dir[q] = ir[q] + cs * sv[q] - rs_ys * iy[q];
            dir[N1] = 0.0;
            h2d(E.dir(), dir.data(), (size_t)N * sizeof(double), st);
        } else {
            E.direction(shift);
            d2h(dir.data(), E.dir(), (size_t)N * sizeof(double), st);
            sync(st);
        }
        // Wolfe line search: one pass per trial
        const double g0d = dot(g, dir);
        auto eval = [&](double step, double* fx, double* dg) {
            for (int q = 0; q < N; ++q) x[q] = gamma[q] + step * dir[q];
            *fx = E.trial(x, step, f, g0d, gx);
            *dg = dot(gx, dir);
        };
        const wolfe::Outcome ls = wolfe::search(std::min(1.0, 1.5 * alpha), f, g0d, eval);
        alpha = ls.step;
        gamma_pre = gamma;
        for (int q = 0; q < N; ++q) gamma[q] = gamma_pre[q] + alpha * dir[q];
        g_pre = g;
        if (!ls.recompute && ls.last_eval != alpha) {
            // The reference keeps T of the last trial (sinkhorn_splr.cpp:147):
            // sums and the sparsification come from T there, the objective's
            // linear terms from the new point.
            for (int q = 0; q < N; ++q) x[q] = gamma_pre[q] + ls.last_eval * dir[q];
            E.set_gamma(x);
            E.grad();
            hs = E.read_state();
            f = hs.f + (lin(x) - lin(gamma));
        } else {
            E.set_gamma(gamma);
            E.grad();
            hs = E.read_state();
            f = hs.f;
        }
        const double gnorm_pre = gnorm;
        gnorm = hs.gnorm;
        read_g();
        if (splr) {
            const bool bad = gnorm_pre < gnorm_init && gnorm > gnorm_pre;
            density *= bad ? 1.1 : 0.99;
        } else {
            const bool bad = gnorm_pre < gnorm_init && gnorm > 1.1 * gnorm_pre;
            density *= bad ? 2.0 : 0.9;
        }
        density = std::min(density_max, std::max(density_min, density));
        E.sparsify_density(density);
        E.set_gamma(gamma);
        sync(st);
        hobj.push_back(f);
        hmar.push_back(gnorm);
        htime.push_back(htime.back() + ms_since(t_it));
        hdens.push_back(density_T2H(density));
    }
    const int L = (int)hobj.size();
    DBuf<double> hist(4 * (size_t)std::max(L, 1), st);
    h2d(hist.get(), hobj.data(), L * sizeof(double), st);
    h2d(hist.get() + L, hmar.data(), L * sizeof(double), st);
    h2d(hist.get() + 2 * L, htime.data(), L * sizeof(double), st);
    h2d(hist.get() + 3 * L, hdens.data(), L * sizeof(double), st);
    finish_erot_result(ops, E.gamma(), hist.get(), hist.get() + L, hist.get() + 2 * L,
                       hist.get() + 3 * L, L, L, i, E.passes(), o, res);
}

template <typename TM>
void sparsify_at(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                 double delta, double density_hint, long long* nnz, int* mask) {
    const int n = P->n, m = P->m;
    regot_opts o;
    regot_opts_init(&o);
    SsnsEngine<TM> E(ctx, P, reg, o);
    std::vector<double> h(n + m, 0.0);
    std::copy(gamma, gamma + n + m - 1, h.begin());
    h2d(E.gamma(), h.data(), (n + m) * sizeof(double), ctx->stream);
    E.grad();
    // delta < 0 selects the density sparsification (density in density_hint)
    if (delta < 0.0) {
        E.sparsify_density(density_hint);
        E.read_state();
    } else {
        E.sparsify(delta, density_hint);
    }
    const SsnState hs = E.read_state();
    const long long stored = (long long)hs.nnz;
    require(E.csc_nnz() == stored, "CSR and CSC copies of the sparsified matrix differ",
            REGOT_ERR_NUMERIC);
    *nnz = delta < 0.0 ? stored : stored + E.zero_count();
    if (mask) E.kept_mask(mask);
    E.ops().check_err();
}

}  // namespace

int force_sparsify_path(int shared_memory) {
    return g_sparsify_legacy.exchange(shared_memory ? 1 : 0);
}

void erot_sparsify_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                       double delta, double density_hint, long long* nnz, int* mask) {
    if (P->prec == REGOT_PREC_MIXED)
        sparsify_at<float>(ctx, P, reg, gamma, delta, density_hint, nnz, mask);
    else
        sparsify_at<double>(ctx, P, reg, gamma, delta, density_hint, nnz, mask);
}

void sinkhorn_ssns_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                       const regot_opts& o, regot_result* res) {
    if (P->prec == REGOT_PREC_MIXED)
        run_ssns<float>(ctx, P, reg, tol, max_iter, o, res);
    else
        run_ssns<double>(ctx, P, reg, tol, max_iter, o, res);
}

void erot_sparsify_density_gpu(regot_ctx* ctx, regot_dproblem* P, double reg,
                               const double* gamma, double density, long long* nnz, int* mask) {
    if (P->prec == REGOT_PREC_MIXED)
        sparsify_at<float>(ctx, P, reg, gamma, -1.0, density, nnz, mask);
    else
        sparsify_at<double>(ctx, P, reg, gamma, -1.0, density, nnz, mask);
}

void sinkhorn_sparse_newton_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol,
                                int max_iter, const regot_opts& o, regot_result* res) {
    if (P->prec == REGOT_PREC_MIXED)
        run_sparse_newton<float>(ctx, P, reg, tol, max_iter, o, res, false);
    else
        run_sparse_newton<double>(ctx, P, reg, tol, max_iter, o, res, false);
}

void sinkhorn_splr_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                       const regot_opts& o, regot_result* res) {
    if (P->prec == REGOT_PREC_MIXED)
        run_sparse_newton<float>(ctx, P, reg, tol, max_iter, o, res, true);
    else
        run_sparse_newton<double>(ctx, P, reg, tol, max_iter, o, res, true);
}

}  // namespace regot
