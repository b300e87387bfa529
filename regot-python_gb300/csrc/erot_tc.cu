// Tensor-core contraction of the weighted plan (FP32 storage): the
// Blackwell-native replacement of the CUDA-core k_tyy for mixed precision.
//
//   row mode:    sums_i = sum_j G_ij,  Z_ik = sum_j G_ij Y_jk   (Z = G Y,  n x d)
//   column mode: sums_j = sum_i G_ij,  Z_jk = sum_i G_ij X_ik   (Z = G'X,  m x d)
//   G_ij = T_ij, or T_ij (u_i + u_{n+j} - W_ij) / reg with an adjoint u,
//   T_ij = exp((alpha_i + beta_j - M_ij)/reg) formed from the stored FP32 M
//   exactly as the dense passes form it (hi/lo split of the FP64 duals,
//   ex2.approx).
// With G = T, row mode gives dL/dx = 2 (sums o x - Z) / scale of a
// squared-Euclidean cost and column mode dL/dy = 2 (sums o y - Z) / scale;
// with the adjoint the same contractions of dL/dM for a loss on the plan.
// No counterpart in the reference, which has no derivatives.
//
// A CTA owns 128 rows (columns) of G: the M = 128 of one tcgen05.mma. It
// walks a contiguous range of K in chunks of 32: every thread forms 16
// entries of the chunk's G tile in registers from a coalesced read of M,
// splits each into BF16 hi + lo (G = hi + lo to about 2^-17 relative) and
// stores them into the two A tiles in shared memory; the chunk of the
// pre-tiled BF16 hi / lo split of Y arrives by two bulk copies on the TMA
// engine. One thread then issues, per 16-wide K step, the three MMAs
// hi*hi + hi*lo + lo*hi (BF16x3: each product to about 2^-16 relative)
// into an FP32 accumulator of 128 lanes x 80 columns in tensor memory:
// columns 0..63 are Z, column 64 the sums (B carries a column of ones).
// Two stages: the tiles of chunk k + 1 are formed while the MMAs of chunk k
// run; a tcgen05.commit on a per-stage mbarrier frees a stage. K is split
// over the grid's y dimension (3 CTAs per SM in total), each split writing
// FP32 partials that one small kernel adds in a fixed order into FP64
// outputs. Every wait is bounded; a wait that gives up sets *err (the host
// returns REGOT_ERR_TIMEOUT) and the CTA waits, again bounded, for its
// issued MMAs before it frees its tensor memory and exits.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "sm100_util.cuh"
#include "solvers.h"

namespace regot {

namespace {

using namespace sm100;

constexpr int kTcOwners = 128;   // MMA M: rows of G per CTA (row mode)
constexpr int kTcKC = 32;        // K per chunk: two MMA K steps of 16
constexpr int kTcN = 80;         // MMA N: 64 outputs, the ones column, 15 zero columns
constexpr int kTcOut = 64;       // outputs per launch
constexpr int kTcOnes = 64;      // D column holding the sums
constexpr int kTcThreads = 256;
// A tile (128 x 32 BF16, K-major, no swizzle): 16 row groups x 4 K groups of
// 8 x 16-byte core matrices; K groups 160 B apart and row groups 640 B
// apart, so that the 32 lanes of a warp store into 32 different banks.
constexpr uint32_t kALbo = 160, kASbo = 640, kABytes = 16 * kASbo;
// B tile (80 x 32 BF16, K-major): packed core matrices, copied as is from
// the pre-tiled global array.
constexpr uint32_t kBLbo = 128, kBSbo = 512, kBBytes = (kTcN / 8) * kBSbo;
constexpr uint32_t kTmemCols = 128;
constexpr size_t kTcSmem = 4 * (size_t)kABytes + 4 * (size_t)kBBytes + 128;  // + alignment
constexpr long long kTcPolls = 1LL << 14;

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ uint32_t a_off(int r, int k) {
    return (uint32_t)((r >> 3) * kASbo + (k >> 3) * kALbo + (r & 7) * 16 + (k & 7) * 2);
}

// BF16 hi / lo split of two K-adjacent values, packed (lower K in the low half).
__device__ __forceinline__ void split2(float g0, float g1, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(g0, g1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(g0 - hf.x, g1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Pre-tiled B: chunk c holds hi then lo tiles of kBBytes each; entry (n, k)
// of a tile at (n >> 3) kBSbo + (k >> 3) kBLbo + (n & 7) 16 + (k & 7) 2 bytes.
// Y is K x dk (row stride ldy, FP64); column kTcOnes is 1 for k < K.
__global__ void k_tc_tile_b(const double* __restrict__ Y, int ldy, int dk, int K, int nch,
                            __nv_bfloat16* __restrict__ Bt) {
    const long long total = (long long)nch * kTcN * kTcKC;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / (kTcN * kTcKC));
        const int rem = (int)(t % (kTcN * kTcKC));
        const int nn = rem / kTcKC, kk = rem % kTcKC;
        const int k = c * kTcKC + kk;
        float v = 0.f;
        if (k < K) {
            if (nn < dk) v = (float)Y[(long long)k * ldy + nn];
            else if (nn == kTcOnes) v = 1.f;
        }
        const __nv_bfloat16 hi = __float2bfloat16_rn(v);
        const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
        const uint32_t off =
            ((nn >> 3) * kBSbo + (kk >> 3) * kBLbo + (nn & 7) * 16 + (kk & 7) * 2) / 2;
        __nv_bfloat16* tile = Bt + (size_t)c * kBBytes;  // 2 tiles of kBBytes / 2 entries
        tile[off] = hi;
        tile[kBBytes / 2 + off] = lo;
    }
}

template <bool COLS, bool ADJ>
__global__ void __launch_bounds__(kTcThreads, 3) k_contract_tc(
    const float* __restrict__ M, long long ldm, int n, int m, const float4* __restrict__ rs,
    const float4* __restrict__ cs, float kexp, float inv_reg, const double* __restrict__ u,
    const double* __restrict__ W, const __nv_bfloat16* __restrict__ Bt, int nch, int per,
    float* __restrict__ part, int owners_pad, int* __restrict__ err) {
    extern __shared__ unsigned char tc_smem_raw[];
    __shared__ __align__(8) uint64_t s_bbar[2];
    __shared__ __align__(8) uint64_t s_mbar[2];
    __shared__ uint32_t s_tmem;
    unsigned char* smem = tc_smem_raw + ((128 - (smem_u32(tc_smem_raw) & 127)) & 127);
    unsigned char* sA = smem;                 // [stage][hi, lo] A tiles
    unsigned char* sB = smem + 4 * kABytes;   // [stage][hi, lo] B tiles

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int o0 = blockIdx.x * kTcOwners;
    const int c0 = blockIdx.y * per;
    const int nloc = min(nch, c0 + per) - c0;  // >= 1 by the host's choice of the split
    if (nloc <= 0) return;

    if (tid == 0) {
        mbar_init(&s_bbar[0], 1);
        mbar_init(&s_bbar[1], 1);
        mbar_init(&s_mbar[0], 1);
        mbar_init(&s_mbar[1], 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(&s_tmem, kTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    constexpr uint32_t idesc = idesc_bf16_f32(kTcOwners, kTcN);

    // ---- per-thread fixed operands ----
    // row mode: rows r_t = 16 warp + 2 t + (lane >> 4) (t < 8), column pair
    // 2 (lane & 15) of every chunk; column mode: column (owner) 32 (warp & 3)
    // + lane, row pairs of the chunk half warp >> 2, taken in an order
    // rotated by lane >> 3 so that a warp's stores hit 32 banks.
    float oh[COLS ? 1 : 8], olk[COLS ? 1 : 8];
    double ou[COLS ? 1 : 8];
    float ch1 = 0.f, clk1 = 0.f;
    double cu1 = 0.0;
    if constexpr (!COLS) {
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int i = o0 + warp * 16 + 2 * t + (lane >> 4);
            oh[t] = 0.f;
            olk[t] = 0.f;
            ou[t] = 0.0;
            if (i < n) {
                const float4 r = rs[i];
                oh[t] = r.x;
                olk[t] = __fmul_rn(r.y, kexp);
                if constexpr (ADJ) ou[t] = u[i];
            }
        }
    } else {
        const int j = o0 + 32 * (warp & 3) + lane;
        if (j < m) {
            const float4 c = cs[j];
            ch1 = c.x;
            clk1 = __fmul_rn(c.y, kexp);
            if constexpr (ADJ) cu1 = u[n + j];
        }
    }

    // M values of a chunk for this thread (row mode: two adjacent columns of
    // 8 rows; column mode: one column of 8 row pairs in the rotated order),
    // loaded one chunk ahead so that the loads of chunk k + 1 are in flight
    // while chunk k's tile is formed and multiplied.
    auto load_m = [&](int c, float2 (&mv)[8]) {
        if constexpr (!COLS) {
            const int j = c * kTcKC + 2 * (lane & 15);
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int i = o0 + warp * 16 + 2 * t + (lane >> 4);
                mv[t] = make_float2(0.f, 0.f);
                if (i < n) {
                    const float* row = M + (long long)i * ldm + j;
                    if (j + 1 < m) mv[t] = *reinterpret_cast<const float2*>(row);
                    else if (j < m) mv[t].x = row[0];
                }
            }
        } else {
            const int j = o0 + 32 * (warp & 3) + lane;
            const bool jv = j < m;
            const int g8 = lane >> 3;
            const int kbase = 16 * (warp >> 2);
#pragma unroll
            for (int pp = 0; pp < 8; ++pp) {
                const int q = (pp & ~3) | ((pp + g8) & 3);
                const int i = c * kTcKC + kbase + 2 * q;
                mv[pp] = make_float2(0.f, 0.f);
                if (jv && i < n) mv[pp].x = M[(long long)i * ldm + j];
                if (jv && i + 1 < n) mv[pp].y = M[(long long)(i + 1) * ldm + j];
            }
        }
    };
    float2 mv[8], mv_next[8];
    load_m(c0, mv);

    bool failed = false;
    int ncommit = 0;        // thread 0: chunks whose MMAs were committed
    int bpending = -1;      // thread 0: chunk whose B copy it gave up waiting for
    for (int it = 0; it < nloc; ++it) {
        const int stage = it & 1;
        const int c = c0 + it;
        bool wfail = false;
        if (it >= 2) wfail = !mbar_wait(&s_mbar[stage], (uint32_t)(((it - 2) >> 1) & 1), kTcPolls);
        if (__syncthreads_or(wfail || failed)) {
            failed = true;
            break;
        }
        // B tiles of this chunk (the MMAs that read this stage are done)
        if (tid == 0) {
            mbar_arrive_expect_tx(&s_bbar[stage], 2 * kBBytes);
            const unsigned char* src = reinterpret_cast<const unsigned char*>(Bt) +
                                       (size_t)c * 2 * kBBytes;
            bulk_g2s(sB + (stage * 2 + 0) * kBBytes, src, kBBytes, &s_bbar[stage]);
            bulk_g2s(sB + (stage * 2 + 1) * kBBytes, src + kBBytes, kBBytes, &s_bbar[stage]);
        }
        unsigned char* Ahi = sA + (stage * 2 + 0) * kABytes;
        unsigned char* Alo = sA + (stage * 2 + 1) * kABytes;
        if constexpr (!COLS) {
            const int kk = 2 * (lane & 15);
            const int j = c * kTcKC + kk;
            float ch[2] = {0.f, 0.f}, clk[2] = {0.f, 0.f};
            double cu[2] = {0.0, 0.0};
            bool cv[2] = {j < m, j + 1 < m};
#pragma unroll
            for (int e = 0; e < 2; ++e)
                if (cv[e]) {
                    const float4 cc = cs[j + e];
                    ch[e] = cc.x;
                    clk[e] = __fmul_rn(cc.y, kexp);
                    if constexpr (ADJ) cu[e] = u[n + j + e];
                }
            if (it + 1 < nloc) load_m(c + 1, mv_next);
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int r = warp * 16 + 2 * t + (lane >> 4);
                const int i = o0 + r;
                float g[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const float mval = e == 0 ? mv[t].x : mv[t].y;
                    const float s = (oh[t] + ch[e]) - mval;
                    float T = ex2_approx(fmaf(s, kexp, __fadd_rn(olk[t], clk[e])));
                    if constexpr (ADJ) {
                        const double w = (i < n && cv[e]) ? W[(long long)i * m + j + e] : 0.0;
                        T = __fmul_rn(__fmul_rn(T, (float)(ou[t] + cu[e] - w)), inv_reg);
                    }
                    g[e] = (i < n && cv[e]) ? T : 0.f;
                }
                uint32_t hi, lo;
                split2(g[0], g[1], hi, lo);
                const uint32_t off = a_off(r, kk);
                *reinterpret_cast<uint32_t*>(Ahi + off) = hi;
                *reinterpret_cast<uint32_t*>(Alo + off) = lo;
            }
        } else {
            const int jj = 32 * (warp & 3) + lane;
            const int j = o0 + jj;
            const bool jv = j < m;
            const int g8 = lane >> 3;
            const int kbase = 16 * (warp >> 2);
            if (it + 1 < nloc) load_m(c + 1, mv_next);
#pragma unroll
            for (int pp = 0; pp < 8; ++pp) {
                const int q = (pp & ~3) | ((pp + g8) & 3);
                const int kk = kbase + 2 * q;
                const int i = c * kTcKC + kk;
                float g[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const bool ok = jv && i + e < n;
                    float rh = 0.f, rlk = 0.f;
                    double ru = 0.0;
                    if (ok) {
                        const float4 rr = rs[i + e];
                        rh = rr.x;
                        rlk = __fmul_rn(rr.y, kexp);
                        if constexpr (ADJ) ru = u[i + e];
                    }
                    const float mval = e == 0 ? mv[pp].x : mv[pp].y;
                    const float s = (rh + ch1) - mval;
                    float T = ex2_approx(fmaf(s, kexp, __fadd_rn(rlk, clk1)));
                    if constexpr (ADJ) {
                        const double w = ok ? W[(long long)(i + e) * m + j] : 0.0;
                        T = __fmul_rn(__fmul_rn(T, (float)(ru + cu1 - w)), inv_reg);
                    }
                    g[e] = ok ? T : 0.f;
                }
                uint32_t hi, lo;
                split2(g[0], g[1], hi, lo);
                const uint32_t off = a_off(jj, kk);
                *reinterpret_cast<uint32_t*>(Ahi + off) = hi;
                *reinterpret_cast<uint32_t*>(Alo + off) = lo;
            }
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) mv[t] = mv_next[t];
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            if (!mbar_wait(&s_bbar[stage], (uint32_t)((it >> 1) & 1), kTcPolls)) {
                failed = true;  // seen by the other threads at the next __syncthreads_or
                bpending = it;
            } else {
                tc_fence_after();
                const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo);
                const uint32_t bh = smem_u32(sB + (stage * 2 + 0) * kBBytes);
                const uint32_t bl = smem_u32(sB + (stage * 2 + 1) * kBBytes);
#pragma unroll
                for (int ks = 0; ks < kTcKC / 16; ++ks) {
                    const uint64_t dah = smem_desc(ah + ks * 2 * kALbo, kALbo, kASbo);
                    const uint64_t dal = smem_desc(al + ks * 2 * kALbo, kALbo, kASbo);
                    const uint64_t dbh = smem_desc(bh + ks * 2 * kBLbo, kBLbo, kBSbo);
                    const uint64_t dbl = smem_desc(bl + ks * 2 * kBLbo, kBLbo, kBSbo);
                    mma_bf16(tmem, dah, dbh, idesc, (it | ks) != 0 ? 1u : 0u);
                    mma_bf16(tmem, dah, dbl, idesc, 1u);
                    mma_bf16(tmem, dal, dbh, idesc, 1u);
                }
                mma_commit(&s_mbar[stage]);
                ncommit = it + 1;
            }
        }
    }
    // Drain: the B copy that a failed wait left in flight (bounded), then the
    // MMAs of the last committed chunk (their commit covers every earlier one).
    __shared__ int s_ncommit;
    if (tid == 0) {
        s_ncommit = ncommit;
        if (bpending >= 0)
            mbar_wait(&s_bbar[bpending & 1], (uint32_t)((bpending >> 1) & 1), kTcPolls);
    }
    failed = __syncthreads_or(failed);
    const int committed = s_ncommit;
    bool done = true;
    if (committed > 0) {
        const int last = committed - 1;
        done = mbar_wait(&s_mbar[last & 1], (uint32_t)((last >> 1) & 1), kTcPolls);
    }
    failed = __syncthreads_or(failed || !done);
    if (failed) {
        if (tid == 0) atomicOr(err, 1);
    } else {
        tc_fence_after();
        const int q = warp & 3, half = warp >> 2;
        const int o = o0 + 32 * q + lane;  // < owners_pad
        float* dst = part + ((size_t)blockIdx.y * owners_pad + o) * kTcN;
#pragma unroll
        for (int x = 0; x < 5; ++x) {
            const int col = half * 40 + 8 * x;
            float v[8];
            tmem_ld8(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)col, v);
#pragma unroll
            for (int e = 0; e < 8; ++e) dst[col + e] = v[e];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// Fixed-order sum of the K-split partials into FP64 outputs.
__global__ void k_tc_reduce(const float* __restrict__ part, int S, int owners_pad, int nown,
                            int dk, double* __restrict__ sums, double* __restrict__ Z, int ldz) {
    const long long total = (long long)nown * (dk + 1);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int o = (int)(t / (dk + 1)), k = (int)(t % (dk + 1));
        const int col = k < dk ? k : kTcOnes;
        double acc = 0.0;
        for (int s = 0; s < S; ++s) acc += (double)part[((size_t)s * owners_pad + o) * kTcN + col];
        if (k < dk) Z[(long long)o * ldz + k] = acc;
        else if (sums) sums[o] = acc;
    }
}

template <bool COLS, bool ADJ>
void launch_contract(dim3 grid, cudaStream_t st, const float* M, long long ldm, int n, int m,
                     const float4* rs, const float4* cs, float kexp, float inv_reg,
                     const double* u, const double* W, const __nv_bfloat16* Bt, int nch, int per,
                     float* part, int owners_pad, int* err) {
    static std::atomic<unsigned long long> configured{0};
    int dev = 0;
    REGOT_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(configured.load() & (1ULL << dev))) {
        REGOT_CUDA(cudaFuncSetAttribute(k_contract_tc<COLS, ADJ>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kTcSmem));
        if (dev < 64) configured.fetch_or(1ULL << dev);
    }
    k_contract_tc<COLS, ADJ><<<grid, kTcThreads, kTcSmem, st>>>(
        M, ldm, n, m, rs, cs, kexp, inv_reg, u, W, Bt, nch, per, part, owners_pad, err);
    REGOT_CHECK_LAUNCH();
    count_launch();
}

}  // namespace

void erot_contract_tc(regot_ctx* ctx, regot_dproblem* P, double reg, const double* d_gamma,
                      const double* d_u, const double* d_W, const double* d_Y, int d, bool cols,
                      double* d_sums, double* d_Z) {
    require(P->prec == REGOT_PREC_MIXED, "the tensor-core contraction needs FP32 storage");
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m;
    const int nown = cols ? m : n, K = cols ? n : m;
    ErotOps ops(P, reg, st);
    DBuf<float4> rs(n, st), cs(m, st);
    DBuf<double> mx(1, st);
    ops.maxabs(d_gamma, n + m, nullptr, 0, mx.get());
    {
        PassParams p = ops.base_params();
        p.ra = d_gamma;
        p.cb = d_gamma + n;
        p.grid = mx.get();
        launch_split(p, rs.get(), cs.get(), nullptr, st);
    }
    const int nch = cdiv(K, kTcKC);
    const int nob = cdiv(nown, kTcOwners);
    // one wave of 3 CTAs per SM (their shared memory allows three)
    const int target = 3 * device_sm_count();
    int S = std::max(1, std::min(nch, target / nob));
    const int per = cdiv(nch, S);
    S = cdiv(nch, per);
    const int owners_pad = nob * kTcOwners;
    DBuf<__nv_bfloat16> Bt((size_t)nch * kBBytes, st);  // 2 tiles of kBBytes / 2 entries per chunk
    DBuf<float> part((size_t)S * owners_pad * kTcN, st);
    DBuf<int> err(1, st);
    err.zero();
    const float kexp = (float)(1.4426950408889634 / reg);
    const float inv_reg = (float)(1.0 / reg);
    const dim3 grid(nob, S);
    for (int k0 = 0; k0 < d || (d == 0 && k0 == 0); k0 += kTcOut) {
        const int dk = std::min(kTcOut, d - k0);
        k_tc_tile_b<<<std::min(cdiv((long long)nch * kTcN * kTcKC, 256), 4096), 256, 0, st>>>(
            d_Y ? d_Y + k0 : nullptr, d, dk, K, nch, Bt.get());
        REGOT_CHECK_LAUNCH();
        count_launch();
        const float* Mf = static_cast<const float*>(P->M);
        if (cols) {
            if (d_u) launch_contract<true, true>(grid, st, Mf, P->ldm, n, m, rs.get(), cs.get(), kexp,
                                                 inv_reg, d_u, d_W, Bt.get(), nch, per, part.get(),
                                                 owners_pad, err.get());
            else launch_contract<true, false>(grid, st, Mf, P->ldm, n, m, rs.get(), cs.get(), kexp,
                                              inv_reg, d_u, d_W, Bt.get(), nch, per, part.get(),
                                              owners_pad, err.get());
        } else {
            if (d_u) launch_contract<false, true>(grid, st, Mf, P->ldm, n, m, rs.get(), cs.get(),
                                                  kexp, inv_reg, d_u, d_W, Bt.get(), nch, per,
                                                  part.get(), owners_pad, err.get());
            else launch_contract<false, false>(grid, st, Mf, P->ldm, n, m, rs.get(), cs.get(),
                                               kexp, inv_reg, d_u, d_W, Bt.get(), nch, per,
                                               part.get(), owners_pad, err.get());
        }
        k_tc_reduce<<<std::min(cdiv((long long)nown * (dk + 1), 256), 4096), 256, 0, st>>>(
            part.get(), S, owners_pad, nown, dk, k0 == 0 ? d_sums : nullptr, d_Z ? d_Z + k0 : nullptr,
            d);
        REGOT_CHECK_LAUNCH();
        count_launch();
        if (d == 0) break;
    }
    int e = 0;
    read_small(ctx, &e, err.get(), sizeof(int), st);
    if (e) throw Error(REGOT_ERR_TIMEOUT, "the tensor-core contraction gave up waiting");
}

}  // namespace regot
