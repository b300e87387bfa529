// Dense streaming passes over the cost matrix M: the n x m hot path of the
// EROT and QROT solvers. Every pass reads M exactly once with 16-byte
// coalesced loads and reduces in registers/shared memory; row results leave
// as per-(row, column-slab) partials, column results as per-(row-block,
// column) partials, scalars as per-CTA partials. The finalize kernels of the
// solvers merge those partials in FP64 in a fixed order (deterministic; no
// floating-point atomics).
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
#include <cfloat>
#include <cmath>
#include <type_traits>

#include "internal.h"

namespace regot {

thread_local long long* g_launch_counter = nullptr;

namespace {

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
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
         : 0;
}
__host__ __device__ constexpr int op_nc(int op) {
    return op == OP_E_COL ? 1 : op == OP_E_ROWCOL ? 1 : op == OP_E_HVP ? 1 : op == OP_E_COLMAX ? 1
         : op == OP_Q_GRAD ? 1 : op == OP_Q_GRADMASK ? 2 : op == OP_Q_P2 ? 1 : op == OP_Q_COLROOT ? 2
         : 0;
}
__host__ __device__ constexpr int op_nt(int op) {
    return op == OP_E_LS ? 4 : op == OP_Q_GRAD ? 1 : op == OP_Q_GRADMASK ? 1 : op == OP_Q_OBJ ? 1
         : op == OP_Q_P3 ? 2 : 0;
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

// Power-of-two grid for the hi/lo split, from a bound on |ra|, |cb|.
__device__ __forceinline__ double split_grid(const double* maxabs) {
    if (!maxabs) return 1.0;
    const double mx = *maxabs;
    if (!(mx > 0.0) || !isfinite(mx)) return 1.0;
    return ldexp(1.0, ilogb(mx) - 21);
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

template <typename TM, int OP>
__global__ void __launch_bounds__(kThreads) dense_pass(const PassParams p) {
    if (p.done && *p.done) return;
    using G = Geo<TM>;
    constexpr int VW = G::VW, LC = G::LC, CW = G::CW;
    constexpr bool MIXED = std::is_same<TM, float>::value;
    constexpr bool COLROOT = (OP == OP_Q_COLROOT);
    using Acc = typename std::conditional<COLROOT, double, TM>::type;
    using VT = typename Vec<TM>::type;
    constexpr int NR = op_nr(OP), NC = op_nc(OP), NT = op_nt(OP);
    constexpr int NRa = NR > 0 ? NR : 1, NCa = NC > 0 ? NC : 1, NTa = NT > 0 ? NT : 1;
    constexpr bool ISMAX = op_is_max(OP);
    constexpr bool EROT = (OP <= OP_E_COLMAX);
    constexpr int RPW = kRB / kWarps;  // rows per warp

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int slab = blockIdx.x, rb = blockIdx.y;
    const int nslabs = gridDim.x, nrb = gridDim.y;
    const int c0 = slab * CW, r0 = rb * kRB;
    const int n = p.n, m = p.m;
    const long long ldm = p.ldm;

    // Constants prepared on the host (no FP64 arithmetic in this kernel:
    // FP64 throughput on this part is a small fraction of FP32).
    const double reg = p.reg;
    const TM kexp = MIXED ? (TM)p.kexp_f : (TM)p.kexp_d;
    const TM inv_reg = MIXED ? (TM)p.inv_reg_f : (TM)p.inv_reg_d;

    // ---- per-row parameters, staged once per CTA in shared memory ----
    __shared__ TM s_rh[kRB], s_rl[kRB], s_rx[kRB], s_rd[kRB];
    __shared__ double s_rad[COLROOT ? kRB : 1];
    if (threadIdx.x < kRB) {
        const int i = r0 + threadIdx.x;
        const bool ok = i < n;
        if constexpr (MIXED) {
            const float4 v = (ok && p.rsplit) ? p.rsplit[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            s_rh[threadIdx.x] = v.x;
            s_rl[threadIdx.x] = v.y;
            s_rx[threadIdx.x] = v.z;
            s_rd[threadIdx.x] = v.w;
        } else {
            s_rh[threadIdx.x] = (ok && p.ra && op_needs_ra(OP)) ? (TM)p.ra[i] : (TM)0;
            s_rl[threadIdx.x] = 0;
            s_rx[threadIdx.x] = (ok && p.rx) ? (TM)p.rx[i] : (TM)0;
            s_rd[threadIdx.x] = (ok && p.rd) ? (TM)p.rd[i] : (TM)0;
        }
        if constexpr (COLROOT) s_rad[threadIdx.x] = (ok && p.ra) ? p.ra[i] : 0.0;
    }

    // ---- per-column parameters in registers ----
    TM ch[LC], cl[LC], cxv[LC], cx2v[LC], cdv[LC];
    double cbd[COLROOT ? LC : 1];
    bool cvalid[LC];
#pragma unroll
    for (int k = 0; k < LC; ++k) {
        const int v = k / VW, e = k % VW;
        const int j = c0 + (v * 32 + lane) * VW + e;
        const bool ok = j < m;
        cvalid[k] = ok;
        if constexpr (COLROOT) cbd[k] = ok ? p.cb[j] : -INFINITY;
        if constexpr (MIXED) {
            const float4 c = (ok && p.csplit) ? p.csplit[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            ch[k] = ok ? c.x : -INFINITY;
            cl[k] = ok ? c.y : 0.f;
            cxv[k] = c.z;
            cx2v[k] = c.w;
            cdv[k] = (ok && p.cdsplit) ? p.cdsplit[j] : 0.f;
        } else {
            ch[k] = ok ? ((p.cb && op_needs_cb(OP)) ? (TM)p.cb[j] : (TM)0) : (TM)(-INFINITY);
            cl[k] = 0;
            cxv[k] = (ok && p.cx) ? (TM)p.cx[j] : (TM)0;
            cx2v[k] = (ok && p.cx2) ? (TM)p.cx2[j] : (TM)0;
            cdv[k] = (ok && p.cd) ? (TM)p.cd[j] : (TM)0;
        }
    }
    __syncthreads();

    const TM init = ISMAX ? (TM)(-INFINITY) : (TM)0;
    Acc cacc[NCa][LC];
#pragma unroll
    for (int c = 0; c < NCa; ++c)
#pragma unroll
        for (int k = 0; k < LC; ++k) cacc[c][k] = (Acc)init;
    Acc tot[NTa];
#pragma unroll
    for (int t = 0; t < NTa; ++t) tot[t] = 0;

    TM steps[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) steps[t] = (TM)p.steps[t];
    const int nsteps = p.nsteps;

    const TM* Mbase = reinterpret_cast<const TM*>(p.M);
    const int rw0 = warp * RPW;

#pragma unroll 1
    for (int u0 = 0; u0 < RPW; u0 += 4) {
        VT mv[4][2];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = r0 + rw0 + u0 + u;
#pragma unroll
            for (int v = 0; v < 2; ++v) {
                const long long col = c0 + (long long)(v * 32 + lane) * VW;
                if (i < n && col < ldm)
                    mv[u][v] = *reinterpret_cast<const VT*>(Mbase + (long long)i * ldm + col);
                else
                    mv[u][v] = Vec<TM>::zero();
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int li = rw0 + u0 + u;
            const int i = r0 + li;
            if (i >= n) break;
            const TM rh = s_rh[li], rl = s_rl[li], rxv = s_rx[li], rdv = s_rd[li];
            const double rad = COLROOT ? s_rad[COLROOT ? li : 0] : 0.0;
            Acc racc[NRa];
#pragma unroll
            for (int r = 0; r < NRa; ++r) racc[r] = (Acc)init;
            uint32_t bits = 0;  // for OP_Q_GRADMASK: one word per column slot
            (void)bits;

#pragma unroll
            for (int k = 0; k < LC; ++k) {
                const TM mval = Vec<TM>::get(mv[u][k / VW], k % VW);
                if constexpr (OP == OP_E_ROWMAX) {
                    TM a;
                    if constexpr (MIXED) a = (ch[k] - mval) + cl[k];
                    else a = ch[k] - mval;
                    racc[0] = fmax(racc[0], a);
                } else if constexpr (OP == OP_E_COLMAX) {
                    TM a;
                    if constexpr (MIXED) a = (rh - mval) + rl;
                    else a = rh - mval;
                    if (cvalid[k]) cacc[0][k] = fmax(cacc[0][k], (Acc)a);
                } else if constexpr (COLROOT) {
                    const double y = (double)mval - rad;
                    if (cvalid[k] && y < cbd[k]) {
                        cacc[0][k] += 1.0;
                        cacc[1][k] += y;
                    }
                } else {
                    TM arg;
                    if constexpr (MIXED) arg = ((rh + ch[k]) - mval) + (rl + cl[k]);
                    else arg = (rh + ch[k]) - mval;
                    if constexpr (EROT) {
                        TM T;
                        if constexpr (MIXED) T = ex2_approx(arg * kexp);
                        else T = exp(arg * kexp);
                        if constexpr (OP == OP_E_ROW) {
                            racc[0] += T;
                        } else if constexpr (OP == OP_E_COL) {
                            cacc[0][k] += T;
                        } else if constexpr (OP == OP_E_ROWCOL) {
                            racc[0] += T;
                            cacc[0][k] += T;
                        } else if constexpr (OP == OP_E_HVP) {
                            racc[0] += T * cxv[k];
                            cacc[0][k] += T * rxv;
                        } else if constexpr (OP == OP_E_LS) {
                            const TM w = (rdv + cdv[k]) * inv_reg;
#pragma unroll
                            for (int t = 0; t < 4; ++t)
                                if (t < nsteps) tot[t] += T * expm1(steps[t] * w);
                        } else if constexpr (OP == OP_E_PLAN) {
                            if (cvalid[k]) {
                                const int j = c0 + ((k / VW) * 32 + lane) * VW + (k % VW);
                                p.out[(long long)i * m + j] = (double)T;
                            }
                        }
                    } else {
                        const TM D = arg > (TM)0 ? arg : (TM)0;
                        if constexpr (OP == OP_Q_GRAD) {
                            racc[0] += D;
                            cacc[0][k] += D;
                            tot[0] += D * D;
                        } else if constexpr (OP == OP_Q_GRADMASK) {
                            const bool pos = arg > (TM)0;
                            racc[0] += D;
                            cacc[0][k] += D;
                            tot[0] += D * D;
                            racc[1] += pos ? (TM)1 : (TM)0;
                            cacc[1][k] += pos ? (TM)1 : (TM)0;
                            const uint32_t word = __ballot_sync(0xffffffffu, pos);
                            if (lane == k) bits = word;
                        } else if constexpr (OP == OP_Q_OBJ) {
                            tot[0] += D * D;
                        } else if constexpr (OP == OP_Q_P1) {
                            racc[0] += D;
                        } else if constexpr (OP == OP_Q_P2) {
                            cacc[0][k] += D * rxv;
                        } else if constexpr (OP == OP_Q_P3) {
                            const TM Dy = D * cxv[k];
                            racc[0] += Dy;
                            racc[1] += Dy * cx2v[k];
                            racc[2] += mval * cx2v[k];
                            const TM R = rxv * Dy;
                            tot[0] += R * mval;
                            tot[1] += R * R;
                        } else if constexpr (OP == OP_Q_PLAN) {
                            if (cvalid[k]) {
                                const int j = c0 + ((k / VW) * 32 + lane) * VW + (k % VW);
                                p.out[(long long)i * m + j] = (double)D * p.inv_reg_d;
                            }
                        }
                    }
                }
            }
            if constexpr (OP == OP_Q_GRADMASK) {
                if (lane < LC) p.bitmask[((long long)i * nslabs + slab) * LC + lane] = bits;
            }
            if constexpr (NR > 0) {
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    racc[r] = ISMAX ? warp_max(racc[r]) : warp_sum(racc[r]);
                }
                if (lane == 0) {
                    Acc* rp = reinterpret_cast<Acc*>(p.rowpart);
#pragma unroll
                    for (int r = 0; r < NR; ++r) rp[((long long)r * nslabs + slab) * n + i] = racc[r];
                }
            }
        }
    }

    // ---- column partials: reduce the 8 warps through shared memory ----
    if constexpr (NC > 0) {
        __shared__ Acc s_c[NC][kWarps][CW];
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
            for (int k = 0; k < LC; ++k) {
                const int off = (k / VW) * 32 * VW + lane * VW + (k % VW);
                s_c[c][warp][off] = cacc[c][k];
            }
        __syncthreads();
        Acc* cp = reinterpret_cast<Acc*>(p.colpart);
        for (int t = threadIdx.x; t < CW; t += kThreads) {
            const int j = c0 + t;
            if (j >= m) continue;
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                Acc s = s_c[c][0][t];
#pragma unroll
                for (int w = 1; w < kWarps; ++w) s = ISMAX ? fmax(s, s_c[c][w][t]) : s + s_c[c][w][t];
                cp[((long long)c * nrb + rb) * m + j] = s;
            }
        }
    }

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
            p.totpart[(long long)threadIdx.x * (nslabs * nrb) + rb * nslabs + slab] = s;
        }
    }
}

// FP32 copies of the per-row / per-column vectors of a mixed pass; the duals
// are split on the common grid G = 2^(floor(log2 bound) - 21).
__global__ void k_split(const PassParams p, float4* rs, float4* cs, float* cds) {
    double g = 1.0, inv_g = 1.0;
    if (p.grid) {
        const double mx = *p.grid;
        if (mx > 0.0 && isfinite(mx)) {
            const int e = ilogb(mx) - 21;
            g = ldexp(1.0, e);
            inv_g = ldexp(1.0, -e);
        }
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < p.n) {
        float hi = 0.f, lo = 0.f;
        if (p.ra) split(p.ra[t], g, inv_g, hi, lo);
        rs[t] = make_float4(hi, lo, p.rx ? (float)p.rx[t] : 0.f, p.rd ? (float)p.rd[t] : 0.f);
    } else if (t < p.n + p.m) {
        const int j = t - p.n;
        float hi = 0.f, lo = 0.f;
        if (p.cb) split(p.cb[j], g, inv_g, hi, lo);
        cs[j] = make_float4(hi, lo, p.cx ? (float)p.cx[j] : 0.f, p.cx2 ? (float)p.cx2[j] : 0.f);
        if (cds) cds[j] = p.cd ? (float)p.cd[j] : 0.f;
    }
}

template <typename TM, int OP>
void launch_one(const PassParams& p, cudaStream_t st) {
    const PassShape s = pass_shape<TM>(p.n, p.m);
    dim3 grid(s.nslabs, s.nrb);
    dense_pass<TM, OP><<<grid, kThreads, 0, st>>>(p);
    REGOT_CHECK_LAUNCH();
    count_launch();
}

template <typename TM>
struct Dispatch {
    template <int OP>
    static void go(int op, const PassParams& p, cudaStream_t st) {
        if constexpr (OP < OP_COUNT) {
            if (op == OP) launch_one<TM, OP>(p, st);
            else go<OP + 1>(op, p, st);
        } else {
            throw Error(REGOT_ERR_INVALID_ARG, "unknown dense pass");
        }
    }
};

}  // namespace

template <typename TM>
void launch_pass(int op, const PassParams& p, cudaStream_t st) {
    if (p.n <= 0 || p.m <= 0) return;
    PassParams q = p;
    q.kexp_f = (float)(1.4426950408889634 / p.reg);
    q.inv_reg_f = (float)(1.0 / p.reg);
    q.kexp_d = 1.0 / p.reg;
    q.inv_reg_d = 1.0 / p.reg;
    Dispatch<TM>::template go<0>(op, q, st);
}

void launch_split(const PassParams& p, float4* rs, float4* cs, float* cds, cudaStream_t st) {
    k_split<<<cdiv(p.n + p.m, 64), 64, 0, st>>>(p, rs, cs, cds);
    REGOT_CHECK_LAUNCH();
    count_launch();
}

template void launch_pass<float>(int, const PassParams&, cudaStream_t);
template void launch_pass<double>(int, const PassParams&, cudaStream_t);

}  // namespace regot
