// Device-side helpers shared by the solver translation units: grid-wide
// deterministic reductions (per-block partials summed in block order by the
// last block to finish), the device clock, and stream-ordered buffers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <utility>

#include "internal.h"

namespace regot {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Running maximum of |v| for the hi/lo split grid (positive doubles order
// like their bit patterns, so an integer atomicMax is exact).
__device__ __forceinline__ void atomic_max_abs(double* target, double v) {
    const double a = fabs(v);
    if (!(a == a)) return;
    atomicMax(reinterpret_cast<unsigned long long*>(target),
              (unsigned long long)__double_as_longlong(a));
}

// Bit pattern of |v| for the running maximum (NaN and infinities count as 0),
// and its maximum over a full warp in integer arithmetic (FP64 instructions
// issue at a small fraction of the integer rate on this part).
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    unsigned long long bits = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
    return (bits >> 52) == 0x7ffULL ? 0ULL : bits;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long bits) {
    const unsigned hi = (unsigned)(bits >> 32), lo = (unsigned)bits;
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    return ((unsigned long long)mhi << 32) | mlo;
}

// Warp-aggregated version: one atomic per warp (all lanes must call it).
__device__ __forceinline__ void warp_atomic_max_abs(double* target, double v) {
    const unsigned long long mx = warp_max_u64(abs_bits(v));
    if ((threadIdx.x & 31) == 0 && mx != 0ULL)
        atomicMax(reinterpret_cast<unsigned long long*>(target), mx);
}

// Block-wide version (all threads of the block must call it): one atomic
// per block instead of one per warp, so that the many blocks of a finalize
// kernel do not serialise on the target's cache line.
__device__ __forceinline__ void block_atomic_max_bits(double* target, unsigned long long bits) {
    __shared__ unsigned long long s_bmax[32];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const unsigned long long a = warp_max_u64(bits);
    if ((tid & 31) == 0) s_bmax[tid >> 5] = a;
    __syncthreads();
    if (tid == 0) {
        unsigned long long mx = 0ULL;
        for (int w = 0; w < (nthreads + 31) >> 5; ++w) mx = s_bmax[w] > mx ? s_bmax[w] : mx;
        if (mx != 0ULL) atomicMax(reinterpret_cast<unsigned long long*>(target), mx);
    }
    __syncthreads();
}

__device__ __forceinline__ void block_atomic_max_abs(double* target, double v) {
    block_atomic_max_bits(target, abs_bits(v));
}

// Sum of count values p[k * stride], k = 0..count-1, in FP64. Loads are
// issued eight at a time into four independent accumulators, so that the
// merge is bound by memory throughput instead of one load latency per term;
// the order is fixed, so results are reproducible.
template <typename Acc>
__device__ __forceinline__ double merge_strided(const Acc* p, int count, size_t stride) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int k = 0;
    for (; k + 8 <= count; k += 8) {
        Acc v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = p[(size_t)(k + q) * stride];
        s0 += (double)v[0] + (double)v[4];
        s1 += (double)v[1] + (double)v[5];
        s2 += (double)v[2] + (double)v[6];
        s3 += (double)v[3] + (double)v[7];
    }
    for (; k < count; ++k) s0 += (double)p[(size_t)k * stride];
    return (s0 + s1) + (s2 + s3);
}

// Knuth's TwoSum in FP32: s + e == a + b exactly (no FMA can be formed, so
// contraction does not change it).
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = a + b;
    const float z = s - a;
    e = (a - (s - z)) + (b - z);
}

// ---- double-word FP32 arithmetic: a value is the unevaluated sum hi + lo
// of two floats (|lo| <= ulp(hi) / 2), about 48 significant bits. Used where
// FP64's issue rate and latency on this part would bound a kernel. The
// algorithms are the published ones: Knuth's TwoSum, Dekker's Fast2Sum, the
// FMA-based TwoProd, and AccurateDWPlusDW, DWTimesDW and DWDivDW of Joldes,
// Muller and Popescu, "Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic" (ACM TOMS 44, 2017). Products that must
// round on their own are written with __fmul_rn so that they are not
// contracted into a neighbouring addition. dw_add(x, y) and dw_add(y, x)
// give the same bits (TwoSum's error term is exact in either order), so a
// butterfly of dw_add leaves every lane with the same result. ----
__device__ __forceinline__ float2 fast_two_sum_f(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return make_float2(s, b - (s - a));
}
__device__ __forceinline__ float2 dw_from(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ double dw_to(float2 v) { return (double)v.x + (double)v.y; }
__device__ __forceinline__ float2 dw_add(float2 x, float2 y) {
    float sh, sl, th, tl;
    two_sum_f(x.x, y.x, sh, sl);
    two_sum_f(x.y, y.y, th, tl);
    const float2 v = fast_two_sum_f(sh, sl + th);
    return fast_two_sum_f(v.x, tl + v.y);
}
__device__ __forceinline__ float2 dw_neg(float2 x) { return make_float2(-x.x, -x.y); }
__device__ __forceinline__ float2 dw_sub(float2 x, float2 y) { return dw_add(x, dw_neg(y)); }
__device__ __forceinline__ float2 dw_mul(float2 x, float2 y) {
    const float ch = __fmul_rn(x.x, y.x);
    const float cl1 = fmaf(x.x, y.x, -ch);
    const float tl1 = fmaf(x.x, y.y, __fmul_rn(x.y, y.y));
    const float cl2 = fmaf(x.y, y.x, tl1);
    return fast_two_sum_f(ch, cl1 + cl2);
}
__device__ __forceinline__ float2 dw_mul_f(float2 x, float y) {
    const float ch = __fmul_rn(x.x, y);
    const float cl1 = fmaf(x.x, y, -ch);
    return fast_two_sum_f(ch, fmaf(x.y, y, cl1));
}
__device__ __forceinline__ float2 dw_div(float2 x, float2 y) {
    const float th = x.x / y.x;
    const float2 r = dw_mul_f(y, th);
    float ph, sl;
    two_sum_f(x.x, -r.x, ph, sl);
    const float d = sl + (x.y - r.y);
    return fast_two_sum_f(th, (ph + d) / y.x);
}
// x < y for normalised double-word values
__device__ __forceinline__ bool dw_lt(float2 x, float2 y) {
    return x.x < y.x || (x.x == y.x && x.y < y.y);
}
// compensated sum (s, e) of a TwoSum accumulation, as a double-word value
__device__ __forceinline__ float2 dw_norm(float s, float e) {
    float h, l;
    two_sum_f(s, e, h, l);
    return make_float2(h, l);
}

// FP32 partials: compensated FP32 sums (TwoSum, two independent
// accumulators with their rounding errors beside them), converted to FP64
// once. FP64 arithmetic issues at a small fraction of the FP32 rate on this
// part; converting and adding every partial in FP64 made the merge kernels
// of the solver loops FP64-bound. The error stays at about count * 2^-48
// relative, the level of the FP64 sum.
template <>
__device__ __forceinline__ double merge_strided<float>(const float* p, int count, size_t stride) {
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
    int k = 0;
    for (; k + 8 <= count; k += 8) {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = p[(size_t)(k + q) * stride];
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
            float t, e;
            two_sum_f(s0, v[q], t, e);
            s0 = t;
            c0 += e;
            two_sum_f(s1, v[q + 1], t, e);
            s1 = t;
            c1 += e;
        }
    }
    for (; k < count; ++k) {
        float t, e;
        two_sum_f(s0, p[(size_t)k * stride], t, e);
        s0 = t;
        c0 += e;
    }
    return ((double)s0 + (double)s1) + ((double)c0 + (double)c1);
}

template <typename Acc>
__device__ __forceinline__ double max_strided(const Acc* p, int count, size_t stride) {
    double s0 = -INFINITY, s1 = -INFINITY;
    int k = 0;
    for (; k + 8 <= count; k += 8) {
        Acc v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = p[(size_t)(k + q) * stride];
        s0 = fmax(s0, fmax(fmax((double)v[0], (double)v[1]), fmax((double)v[2], (double)v[3])));
        s1 = fmax(s1, fmax(fmax((double)v[4], (double)v[5]), fmax((double)v[6], (double)v[7])));
    }
    for (; k < count; ++k) s0 = fmax(s0, (double)p[(size_t)k * stride]);
    return fmax(s0, s1);
}

// Grid-wide sum of K values per thread. Returns true in thread 0 of the last
// block to finish, with the totals in out[]. The last block sums the
// per-block partials with all its threads (thread t takes blocks t, t + bs,
// ... in order, then a fixed butterfly and warp order), so the result does
// not depend on which block finishes last.
// LANE0: only lane 0 of each warp holds nonzero values (warp-per-item
// kernels); the warp sums are then lane 0's values, read without the
// FP64 butterfly (adding the other lanes' zeros would not change them).
template <int K, bool LANE0 = false>
__device__ bool grid_reduce(const double (&vals)[K], double* block_parts, unsigned* counter,
                            double (&out)[K]) {
    __shared__ double s_red[K][32];
    __shared__ bool s_last;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const int lane = tid & 31, warp = tid >> 5;
    const int nw = (nthreads + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double v = LANE0 ? vals[k] : warp_sum_d(vals[k]);
        if (lane == 0) s_red[k][warp] = v;
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += s_red[k][w];
            block_parts[(size_t)blockIdx.x * K + k] = s;
        }
        __threadfence();
        const unsigned ticket = atomicAdd(counter, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double part[K];
#pragma unroll
    for (int k = 0; k < K; ++k) part[k] = 0.0;
    for (unsigned b = tid; b < gridDim.x; b += nthreads) {
#pragma unroll
        for (int k = 0; k < K; ++k) part[k] += __ldcg(&block_parts[(size_t)b * K + k]);
    }
    __syncthreads();  // s_red is reused
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double v = warp_sum_d(part[k]);
        if (lane == 0) s_red[k][warp] = v;
    }
    __syncthreads();
    if (tid != 0) return false;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += s_red[k][w];
        out[k] = s;
    }
    *counter = 0u;
    return true;
}

// Merge of `count` partials p[k * stride] (k = 0 .. count-1) for the 32
// items of a (32, 8) block: item threadIdx.x, partials split over
// threadIdx.y (k = y, y + 8, ...), then summed over y in order. The result
// is valid in the threads with threadIdx.y == 0. Loads of one k are
// coalesced across the 32 items.
template <typename Acc>
__device__ __forceinline__ double merge_2d(const Acc* p, int count, size_t stride, bool valid) {
    __shared__ double s_m2[8][33];
    double a0 = 0.0, a1 = 0.0;
    if (valid) {
        int k = threadIdx.y;
        for (; k + 8 < count; k += 16) {
            a0 += (double)p[(size_t)k * stride];
            a1 += (double)p[(size_t)(k + 8) * stride];
        }
        if (k < count) a0 += (double)p[(size_t)k * stride];
    }
    s_m2[threadIdx.y][threadIdx.x] = a0 + a1;
    __syncthreads();
    double S = 0.0;
    if (threadIdx.y == 0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) S += s_m2[q][threadIdx.x];
    }
    return S;
}

// FP32 partials: the same merge with compensated FP32 sums (TwoSum, the
// rounding errors accumulated beside the sum), converted to FP64 once per
// item. FP64 arithmetic issues at a small fraction of the FP32 rate on this
// part, and converting and adding every partial in FP64 dominated the
// finalize kernels; the compensated sum keeps the merge error at the level of
// the FP64 one (about count * 2^-48 relative instead of count * 2^-24).
template <>
__device__ __forceinline__ double merge_2d<float>(const float* p, int count, size_t stride,
                                                  bool valid) {
    __shared__ float2 s_mf[8][33];
    float s = 0.f, c = 0.f;
    if (valid) {
        int k = threadIdx.y;
        for (; k + 24 < count; k += 32) {
            float v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = p[(size_t)(k + 8 * q) * stride];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float t, e;
                two_sum_f(s, v[q], t, e);
                s = t;
                c += e;
            }
        }
        for (; k < count; k += 8) {
            float t, e;
            two_sum_f(s, p[(size_t)k * stride], t, e);
            s = t;
            c += e;
        }
    }
    s_mf[threadIdx.y][threadIdx.x] = make_float2(s, c);
    __syncthreads();
    double S = 0.0;
    if (threadIdx.y == 0) {
        float ss = 0.f, cc = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float2 v = s_mf[q][threadIdx.x];
            float t, e;
            two_sum_f(ss, v.x, t, e);
            ss = t;
            cc += e + v.y;
        }
        S = (double)ss + (double)cc;
    }
    return S;
}

// Maximum of `count` partials p[k * stride] for the 32 items of a (32, 8)
// block, laid out as in merge_2d (exact in the partials' own type). Valid in
// the threads with threadIdx.y == 0.
template <typename Acc>
__device__ __forceinline__ double max_2d(const Acc* p, int count, size_t stride, bool valid) {
    __shared__ Acc s_mx[8][33];
    Acc v = (Acc)(-INFINITY);
    if (valid)
        for (int k = threadIdx.y; k < count; k += 8) v = fmax(v, p[(size_t)k * stride]);
    s_mx[threadIdx.y][threadIdx.x] = v;
    __syncthreads();
    Acc r = (Acc)(-INFINITY);
    if (threadIdx.y == 0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) r = fmax(r, s_mx[q][threadIdx.x]);
    }
    return (double)r;
}

// Grid-wide sum of K values when one full warp of each block holds them (the
// other warps of the block take no part). Returns true in every lane of that
// warp of the last block to finish, with the totals in out[]. The last warp
// sums the per-block partials lane l taking blocks l, l + 32, ... in order,
// then a fixed butterfly, so the result does not depend on which block
// finishes last.
template <int K>
__device__ bool warp_grid_reduce(const double (&vals)[K], double* block_parts, unsigned* counter,
                                 double (&out)[K]) {
    const int lane = threadIdx.x & 31;
    unsigned last = 0;
    double s[K];
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] = warp_sum_d(vals[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) block_parts[(size_t)blockIdx.x * K + k] = s[k];
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1 ? 1u : 0u;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return false;
    __threadfence();
    double part[K];
#pragma unroll
    for (int k = 0; k < K; ++k) part[k] = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) {
#pragma unroll
        for (int k = 0; k < K; ++k) part[k] += __ldcg(&block_parts[(size_t)b * K + k]);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = warp_sum_d(part[k]);
    if (lane == 0) *counter = 0u;
    return true;
}

// Stream-ordered device buffer (dev_alloc / cudaFreeAsync).
template <typename T>
class DBuf {
public:
    DBuf() = default;
    DBuf(size_t count, cudaStream_t st) { alloc(count, st); }
    ~DBuf() { release(); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept { swap(o); }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            release();
            swap(o);
        }
        return *this;
    }
    void alloc(size_t count, cudaStream_t st) {
        release();
        st_ = st;
        count_ = count;
        if (count) p_ = static_cast<T*>(dev_alloc(count * sizeof(T), st));
    }
    void zero() {
        if (count_) REGOT_CUDA(cudaMemsetAsync(p_, 0, count_ * sizeof(T), st_));
    }
    T* get() const { return p_; }
    size_t size() const { return count_; }
    void release() {
        if (p_) cudaFreeAsync(p_, st_);
        p_ = nullptr;
        count_ = 0;
    }

private:
    void swap(DBuf& o) {
        std::swap(p_, o.p_);
        std::swap(count_, o.count_);
        std::swap(st_, o.st_);
    }
    T* p_ = nullptr;
    size_t count_ = 0;
    cudaStream_t st_ = nullptr;
};

inline void h2d(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    if (bytes) REGOT_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
}
inline void d2h(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    if (bytes) REGOT_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
}
inline void d2d(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    if (bytes) REGOT_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
}
inline void sync(cudaStream_t st) { REGOT_CUDA(cudaStreamSynchronize(st)); }

// Plan output of `count` doubles at `plan` (device or host memory per
// plan_mem); compute(dst) launches the kernel that writes dst. A host
// destination inside a regot_host_alloc block is written by the kernel
// directly (the transfer overlaps the computation and no device copy of the
// plan is made); other host memory goes through a device buffer and one copy.
// The caller synchronises the stream before reading the host result.
// Averaged plans kept in FP32 to the FP64 plan output.
template <typename T>
__global__ void k_widen(const T* x, long long count, double* y) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
         t += (long long)gridDim.x * blockDim.x)
        y[t] = (double)x[t];
}

template <typename F>
void emit_plan(double* plan, int plan_mem, size_t count, cudaStream_t st, F&& compute) {
    if (plan_mem == REGOT_MEM_DEVICE) {
        compute(plan);
        return;
    }
    if (void* view = host_block_view(plan, count * sizeof(double))) {
        compute(static_cast<double*>(view));
        return;
    }
    DBuf<double> out(count, st);
    compute(out.get());
    d2h(plan, out.get(), count * sizeof(double), st);
    sync(st);
}

}  // namespace regot
