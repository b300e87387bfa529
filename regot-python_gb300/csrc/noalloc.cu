// Allocation-free EROT objective/gradient (regot_erot_dual_obj_grad_noalloc).
//
// Some callers cannot call cudaMalloc: code that runs while another
// framework is capturing a CUDA graph (allocation calls are not allowed
// inside a global-mode capture), custom-call / plugin hooks of frameworks
// that own all device memory, and latency-critical loops where cudaMalloc's
// implicit device synchronisation is not acceptable. For them this entry
// point keeps its scratch (FP32 copies of the duals and the per-block
// partial sums of the dense pass) in one file-scope __device__ array of
// kNoallocScratchBytes bytes, which every GPU that loads the library holds
// until the process exits. It calls no allocating routine at all.
//
// The caller passes device pointers for every input and output. All calls
// share the array: calls that overlap on the GPU (on different streams, or
// from different host threads) race on it and must be serialised by the
// caller. The only word that has to start at zero, the pass's error word,
// is cleared by each call before the pass; every other word is overwritten
// before it is read.
//
// Errors on the GPU: the dense pass waits for its parameter copies with a
// bounded wait. If one gives up, the pass sets the error word in the scratch
// and the finishing kernels write NaN into grad and *obj, so the failure
// shows in the outputs without a host synchronisation (the call itself has
// already returned REGOT_OK by then).
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current); make that first call
// before any stream capture begins.
#include <cmath>
#include <mutex>

#include "device_util.cuh"
#include "internal.h"

namespace regot {
namespace {

// 16 MiB. A problem needs about 32 (n + m) + 4 n m (1/512 + 1/64) bytes
// (FP32 row partials per 512-column slab and column partials per 64-row
// block): up to about n = m = 15400; n = m = 14000 always fits.
constexpr size_t kNoallocScratchBytes = REGOT_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (set-up once
// per device).
void* scratch_address(int device) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw Error(REGOT_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                            cudaGetErrorString(e));
        g_noalloc_ptr[device] = ptr;
    }
    return g_noalloc_ptr[device];
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Single block: bound on |alpha|, |beta~| (for the hi/lo grid), then the
// FP32 split of alpha and of beta = (beta~, 0).
__global__ void k_noalloc_split(const double* gamma, int n, int m, double* maxabs, float4* rs,
                                float4* cs, int* err) {
    __shared__ double s_max[32];
    if (threadIdx.x == 0) *err = 0;
    double v = 0.0;
    for (int t = threadIdx.x; t < n + m - 1; t += blockDim.x) {
        const double x = gamma[t];
        if (isfinite(x)) v = fmax(v, fabs(x));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, s_max[w]);
        s_max[0] = mx;
        *maxabs = mx;
    }
    __syncthreads();
    const double mx = s_max[0];
    double g = 1.0, inv_g = 1.0;
    if (mx > 0.0) {
        const int e = ilogb(mx) - 21;
        g = ldexp(1.0, e);
        inv_g = ldexp(1.0, -e);
    }
    for (int t = threadIdx.x; t < n + m; t += blockDim.x) {
        const double x = t < n + m - 1 ? gamma[t] : 0.0;
        float hi = (float)x, lo = 0.f;
        if (isfinite(x)) {
            const double h = rint(x * inv_g) * g;
            hi = (float)h;
            lo = (float)(x - h);
        }
        if (t < n) rs[t] = make_float4(hi, lo, 0.f, 0.f);
        else cs[t - n] = make_float4(hi, lo, 0.f, 0.f);
    }
}

// Merge the pass partials: grad = [T 1 - a ; (T' 1 - b)_{j<m-1}], and per-block
// partials of sum(T 1), gamma_a . a, gamma_b . b.
// A pass whose bounded wait gave up (*err != 0) produced no valid partials:
// grad is then NaN.
__global__ void k_noalloc_grad(const float* rowpart, int nslabs, const float* colpart, int nrb,
                               int n, int m, const double* gamma, const double* a,
                               const double* b, double* grad, double* blockpart,
                               const int* err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool failed = *err != 0;
    double v[3] = {0.0, 0.0, 0.0};
    if (t < n) {
        const double r = merge_strided(rowpart + t, nslabs, (size_t)n);
        grad[t] = failed ? NAN : r - a[t];
        v[0] = r;
        v[1] = gamma[t] * a[t];
    } else if (t < n + m - 1) {
        const int j = t - n;
        const double c = merge_strided(colpart + j, nrb, (size_t)m);
        grad[t] = failed ? NAN : c - b[j];
        v[2] = gamma[t] * b[j];
    }
    __shared__ double s[3][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double x = warp_sum_d(v[q]);
        if (lane == 0) s[q][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double x = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) x += s[threadIdx.x][k];
        blockpart[(size_t)blockIdx.x * 3 + threadIdx.x] = x;
    }
}

// obj = reg * sum(T) - gamma_a . a - gamma_b . b~ (sinkhorn_problem_obj.cpp:389-390).
__global__ void k_noalloc_obj(const double* blockpart, int nblocks, double reg, double* obj,
                              const int* err) {
    if (threadIdx.x != 0) return;
    if (*err) {
        *obj = NAN;
        return;
    }
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = 0; k < nblocks; ++k) {
        s0 += blockpart[(size_t)k * 3 + 0];
        s1 += blockpart[(size_t)k * 3 + 1];
        s2 += blockpart[(size_t)k * 3 + 2];
    }
    *obj = reg * s0 - s1 - s2;
}

}  // namespace
}  // namespace regot

using namespace regot;

extern "C" int regot_erot_dual_obj_grad_noalloc(const float* M, long long ldm, int n, int m,
                                                const double* gamma, const double* a,
                                                const double* b, double reg, double* grad,
                                                double* obj, void* stream) {
    try {
        if (!M || !gamma || !a || !b || !grad || !obj) return REGOT_ERR_INVALID_ARG;
        if (n <= 0 || m <= 1 || ldm < m || ldm % 4 != 0) return REGOT_ERR_INVALID_ARG;
        if (!(reg > 0.0) || !std::isfinite(reg)) return REGOT_ERR_INVALID_ARG;
        if ((reinterpret_cast<uintptr_t>(M) & 15u) != 0) return REGOT_ERR_INVALID_ARG;
        int device = 0;
        REGOT_CUDA(cudaGetDevice(&device));
        if (device < 0 || device >= kMaxDevices) return REGOT_ERR_INVALID_ARG;
        const PassShape sh = pass_shape<float>(n, m);
        const int fin_threads = 64;
        const int fin_blocks = cdiv((long long)n + m - 1, fin_threads);
        // Scratch layout.
        size_t off = 0;
        const size_t o_max = off;
        off = align256(off + sizeof(double));
        const size_t o_err = off;
        off = align256(off + sizeof(int));
        const size_t o_rs = off;
        off = align256(off + (size_t)n * sizeof(float4));
        const size_t o_cs = off;
        off = align256(off + (size_t)m * sizeof(float4));
        const size_t o_row = off;
        off = align256(off + (size_t)sh.nslabs * n * sizeof(float));
        const size_t o_col = off;
        off = align256(off + (size_t)sh.nrb * m * sizeof(float));
        const size_t o_blk = off;
        off = align256(off + (size_t)fin_blocks * 3 * sizeof(double));
        if (off > kNoallocScratchBytes) return REGOT_ERR_TOO_LARGE;

        unsigned char* base = static_cast<unsigned char*>(scratch_address(device));
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        double* maxabs = reinterpret_cast<double*>(base + o_max);
        float4* rs = reinterpret_cast<float4*>(base + o_rs);
        float4* cs = reinterpret_cast<float4*>(base + o_cs);
        float* rowpart = reinterpret_cast<float*>(base + o_row);
        float* colpart = reinterpret_cast<float*>(base + o_col);
        double* blk = reinterpret_cast<double*>(base + o_blk);
        int* err = reinterpret_cast<int*>(base + o_err);

        k_noalloc_split<<<1, 1024, 0, st>>>(gamma, n, m, maxabs, rs, cs, err);
        REGOT_CHECK_LAUNCH();
        PassParams p;
        p.M = M;
        p.ldm = ldm;
        p.n = n;
        p.m = m;
        p.reg = reg;
        p.grid = maxabs;
        p.rsplit = rs;
        p.csplit = cs;
        p.rowpart = rowpart;
        p.colpart = colpart;
        p.err = err;
        launch_pass<float>(OP_E_ROWCOL, p, st);
        k_noalloc_grad<<<fin_blocks, fin_threads, 0, st>>>(rowpart, sh.nslabs, colpart, sh.nrb, n,
                                                           m, gamma, a, b, grad, blk, err);
        REGOT_CHECK_LAUNCH();
        k_noalloc_obj<<<1, 32, 0, st>>>(blk, fin_blocks, reg, obj, err);
        REGOT_CHECK_LAUNCH();
        return REGOT_OK;
    } catch (const Error& e) {
        return e.code;
    } catch (...) {
        return REGOT_ERR_CUDA;
    }
}
