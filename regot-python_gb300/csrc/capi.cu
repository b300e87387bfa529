// C ABI of regot_gb300 (declarations and reference citations in
// include/regot_gb300.h): contexts, device-resident problems, the solver
// entry points and the pass-level entry points. Every entry point converts
// exceptions into a status code and a per-context message.
#include <sys/stat.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <type_traits>
#include <vector>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "internal.h"
#include "solvers.h"

using namespace regot;

namespace {

template <typename F>
int guarded(regot_ctx* ctx, F&& f) {
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

template <typename TS, typename TD>
__global__ void k_convert(const TS* src, long long lds, TD* dst, long long ldd, int n, int m) {
    const long long total = (long long)n * ldd;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long i = t / ldd, j = t - i * ldd;
        dst[t] = j < m ? (TD)src[i * lds + j] : (TD)0;
    }
}

// *flag = 1 if any of the `nvec` 16-byte vectors of M holds a NaN or an
// infinity (padding columns are zero).
template <typename TM>
__global__ void k_nonfinite(const void* M, long long nvec, int* flag) {
    using V = typename std::conditional<sizeof(TM) == 4, float4, double2>::type;
    const V* v = static_cast<const V*>(M);
    bool bad = false;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nvec;
         t += (long long)gridDim.x * blockDim.x) {
        const V x = v[t];
        if constexpr (sizeof(TM) == 4)
            bad |= !(isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(x.w));
        else
            bad |= !(isfinite(x.x) && isfinite(x.y));
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

void check_solver_args(regot_dproblem* P, double reg, double tol, int max_iter, regot_result* res,
                       int dual_len) {
    require(P != nullptr, "problem is NULL");
    require(res != nullptr, "result is NULL");
    require(std::isfinite(reg) && reg > 0.0, "reg must be a positive finite number");
    require(!std::isnan(tol), "tol must not be NaN");
    require(max_iter >= 0, "max_iter must be non-negative");
    require(res->dual != nullptr, "result dual buffer is NULL");
    require(res->hist_cap >= max_iter + 2 ||
                (!res->obj_vals && !res->mar_errs && !res->run_times && !res->densities &&
                 !res->prim_vals),
            "history capacity must be at least max_iter + 2");
    (void)dual_len;
}

regot_opts effective_opts(const regot_opts* o) {
    regot_opts e;
    regot_opts_init(&e);
    if (o) e = *o;
    return e;
}

}  // namespace

namespace regot {

static std::mutex g_pool_mutex;
static std::unordered_map<int, cudaMemPool_t> g_pools;  // per device, kept for the process

void* dev_alloc(size_t bytes, cudaStream_t st) {
    int dev = 0;
    REGOT_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_pool_mutex);
        auto it = g_pools.find(dev);
        if (it != g_pools.end()) {
            pool = it->second;
        } else {
            cudaMemPoolProps props;
            std::memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            REGOT_CUDA(cudaMemPoolCreate(&pool, &props));
            unsigned long long keep = kPoolKeepBytes;
            REGOT_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
            g_pools[dev] = pool;
        }
    }
    void* p = nullptr;
    REGOT_CUDA(cudaMallocFromPoolAsync(&p, bytes, pool, st));
    return p;
}

void* ctx_stage(regot_ctx* ctx, size_t bytes) {
    if (bytes > ctx->stage_bytes) {
        if (ctx->stage) REGOT_CUDA(cudaFreeHost(ctx->stage));
        ctx->stage = nullptr;
        ctx->stage_bytes = 0;
        const size_t want = std::max(bytes, (size_t)64 << 10);
        REGOT_CUDA(cudaHostAlloc(&ctx->stage, want, cudaHostAllocPortable));
        ctx->stage_bytes = want;
    }
    return ctx->stage;
}

void read_small(regot_ctx* ctx, void* dst, const void* src, size_t bytes, cudaStream_t st) {
    void* h = ctx_stage(ctx, bytes);
    d2h(h, src, bytes, st);
    sync(st);
    std::memcpy(dst, h, bytes);
}

void finish_erot_result(ErotOps& ops, const double* d_gamma, const double* hobj,
                        const double* hmar, const double* htime, const double* hdens,
                        int hist_len, int hist_cap, int niter, long long passes,
                        const regot_opts& o, regot_result* res) {
    cudaStream_t st = ops.stream();
    const int n = ops.n(), m = ops.m();
    (void)hist_cap;
    res->niter = niter;
    res->hist_len = hist_len;
    res->passes = passes;
    // Dual, histories and the pass error flag in one staging block, behind
    // one synchronisation.
    const size_t nd = (size_t)n + m - 1, L = (size_t)hist_len;
    double* h = static_cast<double*>(ctx_stage(ops.problem()->ctx, (nd + 4 * L + 1) * sizeof(double)));
    double* h_obj = h + nd;
    double* h_mar = h_obj + L;
    double* h_time = h_mar + L;
    double* h_dens = h_time + L;
    int* h_err = reinterpret_cast<int*>(h_dens + L);
    d2h(h, d_gamma, nd * sizeof(double), st);
    d2h(h_obj, hobj, L * sizeof(double), st);
    d2h(h_mar, hmar, L * sizeof(double), st);
    d2h(h_time, htime, L * sizeof(double), st);
    if (hdens) d2h(h_dens, hdens, L * sizeof(double), st);
    d2h(h_err, ops.err_flag(), sizeof(int), st);
    sync(st);
    if (*h_err) throw Error(REGOT_ERR_TIMEOUT, "a dense pass gave up waiting for its tile copies");
    std::memcpy(res->dual, h, nd * sizeof(double));
    if (res->obj_vals) std::memcpy(res->obj_vals, h_obj, L * sizeof(double));
    if (res->mar_errs) std::memcpy(res->mar_errs, h_mar, L * sizeof(double));
    if (res->run_times) std::memcpy(res->run_times, h_time, L * sizeof(double));
    if (res->densities && hdens) std::memcpy(res->densities, h_dens, L * sizeof(double));
    if (o.plan && res->plan) {
        DBuf<double> mx(1, st);
        emit_plan(res->plan, o.plan_mem, (size_t)n * m, st,
                  [&](double* dst) { ops.plan(d_gamma, d_gamma + n, dst, mx.get()); });
    }
    sync(st);
}

}  // namespace regot

namespace {

// Page-locked host blocks for results. cudaHostAlloc of a large block costs
// milliseconds, so freed blocks are kept (up to kPinnedCacheBytes) and handed
// out again to requests of up to their size.
constexpr size_t kPinnedCacheBytes = size_t(4) << 30;
std::mutex g_pinned_mutex;
std::map<void*, size_t> g_pinned_live;  // ordered: host_block_view finds the enclosing block
std::multimap<size_t, void*> g_pinned_free;
size_t g_pinned_free_bytes = 0;

}  // namespace

extern "C" {

int regot_host_alloc(size_t bytes, void** out) {
    if (!out) return REGOT_ERR_INVALID_ARG;
    *out = nullptr;
    if (bytes == 0) bytes = 1;
    std::lock_guard<std::mutex> lock(g_pinned_mutex);
    auto it = g_pinned_free.lower_bound(bytes);
    if (it != g_pinned_free.end() && it->first <= 2 * bytes) {
        *out = it->second;
        g_pinned_live[it->second] = it->first;
        g_pinned_free_bytes -= it->first;
        g_pinned_free.erase(it);
        return REGOT_OK;
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable | cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        return REGOT_ERR_CUDA;
    }
    g_pinned_live[p] = bytes;
    *out = p;
    return REGOT_OK;
}

void regot_host_free(void* ptr) {
    if (!ptr) return;
    std::lock_guard<std::mutex> lock(g_pinned_mutex);
    auto it = g_pinned_live.find(ptr);
    if (it == g_pinned_live.end()) return;
    const size_t bytes = it->second;
    g_pinned_live.erase(it);
    g_pinned_free.emplace(bytes, ptr);
    g_pinned_free_bytes += bytes;
    while (g_pinned_free_bytes > kPinnedCacheBytes && !g_pinned_free.empty()) {
        auto small = g_pinned_free.begin();  // release the smallest blocks first
        cudaFreeHost(small->second);
        g_pinned_free_bytes -= small->first;
        g_pinned_free.erase(small);
    }
}

}  // extern "C"

namespace regot {

void* host_block_view(void* p, size_t bytes) {
    if (!p) return nullptr;
    std::lock_guard<std::mutex> lock(g_pinned_mutex);
    const char* q = static_cast<const char*>(p);
    auto it = g_pinned_live.upper_bound(p);  // first block starting after p
    if (it == g_pinned_live.begin()) return nullptr;
    --it;
    const char* base = static_cast<const char*>(it->first);
    if (q < base || q + bytes > base + it->second) return nullptr;
    void* dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, it->first, 0) != cudaSuccess || !dev) {
        cudaGetLastError();
        return nullptr;
    }
    return static_cast<char*>(dev) + (q - base);
}

}  // namespace regot

extern "C" {

void regot_opts_init(regot_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precision = REGOT_PREC_MIXED;
    o->method = -1;
    o->mu0 = 1.0;
    o->shift = 1e-3;
    o->density = 0.01;
    o->tau = 0.0;
    o->x0 = nullptr;
    o->x0_len = 0;
    o->cg_tol = 1e-10;
    o->cg_max_iter = 0;
    o->verbose = 0;
    o->plan = 1;
    o->plan_mem = REGOT_MEM_HOST;
    o->prim_vals = 1;
}

int regot_ctx_create(int device, regot_ctx** out) {
    if (!out) return REGOT_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return REGOT_ERR_NO_DEVICE;
    if (device < 0 || device >= count) return REGOT_ERR_INVALID_ARG;
    regot_ctx* ctx = new regot_ctx();
    ctx->device = device;
    const int rc = guarded(ctx, [&] {
        REGOT_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
        ctx->stream = ctx->own_stream;
    });
    if (rc != REGOT_OK) {
        delete ctx;
        return rc;
    }
    *out = ctx;
    return REGOT_OK;
}

void regot_ctx_destroy(regot_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->own_stream);
        cudaStreamDestroy(ctx->own_stream);
    }
    if (ctx->stage) cudaFreeHost(ctx->stage);
    delete ctx;
}

const char* regot_ctx_last_error(const regot_ctx* ctx) {
    return ctx ? ctx->last_error.c_str() : "NULL context";
}

int regot_ctx_set_stream(regot_ctx* ctx, void* stream) {
    if (!ctx) return REGOT_ERR_INVALID_ARG;
    ctx->stream = reinterpret_cast<cudaStream_t>(stream);
    return REGOT_OK;
}

void* regot_ctx_own_stream(const regot_ctx* ctx) {
    return ctx ? reinterpret_cast<void*>(ctx->own_stream) : nullptr;
}

long long regot_ctx_kernel_launches(const regot_ctx* ctx) { return ctx ? ctx->launches : 0; }

int regot_problem_create(regot_ctx* ctx, const regot_problem_desc* d, int precision,
                         regot_dproblem** out) {
    return guarded(ctx, [&] {
        require(d != nullptr && out != nullptr, "NULL argument");
        *out = nullptr;
        require(d->n > 0 && d->m > 0, "M must have at least one row and one column");
        require(d->ldm >= d->m, "ldm must be >= m");
        require(d->M && d->a && d->b, "M, a and b must not be NULL");
        require(d->M_dtype == REGOT_F64 || d->M_dtype == REGOT_F32, "unsupported dtype of M");
        require(precision == REGOT_PREC_FP64 || precision == REGOT_PREC_MIXED,
                "unsupported precision");
        cudaStream_t st = ctx->stream;
        const int n = d->n, m = d->m;
        auto* P = new regot_dproblem();
        try {
            P->ctx = ctx;
            P->n = n;
            P->m = m;
            P->prec = precision;
            const size_t es = precision == REGOT_PREC_FP64 ? 8 : 4;
            const long long vw = 16 / (long long)es;
            P->ldm = (m + vw - 1) / vw * vw;
            P->M = dev_alloc((size_t)n * P->ldm * es, st);
            P->a = static_cast<double*>(dev_alloc(n * sizeof(double), st));
            P->b = static_cast<double*>(dev_alloc(m * sizeof(double), st));
            P->ha.resize(n);
            P->hb.resize(m);
            if (d->ab_mem == REGOT_MEM_DEVICE) {
                d2h(P->ha.data(), d->a, n * sizeof(double), st);
                d2h(P->hb.data(), d->b, m * sizeof(double), st);
                sync(st);
            } else {
                std::memcpy(P->ha.data(), d->a, n * sizeof(double));
                std::memcpy(P->hb.data(), d->b, m * sizeof(double));
            }
            for (int i = 0; i < n; ++i)
                require(std::isfinite(P->ha[i]) && P->ha[i] > 0.0,
                        "a must be finite and positive");
            for (int j = 0; j < m; ++j)
                require(std::isfinite(P->hb[j]) && P->hb[j] > 0.0,
                        "b must be finite and positive");
            for (int i = 0; i < n; ++i) P->sum_a += P->ha[i];
            for (int j = 0; j < m - 1; ++j) P->sum_bt += P->hb[j];
            h2d(P->a, P->ha.data(), n * sizeof(double), st);
            h2d(P->b, P->hb.data(), m * sizeof(double), st);

            const size_t src_es = d->M_dtype == REGOT_F64 ? 8 : 4;
            const bool same = src_es == es;
            const cudaMemcpyKind kind =
                d->M_mem == REGOT_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
            if (same) {
                if (P->ldm != m)
                    REGOT_CUDA(cudaMemsetAsync(P->M, 0, (size_t)n * P->ldm * es, st));
                REGOT_CUDA(cudaMemcpy2DAsync(P->M, P->ldm * es, d->M, d->ldm * src_es, m * es, n,
                                             kind, st));
            } else {
                // Stage the source on the device, then convert row by row.
                void* stage = nullptr;
                const void* src = d->M;
                if (d->M_mem != REGOT_MEM_DEVICE) {
                    stage = dev_alloc((size_t)n * m * src_es, st);
                    REGOT_CUDA(cudaMemcpy2DAsync(stage, m * src_es, d->M, d->ldm * src_es,
                                                 m * src_es, n, kind, st));
                    src = stage;
                }
                const long long lds = d->M_mem == REGOT_MEM_DEVICE ? d->ldm : m;
                if (src_es == 8)
                    k_convert<double, float><<<1024, 256, 0, st>>>(
                        (const double*)src, lds, (float*)P->M, P->ldm, n, m);
                else
                    k_convert<float, double><<<1024, 256, 0, st>>>(
                        (const float*)src, lds, (double*)P->M, P->ldm, n, m);
                count_launch();
                REGOT_CHECK_LAUNCH();
                if (stage) REGOT_CUDA(cudaFreeAsync(stage, st));
            }
            // M must be finite in its storage type (an FP64 entry beyond the
            // FP32 range becomes an infinity in mixed storage).
            {
                DBuf<int> flag(1, st);
                flag.zero();
                const long long nvec = (long long)n * P->ldm * (long long)es / 16;
                const int blocks = (int)std::min<long long>(cdiv(nvec, 256), 4LL * device_sm_count());
                if (es == 4) k_nonfinite<float><<<blocks, 256, 0, st>>>(P->M, nvec, flag.get());
                else k_nonfinite<double><<<blocks, 256, 0, st>>>(P->M, nvec, flag.get());
                count_launch();
                REGOT_CHECK_LAUNCH();
                int bad = 0;
                read_small(ctx, &bad, flag.get(), sizeof(int), st);
                require(!bad, precision == REGOT_PREC_MIXED && d->M_dtype == REGOT_F64
                                  ? "M must be finite (and within the FP32 range in mixed precision)"
                                  : "M must be finite");
            }
            sync(st);
        } catch (...) {
            if (P->M) cudaFreeAsync(P->M, st);
            if (P->a) cudaFreeAsync(P->a, st);
            if (P->b) cudaFreeAsync(P->b, st);
            delete P;
            throw;
        }
        *out = P;
    });
}

static void drop_time_pass_state(regot_dproblem* P);

void regot_problem_destroy(regot_dproblem* P) {
    if (!P) return;
    if (P->ctx) cudaSetDevice(P->ctx->device);
    drop_time_pass_state(P);
    cudaStream_t st = P->ctx ? P->ctx->stream : nullptr;
    if (P->M) cudaFreeAsync(P->M, st);
    if (P->a) cudaFreeAsync(P->a, st);
    if (P->b) cudaFreeAsync(P->b, st);
    if (P->loga) cudaFreeAsync(P->loga, st);
    if (P->logb) cudaFreeAsync(P->logb, st);
    cudaStreamSynchronize(st);
    delete P;
}

#define REGOT_SOLVER_ENTRY(NAME, IMPL, DUAL)                                                 \
    int NAME(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,        \
             const regot_opts* opts, regot_result* res) {                                    \
        return guarded(ctx, [&] {                                                            \
            require(P != nullptr, "problem is NULL");                                        \
            check_solver_args(P, reg, tol, max_iter, res, DUAL);                             \
            const regot_opts o = effective_opts(opts);                                       \
            cudaEvent_t e0, e1;                                                              \
            REGOT_CUDA(cudaEventCreate(&e0));                                                \
            REGOT_CUDA(cudaEventCreate(&e1));                                                \
            REGOT_CUDA(cudaEventRecord(e0, ctx->stream));                                    \
            IMPL(ctx, P, reg, tol, max_iter, o, res);                                        \
            REGOT_CUDA(cudaEventRecord(e1, ctx->stream));                                    \
            REGOT_CUDA(cudaEventSynchronize(e1));                                            \
            float ms = 0.f;                                                                  \
            cudaEventElapsedTime(&ms, e0, e1);                                               \
            res->solve_ms = ms;                                                              \
            cudaEventDestroy(e0);                                                            \
            cudaEventDestroy(e1);                                                            \
        });                                                                                  \
    }

REGOT_SOLVER_ENTRY(regot_sinkhorn_bcd, sinkhorn_bcd_gpu, P->n + P->m - 1)
REGOT_SOLVER_ENTRY(regot_sinkhorn_newton, sinkhorn_newton_gpu, P->n + P->m - 1)
REGOT_SOLVER_ENTRY(regot_sinkhorn_ssns, sinkhorn_ssns_gpu, P->n + P->m - 1)
REGOT_SOLVER_ENTRY(regot_sinkhorn_sparse_newton, sinkhorn_sparse_newton_gpu, P->n + P->m - 1)
REGOT_SOLVER_ENTRY(regot_sinkhorn_splr, sinkhorn_splr_gpu, P->n + P->m - 1)
REGOT_SOLVER_ENTRY(regot_sinkhorn_lbfgs_dual, sinkhorn_lbfgs_dual_gpu, P->n + P->m - 1)
REGOT_SOLVER_ENTRY(regot_sinkhorn_apdagd, sinkhorn_apdagd_gpu, P->n + P->m - 1)
REGOT_SOLVER_ENTRY(regot_qrot_lbfgs_dual, qrot_lbfgs_dual_gpu, P->n + P->m)
REGOT_SOLVER_ENTRY(regot_qrot_assn, qrot_assn_gpu, P->n + P->m)
REGOT_SOLVER_ENTRY(regot_qrot_bcd, qrot_bcd_gpu, P->n + P->m)
REGOT_SOLVER_ENTRY(regot_qrot_gd, qrot_gd_gpu, P->n + P->m)
REGOT_SOLVER_ENTRY(regot_qrot_apdagd, qrot_apdagd_gpu, P->n + P->m)
REGOT_SOLVER_ENTRY(regot_qrot_pdaam, qrot_pdaam_gpu, P->n + P->m)
REGOT_SOLVER_ENTRY(regot_qrot_grssn, qrot_grssn_gpu, P->n + P->m)
REGOT_SOLVER_ENTRY(regot_qrot_lbfgs_semi_dual, qrot_lbfgs_semi_dual_gpu, P->n + P->m)

void regot_pdip_opts_init(regot_pdip_opts* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->inner_solver = 0;
    p->cg_max_iter = 1000;
    p->fixed_threshold = 1e-9;
    p->fp_max_iter = 800;
    p->fp_exit_scale = 1e-2;
    p->fp_stop_gap_mu_only = 1;
    p->cg_stop_gap_mu_only = 0;
    p->cg_mar_tol = 1e-10;
}

int regot_qrot_pdip(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                    const regot_pdip_opts* popts, const regot_opts* opts, regot_result* res,
                    int* converged) {
    return guarded(ctx, [&] {
        require(P != nullptr, "problem is NULL");
        require(res != nullptr, "result is NULL");
        require(!std::isnan(reg), "reg must not be NaN");
        require(!std::isnan(tol), "tol must not be NaN");
        require(max_iter >= 0, "max_iter must be non-negative");
        require(res->hist_cap >= max_iter + 2 || (!res->obj_vals && !res->mar_errs &&
                                                  !res->run_times),
                "history capacity must be at least max_iter + 2");
        regot_pdip_opts po;
        regot_pdip_opts_init(&po);
        if (popts) po = *popts;
        const regot_opts o = effective_opts(opts);
        cudaEvent_t e0, e1;
        REGOT_CUDA(cudaEventCreate(&e0));
        REGOT_CUDA(cudaEventCreate(&e1));
        REGOT_CUDA(cudaEventRecord(e0, ctx->stream));
        qrot_pdip_gpu(ctx, P, reg, tol, max_iter, po, o, res, converged);
        REGOT_CUDA(cudaEventRecord(e1, ctx->stream));
        REGOT_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        res->solve_ms = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    });
}

// ---------------------------------------------------------------- passes --

int regot_erot_optimal_beta(regot_ctx* ctx, regot_dproblem* P, double reg, const double* alpha,
                            double* beta) {
    return guarded(ctx, [&] {
        require(P && alpha && beta, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        cudaStream_t st = ctx->stream;
        ErotOps ops(P, reg, st);
        DBuf<double> da(P->n, st), db(P->m, st), mx(1, st);
        h2d(da.get(), alpha, P->n * sizeof(double), st);
        ops.optimal_beta(da.get(), db.get(), mx.get());
        d2h(beta, db.get(), P->m * sizeof(double), st);
        ops.check_err();
    });
}

int regot_erot_optimal_alpha(regot_ctx* ctx, regot_dproblem* P, double reg, const double* beta,
                             double* alpha) {
    return guarded(ctx, [&] {
        require(P && alpha && beta, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        cudaStream_t st = ctx->stream;
        ErotOps ops(P, reg, st);
        DBuf<double> da(P->n, st), db(P->m, st), mx(1, st);
        h2d(db.get(), beta, P->m * sizeof(double), st);
        ops.optimal_alpha(db.get(), da.get(), mx.get());
        d2h(alpha, da.get(), P->n * sizeof(double), st);
        ops.check_err();
    });
}

// Upload gamma = (alpha, beta~) into device alpha[n], beta[m] with beta_m = 0.
static void upload_gamma(const double* gamma, int n, int m, double* d_ab, cudaStream_t st) {
    std::vector<double> h((size_t)n + m, 0.0);
    std::memcpy(h.data(), gamma, (size_t)(n + m - 1) * sizeof(double));
    h2d(d_ab, h.data(), h.size() * sizeof(double), st);
    sync(st);
}

int regot_erot_dual_obj_grad(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                             double* obj, double* grad) {
    return guarded(ctx, [&] {
        require(P && gamma && obj && grad, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        cudaStream_t st = ctx->stream;
        const int n = P->n, m = P->m;
        ErotOps ops(P, reg, st);
        DBuf<double> g(n + m, st), rc(n + m, st), mx(1, st);
        upload_gamma(gamma, n, m, g.get(), st);
        ops.row_col_sums(g.get(), g.get() + n, rc.get(), rc.get() + n, mx.get());
        std::vector<double> h(n + m);
        d2h(h.data(), rc.get(), (n + m) * sizeof(double), st);
        ops.check_err();
        // sinkhorn_problem_obj.cpp:371-393
        double tsum = 0.0, ga = 0.0, gb = 0.0;
        for (int i = 0; i < n; ++i) {
            tsum += h[i];
            grad[i] = h[i] - P->ha[i];
            ga += gamma[i] * P->ha[i];
        }
        for (int j = 0; j < m - 1; ++j) {
            grad[n + j] = h[n + j] - P->hb[j];
            gb += gamma[n + j] * P->hb[j];
        }
        *obj = reg * tsum - ga - gb;
    });
}

int regot_erot_hvp(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                   const double* x, double* y) {
    return guarded(ctx, [&] {
        require(P && gamma && x && y, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        cudaStream_t st = ctx->stream;
        const int n = P->n, m = P->m;
        ErotOps ops(P, reg, st);
        DBuf<double> g(n + m, st), xv(n + m, st), rc(n + m, st), yy(n + m, st), mx(1, st);
        upload_gamma(gamma, n, m, g.get(), st);
        upload_gamma(x, n, m, xv.get(), st);
        ops.row_col_sums(g.get(), g.get() + n, rc.get(), rc.get() + n, mx.get());
        ops.tmatvec(g.get(), g.get() + n, xv.get(), xv.get() + n, yy.get(), yy.get() + n,
                    mx.get());
        std::vector<double> hrc(n + m), hy(n + m);
        d2h(hrc.data(), rc.get(), (n + m) * sizeof(double), st);
        d2h(hy.data(), yy.get(), (n + m) * sizeof(double), st);
        ops.check_err();
        for (int i = 0; i < n; ++i) y[i] = (hrc[i] * x[i] + hy[i]) / reg;
        for (int j = 0; j < m - 1; ++j) y[n + j] = (hrc[n + j] * x[n + j] + hy[n + j]) / reg;
    });
}

int regot_erot_solve_batched(regot_ctx* ctx, const regot_batch_desc* desc, double reg, double tol,
                             int max_iter, regot_batch_result* res) {
    return regot_erot_solve_batched_grad(ctx, desc, reg, tol, max_iter, res, nullptr, nullptr,
                                         nullptr);
}

int regot_erot_solve_batched_grad(regot_ctx* ctx, const regot_batch_desc* desc, double reg,
                                  double tol, int max_iter, regot_batch_result* res, double* cost,
                                  float* grad_x, float* grad_y) {
    return guarded(ctx, [&] {
        require(desc && res, "NULL argument");
        require(desc->count > 0, "the batch is empty");
        require(desc->n && desc->m && desc->d && desc->x && desc->y && desc->a && desc->b,
                "NULL array in the batch description");
        require(desc->mem == REGOT_MEM_HOST || desc->mem == REGOT_MEM_DEVICE,
                "unknown memory kind");
        require(std::isfinite(reg) && reg > 0.0, "reg must be a positive finite number");
        require(!std::isnan(tol), "tol must not be NaN");
        require(max_iter >= 0, "max_iter must be non-negative");
        erot_solve_batched_gpu(ctx, desc, reg, tol, max_iter, res, cost, grad_x, grad_y);
    });
}

int regot_erot_hess_solve(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                          const double* rhs, double tol, int max_iter, double* x, int* iters) {
    return guarded(ctx, [&] {
        require(P && gamma && rhs && x, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        require(tol >= 0.0, "tol must be non-negative");
        erot_hess_solve_gpu(ctx, P, reg, gamma, rhs, tol, max_iter, x, iters);
    });
}

static void erot_contract_entry(regot_ctx* ctx, regot_dproblem* P, double reg,
                                const double* gamma, const double* u, const double* W,
                                const double* Y, int d, double* sums, double* Z, int mem,
                                bool cols) {
    require(P && gamma, "NULL argument");
    require(reg > 0.0, "reg must be positive");
    require(d >= 0 && (d == 0 || (Y && Z)), "Y and Z are required when d > 0");
    require(mem == REGOT_MEM_HOST || mem == REGOT_MEM_DEVICE, "unknown memory kind");
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m;
    const int nown = cols ? m : n, K = cols ? n : m;
    const size_t nm1 = (size_t)(n + m - 1) * sizeof(double);
    // duals and adjoint with beta_m = 0 appended, on the device
    DBuf<double> g(n + m, st), uu(u ? n + m : 0, st);
    g.zero();
    const cudaMemcpyKind kin = mem == REGOT_MEM_HOST ? cudaMemcpyHostToDevice
                                                     : cudaMemcpyDeviceToDevice;
    REGOT_CUDA(cudaMemcpyAsync(g.get(), gamma, nm1, kin, st));
    if (u) {
        uu.zero();
        REGOT_CUDA(cudaMemcpyAsync(uu.get(), u, nm1, kin, st));
    }
    const double *dW = W, *dY = Y;
    DBuf<double> hW, hY, hZ, hS;
    double *dZ = Z, *dS = sums;
    if (mem == REGOT_MEM_HOST) {
        if (W) {
            hW.alloc((size_t)n * m, st);
            h2d(hW.get(), W, (size_t)n * m * sizeof(double), st);
            dW = hW.get();
        }
        if (d > 0) {
            hY.alloc((size_t)K * d, st);
            h2d(hY.get(), Y, (size_t)K * d * sizeof(double), st);
            dY = hY.get();
            hZ.alloc((size_t)nown * d, st);
            dZ = hZ.get();
        }
        if (sums) {
            hS.alloc(nown, st);
            dS = hS.get();
        }
    }
    erot_contract_gpu(ctx, P, reg, g.get(), u ? uu.get() : nullptr, dW, d > 0 ? dY : nullptr, d,
                      cols, dS, d > 0 ? dZ : nullptr);
    if (mem == REGOT_MEM_HOST) {
        if (d > 0) d2h(Z, dZ, (size_t)nown * d * sizeof(double), st);
        if (sums) d2h(sums, dS, (size_t)nown * sizeof(double), st);
    }
    sync(st);
}

int regot_erot_tyy(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                   const double* u, const double* W, const double* Y, int d, double* rows,
                   double* Z, int mem) {
    return guarded(ctx, [&] {
        erot_contract_entry(ctx, P, reg, gamma, u, W, Y, d, rows, Z, mem, false);
    });
}

int regot_sqeuclid_cost(regot_ctx* ctx, const void* x, const void* y, int n, int m, int d,
                        double scale, int dtype, void* M, long long ldm) {
    return guarded(ctx, [&] {
        require(x && y && M, "NULL argument");
        require(n > 0 && m > 0 && d > 0 && ldm >= m, "invalid sizes");
        require(dtype == REGOT_F32 || dtype == REGOT_F64, "unsupported dtype");
        require(std::isfinite(scale), "scale must be finite");
        sqeuclid_gpu(x, y, n, m, d, scale, dtype == REGOT_F64, M, ldm, ctx->stream);
    });
}

int regot_erot_tty(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                   const double* u, const double* W, const double* X, int d, double* cols,
                   double* Z, int mem) {
    return guarded(ctx, [&] {
        erot_contract_entry(ctx, P, reg, gamma, u, W, X, d, cols, Z, mem, true);
    });
}

int regot_erot_plan(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                    double* plan, int plan_mem) {
    return guarded(ctx, [&] {
        require(P && gamma && plan, "NULL argument");
        cudaStream_t st = ctx->stream;
        const int n = P->n, m = P->m;
        ErotOps ops(P, reg, st);
        DBuf<double> g(n + m, st), mx(1, st);
        upload_gamma(gamma, n, m, g.get(), st);
        emit_plan(plan, plan_mem, (size_t)n * m, st,
                  [&](double* dst) { ops.plan(g.get(), g.get() + n, dst, mx.get()); });
        sync(st);
    });
}

int regot_erot_sparsify(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma,
                        double delta, double density_hint, long long* nnz, int* mask) {
    return guarded(ctx, [&] {
        require(P && gamma && nnz, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        require(delta >= 0.0, "delta must be non-negative");
        erot_sparsify_gpu(ctx, P, reg, gamma, delta, density_hint, nnz, mask);
    });
}

int regot_erot_sparsify_density(regot_ctx* ctx, regot_dproblem* P, double reg,
                                const double* gamma, double density, long long* nnz, int* mask) {
    return guarded(ctx, [&] {
        require(P && gamma && nnz, "NULL argument");
        require(reg > 0.0, "reg must be positive");
        erot_sparsify_density_gpu(ctx, P, reg, gamma, density, nnz, mask);
    });
}

}  // extern "C"

// ------------------------------------------------------------ measurement --
namespace {
struct TimePassState {
    regot_dproblem* P = nullptr;
    double reg = 0.0;
    cudaStream_t stream = nullptr;
    ErotOps* ops = nullptr;
    DBuf<double> vec, mx, plan;
    DBuf<char> xavg;
    DBuf<uint32_t> bitmask;
    int prepared_op = -1;  // pass whose inputs (split) are in place
};
TimePassState* g_tp = nullptr;

// Pass kinds of regot_time_pass, in the order of the REGOT_PASS_* enum.
constexpr int kTimedOps[REGOT_PASS_COUNT] = {
    OP_E_ROW, OP_E_COL, OP_E_ROWCOL, OP_E_HVP, OP_Q_GRAD, OP_E_LS, OP_E_GRADLS, OP_E_AVG,
    OP_E_PLAN, OP_E_ROWMAX, OP_E_COLMAX, OP_Q_GRADMASK, OP_Q_GRADLS, OP_Q_OBJ, OP_Q_P1,
    OP_Q_P2, OP_Q_P3, OP_Q_COLROOT, OP_Q_ROWROOT, OP_Q_AVG, OP_Q_PLAN};

// Deterministic pass inputs: duals (0.1 for the QROT passes, so that a part
// of the entries is positive; 0 for EROT), weights and directions of a few
// hundredths, as in the solvers' late iterations.
__global__ void k_time_pass_inputs(double* v, int n, int m, bool qrot) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int len = 4 * (n + m);
    if (t >= len) return;
    const int block = t / (n + m);  // 0: ra|cb, 1: rx|cx, 2: cx2 (cols), 3: rd|cd
    const int k = t % (n + m);
    double x = 0.0;
    if (block == 0) x = qrot ? 0.1 : 0.0;
    else x = 0.01 * (1 + (k * 7919) % 5) * (block == 3 ? 0.1 : 1.0);
    v[t] = x;
}
}  // namespace

static void drop_time_pass_state(regot_dproblem* P) {
    if (g_tp && g_tp->P == P) {
        delete g_tp->ops;
        delete g_tp;
        g_tp = nullptr;
    }
}

extern "C" long long regot_set_wait_limit(long long spins) { return set_wait_limit(spins); }

extern "C" int regot_force_pass_config(int cfg) { return force_pass_config(cfg); }

extern "C" int regot_force_batch_variant(int variant) { return force_batch_variant(variant); }
extern "C" int regot_set_batch_tail(int max_active) { return set_batch_tail(max_active); }
extern "C" int regot_force_sparsify_path(int shared_memory) {
    return force_sparsify_path(shared_memory);
}
extern "C" int regot_force_qrot_cg_path(int mode) { return force_qrot_cg_path(mode); }

extern "C" int regot_batch_variants(regot_ctx* ctx, int* out) {
    return guarded(ctx, [&] {
        require(out != nullptr, "NULL argument");
        const std::vector<int> v = batch_variants();
        for (size_t c = 0; c < v.size(); ++c) out[c] = v[c];
    });
}

extern "C" int regot_pass_config(regot_ctx* ctx, int kind, int precision, int n, int m) {
    int cfg = -1;
    const int rc = guarded(ctx, [&] {
        require(kind >= 0 && kind < REGOT_PASS_COUNT, "unknown pass kind");
        require(n > 0 && m > 0, "invalid sizes");
        cfg = pass_config(kTimedOps[kind], precision == REGOT_PREC_MIXED, n, m);
    });
    return rc == REGOT_OK ? cfg : -1;
}

extern "C" int regot_autotune_save(const char* path) {
    if (path == nullptr || *path == '\0') {
        // the default location: create its directory
        if (const char* h = std::getenv("HOME")) {
            if (!std::getenv("REGOT_GB300_AUTOTUNE"))
                mkdir((std::string(h) + "/.cache").c_str(), 0755);
        }
    }
    return save_tuning(path);
}
extern "C" int regot_autotune_load(const char* path) { return load_tuning(path); }
extern "C" void regot_autotune_clear(void) { clear_tuning(); }
extern "C" size_t regot_autotune_entries(char* buf, size_t len) {
    const std::string s = tuning_entries();
    if (buf && len) {
        const size_t k = std::min(len - 1, s.size());
        std::memcpy(buf, s.data(), k);
        buf[k] = '\0';
    }
    return s.size();
}

extern "C" int regot_autotune(regot_ctx* ctx, int n, int m, int precision, int reps) {
    int rc = guarded(ctx, [&] {
        require(n > 0 && m > 1, "invalid sizes");
        require(precision == REGOT_PREC_FP64 || precision == REGOT_PREC_MIXED,
                "unsupported precision");
        require(reps > 0, "reps must be positive");
    });
    if (rc != REGOT_OK) return rc;
    // A synthetic problem of the size: M uniform on [0, 1), uniform marginals.
    std::vector<float> M((size_t)n * m);
    unsigned long long x = 0x9E3779B97F4A7C15ULL;
    for (auto& v : M) {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        v = (float)((x >> 40) * (1.0 / (1ULL << 24)));
    }
    std::vector<double> a(n, 1.0 / n), b(m, 1.0 / m);
    regot_problem_desc d{};
    d.M = M.data();
    d.M_dtype = REGOT_F32;
    d.M_mem = REGOT_MEM_HOST;
    d.ldm = m;
    d.n = n;
    d.m = m;
    d.a = a.data();
    d.b = b.data();
    d.ab_mem = REGOT_MEM_HOST;
    regot_dproblem* P = nullptr;
    rc = regot_problem_create(ctx, &d, precision, &P);
    if (rc != REGOT_OK) return rc;
    const int prev = force_pass_config(-1);
    rc = guarded(ctx, [&] {
        cudaStream_t st = ctx->stream;
        cudaEvent_t e0, e1;
        REGOT_CUDA(cudaEventCreate(&e0));
        REGOT_CUDA(cudaEventCreate(&e1));
        const double reg = 0.01;
        try {
            for (int kind = 0; kind < REGOT_PASS_COUNT; ++kind) {
                double us[kPassConfigs];
                for (int cfg = 0; cfg < kPassConfigs; ++cfg) {
                    force_pass_config(cfg);
                    int r = regot_time_pass(ctx, P, kind, reg, 1);  // prepares, warms
                    if (r != REGOT_OK) throw Error(r, ctx->last_error);
                    sync(st);
                    REGOT_CUDA(cudaEventRecord(e0, st));
                    r = regot_time_pass(ctx, P, kind, reg, reps);
                    if (r != REGOT_OK) throw Error(r, ctx->last_error);
                    REGOT_CUDA(cudaEventRecord(e1, st));
                    REGOT_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    REGOT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    us[cfg] = 1e3 * ms / reps;
                }
                int best = 0;
                for (int cfg = 1; cfg < kPassConfigs; ++cfg)
                    if (us[cfg] < us[best]) best = cfg;
                record_tuning(kTimedOps[kind], precision == REGOT_PREC_MIXED, n, m, best, us);
            }
        } catch (...) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    });
    force_pass_config(prev);
    regot_problem_destroy(P);
    return rc;
}

extern "C" long long regot_pass_bytes(regot_dproblem* P, int kind) {
    if (!P || kind < 0 || kind >= REGOT_PASS_COUNT) return -1;
    const long long nm = (long long)P->n * P->m;
    const long long es = P->prec == REGOT_PREC_MIXED ? 4 : 8;
    const int op = kTimedOps[kind];
    long long bytes = nm * es;  // one read of M
    if (op == OP_E_PLAN || op == OP_Q_PLAN) bytes += nm * 8;  // FP64 plan written
    if (op == OP_E_AVG || op == OP_Q_AVG) bytes += 2 * nm * es;  // averaged plan read + written
    if (op == OP_Q_GRADMASK) bytes += nm / 8;  // bitmask written
    return bytes;
}

extern "C" int regot_time_pass(regot_ctx* ctx, regot_dproblem* P, int kind, double reg,
                               int reps) {
    return guarded(ctx, [&] {
        require(P != nullptr && reps >= 0, "invalid argument");
        require(kind >= 0 && kind < REGOT_PASS_COUNT, "unknown pass kind");
        require(reg > 0.0 && std::isfinite(reg), "reg must be a positive finite number");
        cudaStream_t st = ctx->stream;
        const int n = P->n, m = P->m;
        const int op = kTimedOps[kind];
        const bool qrot = op >= OP_Q_GRAD && op != OP_E_GRADLS && op != OP_E_AVG;
        // Workspace kept between calls for the same problem (the timed region
        // should contain the passes only).
        if (!g_tp || g_tp->P != P || g_tp->reg != reg || g_tp->stream != st) {
            if (g_tp) {
                delete g_tp->ops;
                delete g_tp;
            }
            g_tp = new TimePassState();
            g_tp->P = P;
            g_tp->reg = reg;
            g_tp->stream = st;
            g_tp->ops = new ErotOps(P, reg, st);
            g_tp->vec.alloc(4 * ((size_t)n + m), st);
            g_tp->mx.alloc(1, st);
            sync(st);
        }
        ErotOps& ops = *g_tp->ops;
        if (g_tp->prepared_op != op) {
            double* v = g_tp->vec.get();
            k_time_pass_inputs<<<cdiv(4LL * (n + m), 256), 256, 0, st>>>(v, n, m, qrot);
            count_launch();
            REGOT_CHECK_LAUNCH();
            ops.maxabs(v, n + m, nullptr, 0, g_tp->mx.get());
            const size_t es = P->prec == REGOT_PREC_MIXED ? 4 : 8;
            if ((op == OP_E_PLAN || op == OP_Q_PLAN) && !g_tp->plan.get())
                g_tp->plan.alloc((size_t)n * m, st);
            if ((op == OP_E_AVG || op == OP_Q_AVG) && !g_tp->xavg.get()) {
                g_tp->xavg.alloc((size_t)n * m * es, st);
                g_tp->xavg.zero();
            }
            if (op == OP_Q_GRADMASK && !g_tp->bitmask.get()) {
                const PassShape sh = P->prec == REGOT_PREC_MIXED ? pass_shape<float>(n, m)
                                                                 : pass_shape<double>(n, m);
                const int lc = P->prec == REGOT_PREC_MIXED ? Geo<float>::LC : Geo<double>::LC;
                g_tp->bitmask.alloc((size_t)n * sh.nslabs * lc, st);
            }
        }
        double* v = g_tp->vec.get();
        PassParams p = ops.base_params();
        p.ra = v;
        p.cb = v + n;
        p.rx = v + (n + m);
        p.cx = v + (n + m) + n;
        p.cx2 = v + 2 * (n + m) + n;
        p.rd = v + 3 * (n + m);
        p.cd = v + 3 * (n + m) + n;
        p.grid = g_tp->mx.get();
        p.out = g_tp->plan.get();
        p.xavg = g_tp->xavg.get();
        p.bitmask = g_tp->bitmask.get();
        if (op == OP_E_LS) {
            const double s4[4] = {1.0, 0.5, 0.25, 0.1};
            for (int k = 0; k < 4; ++k) p.steps[k] = s4[k];
            p.nsteps = 4;
        } else if (op == OP_E_GRADLS || op == OP_Q_GRADLS) {
            p.steps[0] = 0.5;
            p.nsteps = 1;
        } else if (op == OP_E_AVG) {
            p.steps[0] = 0.1;
            p.nsteps = 1;  // X read and written (an APDAGD iteration after the first)
        } else if (op == OP_Q_AVG) {
            p.steps[0] = 0.9;
            p.steps[1] = 0.1;
            p.nsteps = 1;
        }
        if (g_tp->prepared_op != op) {
            // split once (mixed), run the pass once, then time the dense
            // kernel alone on later calls
            ops.pass(op, p);
            sync(st);
            g_tp->prepared_op = op;
        }
        for (int r = 0; r < reps; ++r) {
            if (P->prec == REGOT_PREC_MIXED) ops.pass_presplit(op, p);
            else ops.pass(op, p);
        }
    });
}
