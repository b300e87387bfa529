// sinkhorn_bcd on the GPU (reference: src/sinkhorn_bcd.cpp:14-124).
//
// One BCD iteration is two streamed passes over M:
//   K1 (row pass, anchor alpha_k):  S_i = sum_j exp((alpha_k,i + beta_k,j - M_ij)/reg)
//        S_i is the row marginal of iterate k, so the gradient, objective and
//        marginal error of iterate k come out of this pass, and
//        alpha_{k+1,i} = alpha_k,i + reg (log a_i - log S_i).
//   K2 (column pass, anchor beta_k): S_j = sum_i exp((alpha_{k+1,i} + beta_k,j - M_ij)/reg)
//        beta_{k+1,j} = beta_k,j + reg (log b_j - log S_j).
// After K2 the column marginals are exact, so the beta part of the gradient
// of the next iterate is zero up to rounding, as in the reference
// (optimal_beta runs last in each sweep). The anchors keep every exponent of
// the passes <= 0 (T <= a_i or b_j <= 1), which makes the FP32 exp safe; a
// row or column sum that still leaves the safe range is redone with an
// explicit max anchor (robust path) without changing the result.
//
// The iteration is captured once in a CUDA graph and replayed in batches;
// every kernel returns immediately once the device-side `done` flag is set,
// so the host only synchronises once per batch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "solvers.h"

namespace regot {

namespace {

// Finalize kernels: (32, 8) blocks, 32 rows (columns) per block with their
// partials merged by 8 threads each (merge_2d), so the merge is not bound by
// the latency of one thread's dependent loads. After the merge only warp 0
// continues: the dual update, the split, the max-abs (integer) and the grid
// sums (warp_grid_reduce) need one thread per row or column, and keeping
// FP64 instructions to that one warp matters on a part whose FP64 rate is a
// small fraction of its FP32 rate.
constexpr int kFinItems = 32;
const dim3 kFinBlock(32, 8);

struct BcdState {
    int done;
    int bad;       // 1: row sums out of range, 2: column sums out of range
    int iter;      // index of the iterate whose gradient the next K1 evaluates
    int niter;
    int hist_len;
    int max_iter;
    unsigned counter;
    int loops;     // bodies of the device-side sweep loop run so far
    int loop_cap;  // hard bound on loops (the loop kernel stops there)
    int pad;
    double tol;
    double sum_bb;     // sum_{j<m-1} b_j beta_j of the current beta
    double beta_last;  // beta_{m-1}
    double gb2_once;   // squared beta-part of the gradient of iterate 0 (x0 given)
    double maxabs;     // running max |alpha|, |beta| (hi/lo split grid)
    double last_gnorm; // marginal error of the last recorded iterate
    // Fixed hi/lo grid of the ping-pong sweeps (k_bcd_init): the split value
    // handed to k_split, the grid g and 1/g, and the bound on |dual| that
    // keeps hi exact on g.
    double gval, sg, sinv, sbound;
    unsigned long long t0;
};

template <bool MIXED>
__device__ __forceinline__ bool sum_ok(double s) {
    return isfinite(s) && s > (MIXED ? 1e-30 : 1e-290);
}

// Fixed hi/lo grid of the ping-pong sweeps: the finalize kernels write the
// FP32 split of the duals they produce, for the next pass, on the grid kept
// in BcdState.
struct SplitOut {
    float4* out = nullptr;  // null: no split written
};

__device__ __forceinline__ float4 split_fixed(double v, const BcdState* st) {
    const double h = rint(v * st->sinv) * st->sg;
    return make_float4((float)h, (float)(v - h), 0.f, 0.f);
}

// Start of the sweeps, after the initial value (sinkhorn_bcd.cpp:49-51): the
// timer, sum_{j<m-1} b_j beta_j and beta_{m-1}, max |alpha|, |beta|, and
// from it the grid of the ping-pong sweeps, g = 2^(e + 3 - 21) with
// e = ilogb(max), i.e. 8x headroom. st->maxabs is zero on entry.
__global__ void k_bcd_init(const double* b, const double* alpha, int n, const double* beta,
                           int m, double* parts, BcdState* st) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    if (gt == 0) st->t0 = globaltimer_ns();
    double v[1] = {0.0};
    unsigned long long mb = 0ULL;
    for (int j = gt; j < m - 1; j += gs) v[0] += b[j] * beta[j];
    for (int t = gt; t < n + m; t += gs) {
        const unsigned long long q = abs_bits(t < n ? alpha[t] : beta[t - n]);
        mb = q > mb ? q : mb;
    }
    block_atomic_max_bits(&st->maxabs, mb);
    __threadfence();
    double out[1];
    if (grid_reduce<1>(v, parts, &st->counter, out)) {
        st->sum_bb = out[0];
        st->beta_last = __ldcg(&beta[m - 1]);
        const double m0 =
            __longlong_as_double((long long)atomicAdd(reinterpret_cast<unsigned long long*>(&st->maxabs), 0ULL));
        const int e = (m0 > 0.0 && isfinite(m0)) ? ilogb(m0) : 0;
        st->gval = ldexp(1.0, e + 3);
        st->sg = ldexp(1.0, e + 3 - 21);
        st->sinv = ldexp(1.0, -(e + 3 - 21));
        st->sbound = ldexp(1.0, e + 4);
    }
}

// Condition of the device-side sweep loop (the last node of its body, run
// on every pass through it): continue while not done and no hand-over is
// pending, and never beyond loop_cap bodies, so the loop ends even if no
// other kernel of the body ran.
__global__ void k_bcd_loop(BcdState* st, cudaGraphConditionalHandle h) {
    const int loops = ++st->loops;
    const bool go = !st->done && !st->bad && loops < st->loop_cap;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

// Graph and executable graph of the sweep loop, destroyed on every exit.
struct LoopGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~LoopGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

// Row finalize of K1: gradient/objective of iterate k, history, stopping
// test, alpha_{k+1}. `anchor` is the row vector the pass used (alpha itself
// on the fast path, -max_j(beta_j - M_ij) on the robust path).
template <typename Acc, bool MIXED>
__global__ void k_bcd_row(const Acc* rp, int nslabs, int n, const double* anchor,
                          const double* alpha, const double* a, const double* loga, double reg,
                          double sum_a, double sum_bt, double* alpha_next, double* hobj,
                          double* hmar, double* htime, double* parts, BcdState* st,
                          int robust, SplitOut so) {
    if (st->done) return;
    const int i = blockIdx.x * kFinItems + threadIdx.x;
    const double S = merge_2d(rp + i, nslabs, (size_t)n, i < n);
    if (threadIdx.y != 0) return;  // the rest runs in warp 0 only
    double v[3] = {0.0, 0.0, 0.0};
    double vmax = 0.0;
    if (i < n) {
        const double al = alpha[i];
        const double an = anchor[i];
        if (!robust && !sum_ok<MIXED>(S)) atomicOr(&st->bad, 1);
        const double r = robust ? exp(log(S) + (al - an) / reg) : S;
        const double g = r - a[i];
        v[0] = g * g;
        v[1] = r;
        v[2] = a[i] * al;
        const double an_next = an + reg * (loga[i] - log(S));
        alpha_next[i] = an_next;
        vmax = an_next;
        if (so.out) {
            if (!(fabs(an_next) < st->sbound)) atomicOr(&st->bad, 4);
            so.out[i] = split_fixed(an_next, st);
        }
    }
    warp_atomic_max_abs(&st->maxabs, vmax);
    __threadfence();
    double out[3];
    if (warp_grid_reduce<3>(v, parts, &st->counter, out) && threadIdx.x == 0) {
        if (atomicAdd(&st->bad, 0)) {
            st->done = 1;
            return;
        }
        const int k = st->iter;
        const double gnorm = sqrt(out[0] + st->gb2_once);
        st->gb2_once = 0.0;
        const double bl = st->beta_last;
        const double obj = reg * out[1] - out[2] - bl * sum_a - st->sum_bb + bl * sum_bt;
        hobj[k] = obj;
        hmar[k] = gnorm;
        st->last_gnorm = gnorm;
        htime[k] = (double)(globaltimer_ns() - st->t0) * 1e-6;
        st->hist_len = k + 1;
        if (gnorm < st->tol || k >= st->max_iter) {
            st->done = 1;
            st->niter = k;
        }
    }
}

// Column finalize of K2: beta_{k+1} into beta_next.
template <typename Acc, bool MIXED>
__global__ void k_bcd_col(const Acc* cp, int nrb, int m, const double* anchor,
                          const double* logb, const double* b, double reg, double* beta_next,
                          double* parts, BcdState* st, int robust, SplitOut so, int advance) {
    if (st->done) return;
    const int j = blockIdx.x * kFinItems + threadIdx.x;
    const double S = merge_2d(cp + j, nrb, (size_t)m, j < m);
    if (threadIdx.y != 0) return;  // the rest runs in warp 0 only
    double v[1] = {0.0};
    double vmax = 0.0;
    if (j < m) {
        if (!robust && !sum_ok<MIXED>(S)) atomicOr(&st->bad, 2);
        const double bn = anchor[j] + reg * (logb[j] - log(S));
        beta_next[j] = bn;
        if (j < m - 1) v[0] = b[j] * bn;
        vmax = bn;
        if (so.out) {
            if (!(fabs(bn) < st->sbound)) atomicOr(&st->bad, 8);
            so.out[j] = split_fixed(bn, st);
        }
    }
    warp_atomic_max_abs(&st->maxabs, vmax);
    __threadfence();
    double out[1];
    if (warp_grid_reduce<1>(v, parts, &st->counter, out) && threadIdx.x == 0) {
        if (atomicAdd(&st->bad, 0)) {
            st->done = 1;
            return;
        }
        st->sum_bb = out[0];
        st->beta_last = __ldcg(&beta_next[m - 1]);
        if (advance) st->iter += 1;
    }
}

// Commit the sweep: alpha <- alpha_next, beta <- beta_next, iter++.
__global__ void k_bcd_commit(int n, int m, double* alpha, const double* alpha_next, double* beta,
                             const double* beta_next, BcdState* st) {
    if (st->done) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) alpha[t] = alpha_next[t];
    if (t < m) beta[t] = beta_next[t];
    if (t == 0) st->iter += 1;
}

__global__ void k_gauge(int n, int m, const double* alpha, const double* beta, double* ga,
                        double* gb) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const double bl = beta[m - 1];
    if (t < n) ga[t] = alpha[t] + bl;
    if (t < m) gb[t] = (t < m - 1) ? beta[t] - bl : 0.0;
}

__global__ void k_colgrad_sq(const double* c, const double* b, int m, double* out) {
    double v = 0.0;
    for (int j = threadIdx.x; j < m - 1; j += blockDim.x) {
        const double g = c[j] - b[j];
        v += g * g;
    }
    __shared__ double s[32];
    v = warp_sum_d(v);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        *out = t;
    }
}

}  // namespace

void sinkhorn_bcd_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                      const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    ErotOps ops(P, reg, st);
    const PassShape sh = ops.buf().shape;
    const int hist_cap = max_iter + 2;

    DBuf<double> alpha(n, st), alpha_next(n, st), beta(m, st), beta_next(m, st), anchor(
        std::max(n, m), st);
    DBuf<double> hist(3 * (size_t)hist_cap, st), parts(3 * (size_t)cdiv(std::max(n, m), kFinItems), st);
    DBuf<double> scratch(std::max(n, m) + 8, st), rsum(n, st), csum(m, st);
    DBuf<BcdState> dst(1, st);
    double* hobj = hist.get();
    double* hmar = hobj + hist_cap;
    double* htime = hmar + hist_cap;

    BcdState h0{};
    h0.max_iter = max_iter;
    h0.tol = tol;
    // two sweeps per body of the device-side loop; iterate max_iter always
    // stops it, this bound only guards the loop itself
    h0.loop_cap = max_iter / 2 + 3;
    h2d(dst.get(), &h0, sizeof(h0), st);
    BcdState* S = dst.get();
    double* mx = scratch.get();

    // Initial value (sinkhorn_bcd.cpp:38-47).
    const bool has_x0 = o.x0 && o.x0_len == n + m - 1;
    if (has_x0) {
        std::vector<double> hb(m, 0.0);
        std::copy(o.x0 + n, o.x0 + n + m - 1, hb.begin());
        h2d(alpha.get(), o.x0, n * sizeof(double), st);
        h2d(beta.get(), hb.data(), m * sizeof(double), st);
    } else {
        alpha.zero();
        ops.optimal_beta(alpha.get(), beta.get(), mx);
    }
    // Timer starts after the initial value (sinkhorn_bcd.cpp:49-51).
    k_bcd_init<<<std::min(cdiv((long long)n + m, 256), 64), 256, 0, st>>>(
        P->b, alpha.get(), n, beta.get(), m, parts.get(), S);
    count_launch();
    if (has_x0) {
        // With a user x0 the beta part of the first gradient is not zero.
        ops.row_col_sums(alpha.get(), beta.get(), rsum.get(), csum.get(), mx);
        k_colgrad_sq<<<1, 256, 0, st>>>(csum.get(), P->b, m, &S->gb2_once);
        count_launch();
    }
    REGOT_CHECK_LAUNCH();

    BcdState hs{};
    auto read_state = [&]() {
        read_small(ctx, &hs, S, sizeof(hs), st);
    };
    // Size the next batch of sweeps from the observed linear convergence
    // rate, so that few sweeps are launched past convergence.
    int prev_iter = -1;
    double prev_g = 0.0;
    auto next_batch = [&](int batch) {
        const int k = hs.hist_len - 1;
        int next = std::min(batch * 2, 64);
        if (prev_iter >= 0 && k > prev_iter && hs.last_gnorm > 0.0 && prev_g > hs.last_gnorm) {
            const double rate = std::log(prev_g / hs.last_gnorm) / (k - prev_iter);
            const double need = std::log(hs.last_gnorm / std::max(tol, 1e-300)) / rate;
            if (std::isfinite(need)) next = (int)std::ceil(need) + 1;
        }
        prev_iter = k;
        prev_g = hs.last_gnorm;
        return std::max(1, std::min(next, std::min(64, max_iter + 1 - k)));
    };
    const int gn = cdiv(n, kFinItems), gm = cdiv(m, kFinItems), gnm = cdiv(std::max(n, m), 256);

    // ---- ping-pong path: 4 kernels per sweep ----
    // The duals alternate between (alpha, beta) for even iterates and
    // (alpha_next, beta_next) for odd ones, so no commit kernel is needed, and
    // the finalize kernels write the FP32 hi/lo split of the duals they
    // produce on a grid fixed for the solve (8x headroom over the initial
    // duals), so no split kernel runs before the passes either. A dual that
    // outgrows the grid, or a sum out of range, hands the solve over to the
    // general path below, which re-splits before every pass.
    int pending = 0;  // robust column half-sweep owed to the general path
    bool finished = false;
    {
        // The grid comes from the initial duals on the device, so the graph
        // below is captured while the initialisation still runs.
        float4* rs = const_cast<float4*>(ops.rsplit());
        float4* cs = const_cast<float4*>(ops.csplit());
        SplitOut so_r, so_c;
        if (mixed) {
            PassParams q = ops.base_params();
            q.ra = alpha.get();
            q.cb = beta.get();
            q.grid = &S->gval;
            launch_split(q, rs, cs, nullptr, st);
            so_r.out = rs;
            so_c.out = cs;
        }
        double* A[2] = {alpha.get(), alpha_next.get()};
        double* B[2] = {beta.get(), beta_next.get()};
        auto half_sweeps = [&](int q) {
            PassParams pr = ops.base_params();
            pr.done = &S->done;
            pr.ra = A[q];
            pr.cb = B[q];
            ops.pass_presplit(OP_E_ROW, pr);
            if (mixed)
                k_bcd_row<float, true><<<gn, kFinBlock, 0, st>>>(
                    (const float*)ops.buf().rowpart.get(), sh.nslabs, n, A[q], A[q], P->a,
                    ops.loga(), reg, ops.sum_a(), ops.sum_bt(), A[1 - q], hobj, hmar, htime,
                    parts.get(), S, 0, so_r);
            else
                k_bcd_row<double, false><<<gn, kFinBlock, 0, st>>>(
                    (const double*)ops.buf().rowpart.get(), sh.nslabs, n, A[q], A[q], P->a,
                    ops.loga(), reg, ops.sum_a(), ops.sum_bt(), A[1 - q], hobj, hmar, htime,
                    parts.get(), S, 0, so_r);
            PassParams pc = pr;
            pc.ra = A[1 - q];
            pc.cb = B[q];
            ops.pass_presplit(OP_E_COL, pc);
            if (mixed)
                k_bcd_col<float, true><<<gm, kFinBlock, 0, st>>>(
                    (const float*)ops.buf().colpart.get(), sh.nrb, m, B[q], ops.logb(), P->b,
                    reg, B[1 - q], parts.get(), S, 0, so_c, 1);
            else
                k_bcd_col<double, false><<<gm, kFinBlock, 0, st>>>(
                    (const double*)ops.buf().colpart.get(), sh.nrb, m, B[q], ops.logb(), P->b,
                    reg, B[1 - q], parts.get(), S, 0, so_c, 1);
            count_launch(2);
        };
        // The sweeps run as a device-side loop: a graph whose only node is a
        // conditional WHILE node; its body is two sweeps and k_bcd_loop,
        // which sets the condition. One launch and one read of the state
        // per solve: no host round trip between sweeps and none launched
        // past convergence.
        LoopGraph lg;
        REGOT_CUDA(cudaGraphCreate(&lg.graph, 0));
        cudaGraphConditionalHandle loop_h;
        REGOT_CUDA(cudaGraphConditionalHandleCreate(&loop_h, lg.graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = loop_h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop_node;
        REGOT_CUDA(cudaGraphAddNode(&loop_node, lg.graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        long long* saved_counter = g_launch_counter;
        long long graph_kernels = 0;
        g_launch_counter = &graph_kernels;
        REGOT_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal));
        try {
            half_sweeps(0);
            half_sweeps(1);
            k_bcd_loop<<<1, 1, 0, st>>>(S, loop_h);
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
        REGOT_CUDA(cudaGraphLaunch(lg.exec, st));
        read_state();
        count_launch(graph_kernels * hs.loops);
        if (!hs.bad) {
            if (!hs.done) throw Error(REGOT_ERR_NUMERIC, "BCD did not terminate");
            finished = true;
        }
        const int k = hs.iter;
        const size_t an = n * sizeof(double), bm = m * sizeof(double);
        if (finished || (hs.bad & (1 | 4))) {
            // iterate k (alpha_k, beta_k) is complete in slot k % 2; when
            // handing over it is not yet recorded
            if (k % 2 == 1) {
                d2d(alpha.get(), alpha_next.get(), an, st);
                d2d(beta.get(), beta_next.get(), bm, st);
            }
        } else {
            // column side: iterate k is recorded, alpha_{k+1} is complete in
            // slot (k + 1) % 2 and beta_k intact in slot k % 2; beta_{k+1} is
            // recomputed from alpha_{k+1} by the robust update
            if ((k + 1) % 2 == 0) d2d(alpha_next.get(), alpha.get(), an, st);
            if (k % 2 == 1) d2d(beta.get(), beta_next.get(), bm, st);
            pending = 2;
        }
        if (!finished) {
            const int zero = 0;
            h2d(&S->bad, &zero, sizeof(int), st);
            h2d(&S->done, &zero, sizeof(int), st);
            sync(st);
        }
    }

    // ---- general path: split before each pass, commit after each sweep ----
    if (!finished) {
        PassParams p1 = ops.base_params();
        p1.grid = &S->maxabs;
        p1.done = &S->done;
        PassParams p2 = p1;
        // K1: anchor alpha_k, column dual beta_k
        p1.ra = alpha.get();
        p1.cb = beta.get();
        // K2: row dual alpha_{k+1}, anchor beta_k
        p2.ra = alpha_next.get();
        p2.cb = beta.get();

        auto launch_row = [&](const double* anc, int robust) {
            if (mixed)
                k_bcd_row<float, true><<<gn, kFinBlock, 0, st>>>(
                    (const float*)ops.buf().rowpart.get(), sh.nslabs, n, anc, alpha.get(), P->a,
                    ops.loga(), reg, ops.sum_a(), ops.sum_bt(), alpha_next.get(), hobj, hmar,
                    htime, parts.get(), S, robust, SplitOut());
            else
                k_bcd_row<double, false><<<gn, kFinBlock, 0, st>>>(
                    (const double*)ops.buf().rowpart.get(), sh.nslabs, n, anc, alpha.get(), P->a,
                    ops.loga(), reg, ops.sum_a(), ops.sum_bt(), alpha_next.get(), hobj, hmar,
                    htime, parts.get(), S, robust, SplitOut());
            count_launch();
        };
        auto launch_col = [&](const double* anc, int robust) {
            if (mixed)
                k_bcd_col<float, true><<<gm, kFinBlock, 0, st>>>(
                    (const float*)ops.buf().colpart.get(), sh.nrb, m, anc, ops.logb(), P->b, reg,
                    beta_next.get(), parts.get(), S, robust, SplitOut(), 0);
            else
                k_bcd_col<double, false><<<gm, kFinBlock, 0, st>>>(
                    (const double*)ops.buf().colpart.get(), sh.nrb, m, anc, ops.logb(), P->b,
                    reg, beta_next.get(), parts.get(), S, robust, SplitOut(), 0);
            count_launch();
        };
        auto launch_commit = [&]() {
            k_bcd_commit<<<gnm, 256, 0, st>>>(n, m, alpha.get(), alpha_next.get(), beta.get(),
                                              beta_next.get(), S);
            count_launch();
        };
        auto sweep = [&]() {
            ops.pass(OP_E_ROW, p1);
            launch_row(alpha.get(), 0);
            ops.pass(OP_E_COL, p2);
            launch_col(beta.get(), 0);
            launch_commit();
        };
        // Robust redo of the half-sweep that left the safe range.
        auto robust = [&](int which) {
            const int zero = 0;
            h2d(&S->bad, &zero, sizeof(int), st);
            h2d(&S->done, &zero, sizeof(int), st);
            PassParams pr = ops.base_params();
            pr.grid = &S->maxabs;
            if (which & 1) {
                // alpha_{k+1} with an explicit max anchor, then the row sums of
                // iterate k measured against it.
                ops.optimal_alpha(beta.get(), anchor.get(), mx);
                ops.maxabs(anchor.get(), n, beta.get(), m, &S->maxabs);
                pr.ra = anchor.get();
                pr.cb = beta.get();
                ops.pass(OP_E_ROW, pr);
                launch_row(anchor.get(), 1);
                ops.maxabs(alpha_next.get(), n, beta.get(), m, &S->maxabs);
                ops.pass(OP_E_COL, p2);
                launch_col(beta.get(), 0);
                launch_commit();
            } else {
                // beta_{k+1} with an explicit max anchor.
                ops.optimal_beta(alpha_next.get(), anchor.get(), mx);
                ops.maxabs(alpha_next.get(), n, anchor.get(), m, &S->maxabs);
                pr.ra = alpha_next.get();
                pr.cb = anchor.get();
                ops.pass(OP_E_COL, pr);
                launch_col(anchor.get(), 1);
                launch_commit();
            }
            REGOT_CHECK_LAUNCH();
            read_state();
            if (hs.bad) throw Error(REGOT_ERR_NONFINITE, "non-finite row or column sums in BCD");
        };
        if (pending) robust(pending);

        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        long long* saved_counter = g_launch_counter;
        long long graph_kernels = 0;
        g_launch_counter = &graph_kernels;
        REGOT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        sweep();
        REGOT_CUDA(cudaStreamEndCapture(st, &graph));
        g_launch_counter = saved_counter;
        REGOT_CUDA(cudaGraphInstantiate(&exec, graph, 0));

        int batch = 4;
        long long launched = 0;
        read_state();
        while (!hs.done) {
            for (int q = 0; q < batch; ++q) REGOT_CUDA(cudaGraphLaunch(exec, st));
            launched += batch;
            count_launch(graph_kernels * batch);
            read_state();
            if (hs.bad) robust(hs.bad);
            if (hs.done) break;
            if (launched > 2LL * max_iter + 64)
                throw Error(REGOT_ERR_NUMERIC, "BCD did not terminate");
            batch = next_batch(batch);
        }
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
    }
    const long long passes = 2LL * hs.hist_len;

    // Results: gauge-fixed dual, plan, histories.
    DBuf<double> gamma(n + m, st);
    k_gauge<<<gnm, 256, 0, st>>>(n, m, alpha.get(), beta.get(), gamma.get(), gamma.get() + n);
    count_launch();
    finish_erot_result(ops, gamma.get(), hobj, hmar, htime, nullptr, hs.hist_len, hist_cap,
                       hs.niter, passes, o, res);
}

}  // namespace regot
