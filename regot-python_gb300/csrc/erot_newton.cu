// sinkhorn_newton on the GPU (reference: src/sinkhorn_newton.cpp:17-129).
//
// The reference forms the dense (n+m-1)^2 dual Hessian
// H = [diag(r) T~; T~' diag(c~)] / reg (sinkhorn_problem_obj.cpp:396-418) and
// solves H d = -g with Eigen::LLT. Here H is never formed: the Newton system
// is solved by conjugate gradients preconditioned with diag(H), where every
// product H p is one dense pass over M (T recomputed from the duals):
//   (H p)_alpha = (r o p_alpha + T p_beta~) / reg
//   (H p)_beta~ = (c~ o p_beta~ + T~' p_alpha) / reg.
// CG stops at ||H d + g|| < cg_tol ||g|| (default 1e-10), so the direction
// agrees with the LLT direction to that relative accuracy. One CG step is
// five kernels captured once in a CUDA graph and replayed in batches; every
// kernel returns immediately once the device-side CG state says `done`.
//
// The Armijo search (theta = kappa = 0.5, <= 20 trials, sinkhorn_newton.cpp:95-104)
// evaluates objective differences directly, four step sizes per pass:
//   f(gamma + s d) - f(gamma) = s g'd + reg * sum_ij T_ij phi(s w_ij),
//   w_ij = (d_i + d_j) / reg,  phi(x) = e^x - 1 - x >= 0,
// (reg * sum_ij T_ij w_ij = g'd + a'd_alpha + b~'d_beta~), so the test is a
// sum of non-negative terms plus an FP64 dot product and stays accurate when
// the decrease is far below the resolution of f itself.
#include <algorithm>
#include <cmath>
#include <vector>

#include "device_util.cuh"
#include "erot_ops.cuh"
#include "solvers.h"

namespace regot {

namespace {

constexpr int kVecThreads = 64;

struct NewtonState {
    int cg_done;
    int cg_it;
    int cg_max;
    unsigned counter;
    double rz;       // r' z of the current CG residual
    double alpha;    // CG step
    double beta;     // CG direction update
    double thresh2;  // stop when ||r||^2 < thresh2
    double rnorm2;
    double f;        // objective at gamma
    double gnorm;
    double gtd;      // g' d
    double ad;       // a' d_alpha + b~' d_beta~
    double maxabs;   // bound on |gamma|, |d| for the hi/lo split
    unsigned long long t0;
};

// Vectors of length n + m hold (alpha part, beta part) with beta_{m-1} = 0.

// Objective, gradient, Hessian diagonal from the row/column sums of T.
template <typename Acc>
__global__ void k_newton_grad(const Acc* rp, int nslabs, const Acc* cp, int nrb, int n, int m,
                              const double* gamma, const double* a, const double* b, double reg,
                              double* g, double* hdiag, double* parts, NewtonState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (t < n) {
        const double r = merge_strided(rp + t, nslabs, (size_t)n);
        const double gi = r - a[t];
        g[t] = gi;
        hdiag[t] = r / reg;
        v[0] = gi * gi;
        v[1] = r;
        v[2] = gamma[t] * a[t];
    } else if (t < n + m) {
        const int j = t - n;
        if (j < m - 1) {
            const double c = merge_strided(cp + j, nrb, (size_t)m);
            const double gj = c - b[j];
            g[t] = gj;
            hdiag[t] = c / reg;
            v[0] = gj * gj;
            v[3] = gamma[t] * b[j];
        } else {
            g[t] = 0.0;
            hdiag[t] = 1.0;
        }
    }
    double out[4];
    __threadfence();
    if (grid_reduce<4>(v, parts, &st->counter, out)) {
        st->gnorm = sqrt(out[0]);
        st->f = reg * out[1] - out[2] - out[3];  // sinkhorn_problem_obj.cpp:389-390
    }
}

// CG set-up for H x = sign v (the Newton system: v = g, sign = -1): x = 0,
// r = sign v, z = r / diag(H), p = z.
__global__ void k_cg_init(int N, const double* g, double sign, const double* hdiag, double tol,
                          double* x, double* r, double* z, double* p, double* parts,
                          NewtonState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (t < N) {
        const double ri = sign * g[t];
        const double zi = ri / hdiag[t];
        x[t] = 0.0;
        r[t] = ri;
        z[t] = zi;
        p[t] = zi;
        v[0] = ri * zi;
        v[1] = ri * ri;
    }
    double out[2];
    __threadfence();
    if (grid_reduce<2>(v, parts, &st->counter, out)) {
        st->rz = out[0];
        st->rnorm2 = out[1];
        st->thresh2 = fmax(tol * tol * out[1], 2.2250738585072014e-308);
        st->cg_it = 0;
        st->cg_done = (out[1] == 0.0 || out[1] < st->thresh2) ? 1 : 0;
    }
}

// y = H p from the HVP pass partials; alpha = r'z / p'y. Blocks of (32, 8)
// threads own 32 entries, rows in the first cdiv(n, 32) blocks and columns
// after them; the eight threads of an entry merge its partials together
// (the columns have one partial per row block: 128 at n = 8192, one chain
// of loads each took most of this kernel's time).
template <typename Acc>
__global__ void __launch_bounds__(256) k_cg_a(const Acc* rp, int nslabs, const Acc* cp, int nrb,
                                              int n, int m, const double* hdiag, const double* p,
                                              double reg, double* y, double* parts,
                                              NewtonState* st) {
    if (st->cg_done) return;
    const int gr = (n + 31) / 32;
    const bool rows = (int)blockIdx.x < gr;
    const int item = (rows ? (int)blockIdx.x : (int)blockIdx.x - gr) * 32 + (int)threadIdx.x;
    const double tp = rows ? merge_2d(rp + item, nslabs, (size_t)n, item < n)
                           : merge_2d(cp + item, nrb, (size_t)m, item < m - 1);
    if (threadIdx.y != 0) return;  // the rest runs in warp 0 only
    double v[1] = {0.0};
    const int t = rows ? item : n + item;
    if (rows ? item < n : item < m) {
        const double yt = (rows || item < m - 1) ? hdiag[t] * p[t] + tp / reg : 0.0;
        y[t] = yt;
        v[0] = p[t] * yt;
    }
    double out[1];
    __threadfence();
    if (warp_grid_reduce<1>(v, parts, &st->counter, out) && threadIdx.x == 0)
        st->alpha = st->rz / out[0];
}

int cg_a_grid(int n, int m) { return (n + 31) / 32 + (m + 31) / 32; }

// x += alpha p, r -= alpha y, z = r / diag(H); beta = r'z_new / r'z_old;
// stop at ||r||^2 < thresh2 or at the iteration limit.
__global__ void k_cg_b(int N, const double* p, const double* y, const double* hdiag, double* x,
                       double* r, double* z, double* parts, NewtonState* st) {
    if (st->cg_done) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const double al = st->alpha;
    double v[2] = {0.0, 0.0};
    if (t < N) {
        x[t] += al * p[t];
        const double ri = r[t] - al * y[t];
        r[t] = ri;
        const double zi = ri / hdiag[t];
        z[t] = zi;
        v[0] = ri * zi;
        v[1] = ri * ri;
    }
    double out[2];
    __threadfence();
    if (grid_reduce<2>(v, parts, &st->counter, out)) {
        st->rnorm2 = out[1];
        st->cg_it += 1;
        if (out[1] < st->thresh2 || st->cg_it >= st->cg_max || !(out[1] == out[1])) {
            st->cg_done = 1;
        } else {
            st->beta = out[0] / st->rz;
            st->rz = out[0];
        }
    }
}

// p = z + beta p; refresh the hi/lo bound with |p|.
// p = z + beta p; with rs / cs (mixed), p's FP32 copies in the z entries of
// the split arrays, which the next HVP pass reads (the duals' hi / lo parts
// in x and y stay as split once per direction).
__global__ void k_cg_c(int N, int n, const double* z, double* p, NewtonState* st, float4* rs,
                       float4* cs) {
    if (st->cg_done) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < N) {
        const double pv = z[t] + st->beta * p[t];
        p[t] = pv;
        if (rs) {
            if (t < n) rs[t].z = (float)pv;
            else cs[t - n].z = (float)pv;
        }
    }
}

// g'd and a'd_alpha + b~'d_beta~ for the line search.
__global__ void k_dir_dots(int n, int m, const double* g, const double* d, const double* a,
                           const double* b, double* parts, NewtonState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    double dv = 0.0;
    if (t < n) {
        dv = d[t];
        v[0] = g[t] * dv;
        v[1] = a[t] * dv;
    } else if (t < n + m - 1) {
        dv = d[t];
        v[0] = g[t] * dv;
        v[1] = b[t - n] * dv;
    }
    block_atomic_max_abs(&st->maxabs, dv);
    double out[2];
    __threadfence();
    if (grid_reduce<2>(v, parts, &st->counter, out)) {
        st->gtd = out[0];
        st->ad = out[1];
    }
}

__global__ void k_axpy_gamma(int N, double s, const double* d, double* gamma, NewtonState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double gv = 0.0;
    if (t < N) {
        gv = gamma[t] + s * d[t];
        gamma[t] = gv;
    }
    block_atomic_max_abs(&st->maxabs, gv);
}

__global__ void k_newton_start(NewtonState* st) { st->t0 = globaltimer_ns(); }
__global__ void k_newton_time(NewtonState* st, double* out) {
    *out = (double)(globaltimer_ns() - st->t0) * 1e-6;
}

// Sum of the per-CTA line-search totals of `nsteps` step sizes.
__global__ void k_ls_totals(const double* totpart, int nblocks, int nsteps, double* out) {
    const int s = threadIdx.x;
    if (s >= nsteps) return;
    double acc = 0.0;
    for (int k = 0; k < nblocks; ++k) acc += totpart[(size_t)s * nblocks + k];
    out[s] = acc;
}

}  // namespace

void sinkhorn_newton_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, double tol, int max_iter,
                         const regot_opts& o, regot_result* res) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    ErotOps ops(P, reg, st);
    const PassShape sh = ops.buf().shape;
    const int hist_cap = max_iter + 2;
    constexpr double theta = 0.5, kappa = 0.5;  // sinkhorn_newton.cpp:29-30
    constexpr int nlinesearch = 20;
    const double cg_tol = o.cg_tol > 0.0 ? o.cg_tol : 1e-10;
    const int cg_max = o.cg_max_iter > 0 ? o.cg_max_iter : 2 * (n + m - 1);

    DBuf<double> gamma(N, st), g(N, st), hdiag(N, st), x(N, st), r(N, st), z(N, st), pv(N, st),
        y(N, st), hist(3 * (size_t)hist_cap, st), scratch(8, st), lsout(4, st);
    DBuf<double> parts(4 * (size_t)std::max(cdiv(N, kVecThreads), cg_a_grid(n, m)), st);
    DBuf<NewtonState> dst(1, st);
    NewtonState h0{};
    h0.cg_max = cg_max;
    h2d(dst.get(), &h0, sizeof(h0), st);
    NewtonState* S = dst.get();
    double* hobj = hist.get();
    double* hmar = hobj + hist_cap;
    double* htime = hmar + hist_cap;
    const int gv = cdiv(N, kVecThreads);

    // Initial value (sinkhorn_newton.cpp:42-52): gamma = x0, or
    // (alpha = 0 + beta_m, beta~ - beta_m) with beta = optimal_beta(0).
    if (o.x0 && o.x0_len == n + m - 1) {
        std::vector<double> h(N, 0.0);
        std::copy(o.x0, o.x0 + n + m - 1, h.begin());
        h2d(gamma.get(), h.data(), N * sizeof(double), st);
    } else {
        DBuf<double> beta(m, st), zero(n, st);
        zero.zero();
        ops.optimal_beta(zero.get(), beta.get(), scratch.get());
        std::vector<double> hb(m);
        d2h(hb.data(), beta.get(), m * sizeof(double), st);
        sync(st);
        std::vector<double> h(N, 0.0);
        for (int i = 0; i < n; ++i) h[i] = hb[m - 1];
        for (int j = 0; j < m - 1; ++j) h[n + j] = hb[j] - hb[m - 1];
        h2d(gamma.get(), h.data(), N * sizeof(double), st);
    }
    k_newton_start<<<1, 1, 0, st>>>(S);
    count_launch();
    ops.maxabs(gamma.get(), N, nullptr, 0, &S->maxabs);

    // f, g at gamma (one fused row+column pass).
    PassParams pg = ops.base_params();
    pg.ra = gamma.get();
    pg.cb = gamma.get() + n;
    pg.grid = &S->maxabs;
    auto grad_pass = [&]() {
        ops.pass(OP_E_ROWCOL, pg);
        if (mixed)
            k_newton_grad<float><<<gv, kVecThreads, 0, st>>>(
                (const float*)ops.buf().rowpart.get(), sh.nslabs,
                (const float*)ops.buf().colpart.get(), sh.nrb, n, m, gamma.get(), P->a, P->b, reg,
                g.get(), hdiag.get(), parts.get(), S);
        else
            k_newton_grad<double><<<gv, kVecThreads, 0, st>>>(
                (const double*)ops.buf().rowpart.get(), sh.nslabs,
                (const double*)ops.buf().colpart.get(), sh.nrb, n, m, gamma.get(), P->a, P->b,
                reg, g.get(), hdiag.get(), parts.get(), S);
        count_launch();
        REGOT_CHECK_LAUNCH();
    };

    // One CG step (captured in a graph).
    PassParams ph = pg;
    ph.rx = pv.get();
    ph.cx = pv.get() + n;
    ph.done = &S->cg_done;
    float4* rs_mut = mixed ? ops.rsplit_mut() : nullptr;
    float4* cs_mut = mixed ? ops.csplit_mut() : nullptr;
    auto cg_step = [&]() {
        ops.pass_presplit(OP_E_HVP, ph);
        if (mixed)
            k_cg_a<float><<<cg_a_grid(n, m), dim3(32, 8), 0, st>>>(
                (const float*)ops.buf().rowpart.get(), sh.nslabs,
                (const float*)ops.buf().colpart.get(), sh.nrb, n, m, hdiag.get(), pv.get(), reg,
                y.get(), parts.get(), S);
        else
            k_cg_a<double><<<cg_a_grid(n, m), dim3(32, 8), 0, st>>>(
                (const double*)ops.buf().rowpart.get(), sh.nslabs,
                (const double*)ops.buf().colpart.get(), sh.nrb, n, m, hdiag.get(), pv.get(), reg,
                y.get(), parts.get(), S);
        k_cg_b<<<gv, kVecThreads, 0, st>>>(N, pv.get(), y.get(), hdiag.get(), x.get(), r.get(),
                                             z.get(), parts.get(), S);
        k_cg_c<<<gv, kVecThreads, 0, st>>>(N, n, z.get(), pv.get(), S, rs_mut, cs_mut);
        count_launch(3);
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long graph_kernels = 0;
    {
        long long* saved = g_launch_counter;
        g_launch_counter = &graph_kernels;
        REGOT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cg_step();
        REGOT_CUDA(cudaStreamEndCapture(st, &graph));
        g_launch_counter = saved;
        REGOT_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    }

    PassParams pl = pg;
    pl.rd = x.get();
    pl.cd = x.get() + n;
    const int ls_blocks = pass_blocks(OP_E_LS, mixed, n, m);

    NewtonState hs{};
    long long passes = 0;
    int hist_len = 0;
    auto record = [&]() {
        k_newton_time<<<1, 1, 0, st>>>(S, htime + hist_len);
        count_launch();
        read_small(ctx, &hs, S, sizeof(hs), st);
        h2d(hobj + hist_len, &hs.f, sizeof(double), st);
        h2d(hmar + hist_len, &hs.gnorm, sizeof(double), st);
        ++hist_len;
    };

    grad_pass();
    ++passes;
    record();
    int i;
    for (i = 0; i < max_iter; i++) {
        if (o.verbose >= 1)
            std::printf("iter = %d, objval = %g, ||grad|| = %g\n", i, hs.f, hs.gnorm);
        if (hs.gnorm < tol || !std::isfinite(hs.f)) break;  // sinkhorn_newton.cpp:87-88

        // Newton direction: H x = -g by preconditioned CG.
        k_cg_init<<<gv, kVecThreads, 0, st>>>(N, g.get(), -1.0, hdiag.get(), cg_tol, x.get(),
                                              r.get(), z.get(), pv.get(), parts.get(), S);
        count_launch();
        // the split of gamma (and of p = z) for the CG's HVP passes
        ops.maxabs(gamma.get(), N, nullptr, 0, &S->maxabs);
        ops.split(ph);
        int batch = 8;
        for (;;) {
            for (int q = 0; q < batch; ++q) REGOT_CUDA(cudaGraphLaunch(exec, st));
            count_launch(graph_kernels * batch);
            int done = 0, it = 0;
            d2h(&done, &S->cg_done, sizeof(int), st);
            d2h(&it, &S->cg_it, sizeof(int), st);
            sync(st);
            if (done) {
                passes += it;
                break;
            }
            batch = std::min(batch * 2, 64);
        }

        // Armijo backtracking on exact objective differences.
        k_dir_dots<<<gv, kVecThreads, 0, st>>>(n, m, g.get(), x.get(), P->a, P->b, parts.get(), S);
        count_launch();
        read_small(ctx, &hs, S, sizeof(hs), st);
        const double thresh = theta * hs.gtd;
        double step = 1.0, accepted = -1.0;
        // The first pass tries the full step alone (accepted in most Newton
        // iterations; one phi per entry instead of four), later passes four
        // steps at a time. The accepted step is the reference's first
        // acceptable one either way.
        for (int k0 = 0; k0 < nlinesearch && accepted < 0.0;) {
            const int ns = std::min(k0 == 0 ? 1 : 4, nlinesearch - k0);
            k0 += ns;
            double steps[4] = {0, 0, 0, 0};
            for (int s = 0; s < ns; ++s) steps[s] = step * std::pow(kappa, s);
            PassParams q = pl;
            for (int s = 0; s < 4; ++s) q.steps[s] = steps[s];
            q.nsteps = ns;
            ops.pass(OP_E_LS, q);
            ++passes;
            k_ls_totals<<<1, 32, 0, st>>>(ops.buf().totpart.get(), ls_blocks, ns, lsout.get());
            count_launch();
            double tots[4];
            d2h(tots, lsout.get(), ns * sizeof(double), st);
            sync(st);
            for (int s = 0; s < ns; ++s) {
                const double df = steps[s] * hs.gtd + reg * tots[s];
                if (df <= steps[s] * thresh) {  // newf <= f + step * thresh
                    accepted = steps[s];
                    break;
                }
            }
            step = steps[ns - 1] * kappa;
        }
        // Without an acceptable step the reference keeps the last trial
        // (step = kappa^19).
        if (accepted < 0.0) accepted = std::pow(kappa, nlinesearch - 1);
        k_axpy_gamma<<<gv, kVecThreads, 0, st>>>(N, accepted, x.get(), gamma.get(), S);
        count_launch();
        grad_pass();
        ++passes;
        record();
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    finish_erot_result(ops, gamma.get(), hobj, hmar, htime, nullptr, hist_len, hist_cap, i,
                       passes, o, res);
}

// H x = rhs for the exact dual Hessian at gamma (the matrix the reference
// factors in sinkhorn_newton.cpp:91-92), by the Jacobi-preconditioned CG of
// the Newton solver above: one HVP pass per step, to
// ||H x - rhs|| < tol ||rhs|| or max_iter steps. Vectors have n + m - 1
// entries (host). Used for implicit derivatives of a solve.
void erot_hess_solve_gpu(regot_ctx* ctx, regot_dproblem* P, double reg, const double* gamma_h,
                         const double* rhs_h, double tol, int max_iter, double* x_h, int* iters) {
    cudaStream_t st = ctx->stream;
    const int n = P->n, m = P->m, N = n + m;
    const bool mixed = P->prec == REGOT_PREC_MIXED;
    ErotOps ops(P, reg, st);
    const PassShape sh = ops.buf().shape;
    DBuf<double> gamma(N, st), g(N, st), hdiag(N, st), x(N, st), r(N, st), z(N, st), pv(N, st),
        y(N, st), rhs(N, st);
    DBuf<double> parts(4 * (size_t)std::max(cdiv(N, kVecThreads), cg_a_grid(n, m)), st);
    DBuf<NewtonState> dst(1, st);
    NewtonState h0{};
    h0.cg_max = max_iter > 0 ? max_iter : 2 * (n + m - 1);
    h2d(dst.get(), &h0, sizeof(h0), st);
    NewtonState* S = dst.get();
    const int gv = cdiv(N, kVecThreads);
    {
        std::vector<double> h(N, 0.0);
        std::copy(gamma_h, gamma_h + n + m - 1, h.begin());
        h2d(gamma.get(), h.data(), N * sizeof(double), st);
        std::copy(rhs_h, rhs_h + n + m - 1, h.begin());
        h[N - 1] = 0.0;
        h2d(rhs.get(), h.data(), N * sizeof(double), st);
    }
    ops.maxabs(gamma.get(), N, nullptr, 0, &S->maxabs);
    PassParams pg = ops.base_params();
    pg.ra = gamma.get();
    pg.cb = gamma.get() + n;
    pg.grid = &S->maxabs;
    ops.pass(OP_E_ROWCOL, pg);  // diag(H) from the row and column sums
    if (mixed)
        k_newton_grad<float><<<gv, kVecThreads, 0, st>>>(
            (const float*)ops.buf().rowpart.get(), sh.nslabs,
            (const float*)ops.buf().colpart.get(), sh.nrb, n, m, gamma.get(), P->a, P->b, reg,
            g.get(), hdiag.get(), parts.get(), S);
    else
        k_newton_grad<double><<<gv, kVecThreads, 0, st>>>(
            (const double*)ops.buf().rowpart.get(), sh.nslabs,
            (const double*)ops.buf().colpart.get(), sh.nrb, n, m, gamma.get(), P->a, P->b, reg,
            g.get(), hdiag.get(), parts.get(), S);
    k_cg_init<<<gv, kVecThreads, 0, st>>>(N, rhs.get(), 1.0, hdiag.get(), tol, x.get(), r.get(),
                                          z.get(), pv.get(), parts.get(), S);
    count_launch(2);
    REGOT_CHECK_LAUNCH();
    PassParams ph = pg;
    ph.rx = pv.get();
    ph.cx = pv.get() + n;
    ph.done = &S->cg_done;
    ops.split(ph);
    float4* rs_mut = mixed ? ops.rsplit_mut() : nullptr;
    float4* cs_mut = mixed ? ops.csplit_mut() : nullptr;
    NewtonState hs{};
    for (;;) {
        read_small(ctx, &hs, S, sizeof(hs), st);
        if (hs.cg_done) break;
        for (int q = 0; q < 8; ++q) {  // steps between state reads
            ops.pass_presplit(OP_E_HVP, ph);
            if (mixed)
                k_cg_a<float><<<cg_a_grid(n, m), dim3(32, 8), 0, st>>>(
                    (const float*)ops.buf().rowpart.get(), sh.nslabs,
                    (const float*)ops.buf().colpart.get(), sh.nrb, n, m, hdiag.get(), pv.get(),
                    reg, y.get(), parts.get(), S);
            else
                k_cg_a<double><<<cg_a_grid(n, m), dim3(32, 8), 0, st>>>(
                    (const double*)ops.buf().rowpart.get(), sh.nslabs,
                    (const double*)ops.buf().colpart.get(), sh.nrb, n, m, hdiag.get(), pv.get(),
                    reg, y.get(), parts.get(), S);
            k_cg_b<<<gv, kVecThreads, 0, st>>>(N, pv.get(), y.get(), hdiag.get(), x.get(), r.get(),
                                                 z.get(), parts.get(), S);
            k_cg_c<<<gv, kVecThreads, 0, st>>>(N, n, z.get(), pv.get(), S, rs_mut, cs_mut);
            count_launch(3);
        }
    }
    read_small(ctx, x_h, x.get(), (size_t)(n + m - 1) * sizeof(double), st);
    if (iters) *iters = hs.cg_it;
    ops.check_err();
}

}  // namespace regot
