"""Batched BCD over point-cloud problems (regot_erot_solve_batched) against
the FP64 oracle's sinkhorn_bcd run on each problem alone."""
import numpy as np
import pytest

import regot_oracle as O

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def _batch(count, seed, nmin=16, nmax=200, dims=range(1, 17)):
    """Uneven problems: n, m log-uniform, d uniform over `dims`, x ~ N(0, I),
    y ~ N(mu, I) with mu ~ N(0, 0.25 I), uniform-random marginals."""
    rng = np.random.default_rng(seed)
    xs, ys, as_, bs, scales = [], [], [], [], []
    dims = list(dims)
    for _ in range(count):
        n, m = np.exp(rng.uniform(np.log(nmin), np.log(nmax), 2)).round().astype(int)
        d = int(rng.choice(dims))
        mu = rng.normal(0.0, 0.5, d)
        xs.append(rng.standard_normal((n, d)).astype(np.float32))
        ys.append((rng.standard_normal((m, d)) + mu).astype(np.float32))
        a = rng.uniform(0.5, 1.5, n)
        b = rng.uniform(0.5, 1.5, m)
        as_.append(a / a.sum())
        bs.append(b / b.sum())
        scales.append(1.0 / d)
    return xs, ys, as_, bs, scales


def _set_tail(v):
    from regot import _lib

    return _lib.load().regot_set_batch_tail(v)


@pytest.fixture(params=["graph", "tail"])
def batch_tail(request):
    """Runs a test with the per-sweep kernels to the end ("graph": tail
    threshold 0) and with the whole solve after the first two sweeps in the
    cluster-per-problem tail kernel ("tail"), restoring the default after."""
    old = _set_tail(0 if request.param == "graph" else 1 << 20)
    try:
        yield request.param
    finally:
        _set_tail(old)


def _cost64(x, y, s):
    x = x.astype(np.float64)
    y = y.astype(np.float64)
    return s * ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)


def test_batched_matches_oracle_per_problem(batch_tail):
    # tol 1e-6 as in the batched workload: the FP32 row sums carry relative
    # errors of a few 1e-7, so much tighter tolerances stall in FP32
    reg, tol = 0.05, 1e-6
    xs, ys, as_, bs, sc = _batch(24, seed=5)
    r = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=tol, max_iter=5000, cost_scale=sc)
    assert len(r.duals) == 24 and r.sweeps >= int(r.niter.max())
    for p in range(24):
        M = _cost64(xs[p], ys[p], sc[p])
        o = O.sinkhorn_bcd(M, as_[p], bs[p], reg, tol=tol, max_iter=5000, plan=False)
        assert r.mar_errs[p] < tol, (p, r.mar_errs[p])
        # the FP32 cost differs from the FP64 one by an ulp of M: the same
        # convergence up to a few iterations, duals to ~1e-6
        assert abs(int(r.niter[p]) - o.niter) <= max(3, 0.05 * o.niter), (p, r.niter[p], o.niter)
        np.testing.assert_allclose(r.duals[p], o.dual, rtol=0, atol=2e-5)
        # the duals are optimal for the FP64 cost to the same accuracy
        _, g = O.erot_dual_obj_grad(M, as_[p], bs[p], reg, r.duals[p])
        assert np.linalg.norm(g) < 5 * tol


def test_batched_max_iter_iterates(batch_tail):
    # every problem stops at max_iter: the duals are the oracle's iterate
    reg = 0.05
    xs, ys, as_, bs, sc = _batch(10, seed=6, dims=(2, 3, 7, 12, 16))
    r = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=1e-14, max_iter=7, cost_scale=sc)
    assert np.all(r.niter == 7)
    for p in range(10):
        M = _cost64(xs[p], ys[p], sc[p])
        o = O.sinkhorn_bcd(M, as_[p], bs[p], reg, tol=1e-14, max_iter=7, plan=False)
        assert o.niter == 7
        np.testing.assert_allclose(r.duals[p], o.dual, rtol=0, atol=2e-5)
        np.testing.assert_allclose(r.mar_errs[p], o.mar_errs[-1], rtol=2e-3, atol=1e-9)


def test_batched_single_problem_equals_batch_member(batch_tail):
    # a problem's result does not depend on the other problems of the batch
    reg, tol = 0.05, 1e-7
    xs, ys, as_, bs, sc = _batch(6, seed=7)
    r = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=tol, max_iter=3000, cost_scale=sc)
    for p in (0, 3, 5):
        r1 = regot.sinkhorn_bcd_batched([xs[p]], [ys[p]], [as_[p]], [bs[p]], reg, tol=tol,
                                        max_iter=3000, cost_scale=sc[p])
        assert r1.niter[0] == r.niter[p]
        np.testing.assert_array_equal(r1.duals[0], r.duals[p])


def test_batched_rejects_bad_input():
    xs, ys, as_, bs, sc = _batch(2, seed=8)
    with pytest.raises(ValueError):
        regot.sinkhorn_bcd_batched(xs, ys[:1], as_, bs, 0.05)
    with pytest.raises(ValueError):
        regot.sinkhorn_bcd_batched([np.zeros((4, 17), np.float32)], [np.zeros((3, 17), np.float32)],
                                   [np.full(4, 0.25)], [np.full(3, 1 / 3)], 0.05)
    with pytest.raises(ValueError):
        regot.sinkhorn_bcd_batched(xs, ys, as_, bs, -1.0)


def test_batched_backward_matches_fp64_at_the_returned_duals(batch_tail):
    # grad=True: each problem's cost a'alpha + b'beta - reg sum T (the negated
    # dual objective of the oracle) and dL/dx = 2 s sum_j T_ij (x_i - y_j),
    # dL/dy = 2 s sum_i T_ij (y_j - x_i), checked in FP64 at the duals the
    # call returned. The kernels evaluate T from the FP32 cost: a relative
    # error of ~1e-7 in M moves the exponent by ~1e-7 M / reg, a few 1e-5 of
    # T at these sizes, hence 3e-4 of the largest gradient entry.
    reg, tol = 0.05, 1e-6
    xs, ys, as_, bs, sc = _batch(14, seed=9, nmin=20, nmax=700, dims=(1, 3, 4, 5, 8, 9, 16))
    r0 = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=tol, max_iter=5000, cost_scale=sc)
    r = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=tol, max_iter=5000, cost_scale=sc,
                                   grad=True)
    np.testing.assert_array_equal(r.niter, r0.niter)
    assert len(r.grad_x) == len(r.grad_y) == len(r.costs) == 14
    for p in range(14):
        np.testing.assert_array_equal(r.duals[p], r0.duals[p])
        x = xs[p].astype(np.float64)
        y = ys[p].astype(np.float64)
        n, m = x.shape[0], y.shape[0]
        M = _cost64(xs[p], ys[p], sc[p])
        f, _ = O.erot_dual_obj_grad(M, as_[p], bs[p], reg, r.duals[p])
        assert abs(r.costs[p] + f) < 5e-6, (p, r.costs[p], -f)
        alpha = r.duals[p][:n]
        beta = np.r_[r.duals[p][n:], 0.0]
        T = np.exp((alpha[:, None] + beta[None, :] - M) / reg)
        gx = 2 * sc[p] * (T.sum(1)[:, None] * x - T @ y)
        gy = 2 * sc[p] * (T.sum(0)[:, None] * y - T.T @ x)
        assert r.grad_x[p].shape == x.shape and r.grad_y[p].shape == y.shape
        assert r.grad_x[p].dtype == np.float32 and r.grad_y[p].dtype == np.float32
        np.testing.assert_allclose(r.grad_x[p], gx, rtol=0, atol=3e-4 * np.abs(gx).max())
        np.testing.assert_allclose(r.grad_y[p], gy, rtol=0, atol=3e-4 * np.abs(gy).max())
        # translating both clouds leaves the cost unchanged: the gradients sum to 0
        np.testing.assert_allclose(r.grad_x[p].sum(0) + r.grad_y[p].sum(0), 0.0,
                                   atol=1e-4 * np.abs(gx).sum())


def test_batched_backward_at_max_iter_iterates(batch_tail):
    # problems stopped by max_iter (odd and even counts, so the last alpha
    # sits in either ping-pong buffer): the backward still uses exactly the
    # returned iterate, whose row sums are still off a by up to 0.1
    reg = 0.05
    xs, ys, as_, bs, sc = _batch(8, seed=10, nmin=40, nmax=400, dims=(2, 6, 11, 16))
    for it in (4, 7):
        r = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=1e-14, max_iter=it,
                                       cost_scale=sc, grad=True)
        assert np.all(r.niter == it)
        for p in range(8):
            n = xs[p].shape[0]
            M = _cost64(xs[p], ys[p], sc[p])
            f, _ = O.erot_dual_obj_grad(M, as_[p], bs[p], reg, r.duals[p])
            assert abs(r.costs[p] + f) < 5e-6 * max(1.0, abs(f)), (it, p)
            alpha = r.duals[p][:n]
            beta = np.r_[r.duals[p][n:], 0.0]
            T = np.exp((alpha[:, None] + beta[None, :] - M) / reg)
            x = xs[p].astype(np.float64)
            y = ys[p].astype(np.float64)
            gx = 2 * sc[p] * (T.sum(1)[:, None] * x - T @ y)
            gy = 2 * sc[p] * (T.sum(0)[:, None] * y - T.T @ x)
            np.testing.assert_allclose(r.grad_x[p], gx, rtol=0, atol=3e-4 * np.abs(gx).max())
            np.testing.assert_allclose(r.grad_y[p], gy, rtol=0, atol=3e-4 * np.abs(gy).max())


def _force(v):
    from regot import _lib

    return _lib.load().regot_force_batch_variant(v)


@pytest.mark.parametrize("scaled", [True, False])
def test_batched_tensor_core_cost_tile(scaled):
    """The tensor-core variant of the half-sweeps (cost tile x y' on tcgen05
    in TF32x3, M = s (|x|^2 + |y|^2 - 2 x.y)) against the CUDA-core direct
    differences and the FP64 oracle. The expansion carries an absolute error
    of about 2^-21 s (|x|^2 + |y|^2) in M, i.e. about 1e-6 s d; at reg 0.05
    that moves T by up to about 1e-4 relative for the unscaled costs of
    d = 16 and the duals by a few 1e-6, which the bounds below state.
    Fixed-iteration runs compare the two variants without the stopping test;
    converged runs check the marginal error of the tensor-core duals in FP64
    on the FP64 cost."""
    reg, tol = 0.05, 1e-6
    xs, ys, as_, bs, sc = _batch(20, seed=8, nmin=40, nmax=400, dims=(3, 6, 8, 11, 16))
    if not scaled:
        sc = [1.0] * len(sc)
    # the tail kernel computes on the CUDA cores: keep every sweep in the
    # per-sweep kernels so that the variants are compared over all six
    old = _force(1)
    old_tail = _set_tail(0)
    try:
        r_tc = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=1e-14, max_iter=6,
                                          cost_scale=sc)
        _force(0)
        r_cc = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=1e-14, max_iter=6,
                                          cost_scale=sc)
        _force(1)
        r_conv = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=tol, max_iter=20000,
                                            cost_scale=sc)
    finally:
        _force(old)
        _set_tail(old_tail)
    worst = 0.0
    for p in range(len(xs)):
        assert r_tc.niter[p] == r_cc.niter[p] == 6
        d = xs[p].shape[1]
        # the cost tile's absolute error (~1e-6 s d) passes into the duals
        # about one to one; 64x headroom
        bound = 6.4e-5 * sc[p] * d
        err = np.abs(r_tc.duals[p] - r_cc.duals[p]).max()
        worst = max(worst, err / bound)
        assert err <= bound, (p, err, bound)
        M = _cost64(xs[p], ys[p], sc[p])
        assert r_conv.mar_errs[p] < tol, (p, r_conv.mar_errs[p])
        _, g = O.erot_dual_obj_grad(M, as_[p], bs[p], reg, r_conv.duals[p])
        # marginal error on the FP64 cost: tol plus the cost tile's perturbation
        assert np.linalg.norm(g) < tol + 2e-4 * sc[p] * d, (p, np.linalg.norm(g))
    print(f"tensor-core vs CUDA-core duals after 6 sweeps: worst error / bound = {worst:.3f}")


@pytest.mark.parametrize("tail", [4, 1 << 20])
def test_batched_tail_handover_keeps_the_iterates(tail):
    """The tail kernel runs the same row and column arithmetic and stopping
    test as the per-sweep kernels (CUDA-core variant forced): handing the
    last problems over mid-solve (tail 4 of 40) or after two sweeps
    (tail 2^20) gives the iteration counts of the per-sweep kernels and their
    duals to FP64 rounding. Only a re-split of the duals on a new grid, which
    the per-sweep loop applies to all running problems and the tail only to
    the problem that needs it, can move the FP32 roundings apart."""
    reg, tol = 0.05, 1e-6
    xs, ys, as_, bs, sc = _batch(40, seed=9, nmin=16, nmax=300)
    old = _force(0)
    old_tail = _set_tail(0)
    try:
        ref = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=tol, max_iter=5000,
                                         cost_scale=sc)
        _set_tail(tail)
        r = regot.sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=tol, max_iter=5000,
                                       cost_scale=sc)
    finally:
        _force(old)
        _set_tail(old_tail)
    np.testing.assert_array_equal(r.niter, ref.niter)
    worst = max(float(np.abs(r.duals[p] - ref.duals[p]).max()) for p in range(len(xs)))
    print(f"tail {tail}: largest dual difference to the per-sweep kernels {worst:.3e}")
    assert worst <= 1e-9
    for p in range(len(xs)):
        assert r.mar_errs[p] < tol
