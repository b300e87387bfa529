"""Parity of the GPU sinkhorn_lbfgs_dual and sinkhorn_apdagd with the FP64
oracle restatements of the reference (sinkhorn_lbfgs_dual.cpp:81-126,
sinkhorn_apdagd.cpp:14-183)."""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


LBFGS_CASES = {
    "points-120x90": (lambda: erot_points(120, 90, seed=3, dtype=np.float64), 0.05),
    "points-200x150": (lambda: erot_points(200, 150, seed=4, dtype=np.float64), 0.02),
}


@pytest.mark.parametrize("case", list(LBFGS_CASES))
def test_lbfgs_dual_fp64_matches_oracle(case):
    make, reg = LBFGS_CASES[case]
    M, a, b = make()
    tol = 1e-8
    r = regot.sinkhorn_lbfgs_dual(M, a, b, reg, tol=tol, max_iter=500, precision="fp64")
    o = O.sinkhorn_lbfgs_dual(M, a, b, reg, tol=tol, max_iter=500)
    L = r.niter + 1
    assert len(r.obj_vals) == len(r.mar_errs) == len(r.run_times) == L
    assert abs(r.niter - o.niter) <= 2, (r.niter, o.niter)
    # the same iterates until the summation-order differences have grown
    k = min(L, len(o.mar_errs), 15)
    np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=1e-6, atol=1e-13)
    np.testing.assert_allclose(r.obj_vals[:k], o.obj_vals[:k], rtol=1e-11, atol=1e-13)
    assert r.mar_errs[-1] < tol
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-6)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-6 * o.plan.max())


@pytest.mark.parametrize("case", list(LBFGS_CASES))
def test_lbfgs_dual_mixed(case):
    # FP32 M: the solve converges to the FP64 solution of the FP32-rounded
    # cost; trials take the objective change from the trial pass itself.
    make, reg = LBFGS_CASES[case]
    M, a, b = make()
    Mq = _as_precision(M, "mixed")
    tol = 1e-7
    r = regot.sinkhorn_lbfgs_dual(M, a, b, reg, tol=tol, max_iter=500, precision="mixed")
    o = O.sinkhorn_lbfgs_dual(Mq, a, b, reg, tol=tol, max_iter=500)
    assert r.mar_errs[-1] < tol
    assert r.niter <= 1.5 * o.niter + 10, (r.niter, o.niter)
    _, g = O.erot_dual_obj_grad(Mq, a, b, reg, r.dual)
    assert np.linalg.norm(g) < 20 * tol
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=2e-5)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=2e-4 * o.plan.max())
    np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-6)


def test_lbfgs_dual_x0_and_max_iter():
    M, a, b = erot_points(80, 60, seed=7, dtype=np.float64)
    reg = 0.05
    r0 = regot.sinkhorn_lbfgs_dual(M, a, b, reg, tol=1e-8, max_iter=500, precision="fp64")
    r1 = regot.sinkhorn_lbfgs_dual(M, a, b, reg, tol=1e-8, max_iter=500, precision="fp64",
                                   x0=r0.dual)
    assert r1.niter == 1 and len(r1.mar_errs) == 1  # converged at the start
    np.testing.assert_allclose(r1.dual, r0.dual, rtol=0, atol=0)
    r2 = regot.sinkhorn_lbfgs_dual(M, a, b, reg, tol=1e-12, max_iter=3, precision="fp64")
    o2 = O.sinkhorn_lbfgs_dual(M, a, b, reg, tol=1e-12, max_iter=3)
    assert r2.niter == o2.niter == 3 and len(r2.mar_errs) == 4
    np.testing.assert_allclose(r2.mar_errs, o2.mar_errs, rtol=1e-8)


def test_lbfgs_dual_line_search_failure_raises():
    # At tol = 1e-9 the FP64 objective can no longer show a sufficient
    # decrease on this problem: the reference's line search throws
    # (LineSearchNocedalWright.h), which reaches Python as RuntimeError.
    M, a, b = erot_points(80, 60, seed=7, dtype=np.float64)
    with pytest.raises(RuntimeError):
        O.sinkhorn_lbfgs_dual(M, a, b, 0.05, tol=1e-9, max_iter=500)
    # The GPU's FP64 sums round differently, so it may fail a step earlier
    # or later, or reach the tolerance: either way it ends cleanly.
    try:
        r = regot.sinkhorn_lbfgs_dual(M, a, b, 0.05, tol=1e-9, max_iter=500, precision="fp64")
    except RuntimeError as e:
        assert "line search" in str(e)
    else:
        assert r.mar_errs[-1] < 1e-9


APDAGD_CASES = {
    "points-120x90": (lambda: erot_points(120, 90, seed=3, dtype=np.float64), 0.05),
    "readme-0.1": (lambda: readme_example(100, 80), 0.1),
}


@pytest.mark.parametrize("case", list(APDAGD_CASES))
def test_apdagd_fp64_matches_oracle(case):
    make, reg = APDAGD_CASES[case]
    M, a, b = make()
    iters = 60
    r = regot.sinkhorn_apdagd(M, a, b, reg, tol=1e-10, max_iter=iters, precision="fp64")
    o = O.sinkhorn_apdagd(M, a, b, reg, tol=1e-10, max_iter=iters)
    assert r.niter == o.niter == iters
    assert len(r.obj_vals) == len(r.mar_errs) == iters + 1
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-6, atol=1e-13)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-8)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-9 * o.plan.max())


def test_apdagd_mixed_follows_oracle():
    M, a, b = erot_points(120, 90, seed=3, dtype=np.float64)
    Mq = _as_precision(M, "mixed")
    reg = 0.05
    iters = 60
    r = regot.sinkhorn_apdagd(M, a, b, reg, tol=1e-10, max_iter=iters, precision="mixed")
    o = O.sinkhorn_apdagd(Mq, a, b, reg, tol=1e-10, max_iter=iters)
    assert r.niter == o.niter == iters
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-6)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=2e-3, atol=1e-9)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-4)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-4 * o.plan.max())


def test_apdagd_stops_on_gap_and_marginals():
    # A loose tolerance that the oracle meets: the GPU stops at the same
    # iteration (duality gap and marginal error of the averaged plan).
    M, a, b = erot_points(60, 50, seed=11, dtype=np.float64)
    reg = 0.1
    o = O.sinkhorn_apdagd(M, a, b, reg, tol=1e-4, max_iter=2000)
    assert o.niter < 2000
    r = regot.sinkhorn_apdagd(M, a, b, reg, tol=1e-4, max_iter=2000, precision="fp64")
    assert r.niter == o.niter
    assert r.mar_errs[-1] <= 1e-4


def test_apdagd_max_iter_zero():
    M, a, b = erot_points(50, 40, seed=12, dtype=np.float64)
    r = regot.sinkhorn_apdagd(M, a, b, 0.1, max_iter=0, precision="fp64")
    o = O.sinkhorn_apdagd(M, a, b, 0.1, max_iter=0)
    assert r.niter == 0 and len(r.mar_errs) == 1
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-12)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-12 * o.plan.max())
