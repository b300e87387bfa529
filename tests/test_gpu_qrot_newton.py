"""Parity of the GPU qrot_grssn (shifted semi-smooth Newton on the Schur CG)
and qrot_lbfgs_semi_dual (L-BFGS on alpha with beta = optimal_beta(alpha)
from the root-finding passes) with the FP64 oracle restatements
(qrot_grssn.cpp:16-133, qrot_lbfgs_semi_dual.cpp:84-126)."""
import numpy as np
import pytest

import regot_oracle as O
from problems import qrot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")

CASES = {
    "points-0.1": (lambda: qrot_points(60, 45, seed=3, dtype=np.float64), 0.1),
    "readme-0.1": (lambda: readme_example(100, 80), 0.1),
    "points-0.01": (lambda: qrot_points(50, 70, seed=8, dtype=np.float64), 0.01),
}


@pytest.mark.parametrize("case", list(CASES))
def test_qrot_grssn_fp64_matches_oracle(case, qrot_cg_path):
    make, reg = CASES[case]
    M, a, b = make()
    iters = 8
    r = regot.qrot_grssn(M, a, b, reg, tol=1e-14, max_iter=iters, precision="fp64")
    o = O.qrot_grssn(M, a, b, reg, tol=1e-14, max_iter=iters)
    assert r.niter == o.niter
    # CG to 1e-8 in a different summation order: directions agree to ~1e-8
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-7, atol=1e-14)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-3, atol=1e-9)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-6)


def test_qrot_grssn_converges_with_the_oracle(qrot_cg_path):
    M, a, b = qrot_points(60, 45, seed=3, dtype=np.float64)
    reg = 0.1
    r = regot.qrot_grssn(M, a, b, reg, tol=1e-8, max_iter=500, precision="fp64")
    o = O.qrot_grssn(M, a, b, reg, tol=1e-8, max_iter=500)
    assert o.niter < 500 and abs(r.niter - o.niter) <= 2
    assert r.mar_errs[-1] * reg < 1e-8
    np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-10)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-6)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-5 * o.plan.max())


def test_qrot_grssn_mixed_converges(qrot_cg_path):
    M, a, b = qrot_points(60, 45, seed=3, dtype=np.float64)
    Mq = M.astype(np.float32).astype(np.float64)
    reg = 0.1
    r = regot.qrot_grssn(M, a, b, reg, tol=1e-7, max_iter=500, precision="mixed")
    o = O.qrot_grssn(Mq, a, b, reg, tol=1e-7, max_iter=500)
    assert r.niter < 500 and r.mar_errs[-1] * reg < 1e-7
    np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-6)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-4)


def test_qrot_grssn_shift_kwarg():
    M, a, b = qrot_points(40, 30, seed=5, dtype=np.float64)
    reg = 0.1
    r = regot.qrot_grssn(M, a, b, reg, tol=1e-14, max_iter=3, precision="fp64", shift=1e-1)
    o = O.qrot_grssn(M, a, b, reg, tol=1e-14, max_iter=3, shift=1e-1)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-8, atol=1e-14)


@pytest.mark.parametrize("case", list(CASES))
def test_qrot_semi_dual_fp64_matches_oracle(case):
    make, reg = CASES[case]
    M, a, b = make()
    iters = 25
    r = regot.qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-14, max_iter=iters, precision="fp64")
    o = O.qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-14, max_iter=iters)
    assert r.niter == o.niter
    assert len(r.obj_vals) == len(r.prim_vals) == len(r.mar_errs) == len(o.obj_vals)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-5, atol=1e-10)
    # primal values (approx_proj of the plan) magnify the last digits of the
    # dual at reg = 0.01
    np.testing.assert_allclose(r.prim_vals, o.prim_vals, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-8)
    # plan = (alpha + beta - M)+ / reg: dual rounding over reg
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-6 * o.plan.max())


def test_qrot_semi_dual_mixed_converges():
    M, a, b = qrot_points(60, 45, seed=3, dtype=np.float64)
    Mq = M.astype(np.float32).astype(np.float64)
    reg = 0.1
    r = regot.qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-7, max_iter=1000, precision="mixed")
    o = O.qrot_lbfgs_semi_dual(Mq, a, b, reg, tol=1e-7, max_iter=1000)
    assert r.niter < 1000 and r.mar_errs[-1] * reg <= 1e-7 * max(1.0, np.linalg.norm(r.dual[:60]))
    np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-6)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-4)


def test_qrot_semi_dual_x0():
    M, a, b = qrot_points(50, 40, seed=9, dtype=np.float64)
    reg = 0.1
    x0 = np.r_[np.full(50, 0.01), np.full(40, 5.0)]  # only alpha is used
    r = regot.qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-14, max_iter=10, precision="fp64", x0=x0)
    o = O.qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-14, max_iter=10, x0=x0)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-8)
