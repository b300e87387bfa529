"""Parity of the GPU qrot_apdagd and qrot_pdaam (averaged-plan pass
OP_Q_AVG, exact block minimisations, cancellation-free line-search tests in
mixed precision) with the FP64 oracle restatements (qrot_apdagd.cpp:14-179,
qrot_pdaam.cpp:14-188)."""
import numpy as np
import pytest

import regot_oracle as O
from problems import qrot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")

SOLVERS = ["qrot_apdagd", "qrot_pdaam"]
CASES = {
    "points-0.1": (lambda: qrot_points(60, 45, seed=3, dtype=np.float64), 0.1),
    "readme-0.1": (lambda: readme_example(100, 80), 0.1),
    "points-0.01": (lambda: qrot_points(50, 70, seed=8, dtype=np.float64), 0.01),
}


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("case", list(CASES))
def test_qrot_accelerated_fp64_matches_oracle(solver, case):
    make, reg = CASES[case]
    M, a, b = make()
    iters = 40
    r = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=iters, precision="fp64")
    o = getattr(O, solver)(M, a, b, reg, tol=1e-14, max_iter=iters)
    assert r.niter == o.niter == iters
    assert len(r.obj_vals) == len(r.prim_vals) == len(r.mar_errs) == iters + 1
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(r.prim_vals, o.prim_vals, rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-9)
    # the averaged plan
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-9 * np.abs(o.plan).max())


@pytest.mark.parametrize("solver", SOLVERS)
def test_qrot_accelerated_mixed_follows_oracle(solver):
    M, a, b = qrot_points(60, 45, seed=3, dtype=np.float64)
    Mq = M.astype(np.float32).astype(np.float64)
    reg, iters = 0.1, 40
    r = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=iters, precision="mixed")
    o = getattr(O, solver)(Mq, a, b, reg, tol=1e-14, max_iter=iters)
    assert r.niter == iters
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-6, atol=1e-10)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-3, atol=1e-7)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-5)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-4 * np.abs(o.plan).max())


@pytest.mark.parametrize("solver", SOLVERS)
def test_qrot_accelerated_stops_with_the_oracle(solver):
    # duality-gap and marginal-error stop at a loose tolerance
    M, a, b = qrot_points(40, 30, seed=7, dtype=np.float64)
    reg = 0.1
    tol = 1e-4
    r = getattr(regot, solver)(M, a, b, reg, tol=tol, max_iter=5000, precision="fp64")
    o = getattr(O, solver)(M, a, b, reg, tol=tol, max_iter=5000)
    assert o.niter < 5000 and r.niter < 5000
    # Over ~1000 accelerated iterations FP64 rounding differences (summation
    # order) move the stopping iteration by a few: compare the stops, not
    # the iterates.
    assert abs(r.niter - o.niter) <= max(2, o.niter // 100)
    assert r.mar_errs[-1] <= tol and o.mar_errs[-1] <= tol
    n_same = min(r.niter, o.niter) // 2
    np.testing.assert_allclose(r.obj_vals[:n_same], o.obj_vals[:n_same], rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-3 * np.abs(o.plan).max())


@pytest.mark.parametrize("solver", SOLVERS)
def test_qrot_accelerated_x0_and_no_plan(solver):
    M, a, b = qrot_points(50, 40, seed=9, dtype=np.float64)
    reg = 0.1
    x0 = np.r_[np.full(50, 0.01), np.full(40, 0.02)]
    r = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=15, precision="fp64", x0=x0)
    o = getattr(O, solver)(M, a, b, reg, tol=1e-14, max_iter=15, x0=x0)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-9)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-9 * o.plan.max())
    rn = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=15, precision="fp64", x0=x0,
                                plan=False, prim_vals=False)
    assert rn.plan is None
    np.testing.assert_allclose(rn.dual, r.dual, rtol=0, atol=0)
