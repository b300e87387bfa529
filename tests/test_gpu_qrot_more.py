"""Parity of the GPU qrot_bcd, qrot_gd and QROT optimal_alpha with the FP64
oracle restatements (qrot_bcd.cpp:14-103, qrot_gd.cpp:14-120,
qrot_problem.cpp:409-419)."""
import numpy as np
import pytest

import regot_oracle as O
from problems import qrot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qrot_optimal_alpha(precision):
    M, a, b = qrot_points(70, 55, seed=4, dtype=np.float64)
    Mq = _as_precision(M, precision)
    reg = 0.1
    beta = np.random.default_rng(0).normal(0.0, 0.1, 55)
    P = regot.Problem(M, a, b, precision=precision)
    al = P.qrot_optimal_alpha(reg, beta)
    ref = O.qrot_optimal_alpha(Mq, a, reg, beta)
    np.testing.assert_allclose(al, ref, rtol=0, atol=1e-12)
    D = np.maximum(al[:, None] + beta[None, :] - Mq, 0.0)
    np.testing.assert_allclose(D.sum(1), reg * a, rtol=1e-10, atol=1e-15)
    P.close()


CASES = {
    "points-0.1": (lambda: qrot_points(60, 45, seed=3, dtype=np.float64), 0.1),
    "readme-0.1": (lambda: readme_example(100, 80), 0.1),
}


@pytest.mark.parametrize("solver", ["qrot_bcd", "qrot_gd"])
@pytest.mark.parametrize("case", list(CASES))
def test_qrot_first_order_fp64_matches_oracle(solver, case):
    make, reg = CASES[case]
    M, a, b = make()
    iters = 40
    r = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=iters, precision="fp64")
    o = getattr(O, solver)(M, a, b, reg, tol=1e-14, max_iter=iters)
    assert r.niter == o.niter == iters
    assert len(r.obj_vals) == len(r.prim_vals) == len(r.mar_errs) == iters + 1
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(r.prim_vals, o.prim_vals, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-10)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-9 * np.abs(o.plan).max())


@pytest.mark.parametrize("solver", ["qrot_bcd", "qrot_gd"])
def test_qrot_first_order_mixed_follows_oracle(solver):
    M, a, b = qrot_points(60, 45, seed=3, dtype=np.float64)
    Mq = _as_precision(M, "mixed")
    reg, iters = 0.1, 40
    r = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=iters, precision="mixed")
    o = getattr(O, solver)(Mq, a, b, reg, tol=1e-14, max_iter=iters)
    assert r.niter == iters
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-6, atol=1e-10)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-3, atol=1e-7)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-5)


def test_qrot_gd_stops_with_the_oracle():
    # a loose tolerance stops both at the same iteration (tau is not a Python
    # keyword: the reference's parse_qrot_opts reads only method and shift)
    M, a, b = qrot_points(40, 30, seed=5, dtype=np.float64)
    reg = 0.1
    r = regot.qrot_gd(M, a, b, reg, tol=1e-3, max_iter=5000, precision="fp64")
    o = O.qrot_gd(M, a, b, reg, tol=1e-3, max_iter=5000)
    assert r.niter == o.niter < 5000
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-9)
