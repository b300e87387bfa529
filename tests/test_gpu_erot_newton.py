"""Parity of the GPU sinkhorn_newton (matrix-free Newton-CG) with the FP64
oracle, which restates the reference's dense-LLT Newton method."""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("reg", [0.1, 0.05])
def test_sinkhorn_newton_matches_oracle(precision, reg):
    M, a, b = readme_example(100, 80)
    Mq = _as_precision(M, precision)
    tol = 1e-9 if precision == "fp64" else 1e-7
    r = regot.sinkhorn_newton(M, a, b, reg, tol=tol, max_iter=200, precision=precision)
    o = O.sinkhorn_newton(Mq, a, b, reg, tol=tol, max_iter=200)
    assert len(r.mar_errs) == r.niter + 1 == len(r.obj_vals) == len(r.run_times)
    # The CG direction agrees with the LLT direction to its 1e-10 relative
    # residual, so the iterates follow the reference path step for step.
    if precision == "fp64":
        # Up to the last steps, where both marginal errors sit at the rounding
        # floor of the two linear solvers, the histories coincide.
        assert abs(r.niter - o.niter) <= 1
        k = sum(1 for v in o.mar_errs if v > 1e-6)
        np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=1e-5, atol=1e-12)
        k2 = min(len(r.obj_vals), len(o.obj_vals))
        np.testing.assert_allclose(r.obj_vals[:k2], o.obj_vals[:k2], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-7)
    else:
        assert abs(r.niter - o.niter) <= 3
        np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-6)
        # the two solves stop at different points of marginal error < tol:
        # measured 1.9e-6 (reg 0.1) and 3.5e-7 (reg 0.05) of the largest entry
        np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=2e-5 * o.plan.max())
    # Newton's last step overshoots tol: the FP64-evaluated gradient norm of
    # the mixed duals measured 0.22 tol at both regs
    f, g = O.erot_dual_obj_grad(Mq, a, b, reg, r.dual)
    assert np.linalg.norm(g) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_agrees_with_bcd(precision):
    # EROT has a unique plan; both solvers must reach it (cross-solver pin).
    M, a, b = erot_points(150, 120, seed=11, dtype=np.float64)
    reg = 0.05
    rn = regot.sinkhorn_newton(M, a, b, reg, tol=1e-8, max_iter=100, precision=precision)
    rb = regot.sinkhorn_bcd(M, a, b, reg, tol=1e-8, max_iter=5000, precision=precision)
    # mixed measured 6.4e-7 of the largest entry and 3.1e-8 on the duals
    np.testing.assert_allclose(rn.plan, rb.plan, rtol=0, atol=1e-5 * rb.plan.max())
    np.testing.assert_allclose(rn.dual, rb.dual, rtol=0, atol=1e-6)
