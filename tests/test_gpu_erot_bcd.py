"""Parity of the GPU EROT passes and sinkhorn_bcd with the FP64 oracle."""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")

# FP64 storage: every element-wise operation in FP64 -> agreement to ~1e-12.
# Mixed: M rounded to FP32 (the oracle sees the same FP32 values), FP32
# exp2/accumulation: T carries about 1e-7 relative error, so single passes
# agree to a few 1e-7 (measured on a GB300: gradient 2.5e-7 of max a, HVP
# 1.2e-7, plan 4.2e-7, optimal_alpha / _beta 2e-8 of reg x 10), and the
# marginal errors to the FP32 rounding of the row sums (absolute ~1e-9,
# bounded here by MAR_ATOL).
TOL = {"fp64": 1e-10, "mixed": 2e-6}
MAR_ATOL = {"fp64": 1e-12, "mixed": 2e-8}


def _problem(kind):
    if kind == "readme":
        return readme_example(100, 80)
    if kind == "odd":
        M, a, b = erot_points(131, 97, seed=5, dtype=np.float64)
        return M, a, b
    raise ValueError(kind)


def _as_precision(M, precision):
    # Mixed mode computes on FP32 M; give the oracle the same rounded values.
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["readme", "odd"])
def test_optimal_beta_alpha(precision, kind):
    M, a, b = _problem(kind)
    Mq = _as_precision(M, precision)
    P = regot.Problem(M, a, b, precision=precision)
    reg = 0.1
    alpha = np.random.default_rng(0).standard_normal(M.shape[0]) * 0.1
    beta_g = P.erot_optimal_beta(reg, alpha)
    beta_o = O.erot_optimal_beta(Mq, b, reg, alpha)
    np.testing.assert_allclose(beta_g, beta_o, rtol=0, atol=TOL[precision] * reg * 10)
    alpha_g = P.erot_optimal_alpha(reg, beta_o)
    alpha_o = O.erot_optimal_alpha(Mq, a, reg, beta_o)
    np.testing.assert_allclose(alpha_g, alpha_o, rtol=0, atol=TOL[precision] * reg * 10)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dual_obj_grad_hvp_plan(precision):
    M, a, b = _problem("odd")
    Mq = _as_precision(M, precision)
    n, m = M.shape
    reg = 0.05
    P = regot.Problem(M, a, b, precision=precision)
    gamma = O.sinkhorn_bcd(Mq, a, b, reg, tol=1e-3, max_iter=50).dual
    f_g, g_g = P.erot_dual_obj_grad(reg, gamma)
    f_o, g_o = O.erot_dual_obj_grad(Mq, a, b, reg, gamma)
    assert abs(f_g - f_o) <= TOL[precision] * max(1.0, abs(f_o))
    scale = np.abs(a).max()
    np.testing.assert_allclose(g_g, g_o, rtol=0, atol=TOL[precision] * scale)
    x = np.random.default_rng(1).standard_normal(n + m - 1)
    y_g = P.erot_hvp(reg, gamma, x)
    y_o = O.erot_hvp(Mq, a, b, reg, gamma, x)
    np.testing.assert_allclose(y_g, y_o, rtol=0, atol=TOL[precision] * np.abs(y_o).max())
    plan_g = P.erot_plan(reg, gamma)
    plan_o = O.erot_plan(Mq, reg, gamma)
    np.testing.assert_allclose(plan_g, plan_o, rtol=0, atol=TOL[precision] * plan_o.max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("reg", [0.1, 0.01])
def test_sinkhorn_bcd_readme(precision, reg):
    M, a, b = _problem("readme")
    Mq = _as_precision(M, precision)
    tol = 1e-8 if precision == "fp64" else 1e-7
    r = regot.sinkhorn_bcd(M, a, b, reg, tol=tol, max_iter=1000, precision=precision)
    o = O.sinkhorn_bcd(Mq, a, b, reg, tol=tol, max_iter=1000)
    assert len(r.mar_errs) == r.niter + 1 == len(r.obj_vals) == len(r.run_times)
    if precision == "fp64":
        assert r.niter == o.niter
        np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-6, atol=1e-14)
        np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-9)
        np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-9 * o.plan.max())
    else:
        assert abs(r.niter - o.niter) <= max(3, o.niter // 20)
        k = min(len(r.mar_errs), len(o.mar_errs), 20)
        np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=1e-3,
                                   atol=MAR_ATOL["mixed"])
        np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-6)
        # measured 2.7e-7 of the largest entry at both regs
        np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=2e-6 * o.plan.max())
    # the returned dual meets the tolerance when checked in FP64 by the
    # oracle; mixed precision stops on its FP32-summed marginal error, which
    # resolves the FP64 one to 2e-7 |a| (measured at reg 0.1: 1.0023 tol)
    f, g = O.erot_dual_obj_grad(Mq, a, b, reg, r.dual)
    if r.niter < 1000:
        bound = tol if precision == "fp64" else tol + 2e-7 * max(np.linalg.norm(a),
                                                                 np.linalg.norm(b))
        assert np.linalg.norm(g) < bound
    assert all(np.diff(r.run_times) >= 0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sinkhorn_bcd_x0_and_max_iter(precision):
    M, a, b = _problem("odd")
    Mq = _as_precision(M, precision)
    reg = 0.05
    x0 = O.sinkhorn_bcd(Mq, a, b, reg, tol=1e-2, max_iter=5).dual
    r = regot.sinkhorn_bcd(M, a, b, reg, tol=1e-12, max_iter=7, precision=precision, x0=x0)
    o = O.sinkhorn_bcd(Mq, a, b, reg, tol=1e-12, max_iter=7, x0=x0)
    assert r.niter == o.niter == 7
    rt = 1e-8 if precision == "fp64" else 1e-3
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=rt, atol=MAR_ATOL[precision])
    r0 = regot.sinkhorn_bcd(M, a, b, reg, tol=1e-12, max_iter=0, precision=precision)
    assert r0.niter == 0 and len(r0.mar_errs) == 1


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sinkhorn_bcd_fallback_paths(precision):
    # Duals far below their final size (x0 ~ 1e-3, final duals ~ 10) and an
    # iterate whose row sums all underflow (alpha = -40 at reg 0.05, handled
    # by the max-anchored updates): the solve must follow the oracle.
    M, a, b = readme_example(100, 80)
    Mq = _as_precision(M, precision)
    n, m = M.shape
    reg = 0.05
    for x0 in (np.full(n + m - 1, 1e-3), np.r_[np.full(n, -40.0), np.zeros(m - 1)]):
        tol = 1e-10 if precision == "fp64" else 2e-4  # solve tolerance of these runs
        r = regot.sinkhorn_bcd(M, a, b, reg, tol=tol, max_iter=3000, precision=precision, x0=x0)
        o = O.sinkhorn_bcd(Mq, a, b, reg, tol=tol, max_iter=3000, x0=x0)
        assert abs(r.niter - o.niter) <= (1 if precision == "fp64" else 0.05 * o.niter + 3)
        k = min(len(o.mar_errs), len(r.mar_errs), 50)
        rt = 1e-8 if precision == "fp64" else 1e-3
        np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=rt, atol=MAR_ATOL[precision])
        np.testing.assert_allclose(r.plan, o.plan, rtol=0,
                                   atol=(1e-9 if precision == "fp64" else 1e-5) * o.plan.max())
