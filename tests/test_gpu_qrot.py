"""Parity of the GPU QROT passes and solvers (qrot_lbfgs_dual, qrot_assn)
with the FP64 oracle restatement of the reference."""
import numpy as np
import pytest

import regot_oracle as O
from problems import qrot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")

TOL = {"fp64": 1e-10, "mixed": 2e-4}


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


def _small(seed=2):
    M, a, b = qrot_points(130, 97, seed=seed, dtype=np.float64)
    return M, a, b


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qrot_pieces(precision):
    M, a, b = _small()
    Mq = _as_precision(M, precision)
    n, m = M.shape
    reg = 0.1
    P = regot.Problem(M, a, b, precision=precision)
    # optimal_beta: sorted-prefix root vs. Newton from above
    alpha = np.random.default_rng(0).standard_normal(n) * 0.05
    beta_g = P.qrot_optimal_beta(reg, alpha)
    beta_o = O.qrot_optimal_beta(Mq, b, reg, alpha)
    np.testing.assert_allclose(beta_g, beta_o, rtol=0, atol=1e-12)
    gamma = O.qrot_lbfgs_dual(Mq, a, b, reg, tol=1e-6, max_iter=30, plan=False).dual
    f_g, g_g = P.qrot_dual_obj_grad(reg, gamma)
    f_o, g_o = O.qrot_dual_obj_grad(Mq, a, b, reg, gamma)
    assert abs(f_g - f_o) <= TOL[precision] * max(1.0, abs(f_o))
    np.testing.assert_allclose(g_g, g_o, rtol=0, atol=TOL[precision] * max(1e-3, np.abs(g_o).max()))
    pv_g = P.qrot_primal_val(reg, gamma)
    pv_o = O.qrot_primal_val(Mq, a, b, reg, gamma)
    assert abs(pv_g - pv_o) <= 10 * TOL[precision] * max(1.0, abs(pv_o))
    np.testing.assert_allclose(P.qrot_plan(reg, gamma), O.qrot_plan(Mq, reg, gamma), rtol=0,
                               atol=TOL[precision] * 10)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qrot_lbfgs_dual(precision):
    # The L-BFGS path follows the oracle's iteration by iteration until
    # rounding differences of the two summation orders grow; both converge
    # (about 950 iterations here) to the same unique plan.
    M, a, b = _small()
    Mq = _as_precision(M, precision)
    reg = 0.1
    tol = 1e-9 if precision == "fp64" else 1e-7
    r = regot.qrot_lbfgs_dual(M, a, b, reg, tol=tol, max_iter=2000, precision=precision)
    o = O.qrot_lbfgs_dual(Mq, a, b, reg, tol=tol, max_iter=2000)
    L = len(r.mar_errs)
    assert L == len(r.obj_vals) == len(r.prim_vals) == len(r.run_times) == r.niter + 1
    k = min(15, L, len(o.mar_errs))
    rt = 1e-6 if precision == "fp64" else 1e-3
    np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=rt, atol=1e-12)
    np.testing.assert_allclose(r.prim_vals[:k], o.prim_vals[:k], rtol=rt)
    assert r.niter < 2000 and o.niter < 2000
    assert r.mar_errs[-1] * reg <= tol * max(1.0, np.linalg.norm(r.dual))
    np.testing.assert_allclose(r.plan, o.plan, rtol=0,
                               atol=(1e-5 if precision == "fp64" else 1e-3) * o.plan.max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qrot_assn(precision, qrot_cg_path):
    # ASSN converges slowly on this problem; its first iterations follow the
    # oracle (same Newton / projection / gradient decisions), with the CG
    # products on the bitmask and on the index lists.
    M, a, b = _small()
    Mq = _as_precision(M, precision)
    reg = 0.1
    r = regot.qrot_assn(M, a, b, reg, tol=1e-9, max_iter=30, precision=precision)
    o = O.qrot_assn(Mq, a, b, reg, tol=1e-9, max_iter=30)
    assert r.niter == o.niter == 30
    k = 10
    rt = 1e-5 if precision == "fp64" else 1e-2
    np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=rt, atol=1e-12)
    np.testing.assert_allclose(r.prim_vals[:k], o.prim_vals[:k], rtol=rt)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qrot_assn_dense_sigma(precision, qrot_cg_path):
    # reg = 100 with uniform weights: D > 0 on about a fifth of the plan, far
    # above the size-based choice's limit for the index lists; both paths
    # still follow the oracle to convergence.
    M, _, _ = _small(seed=4)
    n, m = M.shape
    a = np.full(n, 1.0 / n)
    b = np.full(m, 1.0 / m)
    Mq = _as_precision(M, precision)
    reg = 100.0
    # FP32 M: ||g|| has a floor near 1e-6 here
    tol = 1e-12 if precision == "fp64" else 1e-5
    r = regot.qrot_assn(M, a, b, reg, tol=tol, max_iter=8, precision=precision)
    o = O.qrot_assn(Mq, a, b, reg, tol=tol, max_iter=8)
    gam = o.dual
    D = gam[:n, None] + gam[None, n:] - Mq
    assert (D > 0).mean() > 0.15
    assert abs(r.niter - o.niter) <= (0 if precision == "fp64" else 1)
    rt = 1e-6 if precision == "fp64" else 1e-3
    k = min(sum(1 for v in o.mar_errs if v > (1e-9 if precision == "fp64" else 1e-6)),
            len(r.mar_errs))
    np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=rt, atol=1e-12)
    np.testing.assert_allclose(r.obj_vals[:k], o.obj_vals[:k], rtol=rt * 1e-2, atol=1e-12)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-8 if precision == "fp64" else 1e-5)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qrot_assn_cg_paths_agree(precision):
    # A larger problem on which the size-based choice takes the index lists:
    # the two CG paths give the same iterates up to the CG tolerance.
    from regot import _lib

    lib = _lib.load()
    M, a, b = qrot_points(700, 520, seed=6, dtype=np.float64)
    reg = 0.05
    runs = {}
    for mode in (1, 2, 3, 0):
        old = lib.regot_force_qrot_cg_path(mode)
        try:
            runs[mode] = regot.qrot_assn(M, a, b, reg, tol=1e-10, max_iter=12,
                                         precision=precision, plan=False)
        finally:
            lib.regot_force_qrot_cg_path(old)
    rt = 1e-6 if precision == "fp64" else 1e-4
    for mode in (2, 3, 0):
        assert runs[mode].niter == runs[1].niter
        np.testing.assert_allclose(runs[mode].mar_errs, runs[1].mar_errs, rtol=rt, atol=1e-12)
        np.testing.assert_allclose(runs[mode].obj_vals, runs[1].obj_vals, rtol=1e-9, atol=1e-12)
    np.testing.assert_array_equal(runs[0].mar_errs, runs[2].mar_errs)


def test_qrot_readme_history():
    M, a, b = readme_example(100, 80)
    r = regot.qrot_lbfgs_dual(M, a, b, 0.1, tol=1e-8, max_iter=60)
    o = O.qrot_lbfgs_dual(M, a, b, 0.1, tol=1e-8, max_iter=60)
    assert r.niter == o.niter
    np.testing.assert_allclose(r.mar_errs[:20], o.mar_errs[:20], rtol=1e-6)
