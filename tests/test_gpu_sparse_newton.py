"""Parity of the GPU sinkhorn_sparse_newton and sinkhorn_splr, and of the
density sparsification (sparsify_mat_with_density), with the FP64 oracle
restatements (sinkhorn_sparse_newton.cpp:24-171, sinkhorn_splr.cpp:24-200,
sinkhorn_sparsify4.cpp:77-174, sinkhorn_problem_ls.cpp:226-436)."""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


def _oracle_kept(T, density):
    n, m = T.shape
    outer, inner, _ = O.sparsify_density(T, density)
    K = np.zeros((n, m - 1), dtype=bool)
    for j in range(m - 1):
        K[inner[outer[j]:outer[j + 1]], j] = True
    return K


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("density", [0.0, 1e-4, 0.001, 0.01, 0.2, 1.0])
def test_sparsify_density_pattern(precision, density):
    M, a, b = erot_points(300, 257, seed=5, dtype=np.float64)
    Mq = _as_precision(M, precision)
    reg = 0.02
    gamma = O.sinkhorn_bcd(Mq, a, b, reg, tol=1e-14, max_iter=4, plan=False).dual
    T = O.erot_compute_T(Mq, reg, gamma)
    K_o = _oracle_kept(T, density) & (T[:, :-1] != 0)
    P = regot.Problem(M, a, b, precision=precision)
    nnz_g, K_g = P.erot_sparsify_density(reg, gamma, density)
    assert nnz_g == np.count_nonzero(K_g)
    # row 0 and column 0 always
    assert np.array_equal(K_g[0], T[0, :-1] != 0) and np.array_equal(K_g[:, 0], T[:, 0] != 0)
    bad = np.count_nonzero(K_g != K_o)
    if precision == "fp64":
        # CUDA's exp and the C library's may differ in the last ulp: only
        # the entries at the threshold can change sides
        assert bad <= 2, bad
    else:
        # FP32 T: ties at the FP32 threshold are all kept, and values within
        # FP32 rounding of it can change sides
        assert bad <= max(5, 2e-3 * np.count_nonzero(K_o)), bad
    P.close()


CASES = {
    "points-0.1": (lambda: erot_points(60, 50, seed=11, dtype=np.float64), 0.1, 0.5),
    "readme-0.1": (lambda: readme_example(100, 80), 0.1, 0.01),
    "points-0.02": (lambda: erot_points(80, 70, seed=3, dtype=np.float64), 0.02, 0.1),
}


@pytest.mark.parametrize("solver", ["sinkhorn_sparse_newton", "sinkhorn_splr"])
@pytest.mark.parametrize("case", list(CASES))
def test_sparse_newton_fp64_matches_oracle(solver, case):
    make, reg, density = CASES[case]
    M, a, b = make()
    iters = 12
    r = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=iters, precision="fp64",
                               density=density)
    o = getattr(O, solver)(M, a, b, reg, tol=1e-14, max_iter=iters, density=density)
    assert r.niter == o.niter
    # direct solves: the oracle's Cholesky against Jacobi PCG to 1e-10
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-4, atol=1e-12)
    np.testing.assert_allclose(r.densities, o.densities, rtol=1e-12)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-6)


@pytest.mark.parametrize("solver", ["sinkhorn_sparse_newton", "sinkhorn_splr"])
def test_sparse_newton_cg_method_matches_oracle(solver):
    M, a, b = erot_points(60, 50, seed=11, dtype=np.float64)
    reg = 0.1
    r = getattr(regot, solver)(M, a, b, reg, tol=1e-14, max_iter=8, precision="fp64",
                               density=0.5, method=0)
    o = getattr(O, solver)(M, a, b, reg, tol=1e-14, max_iter=8, density=0.5, method=0)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=1e-5)


@pytest.mark.parametrize("solver,tol", [("sinkhorn_sparse_newton", 1e-7),
                                        ("sinkhorn_splr", 1e-8)])
def test_sparse_newton_converges_with_the_oracle(solver, tol):
    M, a, b = erot_points(40, 30, seed=12, dtype=np.float64)
    reg = 0.1
    r = getattr(regot, solver)(M, a, b, reg, tol=tol, max_iter=2000, precision="fp64",
                               density=0.5)
    o = getattr(O, solver)(M, a, b, reg, tol=tol, max_iter=2000, density=0.5)
    assert r.niter < 2000 and r.mar_errs[-1] < tol
    assert abs(r.niter - o.niter) <= max(2, o.niter // 20)
    np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-10)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-5 * o.plan.max())


@pytest.mark.parametrize("solver", ["sinkhorn_sparse_newton", "sinkhorn_splr"])
def test_sparse_newton_mixed_converges(solver):
    M, a, b = erot_points(80, 70, seed=3, dtype=np.float64)
    Mq = M.astype(np.float32).astype(np.float64)
    reg = 0.05
    tol = 1e-6
    r = getattr(regot, solver)(M, a, b, reg, tol=tol, max_iter=3000, precision="mixed",
                               density=0.2)
    o = getattr(O, solver)(Mq, a, b, reg, tol=tol, max_iter=3000, density=0.2)
    assert r.niter < 3000 and r.mar_errs[-1] < tol
    np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-7)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-4 * o.plan.max())
