"""Parity with the FP64 oracle at the benchmark configurations themselves.

C1  README example, n = 1000, m = 800 (FP64 M): sinkhorn_bcd and
    sinkhorn_ssns at reg 0.1 and 0.01, qrot_lbfgs_dual at reg 0.1, tol 1e-8,
    max_iter 1000.
C2  n = m = 8192, 3-D Gaussian clouds, M = squared distance / max in FP32,
    reg 0.05 and 0.01, tol 1e-6: sinkhorn_bcd against the oracle's BCD on the
    same FP32-rounded M (duals and plan within 1e-6 relative, the marginal
    error re-evaluated in FP64 at most tol); sinkhorn_newton and
    sinkhorn_ssns in mixed precision against the same algorithm in FP64 on
    the GPU (the oracle's dense-LLT Newton at this size is a 1.5 TFLOP
    factorisation per iteration; the FP64 GPU paths are pinned to the oracle
    at small sizes by the other tests).
C3  n = m = 4096 QROT (uniform points, Dirichlet weights), reg 0.1 and
    0.01: qrot_lbfgs_dual and qrot_assn against the oracle run to the same
    iteration count, and the full mixed-precision solve.

"Relative" below means max |x - x_oracle| / max |x_oracle|, after the gauge
beta_m = 0 that both sides return (src/sinkhorn_bcd.cpp:50-51,78).

Mixed precision evaluates T in FP32 (row and column sums to about 1e-7
relative), so the marginal error it reports can differ from the FP64 value
of the same duals by up to about 2e-7 max(|a|_2, |b|_2) (measured: 5.7e-9 on
the C1 marginals, 3e-11 on C2's): 1e-8 for C1, 2.3e-9 for C2. At C2's tol
(1e-6) that is immaterial and the FP64 value is asserted to be at most tol.
C1's tol (1e-8) is at that resolution, so the mixed C1 checks allow tol plus
the resolution term.
"""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, qrot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def rel(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return float(np.abs(x - y).max() / np.abs(y).max())


def fp32_resolution(a, b):
    """Resolution of a marginal error summed in FP32 (see the module notes)."""
    return 2e-7 * max(np.linalg.norm(a), np.linalg.norm(b))


# ---------------------------------------------------------------- C1 ----
@pytest.fixture(scope="module")
def c1():
    return readme_example(1000, 800)


@pytest.mark.parametrize("reg", [0.1, 0.01])
def test_c1_sinkhorn_bcd_fp64(c1, reg):
    M, a, b = c1
    r = regot.sinkhorn_bcd(M, a, b, reg, tol=1e-8, max_iter=1000)
    o = O.sinkhorn_bcd(M, a, b, reg, tol=1e-8, max_iter=1000)
    assert r.niter == o.niter
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-8, atol=0)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-12, atol=0)
    assert rel(r.dual, o.dual) <= 1e-12
    assert rel(r.plan, o.plan) <= 1e-11


@pytest.mark.parametrize("reg", [0.1, 0.01])
def test_c1_sinkhorn_bcd_mixed(c1, reg):
    """FP32 M: the oracle runs on the same FP32-rounded M, to the same
    iteration count as the GPU solve."""
    M, a, b = c1
    Mq = M.astype(np.float32).astype(np.float64)
    tol = 1e-8
    r = regot.sinkhorn_bcd(M, a, b, reg, tol=tol, max_iter=1000, precision="mixed")
    o = O.sinkhorn_bcd(Mq, a, b, reg, tol=0.0, max_iter=r.niter)
    assert rel(r.dual, o.dual) <= 1e-6
    assert rel(r.plan, o.plan) <= 1e-6
    # the oracle's own stopping iteration is the same up to the FP32
    # resolution of the marginal error
    o_stop = O.sinkhorn_bcd(Mq, a, b, reg, tol=tol, max_iter=1000)
    assert abs(o_stop.niter - r.niter) <= max(2, o_stop.niter // 100)
    _, g = O.erot_dual_obj_grad(Mq, a, b, reg, r.dual)
    if r.niter < 1000:
        assert np.linalg.norm(g) <= tol + fp32_resolution(a, b)
    assert abs(np.linalg.norm(g) - r.mar_errs[-1]) <= fp32_resolution(a, b)


def test_c1_sinkhorn_ssns_fp64_reference_cg(c1):
    """method = 0 is the reference's own linear solver (CG on the Schur
    complement, identity preconditioner, tol 1e-8, src/sinkhorn_cg.cpp:9-50).
    CG stops at a relative residual of 1e-8, so two runs that differ only in
    summation order take the same first steps and then drift apart (here by
    one iteration of 62); both reach tol at the same solution. (reg 0.01
    takes the oracle about three minutes and drifts the same way.)"""
    M, a, b = c1
    reg = 0.1
    r = regot.sinkhorn_ssns(M, a, b, reg, tol=1e-8, max_iter=1000, method=0)
    o = O.sinkhorn_ssns(M, a, b, reg, tol=1e-8, max_iter=1000, method=0)
    assert abs(r.niter - o.niter) <= max(2, o.niter // 20)
    np.testing.assert_allclose(r.mar_errs[:10], o.mar_errs[:10], rtol=1e-6, atol=1e-14)
    np.testing.assert_allclose(r.densities[:10], o.densities[:10], rtol=1e-6, atol=0)
    assert r.mar_errs[-1] < 1e-8 and o.mar_errs[-1] < 1e-8
    # Both end below tol, one iteration apart. Solves to 1e-8 that stop at
    # 2 (m - 1) CG steps leave the duals loose along the Hessian's weakest
    # directions, which move single plan entries without moving the
    # marginals: the final plans differ by 9e-5 of the largest entry (the
    # default LDLT-equivalent solve below agrees to 1e-6).
    assert rel(r.plan, o.plan) <= 2e-4


@pytest.mark.parametrize("reg", [0.1, 0.01])
def test_c1_sinkhorn_ssns_fp64_default(c1, reg):
    """method = 1 (default) is a direct SimplicialLDLT solve in the
    reference and preconditioned CG to 1e-10 here: the directions agree to
    that tolerance, so the iteration counts agree to a few percent and both
    final solutions meet tol; the final plans then differ by at most the
    distance between two points of marginal error <= 1e-8 (measured 1.5e-5
    relative at reg 0.01, where the Hessian is worst conditioned)."""
    M, a, b = c1
    r = regot.sinkhorn_ssns(M, a, b, reg, tol=1e-8, max_iter=1000)
    o = O.sinkhorn_ssns(M, a, b, reg, tol=1e-8, max_iter=1000)
    assert abs(r.niter - o.niter) <= max(2, o.niter // 50)
    assert r.mar_errs[-1] < 1e-8 and o.mar_errs[-1] < 1e-8
    assert rel(r.plan, o.plan) <= (1e-6 if reg >= 0.1 else 5e-5)


def test_c1_sinkhorn_ssns_mixed(c1):
    """Mixed precision: the sparsity pattern is chosen from FP32 T, so the
    path differs from the FP64 oracle's; the converged solutions agree."""
    M, a, b = c1
    Mq = M.astype(np.float32).astype(np.float64)
    reg, tol = 0.1, 1e-8
    r = regot.sinkhorn_ssns(M, a, b, reg, tol=tol, max_iter=1000, precision="mixed")
    o = O.sinkhorn_ssns(Mq, a, b, reg, tol=tol, max_iter=1000)
    assert r.niter < 1000
    _, g = O.erot_dual_obj_grad(Mq, a, b, reg, r.dual)
    assert np.linalg.norm(g) <= tol + fp32_resolution(a, b)
    assert rel(r.plan, o.plan) <= 1e-5


def test_c1_qrot_lbfgs_dual(c1):
    """L-BFGS at reg 0.1 does not reach 1e-8 in 1000 iterations on this
    problem (neither does the oracle). In FP64 the first 30 iterations
    coincide with the oracle's to 1e-9 (summation-order differences grow
    from 1e-15 by about a factor of two per iteration; by iteration 35 they
    reach 1e-9). In mixed precision the FP32 sums perturb the first
    gradients by about 1e-7 relative and the iteration amplifies that the same
    way: 3e-6 by iteration 7, 7e-5 by iteration 12; the first 8 iterations are
    compared."""
    M, a, b = c1
    reg = 0.1
    r = regot.qrot_lbfgs_dual(M, a, b, reg, tol=0.0, max_iter=30)
    o = O.qrot_lbfgs_dual(M, a, b, reg, tol=0.0, max_iter=30)
    assert r.niter == o.niter == 30
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-9, atol=0)
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-6, atol=0)
    assert rel(r.dual, o.dual) <= 1e-7
    Mq = M.astype(np.float32).astype(np.float64)
    rm = regot.qrot_lbfgs_dual(M, a, b, reg, tol=0.0, max_iter=8, precision="mixed")
    om = O.qrot_lbfgs_dual(Mq, a, b, reg, tol=0.0, max_iter=8)
    np.testing.assert_allclose(rm.obj_vals, om.obj_vals, rtol=2e-5, atol=0)
    assert rel(rm.dual, om.dual) <= 1e-4
    full = regot.qrot_lbfgs_dual(M, a, b, reg, tol=1e-8, max_iter=1000, plan=False)
    _, g = O.qrot_dual_obj_grad(M, a, b, reg, full.dual)
    np.testing.assert_allclose(np.linalg.norm(g) / reg, full.mar_errs[-1], rtol=1e-9)


# ---------------------------------------------------------------- C2 ----
@pytest.fixture(scope="module")
def c2():
    M, a, b = erot_points(8192, 8192, seed=0, dtype=np.float32)
    Mq = np.asfortranarray(M.astype(np.float64))
    P = regot.Problem(M, a, b, precision="mixed")
    P64 = regot.Problem(Mq, a, b, precision="fp64")
    yield M, Mq, a, b, P, P64
    P.close()
    P64.close()


@pytest.mark.parametrize("reg", [0.05, 0.01])
def test_c2_sinkhorn_bcd_mixed_vs_oracle(c2, reg):
    M, Mq, a, b, P, P64 = c2
    tol = 1e-6
    r = P.sinkhorn_bcd(reg, tol=tol, max_iter=1000)
    o = O.sinkhorn_bcd(Mq, a, b, reg, tol=tol, max_iter=1000)
    assert r.niter == o.niter
    assert rel(r.dual, o.dual) <= 1e-6
    assert rel(r.plan, o.plan) <= 1e-6
    np.testing.assert_allclose(r.mar_errs, o.mar_errs, rtol=1e-4, atol=0)
    # the marginal error of the returned duals, in FP64 on the same M
    _, g = P64.erot_dual_obj_grad(reg, r.dual)
    assert np.linalg.norm(g) <= tol
    # the plain FP64 GPU solve is the oracle's arithmetic
    r64 = P64.sinkhorn_bcd(reg, tol=tol, max_iter=1000, plan=False)
    assert r64.niter == o.niter
    assert rel(r64.dual, o.dual) <= 1e-12


@pytest.mark.parametrize("reg", [0.05, 0.01])
@pytest.mark.parametrize("solver", ["sinkhorn_newton", "sinkhorn_ssns"])
def test_c2_second_order_mixed_vs_fp64(c2, solver, reg):
    M, Mq, a, b, P, P64 = c2
    tol = 1e-6
    r = getattr(P, solver)(reg, tol=tol, max_iter=200, plan=False)
    r64 = getattr(P64, solver)(reg, tol=tol, max_iter=200, plan=False)
    assert r.niter == r64.niter < 200
    np.testing.assert_allclose(r.mar_errs, r64.mar_errs, rtol=2e-3, atol=0)
    assert rel(r.dual, r64.dual) <= 1e-6
    _, g = P64.erot_dual_obj_grad(reg, r.dual)
    assert np.linalg.norm(g) <= tol


# ---------------------------------------------------------------- C3 ----
@pytest.fixture(scope="module")
def c3():
    M, a, b = qrot_points(4096, 4096, seed=1, dtype=np.float32)
    Mq = np.asfortranarray(M.astype(np.float64))
    P = regot.Problem(M, a, b, precision="mixed")
    P64 = regot.Problem(Mq, a, b, precision="fp64")
    yield M, Mq, a, b, P, P64
    P.close()
    P64.close()


@pytest.mark.parametrize("reg", [0.1, 0.01])
def test_c3_qrot_lbfgs_dual(c3, reg):
    M, Mq, a, b, P, P64 = c3
    k = 30
    o = O.qrot_lbfgs_dual(Mq, a, b, reg, tol=0.0, max_iter=k, plan=False)
    r64 = P64.qrot_lbfgs_dual(reg, tol=0.0, max_iter=k, plan=False)
    np.testing.assert_allclose(r64.obj_vals, o.obj_vals, rtol=1e-12, atol=0)
    np.testing.assert_allclose(r64.mar_errs, o.mar_errs, rtol=1e-9, atol=0)
    assert rel(r64.dual, o.dual) <= 1e-10
    r = P.qrot_lbfgs_dual(reg, tol=0.0, max_iter=k, plan=False)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-5, atol=0)
    assert rel(r.dual, o.dual) <= 1e-4
    # the full solve stops by LBFGS++'s test |g| <= tol max(1, |x|)
    # (src/LBFGSpp/LBFGS.h:110-112), and its reported marginal error is the
    # FP64 one of its duals
    full = P.qrot_lbfgs_dual(reg, tol=1e-6, max_iter=20000, plan=False, prim_vals=False)
    assert full.niter < 20000
    _, g = P64.qrot_dual_obj_grad(reg, full.dual)
    # the FP32 row / column sums of D resolve |g| to about 1e-7 reg |(a, b)|
    res = 2e-7 * reg * max(np.linalg.norm(a), np.linalg.norm(b))
    assert abs(np.linalg.norm(g) - reg * full.mar_errs[-1]) <= res
    assert np.linalg.norm(g) <= 1e-6 * max(1.0, np.linalg.norm(full.dual)) + res


@pytest.mark.parametrize("reg", [0.1, 0.01])
def test_c3_qrot_assn(c3, reg):
    M, Mq, a, b, P, P64 = c3
    k = 5
    o = O.qrot_assn(Mq, a, b, reg, tol=0.0, max_iter=k, plan=False)
    r64 = P64.qrot_assn(reg, tol=0.0, max_iter=k, plan=False)
    assert r64.niter == o.niter == k
    np.testing.assert_allclose(r64.obj_vals, o.obj_vals, rtol=1e-10, atol=0)
    np.testing.assert_allclose(r64.mar_errs, o.mar_errs, rtol=1e-7, atol=0)
    assert rel(r64.dual, o.dual) <= 1e-8
    r = P.qrot_assn(reg, tol=0.0, max_iter=k, plan=False)
    np.testing.assert_allclose(r.obj_vals, o.obj_vals, rtol=1e-5, atol=0)
    assert rel(r.dual, o.dual) <= 1e-4
