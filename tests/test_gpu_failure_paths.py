"""Failure paths, injected on the host: invalid inputs and a bounded wait
that runs out.

The reference validates nothing (src/solvers.cpp:463-528 pass the arrays
straight to Eigen) and reports NaN iterates only through its own checks,
e.g. the !isfinite(f) break of src/sinkhorn_newton.cpp:87. This build
rejects bad inputs when the problem is created (ValueError, as pybind11
maps std::invalid_argument), and a dense pass whose bounded wait on its
parameter copies gives up makes the call return REGOT_ERR_TIMEOUT
(RuntimeError) with the context still usable. The wait is made to give up by
lowering its poll limit to 0 (regot_set_wait_limit); the copies are valid
and still land, so nothing on the GPU faults or hangs.
"""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, qrot_points

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def _small(dtype=np.float64):
    return erot_points(40, 30, seed=11, dtype=dtype)


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_cost_is_rejected(bad, precision):
    M, a, b = _small()
    M = M.copy()
    M[7, 3] = bad
    with pytest.raises(ValueError, match="finite"):
        regot.sinkhorn_bcd(M, a, b, 0.1, precision=precision)
    with pytest.raises(ValueError, match="finite"):
        regot.Problem(M, a, b, precision=precision)


def test_cost_beyond_fp32_range_is_rejected_in_mixed_precision():
    M, a, b = _small()
    M = M.copy()
    M[0, 0] = 1e300  # finite in FP64, an infinity once stored in FP32
    with pytest.raises(ValueError, match="FP32"):
        regot.Problem(M, a, b, precision="mixed")
    regot.Problem(M, a, b, precision="fp64").close()  # fine in FP64 storage


def test_nonfinite_cost_on_the_device_is_rejected():
    torch = pytest.importorskip("torch")
    M, a, b = _small(np.float32)
    Md = torch.from_numpy(M).cuda()
    Md[3, 4] = float("nan")
    with pytest.raises(ValueError, match="finite"):
        regot.Problem(Md, a, b, precision="mixed")


@pytest.mark.parametrize("which", ["a", "b"])
@pytest.mark.parametrize("value", [0.0, -1e-3, np.nan])
def test_bad_marginals_are_rejected(which, value):
    M, a, b = _small()
    a, b = a.copy(), b.copy()
    (a if which == "a" else b)[2] = value
    for solver in (regot.sinkhorn_bcd, regot.sinkhorn_newton, regot.qrot_lbfgs_dual):
        with pytest.raises(ValueError, match="positive"):
            solver(M, a, b, 0.1)


def test_shape_mismatch_is_rejected():
    M, a, b = _small()
    for solver in (regot.sinkhorn_bcd, regot.sinkhorn_ssns, regot.qrot_assn):
        with pytest.raises(ValueError):
            solver(M, a[:-1], b, 0.1)
        with pytest.raises(ValueError):
            solver(M, a, np.r_[b, 0.1], 0.1)
        with pytest.raises(ValueError):
            solver(M.ravel(), a, b, 0.1)


def test_bad_scalar_arguments_are_rejected():
    M, a, b = _small()
    with pytest.raises(ValueError):
        regot.sinkhorn_bcd(M, a, b, -0.1)
    with pytest.raises(ValueError):
        regot.sinkhorn_bcd(M, a, b, np.nan)
    with pytest.raises(ValueError):
        regot.sinkhorn_bcd(M, a, b, 0.1, max_iter=-1)
    with pytest.raises(ValueError):
        regot.sinkhorn_bcd(M, a, b, 0.1, precision="fp16")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bounded_wait_that_runs_out_reports_timeout(precision):
    """A wait limit of 0 makes every parameter-copy wait of a mixed pass give
    up at once: the pass records it, drains the copy and the call returns
    REGOT_ERR_TIMEOUT. With the limit restored the same context computes the
    oracle's values again. (FP64 passes stage no parameters, so they never
    wait and are unaffected.)"""
    from regot import _lib

    lib = _lib.load()
    M, a, b = erot_points(300, 260, seed=4, dtype=np.float32)
    Mq = M.astype(np.float64)
    P = regot.Problem(M, a, b, precision=precision)
    reg = 0.05
    gamma = np.random.default_rng(2).standard_normal(300 + 260 - 1) * 0.02
    old = lib.regot_set_wait_limit(0)
    try:
        if precision == "mixed":
            with pytest.raises(RuntimeError, match="gave up"):
                P.erot_dual_obj_grad(reg, gamma)
            with pytest.raises(RuntimeError, match="gave up"):
                P.sinkhorn_bcd(reg, tol=1e-6, max_iter=20)
        else:
            P.erot_dual_obj_grad(reg, gamma)
    finally:
        assert lib.regot_set_wait_limit(old) == 0
    assert lib.regot_set_wait_limit(-1) == old  # default restored
    f, g = P.erot_dual_obj_grad(reg, gamma)
    f_o, g_o = O.erot_dual_obj_grad(Mq, a, b, reg, gamma)
    # random duals: the row and column sums of T are O(100) here, so the
    # gradient is compared relative to its own size
    tol = 1e-13 if precision == "fp64" else 1e-6
    assert abs(f - f_o) <= tol * max(1.0, abs(f_o))
    np.testing.assert_allclose(g, g_o, rtol=0, atol=tol * np.abs(g_o).max())
    P.close()


def test_qrot_bounded_wait_that_runs_out_reports_timeout():
    from regot import _lib

    lib = _lib.load()
    M, a, b = qrot_points(200, 150, seed=3, dtype=np.float32)
    P = regot.Problem(M, a, b, precision="mixed")
    gamma = np.full(350, 0.05)
    old = lib.regot_set_wait_limit(0)
    try:
        with pytest.raises(RuntimeError, match="gave up"):
            P.qrot_dual_obj_grad(0.1, gamma)
    finally:
        lib.regot_set_wait_limit(old)
    f, g = P.qrot_dual_obj_grad(0.1, gamma)
    f_o, g_o = O.qrot_dual_obj_grad(M.astype(np.float64), a, b, 0.1, gamma)
    assert abs(f - f_o) <= 1e-6 * max(1.0, abs(f_o))
    P.close()
