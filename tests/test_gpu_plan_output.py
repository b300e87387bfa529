"""Plans of at least one MiB come back in page-locked blocks of the library
(regot_host_alloc), which the plan kernels write directly across the
host link. They must equal, bit for bit, the plans written through a device
buffer and a copy into ordinary host memory, and match the oracle."""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, qrot_points

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")
from regot import _lib  # noqa: E402

# 257 x 515 doubles = 1.06 MB (above the page-locked threshold); an odd row
# length makes every other row start off the 16-byte grid, so both the
# vector and the element stores of the plan kernels run.
SHAPE = (257, 515)


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


def _pageable(monkeypatch):
    monkeypatch.setattr(_lib, "PINNED_MIN_BYTES", 1 << 62)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_erot_plan_direct_equals_copied(precision, monkeypatch):
    M, a, b = erot_points(*SHAPE, seed=21, dtype=np.float64)
    Mq = _as_precision(M, precision)
    reg = 0.05
    gamma = O.sinkhorn_bcd(Mq, a, b, reg, tol=1e-3, max_iter=40, plan=False).dual
    P = regot.Problem(M, a, b, precision=precision)
    direct = P.erot_plan(reg, gamma)
    assert direct.nbytes >= _lib.PINNED_MIN_BYTES
    _pageable(monkeypatch)
    copied = P.erot_plan(reg, gamma)
    assert np.array_equal(direct, copied)
    ref = O.erot_plan(Mq, reg, gamma)
    tol = 1e-10 if precision == "fp64" else 2e-4
    np.testing.assert_allclose(direct, ref, rtol=0, atol=tol * ref.max())
    P.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_plan_direct_equals_copied(precision, monkeypatch):
    M, a, b = erot_points(*SHAPE, seed=22, dtype=np.float64)
    reg = 0.05
    r1 = regot.sinkhorn_bcd(M, a, b, reg, tol=1e-7, max_iter=3000, precision=precision)
    _pageable(monkeypatch)
    r2 = regot.sinkhorn_bcd(M, a, b, reg, tol=1e-7, max_iter=3000, precision=precision)
    assert np.array_equal(r1.dual, r2.dual)
    assert np.array_equal(r1.plan, r2.plan)
    ref = O.erot_plan(_as_precision(M, precision), reg, r1.dual)
    tol = 1e-10 if precision == "fp64" else 2e-4
    np.testing.assert_allclose(r1.plan, ref, rtol=0, atol=tol * ref.max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qrot_plan_direct_equals_copied(precision, monkeypatch):
    M, a, b = qrot_points(*SHAPE, seed=23, dtype=np.float64)
    Mq = _as_precision(M, precision)
    reg = 0.1
    gamma = O.qrot_lbfgs_dual(Mq, a, b, reg, tol=1e-6, max_iter=30, plan=False).dual
    P = regot.Problem(M, a, b, precision=precision)
    direct = P.qrot_plan(reg, gamma)
    _pageable(monkeypatch)
    copied = P.qrot_plan(reg, gamma)
    assert np.array_equal(direct, copied)
    ref = O.qrot_plan(Mq, reg, gamma)
    tol = 1e-10 if precision == "fp64" else 2e-4
    np.testing.assert_allclose(direct, ref, rtol=0, atol=tol * np.abs(ref).max())
    P.close()
