"""Derivatives of EROT solves: the Hessian solve and the fused weighted-plan
contraction against the FP64 oracle, and the regot.torch autograd wrappers
against FP64 finite differences (no reference counterpart: the reference has
no derivatives)."""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")
torch = pytest.importorskip("torch")
rt = pytest.importorskip("regot.torch")


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


def _solved(n, m, seed, reg, precision="fp64"):
    M, a, b = erot_points(n, m, seed=seed, dtype=np.float64)
    Mq = _as_precision(M, precision)
    gamma = O.sinkhorn_bcd(Mq, a, b, reg, tol=1e-10, max_iter=5000, plan=False).dual
    return M, Mq, a, b, gamma


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hess_solve(precision):
    reg = 0.05
    M, Mq, a, b, gamma = _solved(90, 70, 31, reg, precision)
    P = regot.Problem(M, a, b, precision=precision)
    rhs = np.random.default_rng(1).standard_normal(gamma.size)
    tol = 1e-10 if precision == "fp64" else 1e-6
    x, it = P.erot_hess_solve(reg, gamma, rhs, tol=tol)
    assert 0 < it <= 2 * gamma.size
    r = O.erot_hvp(Mq, a, b, reg, gamma, x) - rhs
    assert np.linalg.norm(r) <= (10 if precision == "fp64" else 50) * tol * np.linalg.norm(rhs)
    P.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("adjoint", [False, True])
def test_tyy_matches_oracle(precision, adjoint):
    reg = 0.05
    n, m, d = 130, 75, 70  # d > 64: two slices of Y
    M, Mq, a, b, gamma = _solved(n, m, 32, reg, precision)
    rng = np.random.default_rng(2)
    Y = rng.standard_normal((m, d))
    T = O.erot_plan(Mq, reg, gamma)
    P = regot.Problem(M, a, b, precision=precision)
    if adjoint:
        u = rng.standard_normal(n + m - 1)
        W = rng.standard_normal((n, m))
        uu = np.r_[u, 0.0]
        G = T * (uu[:n, None] + uu[None, n:] - W) / reg
        rows, Z = P.erot_tyy(reg, gamma, Y, u=u, W=W)
    else:
        G = T
        rows, Z = P.erot_tyy(reg, gamma, Y)
    tol = 1e-11 if precision == "fp64" else 2e-5
    np.testing.assert_allclose(rows, G.sum(1), rtol=0, atol=tol * np.abs(G).sum(1).max())
    np.testing.assert_allclose(Z, G @ Y, rtol=0, atol=tol * (np.abs(G) @ np.abs(Y)).max())
    # the device path gives the same numbers
    dev = torch.device("cuda")
    t = lambda v: torch.from_numpy(np.ascontiguousarray(v)).to(dev)  # noqa: E731
    rows_d, Z_d = P.erot_tyy(reg, t(gamma), t(Y), u=t(u) if adjoint else None,
                             W=t(W) if adjoint else None)
    np.testing.assert_array_equal(rows_d.cpu().numpy(), rows)
    np.testing.assert_array_equal(Z_d.cpu().numpy(), Z)
    P.close()


def _cuda64(x):
    return torch.tensor(x, dtype=torch.float64, device="cuda")


def test_ot_cost_gradients_match_finite_differences():
    reg = 0.05
    M, a, b = erot_points(30, 25, seed=33, dtype=np.float64)
    Mt = _cuda64(M).requires_grad_(True)
    at = _cuda64(a).requires_grad_(True)
    bt = _cuda64(b).requires_grad_(True)
    L = rt.ot_cost(Mt, at, bt, reg, tol=1e-12)
    L.backward()
    f = lambda MM, aa, bb: float(rt.ot_cost(_cuda64(MM), _cuda64(aa), _cuda64(bb), reg,  # noqa
                                            tol=1e-12))
    h = 1e-5
    for (i, j) in [(0, 0), (3, 7), (29, 24), (12, 5)]:
        E = np.zeros_like(M)
        E[i, j] = h
        fd = (f(M + E, a, b) - f(M - E, a, b)) / (2 * h)
        np.testing.assert_allclose(Mt.grad[i, j].item(), fd, rtol=1e-5, atol=1e-12)
    for (i, k) in [(0, 1), (4, 20)]:
        e = np.zeros_like(a)
        e[i], e[k] = h, -h
        fd = (f(M, a + e, b) - f(M, a - e, b)) / (2 * h)
        np.testing.assert_allclose((at.grad[i] - at.grad[k]).item(), fd, rtol=1e-5, atol=1e-10)
        e = np.zeros_like(b)
        e[i], e[k] = h, -h
        fd = (f(M, a, b + e) - f(M, a, b - e)) / (2 * h)
        np.testing.assert_allclose((bt.grad[i] - bt.grad[k]).item(), fd, rtol=1e-5, atol=1e-10)


def test_sqeuclid_cost_dx_matches_finite_differences():
    # n = m = 256 points in d = 8, FP64 (the differentiable-loss check). With
    # scale 64 the costs stay below 1.2; at scale 8 (costs up to 9, M/reg up
    # to 185) the reference's first full Newton step already overflows.
    rng = np.random.default_rng(3)
    n, d, scale, reg = 256, 8, 64.0, 0.05
    x = rng.standard_normal((n, d))
    y = rng.standard_normal((n, d))
    a = np.full(n, 1.0 / n)
    b = np.full(n, 1.0 / n)
    xt = _cuda64(x).requires_grad_(True)
    L = rt.sqeuclid_ot_cost(xt, _cuda64(y), _cuda64(a), _cuda64(b), reg, scale=scale, tol=1e-12)
    L.backward()
    f = lambda xx: float(rt.sqeuclid_ot_cost(_cuda64(xx), _cuda64(y), _cuda64(a), _cuda64(b),  # noqa
                                             reg, scale=scale, tol=1e-12))
    h = 1e-5
    for (i, k) in [(0, 0), (17, 3), (255, 7), (100, 5)]:
        e = np.zeros_like(x)
        e[i, k] = h
        fd = (f(x + e) - f(x - e)) / (2 * h)
        np.testing.assert_allclose(xt.grad[i, k].item(), fd, rtol=1e-4, atol=1e-9)


def test_plan_loss_implicit_gradients_match_finite_differences():
    rng = np.random.default_rng(4)
    n, m, d, scale, reg = 64, 48, 8, 8.0, 0.05
    x = rng.standard_normal((n, d))
    y = rng.standard_normal((m, d))
    a = np.full(n, 1.0 / n)
    b = np.full(m, 1.0 / m)
    W = _cuda64(rng.standard_normal((n, m)))
    xt = _cuda64(x).requires_grad_(True)
    at = _cuda64(a).requires_grad_(True)
    L = rt.sqeuclid_plan_loss(xt, _cuda64(y), at, _cuda64(b), reg, W, scale=scale, tol=1e-12)
    L.backward()
    f = lambda xx, aa: float(rt.sqeuclid_plan_loss(  # noqa: E731
        _cuda64(xx), _cuda64(y), _cuda64(aa), _cuda64(b), reg, W, scale=scale, tol=1e-12))
    h = 1e-5
    for (i, k) in [(0, 0), (9, 4), (63, 7)]:
        e = np.zeros_like(x)
        e[i, k] = h
        fd = (f(x + e, a) - f(x - e, a)) / (2 * h)
        np.testing.assert_allclose(xt.grad[i, k].item(), fd, rtol=1e-4, atol=1e-8)
    for (i, k) in [(0, 1), (30, 50)]:
        e = np.zeros_like(a)
        e[i], e[k] = h, -h
        fd = (f(x, a + e) - f(x, a - e)) / (2 * h)
        np.testing.assert_allclose((at.grad[i] - at.grad[k]).item(), fd, rtol=1e-4, atol=1e-8)
    # ot_plan composed with the same cost through torch autograd agrees
    xt2 = _cuda64(x).requires_grad_(True)
    yt = _cuda64(y)
    Mx = ((xt2[:, None, :] - yt[None, :, :]) ** 2).sum(-1) / scale
    T = rt.ot_plan(Mx, _cuda64(a), _cuda64(b), reg, tol=1e-12)
    (W * T).sum().backward()
    np.testing.assert_allclose(xt2.grad.cpu().numpy(), xt.grad.cpu().numpy(), rtol=1e-6,
                               atol=1e-10)
