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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("adjoint", [False, True])
@pytest.mark.parametrize("shape", [(130, 75, 70), (300, 257, 8), (40, 520, 64)])
def test_tty_matches_oracle(precision, adjoint, shape):
    """Column-side contraction cols = G'1, Z = G'X (tensor cores for FP32
    storage: BF16 hi/lo split operands, FP32 accumulation, so about 1e-5 of
    sum |G||X|; FP64 storage to rounding)."""
    reg = 0.05
    n, m, d = shape
    M, Mq, a, b, gamma = _solved(n, m, 34, reg, precision)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((n, d))
    T = O.erot_plan(Mq, reg, gamma)
    P = regot.Problem(M, a, b, precision=precision)
    if adjoint:
        u = rng.standard_normal(n + m - 1)
        W = rng.standard_normal((n, m))
        uu = np.r_[u, 0.0]
        G = T * (uu[:n, None] + uu[None, n:] - W) / reg
        cols, Z = P.erot_tty(reg, gamma, X, u=u, W=W)
    else:
        G = T
        cols, Z = P.erot_tty(reg, gamma, X)
    tol = 1e-11 if precision == "fp64" else 2e-5
    np.testing.assert_allclose(cols, G.sum(0), rtol=0, atol=tol * np.abs(G).sum(0).max())
    np.testing.assert_allclose(Z, G.T @ X, rtol=0, atol=tol * (np.abs(G).T @ np.abs(X)).max())
    rows, Zr = P.erot_tyy(reg, gamma, X[:m] if n >= m else np.resize(X, (m, d)),
                          u=u if adjoint else None, W=W if adjoint else None)
    np.testing.assert_allclose(rows, G.sum(1), rtol=0, atol=tol * np.abs(G).sum(1).max())
    P.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sqeuclid_cost_kernel(dtype):
    from regot import _lib
    import ctypes as C

    rng = np.random.default_rng(6)
    n, m, d, scale = 150, 97, 70, 1.0 / 64
    x = rng.standard_normal((n, d)).astype(dtype)
    y = rng.standard_normal((m, d)).astype(dtype)
    ref = ((x.astype(np.float64)[:, None, :] - y.astype(np.float64)[None, :, :]) ** 2).sum(-1)
    ref *= scale
    xt, yt = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    Mt = torch.empty((n, m), dtype=xt.dtype, device="cuda")
    ctx = _lib.context(0)
    ctx.check(_lib.load().regot_sqeuclid_cost(
        ctx.handle, C.c_void_p(xt.data_ptr()), C.c_void_p(yt.data_ptr()), n, m, d, scale,
        _lib.REGOT_F64 if dtype == np.float64 else _lib.REGOT_F32, C.c_void_p(Mt.data_ptr()), m))
    torch.cuda.synchronize()
    got = Mt.cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(got, ref, rtol=1e-13 if dtype == np.float64 else 2e-6, atol=0)


def _cuda64(x):
    return torch.tensor(x, dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sqeuclid_gradients_match_the_oracle_solve(precision):
    """dL/dx and dL/dy of the differentiable OT cost against the gradient
    formed from the oracle's own solve: duals of the FP64 oracle's Newton
    iteration on the same cost matrix, its plan T, dL/dx = 2 (T1 o x - T y)
    / scale and dL/dy = 2 (T'1 o y - T'x) / scale in FP64. FP32 points (mixed)
    are compared with 1e-4 of the largest gradient entry: the FP32 cost and
    the BF16x3 tensor-core contraction move the result by a few 1e-6."""
    rng = np.random.default_rng(7)
    n, m, d, scale, reg = 256, 200, 8, 64.0, 0.05
    dt = np.float64 if precision == "fp64" else np.float32
    x = rng.standard_normal((n, d)).astype(dt)
    y = rng.standard_normal((m, d)).astype(dt)
    a = np.full(n, 1.0 / n)
    b = np.full(m, 1.0 / m)
    xt = torch.from_numpy(x).cuda().requires_grad_(True)
    yt = torch.from_numpy(y).cuda().requires_grad_(True)
    L = rt.sqeuclid_ot_cost(xt, yt, _cuda64(a), _cuda64(b), reg, scale=scale,
                            tol=1e-12 if precision == "fp64" else 1e-8)
    L.backward()
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    M = ((x64[:, None, :] - y64[None, :, :]) ** 2).sum(-1) / scale
    if precision == "mixed":
        M = M.astype(np.float32).astype(np.float64)
    o = O.sinkhorn_newton(M, a, b, reg, tol=1e-12, max_iter=200)
    T = O.erot_plan(M, reg, o.dual)
    gx = 2.0 * (T.sum(1)[:, None] * x64 - T @ y64) / scale
    gy = 2.0 * (T.sum(0)[:, None] * y64 - T.T @ x64) / scale
    tol = 1e-8 if precision == "fp64" else 1e-4
    np.testing.assert_allclose(xt.grad.cpu().numpy(), gx, rtol=0, atol=tol * np.abs(gx).max())
    np.testing.assert_allclose(yt.grad.cpu().numpy(), gy, rtol=0, atol=tol * np.abs(gy).max())
    assert abs(L.item() + o.obj_vals[-1]) <= (1e-10 if precision == "fp64" else 1e-6)


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
    # dL/dy through the column-side contraction
    yt = _cuda64(y).requires_grad_(True)
    L = rt.sqeuclid_ot_cost(_cuda64(x), yt, _cuda64(a), _cuda64(b), reg, scale=scale, tol=1e-12)
    L.backward()
    g = lambda yy: float(rt.sqeuclid_ot_cost(_cuda64(x), _cuda64(yy), _cuda64(a), _cuda64(b),  # noqa
                                             reg, scale=scale, tol=1e-12))
    for (j, k) in [(0, 0), (31, 6), (255, 2)]:
        e = np.zeros_like(y)
        e[j, k] = h
        fd = (g(y + e) - g(y - e)) / (2 * h)
        np.testing.assert_allclose(yt.grad[j, k].item(), fd, rtol=1e-4, atol=1e-9)


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
    # dL/dy of the plan loss (column-side contraction with the adjoint)
    yt = _cuda64(y).requires_grad_(True)
    Ly = rt.sqeuclid_plan_loss(_cuda64(x), yt, _cuda64(a), _cuda64(b), reg, W, scale=scale,
                               tol=1e-12)
    Ly.backward()
    fy = lambda yy: float(rt.sqeuclid_plan_loss(  # noqa: E731
        _cuda64(x), _cuda64(yy), _cuda64(a), _cuda64(b), reg, W, scale=scale, tol=1e-12))
    for (j, k) in [(0, 3), (47, 1)]:
        e = np.zeros_like(y)
        e[j, k] = h
        fd = (fy(y + e) - fy(y - e)) / (2 * h)
        np.testing.assert_allclose(yt.grad[j, k].item(), fd, rtol=1e-4, atol=1e-8)
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
