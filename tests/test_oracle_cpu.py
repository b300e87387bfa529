"""CPU checks of the FP64 oracle (the restatement every GPU parity test
compares against). The reference ships no tests or golden vectors, so the
oracle is pinned here by closed-form cases, finite differences, independent
numpy restatements written from the same published formulas, and
cross-solver agreement."""
import numpy as np
import pytest
from scipy.optimize import minimize

import regot_oracle as O
from problems import erot_points, qrot_points, readme_example


def _erot_dual_np(M, a, b, reg, gamma):
    """Dual objective and gradient of EROT (sinkhorn_problem_obj.cpp:324-393)
    written directly in numpy, beta_m = 0."""
    n, m = M.shape
    al = gamma[:n]
    be = np.r_[gamma[n:], 0.0]
    T = np.exp((al[:, None] + be[None, :] - M) / reg)
    f = reg * T.sum() - al @ a - be[:-1] @ b[:-1]
    g = np.r_[T.sum(1) - a, (T.sum(0) - b)[:-1]]
    return f, g, T


def _qrot_dual_np(M, a, b, reg, gamma):
    n, m = M.shape
    D = np.maximum(gamma[:n, None] + gamma[None, n:] - M, 0.0)
    f = 0.5 * (D ** 2).sum() - reg * (gamma[:n] @ a + gamma[n:] @ b)
    g = np.r_[D.sum(1) - reg * a, D.sum(0) - reg * b]
    return f, g, D


def test_erot_obj_grad_matches_numpy_and_fd():
    M, a, b = erot_points(40, 30, seed=2, dtype=np.float64)
    reg = 0.1
    rng = np.random.default_rng(0)
    gamma = rng.standard_normal(M.shape[0] + M.shape[1] - 1) * 0.05
    f, g = O.erot_dual_obj_grad(M, a, b, reg, gamma)
    f2, g2, _ = _erot_dual_np(M, a, b, reg, gamma)
    assert abs(f - f2) <= 1e-12 * max(1.0, abs(f2))
    np.testing.assert_allclose(g, g2, rtol=1e-11, atol=1e-14)
    h = 1e-6
    for k in rng.choice(gamma.size, 8, replace=False):
        e = np.zeros_like(gamma)
        e[k] = h
        fd = (O.erot_dual_obj(M, a, b, reg, gamma + e) - O.erot_dual_obj(M, a, b, reg, gamma - e)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k]))


def test_erot_hvp_is_gradient_derivative():
    M, a, b = erot_points(30, 25, seed=3, dtype=np.float64)
    reg = 0.2
    rng = np.random.default_rng(1)
    N = M.shape[0] + M.shape[1] - 1
    gamma = rng.standard_normal(N) * 0.05
    x = rng.standard_normal(N)
    hx = O.erot_hvp(M, a, b, reg, gamma, x)
    h = 1e-6
    _, gp = O.erot_dual_obj_grad(M, a, b, reg, gamma + h * x)
    _, gm = O.erot_dual_obj_grad(M, a, b, reg, gamma - h * x)
    np.testing.assert_allclose(hx, (gp - gm) / (2 * h), rtol=1e-5, atol=1e-8)


def test_erot_newton_direction_solves_hessian_system():
    M, a, b = readme_example(40, 30)
    reg = 0.1
    rng = np.random.default_rng(2)
    gamma = rng.standard_normal(M.shape[0] + M.shape[1] - 1) * 0.1
    _, g = O.erot_dual_obj_grad(M, a, b, reg, gamma)
    d = O.erot_newton_direction(M, a, b, reg, gamma)
    np.testing.assert_allclose(O.erot_hvp(M, a, b, reg, gamma, d), -g, rtol=1e-8, atol=1e-12)


def test_erot_optimal_beta_alpha_match_marginals():
    M, a, b = readme_example(50, 40)
    reg = 0.05
    alpha = np.random.default_rng(4).standard_normal(50) * 0.1
    beta = O.erot_optimal_beta(M, b, reg, alpha)
    T = np.exp((alpha[:, None] + beta[None, :] - M) / reg)
    np.testing.assert_allclose(T.sum(0), b, rtol=1e-12)
    alpha2 = O.erot_optimal_alpha(M, a, reg, beta)
    T = np.exp((alpha2[:, None] + beta[None, :] - M) / reg)
    np.testing.assert_allclose(T.sum(1), a, rtol=1e-12)


@pytest.mark.parametrize("solver", ["sinkhorn_bcd", "sinkhorn_newton", "sinkhorn_ssns"])
def test_erot_separable_cost_known_answer(solver):
    # M_ij = u_i + v_j: the EROT plan is exactly a b' for every reg.
    rng = np.random.default_rng(5)
    n, m = 35, 28
    u, v = rng.uniform(0, 1, n), rng.uniform(0, 1, m)
    M = u[:, None] + v[None, :]
    a = rng.uniform(0.5, 1.5, n)
    a /= a.sum()
    b = rng.uniform(0.5, 1.5, m)
    b /= b.sum()
    r = getattr(O, solver)(M, a, b, 0.05, tol=1e-11, max_iter=500)
    np.testing.assert_allclose(r.plan, np.outer(a, b), rtol=1e-8, atol=1e-14)
    assert r.mar_errs[-1] < 1e-11


def test_erot_solvers_agree_with_generic_minimiser():
    M, a, b = readme_example(30, 24)
    reg = 0.1
    n, m = M.shape
    fun = lambda x: _erot_dual_np(M, a, b, reg, x)[:2]  # noqa: E731
    res = minimize(fun, np.zeros(n + m - 1), jac=True, method="L-BFGS-B",
                   options={"maxiter": 20000, "gtol": 1e-12, "ftol": 1e-15})
    for solver in ("sinkhorn_bcd", "sinkhorn_newton", "sinkhorn_ssns"):
        r = getattr(O, solver)(M, a, b, reg, tol=1e-10, max_iter=2000)
        assert r.obj_vals[-1] <= res.fun + 1e-10
        np.testing.assert_allclose(r.obj_vals[-1], res.fun, rtol=1e-8)
        np.testing.assert_allclose(r.plan, _erot_dual_np(M, a, b, reg, r.dual)[2], rtol=1e-12)


def test_erot_lbfgs_dual_matches_generic_minimiser():
    # sinkhorn_lbfgs_dual minimises the same dual as BCD: same optimum as an
    # independent minimiser of the numpy dual.
    M, a, b = erot_points(40, 30, seed=8, dtype=np.float64)
    reg = 0.05
    n, m = M.shape
    fun = lambda x: _erot_dual_np(M, a, b, reg, x)[:2]  # noqa: E731
    res = minimize(fun, np.zeros(n + m - 1), jac=True, method="L-BFGS-B",
                   options={"maxiter": 20000, "gtol": 1e-12, "ftol": 1e-15})
    r = O.sinkhorn_lbfgs_dual(M, a, b, reg, tol=1e-8, max_iter=1000)
    assert r.mar_errs[-1] < 1e-8 and len(r.mar_errs) == r.niter + 1
    np.testing.assert_allclose(r.obj_vals[-1], res.fun, rtol=1e-9)
    f, g, T = _erot_dual_np(M, a, b, reg, r.dual)
    np.testing.assert_allclose(r.mar_errs[-1], np.linalg.norm(g), rtol=1e-9)
    np.testing.assert_allclose(r.plan, T, rtol=1e-12)


def test_erot_apdagd_averaged_plan_and_gap():
    # APDAGD's plan is the running average of T along the extrapolated
    # points; its marginal error falls and its duality gap closes.
    M, a, b = erot_points(60, 50, seed=11, dtype=np.float64)
    reg = 0.1
    r = O.sinkhorn_apdagd(M, a, b, reg, tol=1e-4, max_iter=2000)
    assert r.niter < 2000 and r.mar_errs[-1] <= 1e-4
    P = r.plan
    mar = np.sqrt(((P.sum(1) - a) ** 2).sum() + ((P.sum(0) - b) ** 2).sum())
    np.testing.assert_allclose(r.mar_errs[-1], mar, rtol=1e-10)
    primal = (M * P).sum() - reg * (P * (1 - np.log(P))).sum()
    assert primal - (-r.obj_vals[-1]) <= 1e-4
    rb = O.sinkhorn_bcd(M, a, b, reg, tol=1e-11, max_iter=20000)
    np.testing.assert_allclose(P, rb.plan, rtol=0, atol=2e-3 * rb.plan.max())


def test_erot_bcd_objective_is_monotone():
    M, a, b = erot_points(60, 50, seed=6, dtype=np.float64)
    r = O.sinkhorn_bcd(M, a, b, 0.05, tol=1e-10, max_iter=300)
    f = np.array(r.obj_vals)
    assert np.all(np.diff(f) <= 1e-14 * np.abs(f[1:]) + 1e-15)


def _sparsify_np(T, delta, from_large):
    """sparsify_mat3 by its defining property (not its algorithm): per column
    drop the smallest entries while their sum stays <= delta; per row, when
    the dropped sum exceeds 2 delta, keep the largest dropped entries until
    it does not; exact zeros count as kept."""
    n, m = T.shape
    m1 = m - 1
    x = np.empty(m1)
    for j in range(m1):
        c = np.sort(T[:, j])
        cs = np.cumsum(c)
        if not cs[-1] > delta:
            x[j] = c[-1] if from_large else np.inf
            continue
        x[j] = c[np.argmax(cs > delta)]
    keep = T[:, :m1] >= x[None, :]
    D = np.where(keep, 0.0, T[:, :m1])
    for i in range(n):
        if D[i].sum() > 2 * delta:
            c = np.sort(D[i])
            y = c[np.argmax(np.cumsum(c) > 2 * delta)]
            keep[i] |= D[i] >= y
    return keep | (T[:, :m1] == 0)


@pytest.mark.parametrize("hint", [0.001, 0.5])
def test_sparsify_mat3_matches_definition(hint):
    rng = np.random.default_rng(7)
    for trial in range(4):
        n, m = rng.integers(20, 90), rng.integers(20, 90)
        T = np.exp(rng.standard_normal((n, m)) * 4.0 - 6.0) / (n * m)
        T[rng.random((n, m)) < 0.05] = 0.0
        for delta in [0.0, 1e-4 * T.sum(), 0.01 * T.sum(), 10.0 * T.sum()]:
            outer, inner, vals = O.sparsify_mat3(T, delta, hint)
            K = np.zeros((n, m - 1), dtype=bool)
            for j in range(m - 1):
                K[inner[outer[j]:outer[j + 1]], j] = True
            np.testing.assert_array_equal(K, _sparsify_np(T, delta, hint <= 0.2))
            np.testing.assert_array_equal(vals, T[:, :-1].T[K.T])


def test_qrot_obj_grad_and_fd():
    M, a, b = qrot_points(40, 30, seed=3, dtype=np.float64)
    reg = 0.1
    rng = np.random.default_rng(8)
    gamma = rng.standard_normal(70) * 0.1
    f, g = O.qrot_dual_obj_grad(M, a, b, reg, gamma)
    f2, g2, _ = _qrot_dual_np(M, a, b, reg, gamma)
    assert abs(f - f2) <= 1e-12 * max(1.0, abs(f2))
    np.testing.assert_allclose(g, g2, rtol=1e-11, atol=1e-14)
    h = 1e-7
    for k in rng.choice(70, 8, replace=False):
        e = np.zeros(70)
        e[k] = h
        fd = (O.qrot_dual_obj(M, a, b, reg, gamma + e) - O.qrot_dual_obj(M, a, b, reg, gamma - e)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-5 * max(1e-3, abs(g[k]))


def test_qrot_optimal_beta_root():
    M, a, b = qrot_points(50, 40, seed=4, dtype=np.float64)
    reg = 0.05
    alpha = np.random.default_rng(9).standard_normal(50) * 0.1
    beta = O.qrot_optimal_beta(M, b, reg, alpha)
    lhs = np.maximum(beta[None, :] - (M - alpha[:, None]), 0.0).sum(0)
    np.testing.assert_allclose(lhs, reg * b, rtol=1e-10)


def test_qrot_primal_val_of_feasible_plan():
    # primal_val projects D/reg onto the marginals (approx_proj.h:6-26) and
    # evaluates <P, M> + reg/2 ||P||^2; at the optimum the plan is already
    # feasible, so the value equals that of the unprojected plan.
    M, a, b = qrot_points(30, 25, seed=5, dtype=np.float64)
    reg = 0.1
    # (tol 1e-9 makes the FP64 line search fail here, in the reference too)
    r = O.qrot_lbfgs_dual(M, a, b, reg, tol=1e-8, max_iter=5000)
    P = O.qrot_plan(M, reg, r.dual)
    np.testing.assert_allclose(P.sum(1), a, atol=1e-6)
    np.testing.assert_allclose(P.sum(0), b, atol=1e-6)
    direct = (P * M).sum() + 0.5 * reg * (P ** 2).sum()
    np.testing.assert_allclose(O.qrot_primal_val(M, a, b, reg, r.dual), direct, rtol=1e-5)
    # strong duality: primal value = -dual objective / reg
    np.testing.assert_allclose(direct, -r.obj_vals[-1] / reg, rtol=1e-5)


def test_qrot_solvers_agree_with_generic_minimiser():
    M, a, b = qrot_points(25, 20, seed=6, dtype=np.float64)
    reg = 0.1
    fun = lambda x: _qrot_dual_np(M, a, b, reg, x)[:2]  # noqa: E731
    res = minimize(fun, np.zeros(45), jac=True, method="L-BFGS-B",
                   options={"maxiter": 50000, "gtol": 1e-13, "ftol": 1e-16})
    r = O.qrot_lbfgs_dual(M, a, b, reg, tol=1e-8, max_iter=5000)
    np.testing.assert_allclose(r.obj_vals[-1], res.fun, rtol=1e-7)
    P_ref = _qrot_dual_np(M, a, b, reg, res.x)[2] / reg
    np.testing.assert_allclose(O.qrot_plan(M, reg, r.dual), P_ref, atol=1e-4 * P_ref.max())


def test_qrot_assn_matches_numpy_restatement():
    """ASSN (qrot_assn.cpp:16-170) restated in numpy with a dense solve of the
    regularised generalised Jacobian; the oracle's CG (tol 1e-8) must take
    the same Newton / projection / gradient decisions."""
    M, a, b = readme_example(60, 50)
    n, m = M.shape
    reg = 0.1
    gam = np.r_[np.zeros(n), O.qrot_optimal_beta(M, b, reg, np.zeros(n))]

    def fg(x):
        f, g, D = _qrot_dual_np(M, a, b, reg, x)
        return f, g, (D > 0).astype(float)

    f, g, s = fg(gam)
    gn = np.linalg.norm(g)
    lam, xi = 1.0, gn
    errs = [gn / reg]
    for _ in range(12):
        if gn < 1e-12:
            break
        mu = lam * gn
        H = np.block([[np.diag(s.sum(1)), s], [s.T, np.diag(s.sum(0))]]) + mu * np.eye(n + m)
        d = np.linalg.solve(H, -g)
        _, gu, _ = fg(gam + d)
        gun = np.linalg.norm(gu)
        if gun <= 0.99 * xi:
            gam, xi = gam + d, gun
        else:
            numer = -gu @ d
            rho = numer / (d @ d)
            v = gam - (numer / gun ** 2) * gu
            gvn = np.linalg.norm(fg(v)[1])
            if rho >= 0.25 and gvn <= gn:
                gam = v
            else:
                gam = gam - 0.5 * g
            lam = 0.5 * (0.01 + lam) if rho >= 0.75 else (2 * lam if rho >= 0.25 else 4 * lam)
        f, g, s = fg(gam)
        gn = np.linalg.norm(g)
        errs.append(gn / reg)
    r = O.qrot_assn(M, a, b, reg, tol=1e-12, max_iter=len(errs) - 1, plan=False)
    np.testing.assert_allclose(r.mar_errs[:len(errs)], errs, rtol=1e-5)


@pytest.mark.parametrize("solver", ["qrot_apdagd", "qrot_pdaam"])
def test_qrot_accelerated_averaged_plan_and_gap(solver):
    # The plan of the accelerated QROT methods is the running average of
    # D/reg along the extrapolated points: its marginal error is the recorded
    # one, its duality gap against the last dual value closes, and it tends
    # to the optimal plan.
    M, a, b = qrot_points(40, 30, seed=7, dtype=np.float64)
    reg = 0.1
    r = getattr(O, solver)(M, a, b, reg, tol=1e-5, max_iter=5000)
    assert r.niter < 5000 and r.mar_errs[-1] <= 1e-5
    P = r.plan
    mar = np.sqrt(((P.sum(1) - a) ** 2).sum() + ((P.sum(0) - b) ** 2).sum())
    np.testing.assert_allclose(r.mar_errs[-1], mar, rtol=1e-10)
    primal = (M * P).sum() + 0.5 * reg * (P * P).sum()
    assert primal - (-r.obj_vals[-1] / reg) <= 1e-5
    rl = O.qrot_lbfgs_dual(M, a, b, reg, tol=1e-8, max_iter=20000)
    P_opt = O.qrot_plan(M, reg, rl.dual)
    np.testing.assert_allclose(P, P_opt, rtol=0, atol=0.05 * P_opt.max())
    np.testing.assert_allclose(r.obj_vals[-1], rl.obj_vals[-1], rtol=1e-4)


def test_qrot_grssn_and_semi_dual_reach_the_optimum():
    # Both reach the optimum of the generic minimiser; GRSSN's first step is
    # the Newton direction of the shifted generalized Jacobian, and the
    # semi-dual's dual is (alpha, optimal_beta(alpha)).
    M, a, b = qrot_points(25, 20, seed=6, dtype=np.float64)
    reg = 0.1
    fun = lambda x: _qrot_dual_np(M, a, b, reg, x)[:2]  # noqa: E731
    res = minimize(fun, np.zeros(45), jac=True, method="L-BFGS-B",
                   options={"maxiter": 50000, "gtol": 1e-13, "ftol": 1e-16})
    rg = O.qrot_grssn(M, a, b, reg, tol=1e-9, max_iter=500)
    assert rg.niter < 500 and rg.mar_errs[-1] * reg < 1e-9
    np.testing.assert_allclose(rg.obj_vals[-1], res.fun, rtol=1e-7)
    rs = O.qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-8, max_iter=2000)
    np.testing.assert_allclose(rs.obj_vals[-1], res.fun, rtol=1e-7)
    beta = O.qrot_optimal_beta(M, b, reg, rs.dual[:25])
    np.testing.assert_allclose(rs.dual[25:], beta, rtol=0, atol=0)
    # first GRSSN step: (H + shift I) d = -g with H the generalized Jacobian
    gam = np.r_[np.zeros(25), O.qrot_optimal_beta(M, b, reg, np.zeros(25))]
    f, g, D = _qrot_dual_np(M, a, b, reg, gam)
    s = (D > 0).astype(float)
    H = np.block([[np.diag(s.sum(1)), s], [s.T, np.diag(s.sum(0))]]) + 1e-3 * np.eye(45)
    d = np.linalg.solve(H, -g)
    step = 1.0
    for _ in range(20):
        if _qrot_dual_np(M, a, b, reg, gam + step * d)[0] <= f + step * 0.5 * (g @ d):
            break
        step *= 0.5
    r1 = O.qrot_grssn(M, a, b, reg, tol=1e-14, max_iter=1, plan=False)
    np.testing.assert_allclose(r1.dual, gam + step * d, rtol=0, atol=1e-7)


def _sparsify_density_np(T, density):
    """sparsify_mat_with_density restated in numpy (distinct values)."""
    n, m = T.shape
    Tt = T[:, :-1]
    k = int(Tt.size * min(max(density, 0.0), 1.0))
    K = np.zeros(Tt.shape, dtype=bool)
    if k > 0:
        order = np.argsort(Tt.ravel(order="F"), kind="stable")
        K.ravel(order="F")[order[Tt.size - k:]] = True
        K = K.reshape(Tt.shape, order="F") if not K.flags.f_contiguous else K
        flat = np.zeros(Tt.size, dtype=bool)
        flat[order[Tt.size - k:]] = True
        K = flat.reshape(Tt.shape, order="F")
    K[:, 0] = True
    K[0, :] = True
    return K


@pytest.mark.parametrize("density", [0.0, 0.003, 0.05, 0.4, 1.0])
def test_sparsify_density_matches_definition(density):
    rng = np.random.default_rng(17)
    for trial in range(3):
        n, m = rng.integers(20, 90), rng.integers(20, 90)
        T = np.exp(rng.standard_normal((n, m)) * 4.0 - 6.0) / (n * m)
        outer, inner, vals = O.sparsify_density(T, density)
        K = np.zeros((n, m - 1), dtype=bool)
        for j in range(m - 1):
            K[inner[outer[j]:outer[j + 1]], j] = True
        np.testing.assert_array_equal(K, _sparsify_density_np(T, density))
        np.testing.assert_array_equal(vals, T[:, :-1].T[K.T])


@pytest.mark.parametrize("coefs,init", [
    ([0.0, -1.0, 0.5, 0.0, 0.0], 1.0),     # minimiser at 1: accepted at once
    ([0.0, -1.0, 50.0, 0.0, 0.0], 1.0),    # minimiser at 0.01: interpolation
    ([0.0, -1.0, 0.01, 0.0, 0.0], 1.0),    # minimiser at 50: extrapolation to 2
    ([0.0, -1.0, 0.3, -0.4, 0.2], 0.5),    # quartic
    ([1.0, -3.0, 0.0, 2.0, 0.5], 1.5),
])
def test_wolfe_line_search_conditions(coefs, init):
    """line_search_wolfe (sinkhorn_problem_ls.cpp:226-436): the returned step
    satisfies the strong Wolfe conditions, or is the upper bound 2 with
    sufficient decrease."""
    c = np.array(coefs, dtype=float)
    f = np.polynomial.Polynomial(c)
    df = f.deriv()
    step, recompute, nev = O.wolfe_poly(c, init)
    assert 1 <= nev <= 20 and not recompute
    suff = f(step) <= f(0) + 1e-4 * step * df(0)
    curv = abs(df(step)) <= 0.9 * abs(df(0))
    assert suff and (curv or step == 2.0)


def test_wolfe_line_search_ascent_direction():
    step, recompute, nev = O.wolfe_poly([0.0, 1.0, 1.0, 0.0, 0.0], 0.7)
    assert step == 0.7 and recompute and nev == 0


@pytest.mark.parametrize("solver,tol", [("sinkhorn_sparse_newton", 1e-7), ("sinkhorn_splr", 1e-8)])
def test_erot_sparse_newton_and_splr_reach_the_optimum(solver, tol):
    # The sparsified Newton steps converge linearly (the density falls to
    # 1 % of its maximum); SPLR's low-rank correction converges much faster.
    M, a, b = erot_points(40, 30, seed=12, dtype=np.float64)
    reg = 0.1
    rn = O.sinkhorn_newton(M, a, b, reg, tol=1e-11, max_iter=100)
    r = getattr(O, solver)(M, a, b, reg, tol=tol, max_iter=2000, density=0.5)
    assert r.niter < 2000 and r.mar_errs[-1] < tol
    np.testing.assert_allclose(r.obj_vals[-1], rn.obj_vals[-1], rtol=1e-9)
    np.testing.assert_allclose(r.plan, rn.plan, rtol=0, atol=1e-5 * rn.plan.max())
    # densities record density_T2H of the density parameter
    n, m = M.shape
    d0 = 0.1 * 0.5
    np.testing.assert_allclose(r.densities[0], (2 * d0 * n * (m - 1) + n + m - 1) / (n + m - 1) ** 2)


@pytest.mark.parametrize("mode", ["cg", "fp"])
@pytest.mark.parametrize("reg", [0.1, 0.01])
def test_qrot_pdip_reaches_the_qrot_optimum(mode, reg):
    """qrot_pdip (pdip_cg.cpp / pdip_fp.cpp): the interior-point plan is
    feasible to the stopping tolerance and tends to the QROT optimum found
    by the dual Newton method."""
    M, a, b = qrot_points(40, 30, seed=3, dtype=np.float64)
    r = O.qrot_pdip(M, a, b, reg, tol=1e-8, max_iter=200, inner_solver=mode)
    assert r.converged and r.niter < 200
    assert len(r.obj_vals) == len(r.mar_errs) == r.niter
    P = r.plan
    mar = max(np.linalg.norm(P.sum(1) - a), np.linalg.norm(P.sum(0) - b))
    np.testing.assert_allclose(r.mar_errs[-1], mar, rtol=1e-6, atol=1e-14)
    np.testing.assert_allclose(r.obj_vals[-1], (M * P).sum() + reg / 2 * (P * P).sum(), rtol=1e-12)
    assert P.min() > 0
    rg = O.qrot_grssn(M, a, b, reg, tol=1e-11, max_iter=2000)
    Pg = O.qrot_plan(M, reg, rg.dual)
    # the barrier stop leaves a few entries near the support boundary off
    np.testing.assert_allclose(P, Pg, rtol=0, atol=2e-2 * Pg.max())
    np.testing.assert_allclose(r.obj_vals[-1], (M * Pg).sum() + reg / 2 * (Pg * Pg).sum(),
                               rtol=2e-3)
