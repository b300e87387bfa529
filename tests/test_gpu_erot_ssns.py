"""Parity of the GPU sinkhorn_ssns and of its sparsification (sparsify_mat3)
with the FP64 oracle restatement of the reference."""
import numpy as np
import pytest

import regot_oracle as O
from problems import erot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")


def _as_precision(M, precision):
    return M.astype(np.float32).astype(np.float64) if precision == "mixed" else M


def _oracle_kept(T, delta, hint):
    """Kept mask (n x (m-1)) and nnz of the oracle's sparsify_mat3."""
    n, m = T.shape
    outer, inner, _ = O.sparsify_mat3(T, delta, hint)
    K = np.zeros((n, m - 1), dtype=bool)
    for j in range(m - 1):
        K[inner[outer[j]:outer[j + 1]], j] = True
    return K, len(inner)


def _partial_duals(M, a, b, reg, iters):
    return O.sinkhorn_bcd(M, a, b, reg, tol=1e-14, max_iter=iters, plan=False).dual


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("hint", [0.001, 0.5])
@pytest.mark.parametrize("shape", [(300, 257), (304, 260)])
def test_sparsify_pattern(precision, hint, shape):
    # Same T, same delta: the kept set of the radix-select thresholds equals
    # the nth_element/sort selection of the reference entry by entry. (With
    # m a multiple of 4, FP32 rows are 16-byte aligned and T' is formed by
    # the vectorised transpose.)
    M, a, b = erot_points(*shape, seed=5, dtype=np.float64)
    Mq = _as_precision(M, precision)
    reg = 0.02
    gamma = _partial_duals(Mq, a, b, reg, 4)
    _, g = O.erot_dual_obj_grad(Mq, a, b, reg, gamma)
    T = O.erot_compute_T(Mq, reg, gamma)
    P = regot.Problem(M, a, b, precision=precision)
    gn = np.linalg.norm(g)
    for delta in [0.01 * gn, 0.3 * gn, 1e-4, 0.0]:
        K_o, nnz_o = _oracle_kept(T, delta, hint)
        nnz_g, K_g = P.erot_sparsify(reg, gamma, delta, hint)
        stored_o = K_o & (T[:, :-1] != 0)
        if precision == "fp64":
            assert nnz_g == nnz_o, delta
            assert np.array_equal(K_g, stored_o), (delta, np.count_nonzero(K_g != stored_o))
        else:
            # FP32 T: selections can differ where a partial sum sits within
            # FP32 rounding of delta.
            bad = np.count_nonzero(K_g != stored_o)
            assert bad <= max(3, 2e-3 * nnz_o), (delta, bad, nnz_o)
            assert abs(nnz_g - nnz_o) <= max(3, 2e-3 * nnz_o)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("shape", [(300, 257), (1000, 1537), (2100, 700)])
def test_sparsify_register_path_matches_shared_memory_path(precision, shape):
    # The selection stages have two implementations (rows and columns in
    # registers, or in shared memory for longer ones); on the same T they
    # keep exactly the same entries, in both sparsifications. The shapes give
    # 4, 8 and 16 register values per thread.
    from regot import _lib

    lib = _lib.load()
    n, m = shape
    M, a, b = erot_points(n, m, seed=6, dtype=np.float64)
    Mq = _as_precision(M, precision)
    reg = 0.02
    gamma = _partial_duals(Mq, a, b, reg, 4)
    _, g = O.erot_dual_obj_grad(Mq, a, b, reg, gamma)
    gn = np.linalg.norm(g)
    P = regot.Problem(M, a, b, precision=precision)

    def both(fn):
        first = fn()
        old = lib.regot_force_sparsify_path(1)
        try:
            second = fn()
        finally:
            assert lib.regot_force_sparsify_path(old) == 1
        return first, second

    for delta, hint in [(0.01 * gn, 0.001), (0.3 * gn, 0.5), (1e-4, 0.001), (0.0, 0.5)]:
        (nr, Kr), (ns, Ks) = both(lambda: P.erot_sparsify(reg, gamma, delta, hint))
        assert nr == ns, delta
        assert np.array_equal(Kr, Ks), (delta, np.count_nonzero(Kr != Ks))
    for density in (0.02, 0.3):
        (nr, Kr), (ns, Ks) = both(lambda: P.erot_sparsify_density(reg, gamma, density))
        assert nr == ns, density
        assert np.array_equal(Kr, Ks), (density, np.count_nonzero(Kr != Ks))
    P.close()


@pytest.mark.parametrize("hint", [0.001, 0.5])
def test_sparsify_large_delta_branches(hint):
    # Column sums below delta: find_small drops every entry, find_large keeps
    # each column's largest (sinkhorn_sparsify3.cpp:303 and the two searches).
    M, a, b = readme_example(120, 90)
    reg = 0.1
    gamma = _partial_duals(M, a, b, reg, 3)
    T = O.erot_compute_T(M, reg, gamma)
    delta = 10.0 * T.sum(axis=0).max()
    K_o, nnz_o = _oracle_kept(T, delta, hint)
    nnz_g, K_g = regot.Problem(M, a, b).erot_sparsify(reg, gamma, delta, hint)
    assert nnz_g == nnz_o
    assert np.array_equal(K_g, K_o & (T[:, :-1] != 0))
    if hint > 0.2:
        assert nnz_o == np.count_nonzero(T[:, :-1] == 0)
    else:
        assert nnz_o >= T.shape[1] - 1


def test_sparsify_counts_exact_zeros():
    # Entries whose FP64 T underflows to 0 are kept (Delta == 0) and count
    # towards nnz without being stored.
    M, a, b = erot_points(160, 130, seed=9, dtype=np.float64)
    M = M * 40.0
    reg = 0.02
    gamma = _partial_duals(M, a, b, reg, 2)
    T = O.erot_compute_T(M, reg, gamma)
    assert np.count_nonzero(T == 0) > 50
    _, g = O.erot_dual_obj_grad(M, a, b, reg, gamma)
    for precision in ["fp64", "mixed"]:
        Mq = _as_precision(M, precision)
        Tq = O.erot_compute_T(Mq, reg, gamma)
        delta = 0.01 * np.linalg.norm(g)
        K_o, nnz_o = _oracle_kept(Tq, delta, 0.001)
        nnz_g, K_g = regot.Problem(M, a, b, precision=precision).erot_sparsify(
            reg, gamma, delta, 0.001)
        if precision == "fp64":
            # Whether exp returns 0 or the smallest subnormal depends on its
            # last-ulp rounding there (CUDA's exp and the C library's differ):
            # only those entries may change sides.
            tiny = (Tq[:, :-1] > 0) & (Tq[:, :-1] < 2.0**-1060)
            diff = K_g != (K_o & (Tq[:, :-1] != 0))
            assert not np.any(diff & ~tiny)
            assert abs(nnz_g - nnz_o) <= np.count_nonzero(tiny)
        else:
            assert abs(nnz_g - nnz_o) <= max(3, 2e-3 * nnz_o)


CASES = {
    "readme-0.1": (lambda: readme_example(100, 80), 0.1),
    "readme-0.01": (lambda: readme_example(100, 80), 0.01),
    "points-0.05": (lambda: erot_points(200, 150, seed=3, dtype=np.float64), 0.05),
}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", list(CASES))
def test_sinkhorn_ssns_matches_oracle(precision, case):
    make, reg = CASES[case]
    M, a, b = make()
    Mq = _as_precision(M, precision)
    tol = 1e-9 if precision == "fp64" else 1e-7
    r = regot.sinkhorn_ssns(M, a, b, reg, tol=tol, max_iter=400, precision=precision)
    o = O.sinkhorn_ssns(Mq, a, b, reg, tol=tol, max_iter=400)
    L = r.niter + 1
    assert len(r.mar_errs) == len(r.obj_vals) == len(r.run_times) == len(r.densities) == L
    dim = M.shape[0] + M.shape[1] - 1
    if precision == "fp64":
        # The direction comes from CG to 1e-10 instead of a sparse LDLT, so
        # the safe-step decisions and the iteration histories coincide until
        # the differences of the two solves have grown (about 50 iterations
        # at reg = 0.01).
        assert abs(r.niter - o.niter) <= 2, (r.niter, o.niter)
        k = min(sum(1 for v in o.mar_errs if v > 1e-6), L, 40)
        np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=1e-5, atol=1e-12)
        np.testing.assert_allclose(r.obj_vals[:k], o.obj_vals[:k], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(r.densities[:k], o.densities[:k], rtol=0, atol=8.0 / dim**2)
        # Both stop at ||grad|| < 1e-9; at reg = 0.01 the duals are then only
        # determined to about 1e-6.
        np.testing.assert_allclose(r.dual, o.dual, rtol=0, atol=2e-6)
    else:
        assert r.niter <= 1.5 * o.niter + 10, (r.niter, o.niter)
        np.testing.assert_allclose(r.obj_vals[-1], o.obj_vals[-1], rtol=1e-6)
        np.testing.assert_allclose(r.densities[0], o.densities[0], rtol=2e-3)
    # mixed: the solves stop at different points of marginal error < tol,
    # measured 2.2e-6 (README cases) and 2.4e-7 (points) of the largest entry
    np.testing.assert_allclose(r.plan, o.plan, rtol=0,
                               atol=(1e-7 if precision == "fp64" else 2e-5) * o.plan.max())
    # mixed: the FP64-evaluated gradient norm measured 0.27-0.43 tol
    _, g = O.erot_dual_obj_grad(Mq, a, b, reg, r.dual)
    assert np.linalg.norm(g) < tol


def test_sinkhorn_ssns_cg_method():
    # method=0: the reference's CG (identity preconditioner, 1e-8 relative).
    M, a, b = readme_example(100, 80)
    reg = 0.1
    r = regot.sinkhorn_ssns(M, a, b, reg, tol=1e-9, max_iter=300, method=0)
    o = O.sinkhorn_ssns(M, a, b, reg, tol=1e-9, max_iter=300, method=0)
    # CG to 1e-8 on both sides: the histories agree until the rounding of
    # the two CG runs has grown.
    assert abs(r.niter - o.niter) <= 0.2 * o.niter, (r.niter, o.niter)
    k = min(sum(1 for v in o.mar_errs if v > 1e-5), r.niter + 1, 15)
    np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=1e-4, atol=1e-12)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-7 * o.plan.max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ssns_agrees_with_bcd(precision):
    M, a, b = erot_points(180, 140, seed=13, dtype=np.float64)
    reg = 0.05
    rs = regot.sinkhorn_ssns(M, a, b, reg, tol=1e-8, max_iter=200, precision=precision)
    rb = regot.sinkhorn_bcd(M, a, b, reg, tol=1e-8, max_iter=5000, precision=precision)
    # mixed measured 6.5e-7 of the largest entry and 2.4e-7 on the duals
    np.testing.assert_allclose(rs.plan, rb.plan, rtol=0, atol=1e-5 * rb.plan.max())
    np.testing.assert_allclose(rs.dual, rb.dual, rtol=0, atol=2e-6)


def test_ssns_x0_and_errors():
    M, a, b = readme_example(60, 50)
    reg = 0.1
    r0 = regot.sinkhorn_ssns(M, a, b, reg, tol=1e-10, max_iter=200)
    r1 = regot.sinkhorn_ssns(M, a, b, reg, tol=1e-10, max_iter=200, x0=r0.dual)
    assert r1.niter == 0
    np.testing.assert_allclose(r1.dual, r0.dual, rtol=0, atol=0)
    with pytest.raises(ValueError):
        regot.sinkhorn_ssns(M, a, b, reg, method=7)
