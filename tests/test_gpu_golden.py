"""GPU solves (FP64 passes, through the C ABI) against the committed golden
fixtures of the oracle (tests/golden/)."""
import glob
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_matches_fixture(path):
    g = np.load(path)
    solver = str(g["solver"])
    reg, tol, max_iter = float(g["reg"]), float(g["tol"]), int(g["max_iter"])
    kw = json.loads(str(g["kwargs"])) if "kwargs" in g else {}
    r = getattr(regot, solver)(g["M"], g["a"], g["b"], reg, tol=tol, max_iter=max_iter,
                               precision="fp64", **kw)
    ref_mar = g["mar_errs"]
    P = g["plan"]
    if solver == "qrot_pdip":
        # converged interior-point solve: same stop, same iterates to rounding
        assert r.converged == bool(g["converged"])
        assert abs(r.niter - int(g["niter"])) <= 1
        k = min(len(r.obj_vals), len(g["obj_vals"])) - 1
        np.testing.assert_allclose(r.obj_vals[:k], g["obj_vals"][:k], rtol=1e-7)
        np.testing.assert_allclose(r.plan, P, rtol=0, atol=1e-6 * P.max())
        return
    if solver == "qrot_assn" or tol <= 1e-13:
        # fixed iteration count: the histories follow the oracle step for step
        assert r.niter == int(g["niter"])
        k = len(ref_mar)
        np.testing.assert_allclose(r.mar_errs[:k], ref_mar, rtol=1e-5 if solver == "qrot_assn"
                                   else 1e-4, atol=1e-12)
        if "prim_vals" in g:
            np.testing.assert_allclose(r.prim_vals[:k], g["prim_vals"], rtol=1e-6)
        if solver == "qrot_assn":
            return
        np.testing.assert_allclose(r.obj_vals[:k], g["obj_vals"], rtol=1e-8, atol=1e-14)
        np.testing.assert_allclose(r.dual, g["dual"], rtol=0,
                                   atol=1e-6 * max(1.0, np.abs(g["dual"]).max()))
        np.testing.assert_allclose(r.plan, P, rtol=0, atol=1e-5 * P.max())
        if "densities" in g:
            np.testing.assert_allclose(r.densities[:k], g["densities"][:k], rtol=1e-12)
        return
    # converged solves: same iteration count up to the last steps at the
    # rounding floor, same histories while the marginal error is well above
    # it, and the same unique plan
    # (L-BFGS amplifies rounding differences of the summation order: its
    # histories agree for the first tens of iterations only)
    assert abs(r.niter - int(g["niter"])) <= max(3, int(g["niter"]) // 5)
    k = min(sum(1 for v in ref_mar if v > 1e3 * tol), len(r.mar_errs))
    if solver == "qrot_lbfgs_dual":
        k = min(k, 30)
    np.testing.assert_allclose(r.mar_errs[:k], ref_mar[:k], rtol=1e-5, atol=1e-14)
    np.testing.assert_allclose(r.obj_vals[:k], g["obj_vals"][:k], rtol=1e-9, atol=1e-14)
    # both plans are within the stopping tolerance of the unique optimum
    # (QROT L-BFGS stops at ||grad|| <= 1e-8, i.e. plan errors ~ 1e-7)
    ptol = 1e-5 if solver == "qrot_lbfgs_dual" else 1e-6
    np.testing.assert_allclose(r.plan, P, rtol=0, atol=ptol * P.max())
    if "densities" in g:
        np.testing.assert_allclose(r.densities[:k], g["densities"][:k], rtol=0,
                                   atol=8.0 / (P.shape[0] + P.shape[1] - 1) ** 2)
