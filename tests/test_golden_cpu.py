"""The oracle reproduces the committed golden fixtures (tests/golden/,
generated by tests/golden/make_golden.py from the oracle itself)."""
import glob
import json
import os

import numpy as np
import pytest

import regot_oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def test_fixtures_present():
    assert len(GOLDEN) >= 19


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_reproduces_fixture(path):
    g = np.load(path)
    solver = str(g["solver"])
    kw = json.loads(str(g["kwargs"])) if "kwargs" in g else {}
    r = getattr(O, solver)(g["M"], g["a"], g["b"], float(g["reg"]), tol=float(g["tol"]),
                           max_iter=int(g["max_iter"]), **kw)
    assert r.niter == int(g["niter"])
    np.testing.assert_allclose(r.mar_errs, g["mar_errs"], rtol=1e-8, atol=1e-15)
    np.testing.assert_allclose(r.obj_vals, g["obj_vals"], rtol=1e-11, atol=1e-15)
    if "dual" in g:
        np.testing.assert_allclose(r.dual, g["dual"], rtol=1e-9, atol=1e-12)
    if "converged" in g:
        assert r.converged == bool(g["converged"])
    np.testing.assert_allclose(r.plan, g["plan"], rtol=1e-9, atol=1e-15)
    if "densities" in g:
        np.testing.assert_array_equal(r.densities, g["densities"])
    if "prim_vals" in g:
        np.testing.assert_allclose(r.prim_vals, g["prim_vals"], rtol=1e-9)
