"""Parity of the GPU qrot_pdip (primal-dual interior point: device passes
over the n x m primal vectors, host factorizations of the block matrix)
with the FP64 oracle restatement of pdip_cg.cpp:206-413 and
pdip_fp.cpp:278-667."""
import numpy as np
import pytest

import regot_oracle as O
from problems import qrot_points, readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")

CASES = {
    "readme-0.1": (lambda: readme_example(100, 80), 0.1),
    "readme-0.01": (lambda: readme_example(100, 80), 0.01),
    "points-0.1": (lambda: qrot_points(60, 45, seed=3, dtype=np.float64), 0.1),
}


@pytest.mark.parametrize("mode", ["cg", "fp"])
@pytest.mark.parametrize("case", list(CASES))
def test_pdip_matches_oracle(mode, case):
    make, reg = CASES[case]
    M, a, b = make()
    r = regot.qrot_pdip(M, a, b, reg, tol=1e-8, max_iter=200, inner_solver=mode,
                        precision="fp64")
    o = O.qrot_pdip(M, a, b, reg, tol=1e-8, max_iter=200, inner_solver=mode)
    assert r.converged == o.converged
    assert abs(r.niter - o.niter) <= 1
    k = min(len(r.obj_vals), len(o.obj_vals)) - 1
    # the iterates agree to rounding until the barrier drives entries to 0
    np.testing.assert_allclose(r.obj_vals[:k], o.obj_vals[:k], rtol=1e-7)
    np.testing.assert_allclose(r.mar_errs[:k], o.mar_errs[:k], rtol=1e-3, atol=1e-11)
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-6 * o.plan.max())
    assert len(r.run_times) == len(r.obj_vals)


def test_pdip_aliases_and_options():
    M, a, b = readme_example(60, 50)
    reg = 0.1
    r1 = regot.pdip_cg(M, a, b, reg, max_iter=5, precision="fp64")
    r2 = regot.qrot_pdip(M, a, b, reg, max_iter=5, precision="fp64", inner_solver="CG")
    np.testing.assert_array_equal(r1.obj_vals, r2.obj_vals)
    r3 = regot.pdip_fp(M, a, b, reg, max_iter=5, precision="fp64", fixed_threshold=1e-6)
    o3 = O.qrot_pdip(M, a, b, reg, max_iter=5, inner_solver="fp", fixed_threshold=1e-6)
    np.testing.assert_allclose(r3.obj_vals, o3.obj_vals, rtol=1e-8)
    with pytest.raises(RuntimeError):
        regot.qrot_pdip(M, a, b, reg, inner_solver="lu")
    with pytest.raises(RuntimeError):
        regot.qrot_pdip(M, a, b, reg, inner_solver=1)
    # gap-only stop on the CG path, and a small cg_max_iter
    r4 = regot.qrot_pdip(M, a, b, reg, max_iter=12, precision="fp64", cg_stop_gap_mu_only=True,
                         cg_max_iter=50)
    o4 = O.qrot_pdip(M, a, b, reg, max_iter=12, cg_stop_gap_mu_only=True, cg_max_iter=50)
    assert r4.niter == o4.niter == 12
    np.testing.assert_allclose(r4.obj_vals, o4.obj_vals, rtol=1e-7)


def test_pdip_mixed_storage_reads_fp32_cost():
    # PDIP computes in FP64; in mixed storage the cost is the FP32 copy of M
    M, a, b = readme_example(80, 70)
    Mq = M.astype(np.float32).astype(np.float64)
    r = regot.qrot_pdip(M, a, b, 0.1, precision="mixed")
    o = O.qrot_pdip(Mq, a, b, 0.1)
    assert r.converged and abs(r.niter - o.niter) <= 1
    np.testing.assert_allclose(r.plan, o.plan, rtol=0, atol=1e-6 * o.plan.max())
