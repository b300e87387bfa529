"""The GPU solvers against the reference's own outputs: the plans of the four
solves that the reference rendered as figs/plan_*.png (README example,
100 x 80), read back into tests/golden/reference_images/.

Each GPU plan must fall, entry for entry, in the colormap bins of the
reference's image (1 bin = 1/256 of the plan's range). Measured on a GB300,
all eight cases need no tolerance at all: every entry of every plan lies in
its bin. The tolerances below (in bins) excuse only entries within them of a
bin edge:
  - FP64 follows the reference's iterates to rounding (the GPU tests hold
    sinkhorn_bcd and qrot_pdip to 1e-6 of the largest entry or better; FP64
    sinkhorn_ssns solves its Newton systems by preconditioned CG where the
    reference factorises): 1e-4 bins;
  - mixed precision stores M in FP32 and forms T in FP32, so entries may
    move by a few ulps of the largest one: 1e-3 bins.
"""
import numpy as np
import pytest

import plan_image as P
from problems import readme_example

pytestmark = pytest.mark.gpu

regot = pytest.importorskip("regot")

TOL_BINS = {"fp64": 1e-4, "mixed": 1e-3}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", P.IMAGES)
def test_gpu_plan_reproduces_reference_image(name, precision):
    labels, rgb, call = P.load(name)
    M, a, b = readme_example(100, 80)
    r = getattr(regot, call["solver"])(M, a, b, call["reg"], tol=call["tol"],
                                       max_iter=call["max_iter"], precision=precision,
                                       **call["kwargs"])
    T = np.asarray(r.plan)
    tol = TOL_BINS[precision]
    bad = P.violations(T, labels, rgb, tol=tol)
    assert bad == 0, (f"{bad} constraints broken at {tol} bins; "
                      f"needed {P.needed_tol(T, labels, rgb)}")


# EROT's plan is unique: the GPU's other EROT solvers, converged well below
# the reference's tol, reproduce its images too (the oracle's do at
# tolerance 0, tests/test_reference_images_cpu.py).
CROSS = [
    ("plan_erot_bcd_reg0_1", "sinkhorn_newton", 1e-9, 1000),
    ("plan_erot_bcd_reg0_1", "sinkhorn_ssns", 1e-9, 1000),
    ("plan_erot_ssns_reg0_01", "sinkhorn_newton", 1e-9, 1000),
    ("plan_erot_ssns_reg0_01", "sinkhorn_bcd", 1e-9, 20000),
]


@pytest.mark.parametrize("name,solver,tol,max_iter", CROSS,
                         ids=[f"{c[0][5:]}-{c[1]}" for c in CROSS])
def test_gpu_other_erot_solvers_reproduce_reference_image(name, solver, tol, max_iter):
    labels, rgb, call = P.load(name)
    M, a, b = readme_example(100, 80)
    r = getattr(regot, solver)(M, a, b, call["reg"], tol=tol, max_iter=max_iter,
                               precision="fp64")
    assert r.mar_errs[-1] < tol
    T = np.asarray(r.plan)
    bad = P.violations(T, labels, rgb, tol=TOL_BINS["fp64"])
    assert bad == 0, (f"{bad} constraints broken; needed {P.needed_tol(T, labels, rgb)}")
