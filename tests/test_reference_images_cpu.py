"""The oracle against the reference's own outputs: the four transport plans
that the reference's solvers computed on the README example and rendered as
figs/plan_*.png (read back into tests/golden/reference_images/ by
make_reference_images.py there).

The oracle's plans fall, entry for entry, in the colormap bins that the
reference's images show (tol = 0: 8-bit resolution of the plan's range, no
entry excused). The same check rejects planted mistakes and solves that
differ from the reference's call only slightly (an earlier stop, a 1 %
different reg), so it pins the oracle at that resolution.
"""
import numpy as np
import pytest

import plan_image as P
import regot_oracle as O
from problems import readme_example


@pytest.fixture(scope="module")
def readme():
    return readme_example(100, 80)


def _solve(readme, call, **over):
    M, a, b = readme
    kw = dict(call["kwargs"])
    args = dict(tol=call["tol"], max_iter=call["max_iter"])
    args.update(over)
    reg = args.pop("reg", call["reg"])
    return getattr(O, call["solver"])(M, a, b, reg, **args, **kw)


@pytest.fixture(scope="module")
def oracle_plans(readme):
    out = {}
    for name in P.IMAGES:
        labels, rgb, call = P.load(name)
        out[name] = np.asarray(_solve(readme, call).plan)
    return out


def test_fixture_matches_the_calls():
    for name in P.IMAGES:
        labels, rgb, call = P.load(name)
        assert labels.shape == (100, 80) and labels.max() == len(rgb) - 1
        assert (call["n"], call["m"]) == (100, 80)
        # viridis's first and last entries truncated to 8 bits
        assert tuple(rgb[np.argmin(rgb[:, 1])]) == (68, 1, 84)
        assert tuple(rgb[np.argmax(rgb[:, 1])]) == (253, 231, 36)


@pytest.mark.parametrize("name", P.IMAGES)
def test_oracle_reproduces_reference_image(name, oracle_plans):
    labels, rgb, _ = P.load(name)
    assert P.violations(oracle_plans[name], labels, rgb, tol=0.0) == 0


@pytest.mark.parametrize("name", P.IMAGES)
def test_planted_mistakes_are_detected(name, oracle_plans):
    """Mistakes planted in the oracle's plan: one entry moved by two bins, a
    1 % drift across the rows, two rows swapped."""
    labels, rgb, _ = P.load(name)
    T = oracle_plans[name]
    span = T.max() - T.min()
    moved = T.copy()
    i, j = np.unravel_index(np.argsort(T, axis=None)[T.size // 2 + 3000], T.shape)
    moved[i, j] += 2.0 / 256 * span
    drift = T * (1.0 + 0.01 * np.arange(T.shape[0])[:, None] / T.shape[0])
    swapped = T.copy()
    swapped[[10, 11]] = swapped[[11, 10]]
    for bad in (moved, drift, swapped):
        assert P.violations(bad, labels, rgb, tol=0.0) > 0


def test_close_but_different_solves_are_rejected(readme):
    """sinkhorn_bcd stopped at tol 1e-5 instead of 1e-6, or run at reg 0.099
    or 0.101 instead of 0.1, does not reproduce the reference's image."""
    labels, rgb, call = P.load("plan_erot_bcd_reg0_1")
    assert P.violations(_solve(readme, call, tol=1e-5).plan, labels, rgb) > 0
    for reg in (0.099, 0.101):
        assert P.violations(_solve(readme, call, reg=reg).plan, labels, rgb) > 0


# EROT has a unique plan, so solvers other than the one the reference ran
# reproduce its image once they are converged well below the reference's
# tol 1e-6 (the QROT solvers other than PDIP converge too slowly on this
# problem to be compared the same way).
CROSS = [
    ("plan_erot_bcd_reg0_1", "sinkhorn_newton", 1e-9, 1000),
    ("plan_erot_bcd_reg0_1", "sinkhorn_ssns", 1e-9, 1000),
    ("plan_erot_bcd_reg0_1", "sinkhorn_bcd", 1e-10, 5000),
    ("plan_erot_ssns_reg0_01", "sinkhorn_newton", 1e-9, 1000),
    ("plan_erot_ssns_reg0_01", "sinkhorn_bcd", 1e-9, 20000),
]


@pytest.mark.parametrize("name,solver,tol,max_iter", CROSS,
                         ids=[f"{c[0][5:]}-{c[1]}" for c in CROSS])
def test_other_erot_solvers_reproduce_reference_image(readme, name, solver, tol, max_iter):
    labels, rgb, call = P.load(name)
    M, a, b = readme
    r = getattr(O, solver)(M, a, b, call["reg"], tol=tol, max_iter=max_iter)
    assert r.mar_errs[-1] < tol
    assert P.violations(r.plan, labels, rgb, tol=0.0) == 0


def test_checker_edge_cases():
    """The checker refuses a plan of another shape and finds no tolerance at
    which an unrelated plan matches."""
    labels, rgb, _ = P.load("plan_erot_bcd_reg0_1")
    with pytest.raises(ValueError):
        P.violations(np.ones((80, 100)), labels, rgb)
    noise = np.random.default_rng(0).random(labels.shape)
    assert P.needed_tol(noise, labels, rgb) == float("inf")
