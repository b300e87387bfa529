"""Regenerate the golden fixtures of tests/golden/ from the FP64 oracle.

The reference ships no golden vectors and cannot be built here (its numerics
need Eigen, which is not available offline), so these fixtures are outputs of
the oracle restatement on small seeded inputs. They pin the oracle against
regressions (tests/test_golden_cpu.py) and give the GPU tests a fixed target
(tests/test_gpu_golden.py).

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")]

import regot_oracle as O  # noqa: E402
from problems import erot_points, qrot_points, readme_example  # noqa: E402

# name -> (problem builder, solver, reg, tol, max_iter, kwargs)
CASES = {
    "bcd_readme_40x30_r0.1": (lambda: readme_example(40, 30), "sinkhorn_bcd", 0.1, 1e-10, 1000, {}),
    "bcd_points_48x36_r0.05": (lambda: erot_points(48, 36, seed=21, dtype=np.float64),
                               "sinkhorn_bcd", 0.05, 1e-10, 2000, {}),
    "newton_readme_40x30_r0.05": (lambda: readme_example(40, 30), "sinkhorn_newton", 0.05,
                                  1e-10, 200, {}),
    "ssns_readme_40x30_r0.05": (lambda: readme_example(40, 30), "sinkhorn_ssns", 0.05, 1e-10,
                                300, {}),
    "ssns_points_48x36_r0.02": (lambda: erot_points(48, 36, seed=22, dtype=np.float64),
                                "sinkhorn_ssns", 0.02, 1e-10, 300, {}),
    "lbfgs_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=23, dtype=np.float64),
                                "qrot_lbfgs_dual", 0.1, 1e-8, 3000, {}),
    "assn_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=24, dtype=np.float64),
                               "qrot_assn", 0.1, 1e-10, 20, {}),
    # fixed iteration counts (tol 1e-14): the histories follow step for step
    "lbfgsdual_readme_40x30_r0.1": (lambda: readme_example(40, 30), "sinkhorn_lbfgs_dual", 0.1,
                                    1e-14, 15, {}),
    "apdagd_readme_40x30_r0.1": (lambda: readme_example(40, 30), "sinkhorn_apdagd", 0.1,
                                 1e-14, 30, {}),
    "sparsenewton_points_48x36_r0.05": (lambda: erot_points(48, 36, seed=25, dtype=np.float64),
                                        "sinkhorn_sparse_newton", 0.05, 1e-14, 10,
                                        {"density": 0.3}),
    "splr_points_48x36_r0.05": (lambda: erot_points(48, 36, seed=26, dtype=np.float64),
                                "sinkhorn_splr", 0.05, 1e-14, 10, {"density": 0.3}),
    "qbcd_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=27, dtype=np.float64),
                               "qrot_bcd", 0.1, 1e-14, 20, {}),
    "qgd_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=28, dtype=np.float64),
                              "qrot_gd", 0.1, 1e-14, 20, {}),
    "qapdagd_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=29, dtype=np.float64),
                                  "qrot_apdagd", 0.1, 1e-14, 20, {}),
    "qpdaam_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=30, dtype=np.float64),
                                 "qrot_pdaam", 0.1, 1e-14, 20, {}),
    "grssn_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=31, dtype=np.float64),
                                "qrot_grssn", 0.1, 1e-14, 6, {}),
    "semidual_points_32x24_r0.1": (lambda: qrot_points(32, 24, seed=32, dtype=np.float64),
                                   "qrot_lbfgs_semi_dual", 0.1, 1e-14, 15, {}),
    # converged interior-point solves
    "pdipcg_points_30x25_r0.1": (lambda: qrot_points(30, 25, seed=33, dtype=np.float64),
                                 "qrot_pdip", 0.1, 1e-8, 200, {"inner_solver": "cg"}),
    "pdipfp_points_30x25_r0.1": (lambda: qrot_points(30, 25, seed=34, dtype=np.float64),
                                 "qrot_pdip", 0.1, 1e-8, 200, {"inner_solver": "fp"}),
}


def solve(name):
    make, solver, reg, tol, max_iter, kw = CASES[name]
    M, a, b = make()
    r = getattr(O, solver)(M, a, b, reg, tol=tol, max_iter=max_iter, **kw)
    out = dict(M=M, a=a, b=b, reg=reg, tol=tol, max_iter=max_iter, solver=solver,
               kwargs=json.dumps(kw), niter=r.niter, plan=r.plan,
               obj_vals=np.array(r.obj_vals), mar_errs=np.array(r.mar_errs))
    if hasattr(r, "dual"):
        out["dual"] = r.dual
    if hasattr(r, "converged"):
        out["converged"] = r.converged
    if hasattr(r, "densities"):
        out["densities"] = np.array(r.densities)
    if hasattr(r, "prim_vals"):
        out["prim_vals"] = np.array(r.prim_vals)
    return out


def main():
    for name in CASES:
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **solve(name))
        print("wrote", name)


if __name__ == "__main__":
    main()
