"""ctypes front end of the FP64 CPU oracle (test infrastructure only).

The oracle restates the reference solvers of yixuan/regot-python in plain
C++ (see oracle.h for the per-function citations). This module exposes it
with the reference's Python signatures, ``regot.<solver>(M, a, b, reg,
tol=1e-6, max_iter=1000, verbose=0, **kwargs)`` (src/solvers.cpp:463-528),
so tests can call the oracle and the CUDA path the same way.

Only tests, ``__graft_entry__.smoke()`` and the CPU baseline of ``bench.py``
use this module. Parity status: pinned at 8-bit resolution to the
reference's own README plan images (four solves on the 100 x 80 README
example, tests/test_reference_images_cpu.py); the reference ships no golden
vectors and cannot be compiled here.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from types import SimpleNamespace

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Opts(C.Structure):
    _fields_ = [
        ("x0", _dp),
        ("x0_len", C.c_int),
        ("method", C.c_int),
        ("mu0", C.c_double),
        ("shift", C.c_double),
        ("density", C.c_double),
        ("tau", C.c_double),
    ]


class _Result(C.Structure):
    _fields_ = [
        ("niter", C.c_int),
        ("hist_len", C.c_int),
        ("hist_cap", C.c_int),
        ("dual", _dp),
        ("plan", _dp),
        ("obj_vals", _dp),
        ("mar_errs", _dp),
        ("run_times", _dp),
        ("densities", _dp),
        ("prim_vals", _dp),
        ("err", C.c_char * 256),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, no other dependency)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _lib.oracle_erot_dual_obj.restype = C.c_double
        _lib.oracle_erot_dual_obj_grad.restype = C.c_double
        _lib.oracle_erot_compute_T.restype = C.c_double
        _lib.oracle_sparsify_mat3.restype = C.c_long
        _lib.oracle_sparsify_density.restype = C.c_long
        _lib.oracle_wolfe_poly.restype = C.c_double
        _lib.oracle_qrot_dual_obj.restype = C.c_double
        _lib.oracle_qrot_dual_obj_grad.restype = C.c_double
        _lib.oracle_qrot_primal_val.restype = C.c_double
        for name in ("oracle_sparsify_mat3",):
            getattr(_lib, name).argtypes = [
                _dp, C.c_int, C.c_int, C.c_double, C.c_double, _ip, _ip, _dp, C.c_long]
    return _lib


def _d(x):
    return x.ctypes.data_as(_dp)


def _f64(x, order="C"):
    return np.require(np.asarray(x, dtype=np.float64), requirements=[order[0], "A"])


def _colmajor(M):
    return np.asfortranarray(np.asarray(M, dtype=np.float64))


def _opts(kwargs, method_default, n_dual):
    o = _Opts()
    x0 = kwargs.get("x0")
    keep = []
    if x0 is not None:
        x0 = _f64(x0).ravel()
        keep.append(x0)
        o.x0 = _d(x0)
        o.x0_len = x0.size
    o.method = int(kwargs.get("method", method_default))
    o.mu0 = float(kwargs.get("mu0", 1.0))
    o.shift = float(kwargs.get("shift", 1e-3))
    o.density = float(kwargs.get("density", 0.01))
    o.tau = float(kwargs.get("tau", 0.0))
    return o, keep


def _run(fn, M, a, b, reg, tol, max_iter, verbose, kwargs, dual_len, method_default,
         with_prim=False, with_dens=False, plan=True):
    M = _colmajor(M)
    n, m = M.shape
    a = _f64(a).ravel()
    b = _f64(b).ravel()
    cap = max_iter + 2
    bufs = {k: np.zeros(cap) for k in ("obj_vals", "mar_errs", "run_times", "densities", "prim_vals")}
    dual = np.zeros(dual_len(n, m))
    P = np.zeros((n, m)) if plan else None
    r = _Result()
    r.hist_cap = cap
    r.dual = _d(dual)
    r.plan = _d(P) if plan else _dp()
    for k, v in bufs.items():
        setattr(r, k, _d(v))
    o, keep = _opts(kwargs, method_default, dual_len(n, m))
    rc = fn(_d(M), n, m, _d(a), _d(b), C.c_double(reg), C.c_double(tol), int(max_iter),
            int(verbose), C.byref(o), C.byref(r))
    del keep
    if rc == 2:
        raise ValueError(r.err.decode())
    if rc != 0:
        raise RuntimeError(r.err.decode())
    L = r.hist_len
    out = SimpleNamespace(niter=r.niter, dual=dual, plan=P,
                          obj_vals=list(bufs["obj_vals"][:L]),
                          mar_errs=list(bufs["mar_errs"][:L]),
                          run_times=list(bufs["run_times"][:L]))
    if with_dens:
        out.densities = list(bufs["densities"][:L])
    if with_prim:
        out.prim_vals = list(bufs["prim_vals"][:L])
    return out


_EROT_DUAL = lambda n, m: n + m - 1  # noqa: E731
_QROT_DUAL = lambda n, m: n + m  # noqa: E731


def sinkhorn_bcd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_sinkhorn_bcd, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _EROT_DUAL, 1, with_dens=False, plan=kwargs.get("plan", True))


def sinkhorn_newton(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_sinkhorn_newton, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _EROT_DUAL, 1, plan=kwargs.get("plan", True))


def sinkhorn_ssns(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_sinkhorn_ssns, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _EROT_DUAL, 1, with_dens=True, plan=kwargs.get("plan", True))


def sinkhorn_sparse_newton(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_sinkhorn_sparse_newton, M, a, b, reg, tol, max_iter, verbose,
                kwargs, _EROT_DUAL, 1, with_dens=True, plan=kwargs.get("plan", True))


def sinkhorn_splr(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_sinkhorn_splr, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _EROT_DUAL, 1, with_dens=True, plan=kwargs.get("plan", True))


def sinkhorn_lbfgs_dual(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_sinkhorn_lbfgs_dual, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _EROT_DUAL, 1, plan=kwargs.get("plan", True))


def sinkhorn_apdagd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_sinkhorn_apdagd, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _EROT_DUAL, 1, plan=kwargs.get("plan", True))


def qrot_lbfgs_dual(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_lbfgs_dual, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


def qrot_bcd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_bcd, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


def qrot_gd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_gd, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


def qrot_apdagd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_apdagd, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


def qrot_pdaam(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_pdaam, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


def qrot_grssn(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_grssn, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


def qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_lbfgs_semi_dual, M, a, b, reg, tol, max_iter, verbose,
                kwargs, _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


_PDIP_KEYS = ("cg_max_iter", "fixed_threshold", "fp_max_iter", "fp_exit_scale",
              "fp_stop_gap_mu_only", "cg_stop_gap_mu_only", "cg_mar_tol")
_PDIP_DEFAULTS = (1000, 1e-9, 800, 1e-2, True, False, 1e-10)


def qrot_pdip(M, a, b, reg, tol=1e-8, max_iter=1000, verbose=0, **kwargs):
    """qrot_pdip restated: namespace(niter, converged, plan, obj_vals,
    mar_errs, run_times)."""
    M = _colmajor(M)
    n, m = M.shape
    a = _f64(a).ravel()
    b = _f64(b).ravel()
    mode = str(kwargs.get("inner_solver", "cg")).lower()
    popts = np.array([float(kwargs.get(k, dflt)) for k, dflt in zip(_PDIP_KEYS, _PDIP_DEFAULTS)])
    cap = max_iter + 2
    hist = np.zeros((3, cap))
    plan = np.zeros((n, m))
    flag = np.zeros(1)
    r = _Result()
    r.hist_cap = cap
    r.dual = _d(flag)
    r.plan = _d(plan)
    r.obj_vals = _d(hist[0])
    r.mar_errs = _d(hist[1])
    r.run_times = _d(hist[2])
    rc = lib().oracle_qrot_pdip(_d(M), n, m, _d(a), _d(b), C.c_double(reg), C.c_double(tol),
                                int(max_iter), 1 if mode == "fp" else 0, _d(popts), C.byref(r))
    if rc != 0:
        raise RuntimeError(r.err.decode())
    k = r.hist_len
    return SimpleNamespace(niter=r.niter, converged=bool(flag[0]), plan=plan,
                           obj_vals=hist[0, :k].tolist(), mar_errs=hist[1, :k].tolist(),
                           run_times=hist[2, :k].tolist())


def qrot_optimal_alpha(M, a, reg, beta):
    M = _colmajor(M)
    n, m = M.shape
    alpha = np.zeros(n)
    lib().oracle_qrot_optimal_alpha(_d(M), n, m, _d(_f64(a)), C.c_double(reg), _d(_f64(beta)),
                                    _d(alpha))
    return alpha


def qrot_assn(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    return _run(lib().oracle_qrot_assn, M, a, b, reg, tol, max_iter, verbose, kwargs,
                _QROT_DUAL, 0, with_prim=True, plan=kwargs.get("plan", True))


# ---------------- problem pieces ----------------

def erot_optimal_beta(M, b, reg, alpha):
    M = _colmajor(M)
    n, m = M.shape
    alpha = _f64(alpha).ravel()
    b = _f64(b).ravel()
    out = np.zeros(m)
    lib().oracle_erot_optimal_beta(_d(M), n, m, _d(b), C.c_double(reg), _d(alpha), _d(out))
    return out


def erot_optimal_alpha(M, a, reg, beta):
    M = _colmajor(M)
    n, m = M.shape
    beta = _f64(beta).ravel()
    a = _f64(a).ravel()
    out = np.zeros(n)
    lib().oracle_erot_optimal_alpha(_d(M), n, m, _d(a), C.c_double(reg), _d(beta), _d(out))
    return out


def erot_dual_obj(M, a, b, reg, gamma):
    M = _colmajor(M)
    n, m = M.shape
    return lib().oracle_erot_dual_obj(_d(M), n, m, _d(_f64(a)), _d(_f64(b)), C.c_double(reg),
                                      _d(_f64(gamma)))


def erot_dual_obj_grad(M, a, b, reg, gamma):
    M = _colmajor(M)
    n, m = M.shape
    g = np.zeros(n + m - 1)
    f = lib().oracle_erot_dual_obj_grad(_d(M), n, m, _d(_f64(a)), _d(_f64(b)), C.c_double(reg),
                                        _d(_f64(gamma)), _d(g))
    return f, g


def erot_hvp(M, a, b, reg, gamma, x):
    M = _colmajor(M)
    n, m = M.shape
    y = np.zeros(n + m - 1)
    lib().oracle_erot_hvp(_d(M), n, m, _d(_f64(a)), _d(_f64(b)), C.c_double(reg),
                          _d(_f64(gamma)), _d(_f64(x)), _d(y))
    return y


def erot_newton_direction(M, a, b, reg, gamma):
    M = _colmajor(M)
    n, m = M.shape
    d = np.zeros(n + m - 1)
    rc = lib().oracle_erot_newton_direction(_d(M), n, m, _d(_f64(a)), _d(_f64(b)),
                                            C.c_double(reg), _d(_f64(gamma)), _d(d))
    if rc != 0:
        raise RuntimeError("Hessian not positive definite")
    return d


def erot_compute_T(M, reg, gamma):
    """T column-major as an (n, m) array."""
    M = _colmajor(M)
    n, m = M.shape
    T = np.zeros((n, m), order="F")
    lib().oracle_erot_compute_T(_d(M), n, m, C.c_double(reg), _d(_f64(gamma)), _d(T))
    return T


def sparsify_mat3(T, delta, density_hint):
    """Returns (outer[m], inner[nnz], values[nnz]) of the CSC of kept entries."""
    T = _colmajor(T)
    n, m = T.shape
    cap = n * max(m - 1, 0) + 1
    outer = np.zeros(m, dtype=np.int32)
    inner = np.zeros(cap, dtype=np.int32)
    vals = np.zeros(cap)
    nnz = lib().oracle_sparsify_mat3(_d(T), n, m, C.c_double(delta), C.c_double(density_hint),
                                     outer.ctypes.data_as(_ip), inner.ctypes.data_as(_ip),
                                     _d(vals), C.c_long(cap))
    return outer, inner[:nnz].copy(), vals[:nnz].copy()


def sparsify_density(T, density):
    """sparsify_mat_with_density: (outer[m], inner[nnz], values[nnz]) CSC."""
    T = _colmajor(T)
    n, m = T.shape
    cap = n * max(m - 1, 0) + 1
    outer = np.zeros(m, dtype=np.int32)
    inner = np.zeros(cap, dtype=np.int32)
    vals = np.zeros(cap)
    nnz = lib().oracle_sparsify_density(_d(T), n, m, C.c_double(density),
                                        outer.ctypes.data_as(_ip), inner.ctypes.data_as(_ip),
                                        _d(vals), C.c_long(cap))
    return outer, inner[:nnz].copy(), vals[:nnz].copy()


def wolfe_poly(coefs, init_step):
    """More-Thuente line search on a quartic: (step, recompute, evaluations)."""
    c = _f64(coefs).ravel()
    flag = C.c_int(0)
    nev = C.c_int(0)
    step = lib().oracle_wolfe_poly(_d(c), C.c_double(init_step), C.byref(flag), C.byref(nev))
    return step, bool(flag.value), nev.value


def erot_plan(M, reg, gamma):
    M = _colmajor(M)
    n, m = M.shape
    P = np.zeros((n, m))
    lib().oracle_erot_plan(_d(M), n, m, C.c_double(reg), _d(_f64(gamma)), _d(P))
    return P


def qrot_dual_obj(M, a, b, reg, gamma, tau=0.0):
    M = _colmajor(M)
    n, m = M.shape
    return lib().oracle_qrot_dual_obj(_d(M), n, m, _d(_f64(a)), _d(_f64(b)), C.c_double(reg),
                                      C.c_double(tau), _d(_f64(gamma)))


def qrot_dual_obj_grad(M, a, b, reg, gamma, tau=0.0):
    M = _colmajor(M)
    n, m = M.shape
    g = np.zeros(n + m)
    f = lib().oracle_qrot_dual_obj_grad(_d(M), n, m, _d(_f64(a)), _d(_f64(b)), C.c_double(reg),
                                        C.c_double(tau), _d(_f64(gamma)), _d(g))
    return f, g


def qrot_optimal_beta(M, b, reg, alpha):
    M = _colmajor(M)
    n, m = M.shape
    out = np.zeros(m)
    lib().oracle_qrot_optimal_beta(_d(M), n, m, _d(_f64(b)), C.c_double(reg),
                                   _d(_f64(alpha)), _d(out))
    return out


def qrot_primal_val(M, a, b, reg, gamma):
    M = _colmajor(M)
    n, m = M.shape
    return lib().oracle_qrot_primal_val(_d(M), n, m, _d(_f64(a)), _d(_f64(b)), C.c_double(reg),
                                        _d(_f64(gamma)))


def qrot_hess_cg(M, gamma, rhs, shift, tau=0.0, cg_tol=1e-8):
    M = _colmajor(M)
    n, m = M.shape
    out = np.zeros(n + m)
    lib().oracle_qrot_hess_cg(_d(M), n, m, _d(_f64(gamma)), _d(_f64(rhs)), C.c_double(shift),
                              C.c_double(tau), C.c_double(cg_tol), _d(out))
    return out


def qrot_plan(M, reg, gamma):
    M = _colmajor(M)
    n, m = M.shape
    P = np.zeros((n, m))
    lib().oracle_qrot_plan(_d(M), n, m, C.c_double(reg), _d(_f64(gamma)), _d(P))
    return P
