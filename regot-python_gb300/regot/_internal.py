"""GPU mirror of the reference's ``regot._internal`` module.

Same names, positional/keyword arguments and defaults as the pybind11
bindings of src/solvers.cpp:463-528:

    sinkhorn_bcd / sinkhorn_newton / sinkhorn_ssns
    qrot_lbfgs_dual / qrot_assn
        (M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs)

and the same result classes (``sinkhorn_result`` with niter, dual, plan,
obj_vals, mar_errs, run_times, densities; ``qrot_result`` with niter, dual,
plan, obj_vals, prim_vals, mar_errs, run_times; solvers.cpp:531-564).

Reference kwargs: ``method``, ``mu0``, ``shift``, ``density`` (EROT) and
``method``, ``shift`` (QROT), with the reference defaults; unknown kwargs are
ignored as in the reference. Additional kwargs of this implementation:

    precision  "fp64" (M stored and processed in FP64) or "mixed" (M in FP32,
               FP64 duals); default "fp64" for float64 M, "mixed" for float32 M
    x0         initial dual vector (n+m-1 for EROT, n+m for QROT)
    device     CUDA device index (default 0)
    plan       False to skip computing the plan (default True)
    prim_vals  QROT: False to skip the per-iteration primal value
    cg_tol     Newton-CG relative residual target

M may be a NumPy array (C or Fortran order, float64 or float32) or a CUDA
torch tensor (used in place, no host round trip). The solve runs on the GPU;
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

__all__ = [
    "sinkhorn_bcd", "sinkhorn_newton", "sinkhorn_ssns", "sinkhorn_lbfgs_dual", "sinkhorn_apdagd",
    "sinkhorn_sparse_newton", "sinkhorn_splr",
    "qrot_lbfgs_dual", "qrot_assn", "qrot_bcd", "qrot_gd", "qrot_apdagd", "qrot_pdaam",
    "qrot_grssn", "qrot_lbfgs_semi_dual", "qrot_pdip", "pdip_cg", "pdip_fp", "pdip_result", "sinkhorn_result", "qrot_result",
    "Problem",
    "sinkhorn_bcd_batched", "batch_result",
]


class sinkhorn_result:
    """Result of an EROT solver (src/sinkhorn_result.h:13-30)."""

    def __init__(self):
        self.niter = 0
        self.dual = np.zeros(0)
        self.plan = np.zeros((0, 0))
        self.obj_vals = []
        self.mar_errs = []
        self.run_times = []
        self.densities = []

    def __repr__(self):
        return f"<sinkhorn_result niter={self.niter}>"


class qrot_result:
    """Result of a QROT solver (src/qrot_result.h:13-30)."""

    def __init__(self):
        self.niter = 0
        self.dual = np.zeros(0)
        self.plan = np.zeros((0, 0))
        self.obj_vals = []
        self.prim_vals = []
        self.mar_errs = []
        self.run_times = []

    def __repr__(self):
        return f"<qrot_result niter={self.niter}>"


class pdip_result:
    """Result of qrot_pdip (src/pdip_result.h:13-33). The per-phase timing
    fields are filled only by the reference's developer build; they are 0."""

    def __init__(self):
        self.niter = 0
        self.converged = False
        self.plan = np.zeros((0, 0))
        self.obj_vals = []
        self.mar_errs = []
        self.run_times = []
        self.t_build_B = 0.0
        self.t_chol_factor = 0.0
        self.t_chol_solve = 0.0
        self.t_eq_matvec = 0.0
        self.t_other = 0.0

    def __repr__(self):
        return f"<pdip_result niter={self.niter} converged={self.converged}>"


def _is_torch_cuda(x) -> bool:
    t = type(x)
    return t.__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _check_cuda_f64(t, shape, name):
    import torch

    if not (_is_torch_cuda(t) and t.dtype == torch.float64 and t.is_contiguous()
            and tuple(t.shape) == tuple(shape)):
        raise ValueError(f"{name} must be a contiguous float64 CUDA tensor of shape {shape}")


def _precision_code(precision, dtype) -> int:
    if precision is None:
        return L.REGOT_PREC_FP64 if dtype == np.float64 else L.REGOT_PREC_MIXED
    p = str(precision).lower()
    if p in ("fp64", "float64", "double", "plain"):
        return L.REGOT_PREC_FP64
    if p in ("mixed", "fp32", "float32"):
        return L.REGOT_PREC_MIXED
    raise ValueError(f"unknown precision {precision!r}; use 'fp64' or 'mixed'")


class Problem:
    """A cost matrix and marginals resident on one GPU (regot_dproblem).

    Reusing a Problem for several solves uploads M once.
    """

    def __init__(self, M, a, b, precision=None, device: int = 0):
        self.ctx = L.context(device)
        lib = L.load()
        self._keep = []
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())
        b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).ravel())
        d = L.ProblemDesc()
        if _is_torch_cuda(M):
            import torch  # only when a torch tensor is passed

            if M.dim() != 2:
                raise ValueError("M must be a 2-D matrix")
            if M.dtype not in (torch.float32, torch.float64):
                M = M.to(torch.float64)
            if M.stride(1) != 1:
                M = M.contiguous()
            n, m = M.shape
            d.M = C.c_void_p(M.data_ptr())
            d.M_dtype = L.REGOT_F64 if M.dtype == torch.float64 else L.REGOT_F32
            d.M_mem = L.REGOT_MEM_DEVICE
            d.ldm = M.stride(0)
            dtype = np.float64 if M.dtype == torch.float64 else np.float32
            self._keep.append(M)
        else:
            M = np.asarray(M)
            if M.ndim != 2:
                raise ValueError("M must be a 2-D matrix")
            if M.dtype not in (np.float64, np.float32):
                M = M.astype(np.float64)
            M = np.ascontiguousarray(M)
            n, m = M.shape
            d.M = C.c_void_p(M.ctypes.data)
            d.M_dtype = L.REGOT_F64 if M.dtype == np.float64 else L.REGOT_F32
            d.M_mem = L.REGOT_MEM_HOST
            d.ldm = m
            dtype = M.dtype
            self._keep.append(M)
        if a.size != n or b.size != m:
            raise ValueError(f"a must have {n} entries and b {m} entries (M is {n}x{m})")
        d.n, d.m = n, m
        d.a = C.c_void_p(a.ctypes.data)
        d.b = C.c_void_p(b.ctypes.data)
        d.ab_mem = L.REGOT_MEM_HOST
        self.n, self.m = n, m
        self.precision = _precision_code(precision, dtype)
        h = C.c_void_p()
        self.ctx.check(lib.regot_problem_create(self.ctx.handle, C.byref(d), self.precision,
                                                C.byref(h)))
        self.handle = h
        self._keep = []
        self._lib = lib

    def close(self):
        if getattr(self, "handle", None):
            self._lib.regot_problem_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- solver calls -------------------------------------------------
    def _solve(self, fname, reg, tol, max_iter, verbose, kwargs, qrot):
        n, m = self.n, self.m
        o = L.Opts()
        self._lib.regot_opts_init(C.byref(o))
        o.precision = self.precision
        if "method" in kwargs:
            o.method = int(kwargs["method"])
        if "mu0" in kwargs:
            o.mu0 = float(kwargs["mu0"])
        if "shift" in kwargs:
            o.shift = float(kwargs["shift"])
        if "density" in kwargs:
            o.density = float(kwargs["density"])
        if "cg_tol" in kwargs:
            o.cg_tol = float(kwargs["cg_tol"])
        if "cg_max_iter" in kwargs:
            o.cg_max_iter = int(kwargs["cg_max_iter"])
        o.verbose = int(verbose)
        want_plan = bool(kwargs.get("plan", True))
        o.plan = 1 if want_plan else 0
        o.prim_vals = 1 if kwargs.get("prim_vals", True) else 0
        x0 = kwargs.get("x0")
        keep = []
        if x0 is not None:
            x0 = np.ascontiguousarray(np.asarray(x0, dtype=np.float64).ravel())
            keep.append(x0)
            o.x0 = x0.ctypes.data_as(C.POINTER(C.c_double))
            o.x0_len = x0.size
        max_iter = int(max_iter)
        if max_iter < 0:
            raise ValueError("max_iter must be non-negative")
        cap = max_iter + 2
        dual = np.zeros(n + m if qrot else n + m - 1)
        plan = L.host_empty((n, m)) if want_plan else None
        hist = np.zeros((5, cap))
        r = L.Result()
        r.hist_cap = cap
        r.dual = dual.ctypes.data
        r.plan = plan.ctypes.data if want_plan else None
        r.obj_vals = hist[0].ctypes.data
        r.mar_errs = hist[1].ctypes.data
        r.run_times = hist[2].ctypes.data
        r.densities = hist[3].ctypes.data
        r.prim_vals = hist[4].ctypes.data
        fn = getattr(self._lib, fname)
        self.ctx.check(fn(self.ctx.handle, self.handle, float(reg), float(tol), max_iter,
                          C.byref(o), C.byref(r)))
        k = r.hist_len
        res = qrot_result() if qrot else sinkhorn_result()
        res.niter = int(r.niter)
        res.dual = dual
        res.plan = plan
        res.obj_vals = hist[0, :k].tolist()
        res.mar_errs = hist[1, :k].tolist()
        res.run_times = hist[2, :k].tolist()
        if qrot:
            res.prim_vals = hist[4, :k].tolist()
        elif fname in ("regot_sinkhorn_ssns", "regot_sinkhorn_sparse_newton",
                       "regot_sinkhorn_splr"):
            res.densities = hist[3, :k].tolist()
        res.passes = int(r.passes)
        res.solve_ms = float(r.solve_ms)
        if verbose:
            for i in range(k):
                print(f"iter = {i}, objval = {res.obj_vals[i]}, ||grad|| = {res.mar_errs[i]}")
        return res

    def sinkhorn_bcd(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_sinkhorn_bcd", reg, tol, max_iter, verbose, kw, False)

    def sinkhorn_newton(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_sinkhorn_newton", reg, tol, max_iter, verbose, kw, False)

    def sinkhorn_ssns(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_sinkhorn_ssns", reg, tol, max_iter, verbose, kw, False)

    def sinkhorn_sparse_newton(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_sinkhorn_sparse_newton", reg, tol, max_iter, verbose, kw, False)

    def sinkhorn_splr(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_sinkhorn_splr", reg, tol, max_iter, verbose, kw, False)

    def sinkhorn_lbfgs_dual(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_sinkhorn_lbfgs_dual", reg, tol, max_iter, verbose, kw, False)

    def sinkhorn_apdagd(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_sinkhorn_apdagd", reg, tol, max_iter, verbose, kw, False)

    def qrot_lbfgs_dual(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_lbfgs_dual", reg, tol, max_iter, verbose, kw, True)

    def qrot_assn(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_assn", reg, tol, max_iter, verbose, kw, True)

    def qrot_bcd(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_bcd", reg, tol, max_iter, verbose, kw, True)

    def qrot_gd(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_gd", reg, tol, max_iter, verbose, kw, True)

    def qrot_apdagd(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_apdagd", reg, tol, max_iter, verbose, kw, True)

    def qrot_pdaam(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_pdaam", reg, tol, max_iter, verbose, kw, True)

    def qrot_pdip(self, reg, tol=1e-8, max_iter=1000, verbose=0, **kw):
        """qrot_pdip (solvers.cpp:268-292): kwargs inner_solver ("cg" | "fp")
        and the PDIPSolverOpts fields parsed by parse_pdip_opts (203-239)."""
        mode = kw.get("inner_solver", "cg")
        if not isinstance(mode, str):
            raise RuntimeError(
                'qrot_pdip: inner_solver must be a string, e.g. "cg" or "fp"')
        mode = mode.lower()
        if mode not in ("cg", "fp"):
            raise RuntimeError('qrot_pdip: inner_solver must be "cg" or "fp"')
        n, m = self.n, self.m
        po = L.PdipOpts()
        self._lib.regot_pdip_opts_init(C.byref(po))
        po.inner_solver = 1 if mode == "fp" else 0
        for key, conv in (("cg_max_iter", int), ("fixed_threshold", float),
                          ("fp_max_iter", int), ("fp_exit_scale", float),
                          ("fp_stop_gap_mu_only", bool), ("cg_stop_gap_mu_only", bool),
                          ("cg_mar_tol", float)):
            if key in kw:
                setattr(po, key, conv(kw[key]))
        o = L.Opts()
        self._lib.regot_opts_init(C.byref(o))
        o.verbose = int(verbose)
        want_plan = bool(kw.get("plan", True))
        o.plan = 1 if want_plan else 0
        max_iter = int(max_iter)
        if max_iter < 0:
            raise ValueError("max_iter must be non-negative")
        cap = max_iter + 2
        hist = np.zeros((3, cap))
        plan = L.host_empty((n, m)) if want_plan else None
        r = L.Result()
        r.hist_cap = cap
        r.plan = plan.ctypes.data if want_plan else None
        r.obj_vals = hist[0].ctypes.data
        r.mar_errs = hist[1].ctypes.data
        r.run_times = hist[2].ctypes.data
        conv = C.c_int(0)
        self.ctx.check(self._lib.regot_qrot_pdip(
            self.ctx.handle, self.handle, float(reg), float(tol), max_iter, C.byref(po),
            C.byref(o), C.byref(r), C.byref(conv)))
        k = r.hist_len
        res = pdip_result()
        res.niter = int(r.niter)
        res.converged = bool(conv.value)
        res.plan = plan
        res.obj_vals = hist[0, :k].tolist()
        res.mar_errs = hist[1, :k].tolist()
        res.run_times = hist[2, :k].tolist()
        res.solve_ms = float(r.solve_ms)
        return res

    def qrot_grssn(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_grssn", reg, tol, max_iter, verbose, kw, True)

    def qrot_lbfgs_semi_dual(self, reg, tol=1e-6, max_iter=1000, verbose=0, **kw):
        return self._solve("regot_qrot_lbfgs_semi_dual", reg, tol, max_iter, verbose, kw, True)

    # ---- pass-level calls --------------------------------------------
    def _vec(self, x, size):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
        if x.size != size:
            raise ValueError(f"expected a vector of length {size}")
        return x

    def erot_optimal_beta(self, reg, alpha):
        alpha = self._vec(alpha, self.n)
        out = np.zeros(self.m)
        self.ctx.check(self._lib.regot_erot_optimal_beta(
            self.ctx.handle, self.handle, float(reg), alpha.ctypes.data, out.ctypes.data))
        return out

    def erot_optimal_alpha(self, reg, beta):
        beta = self._vec(beta, self.m)
        out = np.zeros(self.n)
        self.ctx.check(self._lib.regot_erot_optimal_alpha(
            self.ctx.handle, self.handle, float(reg), beta.ctypes.data, out.ctypes.data))
        return out

    def erot_dual_obj_grad(self, reg, gamma):
        gamma = self._vec(gamma, self.n + self.m - 1)
        obj = np.zeros(1)
        grad = np.zeros(self.n + self.m - 1)
        self.ctx.check(self._lib.regot_erot_dual_obj_grad(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, obj.ctypes.data,
            grad.ctypes.data))
        return float(obj[0]), grad

    def erot_hvp(self, reg, gamma, x):
        gamma = self._vec(gamma, self.n + self.m - 1)
        x = self._vec(x, self.n + self.m - 1)
        y = np.zeros(self.n + self.m - 1)
        self.ctx.check(self._lib.regot_erot_hvp(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, x.ctypes.data,
            y.ctypes.data))
        return y

    def erot_plan(self, reg, gamma, out=None):
        """T(gamma) as an n x m FP64 array (sinkhorn_result.h:32-50); with
        `out` a contiguous float64 CUDA tensor of that shape, written there."""
        gamma = self._vec(gamma, self.n + self.m - 1)
        if out is not None:
            import torch

            _check_cuda_f64(out, (self.n, self.m), "out")
            torch.cuda.current_stream(out.device).synchronize()
            self.ctx.check(self._lib.regot_erot_plan(
                self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, out.data_ptr(),
                L.REGOT_MEM_DEVICE))
            return out
        P = L.host_empty((self.n, self.m))
        self.ctx.check(self._lib.regot_erot_plan(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, P.ctypes.data,
            L.REGOT_MEM_HOST))
        return P

    def erot_hess_solve(self, reg, gamma, rhs, tol=1e-10, max_iter=0):
        """x with H x = rhs for the exact dual Hessian at gamma (the Newton
        system of sinkhorn_newton.cpp:91-92), by preconditioned CG; returns
        (x, CG steps)."""
        gamma = self._vec(gamma, self.n + self.m - 1)
        rhs = self._vec(rhs, self.n + self.m - 1)
        x = np.zeros(self.n + self.m - 1)
        it = C.c_int(0)
        self.ctx.check(self._lib.regot_erot_hess_solve(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, rhs.ctypes.data,
            float(tol), int(max_iter), x.ctypes.data, C.byref(it)))
        return x, int(it.value)

    def erot_tyy(self, reg, gamma, Y, u=None, W=None):
        """(rows, Z): rows = G 1 and Z = G Y for G = T(gamma), or
        G = T o (u_i + u_j - W_ij) / reg when the adjoint u is given. numpy
        arguments run through host memory; float64 CUDA tensors (gamma, u,
        W, Y) stay on the device and the results are CUDA tensors."""
        return self._contract(reg, gamma, Y, u, W, cols=False)

    def erot_tty(self, reg, gamma, X, u=None, W=None):
        """(cols, Z): cols = G'1 and Z = G'X (X n x d) for the same G as
        erot_tyy."""
        return self._contract(reg, gamma, X, u, W, cols=True)

    def _contract(self, reg, gamma, Y, u, W, cols):
        n, m = self.n, self.m
        K, nown = (n, m) if cols else (m, n)
        fn = self._lib.regot_erot_tty if cols else self._lib.regot_erot_tyy
        if _is_torch_cuda(Y):
            import torch

            d = int(Y.shape[1])
            _check_cuda_f64(Y, (K, d), "Y")
            for name, t, shape in (("gamma", gamma, (n + m - 1,)), ("u", u, (n + m - 1,)),
                                   ("W", W, (n, m))):
                if t is not None:
                    _check_cuda_f64(t, shape, name)
            sums = torch.empty(nown, dtype=torch.float64, device=Y.device)
            Z = torch.empty((nown, d), dtype=torch.float64, device=Y.device)
            torch.cuda.current_stream(Y.device).synchronize()
            self.ctx.check(fn(
                self.ctx.handle, self.handle, float(reg), gamma.data_ptr(),
                u.data_ptr() if u is not None else None, W.data_ptr() if W is not None else None,
                Y.data_ptr(), d, sums.data_ptr(), Z.data_ptr(), L.REGOT_MEM_DEVICE))
            return sums, Z
        gamma = self._vec(gamma, n + m - 1)
        Y = np.ascontiguousarray(np.asarray(Y, dtype=np.float64))
        if Y.ndim != 2 or Y.shape[0] != K:
            raise ValueError(f"the contracted matrix must be {K} x d")
        d = Y.shape[1]
        keep = []
        if u is not None:
            u = self._vec(u, n + m - 1)
            keep.append(u)
        if W is not None:
            W = np.ascontiguousarray(np.asarray(W, dtype=np.float64))
            if W.shape != (n, m):
                raise ValueError(f"W must be {n} x {m}")
            keep.append(W)
        sums = np.zeros(nown)
        Z = np.zeros((nown, d))
        self.ctx.check(fn(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data,
            u.ctypes.data if u is not None else None, W.ctypes.data if W is not None else None,
            Y.ctypes.data, d, sums.ctypes.data, Z.ctypes.data, L.REGOT_MEM_HOST))
        return sums, Z

    def erot_sparsify(self, reg, gamma, delta, density_hint, mask=True):
        """sparsify_mat3 of T(gamma) (sinkhorn_sparsify3.cpp:276-405): returns
        (nnz, kept) with nnz counted as the reference does (exact zeros of T
        included) and kept the n x (m-1) boolean mask of stored entries."""
        gamma = self._vec(gamma, self.n + self.m - 1)
        nnz = np.zeros(1, dtype=np.int64)
        K = np.zeros((self.n, self.m - 1), dtype=np.int32) if mask else None
        self.ctx.check(self._lib.regot_erot_sparsify(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, float(delta),
            float(density_hint), nnz.ctypes.data, K.ctypes.data if mask else None))
        return int(nnz[0]), (K.astype(bool) if mask else None)

    def erot_sparsify_density(self, reg, gamma, density, mask=True):
        """sparsify_mat_with_density of T(gamma) (sinkhorn_sparsify4.cpp:77-174,
        first row and column preserved): returns (nnz, kept) as erot_sparsify."""
        gamma = self._vec(gamma, self.n + self.m - 1)
        nnz = np.zeros(1, dtype=np.int64)
        K = np.zeros((self.n, self.m - 1), dtype=np.int32) if mask else None
        self.ctx.check(self._lib.regot_erot_sparsify_density(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, float(density),
            nnz.ctypes.data, K.ctypes.data if mask else None))
        return int(nnz[0]), (K.astype(bool) if mask else None)

    def qrot_dual_obj_grad(self, reg, gamma):
        gamma = self._vec(gamma, self.n + self.m)
        obj = np.zeros(1)
        grad = np.zeros(self.n + self.m)
        self.ctx.check(self._lib.regot_qrot_dual_obj_grad(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, obj.ctypes.data,
            grad.ctypes.data))
        return float(obj[0]), grad

    def qrot_optimal_beta(self, reg, alpha):
        alpha = self._vec(alpha, self.n)
        out = np.zeros(self.m)
        self.ctx.check(self._lib.regot_qrot_optimal_beta(
            self.ctx.handle, self.handle, float(reg), alpha.ctypes.data, out.ctypes.data))
        return out

    def qrot_optimal_alpha(self, reg, beta):
        beta = self._vec(beta, self.m)
        out = np.zeros(self.n)
        self.ctx.check(self._lib.regot_qrot_optimal_alpha(
            self.ctx.handle, self.handle, float(reg), beta.ctypes.data, out.ctypes.data))
        return out

    def qrot_primal_val(self, reg, gamma):
        gamma = self._vec(gamma, self.n + self.m)
        out = np.zeros(1)
        self.ctx.check(self._lib.regot_qrot_primal_val(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, out.ctypes.data))
        return float(out[0])

    def qrot_plan(self, reg, gamma):
        gamma = self._vec(gamma, self.n + self.m)
        P = L.host_empty((self.n, self.m))
        self.ctx.check(self._lib.regot_qrot_plan(
            self.ctx.handle, self.handle, float(reg), gamma.ctypes.data, P.ctypes.data,
            L.REGOT_MEM_HOST))
        return P


def _solve(name, M, a, b, reg, tol, max_iter, verbose, kwargs):
    prob = Problem(M, a, b, precision=kwargs.get("precision"), device=int(kwargs.get("device", 0)))
    try:
        return getattr(prob, name)(reg, tol, max_iter, verbose, **kwargs)
    finally:
        prob.close()


def sinkhorn_bcd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """BCD (Sinkhorn) for EROT; reference src/sinkhorn_bcd.cpp:14-124."""
    return _solve("sinkhorn_bcd", M, a, b, reg, tol, max_iter, verbose, kwargs)


def sinkhorn_newton(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Newton's method for EROT; reference src/sinkhorn_newton.cpp:17-129."""
    return _solve("sinkhorn_newton", M, a, b, reg, tol, max_iter, verbose, kwargs)


def sinkhorn_ssns(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Safe and sparse Newton for EROT; reference src/sinkhorn_ssns.cpp:16-234."""
    return _solve("sinkhorn_ssns", M, a, b, reg, tol, max_iter, verbose, kwargs)


def sinkhorn_sparse_newton(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Newton's method with a density-sparsified Hessian for EROT; reference
    src/sinkhorn_sparse_newton.cpp:24-171. kwargs: ``density`` (0.01),
    ``shift`` (1e-3), ``method`` (1)."""
    return _solve("sinkhorn_sparse_newton", M, a, b, reg, tol, max_iter, verbose, kwargs)


def sinkhorn_splr(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Sparse-plus-low-rank quasi-Newton method for EROT; reference
    src/sinkhorn_splr.cpp:24-200. kwargs: ``density`` (0.01), ``shift``
    (1e-3), ``method`` (1)."""
    return _solve("sinkhorn_splr", M, a, b, reg, tol, max_iter, verbose, kwargs)


def sinkhorn_lbfgs_dual(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """L-BFGS on the EROT dual; reference src/sinkhorn_lbfgs_dual.cpp:81-126."""
    return _solve("sinkhorn_lbfgs_dual", M, a, b, reg, tol, max_iter, verbose, kwargs)


def sinkhorn_apdagd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Accelerated primal-dual adaptive gradient descent for EROT; reference
    src/sinkhorn_apdagd.cpp:14-183. The plan is the averaged primal plan."""
    return _solve("sinkhorn_apdagd", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_lbfgs_dual(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """L-BFGS on the QROT dual; reference src/qrot_lbfgs_dual.cpp:81-126."""
    return _solve("qrot_lbfgs_dual", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_bcd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Block coordinate descent for QROT; reference src/qrot_bcd.cpp:14-103."""
    return _solve("qrot_bcd", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_gd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Gradient descent for QROT; reference src/qrot_gd.cpp:14-120."""
    return _solve("qrot_gd", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_apdagd(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Accelerated primal-dual adaptive gradient descent for QROT; reference
    src/qrot_apdagd.cpp:14-179. The plan is the averaged primal plan."""
    return _solve("qrot_apdagd", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_pdaam(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Primal-dual accelerated alternating minimisation for QROT; reference
    src/qrot_pdaam.cpp:14-188. The plan is the averaged primal plan."""
    return _solve("qrot_pdaam", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_grssn(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Regularized semi-smooth Newton for QROT; reference src/qrot_grssn.cpp:16-133.
    kwargs: ``shift`` (1e-3), ``method`` (the system is solved by CG)."""
    return _solve("qrot_grssn", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_lbfgs_semi_dual(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """L-BFGS on the QROT semi-dual; reference src/qrot_lbfgs_semi_dual.cpp:84-126."""
    return _solve("qrot_lbfgs_semi_dual", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_pdip(M, a, b, reg, tol=1e-8, max_iter=1000, verbose=0, **kwargs):
    """Primal-dual interior point for QROT; reference src/solvers.cpp:268-292
    (pdip_cg.cpp:206-413, pdip_fp.cpp:278-667). kwargs: ``inner_solver``
    ("cg" or "fp"), ``cg_max_iter``, ``fixed_threshold``, ``fp_max_iter``,
    ``fp_exit_scale``, ``fp_stop_gap_mu_only``, ``cg_stop_gap_mu_only``,
    ``cg_mar_tol``. Returns a ``pdip_result``."""
    return _solve("qrot_pdip", M, a, b, reg, tol, max_iter, verbose, kwargs)


def pdip_cg(M, a, b, reg, tol=1e-8, max_iter=1000, verbose=0, **kwargs):
    """``qrot_pdip`` with the CG inner solver (solvers.cpp:294-300)."""
    kwargs = dict(kwargs, inner_solver="cg")
    return _solve("qrot_pdip", M, a, b, reg, tol, max_iter, verbose, kwargs)


def pdip_fp(M, a, b, reg, tol=1e-8, max_iter=1000, verbose=0, **kwargs):
    """``qrot_pdip`` with the fixed-point inner solver (solvers.cpp:302-308)."""
    kwargs = dict(kwargs, inner_solver="fp")
    return _solve("qrot_pdip", M, a, b, reg, tol, max_iter, verbose, kwargs)


def qrot_assn(M, a, b, reg, tol=1e-6, max_iter=1000, verbose=0, **kwargs):
    """Adaptive semi-smooth Newton for QROT; reference src/qrot_assn.cpp:16-170."""
    return _solve("qrot_assn", M, a, b, reg, tol, max_iter, verbose, kwargs)


class batch_result:
    """Result of sinkhorn_bcd_batched: per-problem iteration counts, final
    marginal errors and gauge-fixed duals (alpha, beta~) as sinkhorn_bcd
    returns them, plus the sweeps and device time of the whole batch. With
    grad=True also each problem's regularised OT cost (costs) and its
    gradients with respect to the points (grad_x, grad_y: lists of (n_p, d_p)
    and (m_p, d_p) arrays)."""

    def __init__(self):
        self.niter = None
        self.mar_errs = None
        self.duals = []
        self.sweeps = 0
        self.solve_ms = 0.0
        self.costs = None
        self.grad_x = None
        self.grad_y = None

    def __repr__(self):
        return (f"batch_result(problems={len(self.duals)}, sweeps={self.sweeps}, "
                f"max niter={int(self.niter.max()) if len(self.duals) else 0})")


def sinkhorn_bcd_batched(xs, ys, as_, bs, reg, tol=1e-6, max_iter=1000, cost_scale=None,
                         device: int = 0, grad: bool = False):
    """sinkhorn_bcd (reference src/sinkhorn_bcd.cpp:14-124) on many problems
    at once, each with the squared-Euclidean cost M_ij = s_p |x_i - y_j|^2
    computed on the fly in FP32 (no n x m matrix is stored). xs, ys: lists
    of (n_p, d_p) and (m_p, d_p) point arrays (d_p <= 16); as_, bs: lists of
    marginals; cost_scale: None, a number or one number per problem. Each
    problem stops at its own iteration (marginal error < tol or max_iter).
    grad=True adds the backward in the same call: each problem's cost
    L = a'alpha + b'beta - reg sum T and dL/dx = 2 s sum_j T_ij (x_i - y_j),
    dL/dy = 2 s sum_i T_ij (y_j - x_i) at the returned duals (the envelope
    theorem, dL/dM = T), as float32 arrays like the points."""
    P = len(xs)
    if not (len(ys) == len(as_) == len(bs) == P) or P == 0:
        raise ValueError("xs, ys, as_ and bs must be non-empty lists of the same length")
    xs = [np.ascontiguousarray(np.asarray(x, dtype=np.float32)) for x in xs]
    ys = [np.ascontiguousarray(np.asarray(y, dtype=np.float32)) for y in ys]
    as_ = [np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel()) for v in as_]
    bs = [np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel()) for v in bs]
    n = np.array([x.shape[0] for x in xs], dtype=np.int32)
    m = np.array([y.shape[0] for y in ys], dtype=np.int32)
    d = np.array([x.shape[1] if x.ndim == 2 else 0 for x in xs], dtype=np.int32)
    for p in range(P):
        if xs[p].ndim != 2 or ys[p].ndim != 2 or ys[p].shape[1] != d[p]:
            raise ValueError(f"problem {p}: x and y must be 2-D with the same dimension")
        if as_[p].size != n[p] or bs[p].size != m[p]:
            raise ValueError(f"problem {p}: a must have {n[p]} entries and b {m[p]}")
        if not (1 <= d[p] <= L.BATCH_MAX_DIM):
            raise ValueError(f"problem {p}: point dimension must be in 1..{L.BATCH_MAX_DIM}")
    if cost_scale is None:
        sc = None
    else:
        sc = np.ascontiguousarray(np.broadcast_to(np.asarray(cost_scale, dtype=np.float64),
                                                  (P,)))
    X = np.concatenate([x.ravel() for x in xs])
    Y = np.concatenate([y.ravel() for y in ys])
    A = np.concatenate(as_)
    B = np.concatenate(bs)
    ctx = L.context(device)
    lib = L.load()
    desc = L.BatchDesc()
    desc.count = P
    desc.n, desc.m, desc.d = n.ctypes.data, m.ctypes.data, d.ctypes.data
    desc.cost_scale = sc.ctypes.data if sc is not None else None
    desc.x, desc.y, desc.a, desc.b = X.ctypes.data, Y.ctypes.data, A.ctypes.data, B.ctypes.data
    desc.mem = L.REGOT_MEM_HOST
    alpha = np.zeros(A.size)
    beta = np.zeros(B.size)
    niter = np.zeros(P, dtype=np.int32)
    mar = np.zeros(P)
    r = L.BatchResult()
    r.alpha, r.beta = alpha.ctypes.data, beta.ctypes.data
    r.niter, r.mar_err = niter.ctypes.data, mar.ctypes.data
    if grad:
        costs = np.zeros(P)
        gx = np.zeros(X.size, dtype=np.float32)
        gy = np.zeros(Y.size, dtype=np.float32)
        ctx.check(lib.regot_erot_solve_batched_grad(
            ctx.handle, C.byref(desc), float(reg), float(tol), int(max_iter), C.byref(r),
            costs.ctypes.data, gx.ctypes.data, gy.ctypes.data))
    else:
        ctx.check(lib.regot_erot_solve_batched(ctx.handle, C.byref(desc), float(reg),
                                               float(tol), int(max_iter), C.byref(r)))
    out = batch_result()
    if grad:
        xo = np.r_[0, np.cumsum(n.astype(np.int64) * d)]
        yo = np.r_[0, np.cumsum(m.astype(np.int64) * d)]
        out.costs = costs
        out.grad_x = [gx[xo[p]:xo[p + 1]].reshape(n[p], d[p]) for p in range(P)]
        out.grad_y = [gy[yo[p]:yo[p + 1]].reshape(m[p], d[p]) for p in range(P)]
    out.niter = niter
    out.mar_errs = mar
    ro = np.r_[0, np.cumsum(n)]
    co = np.r_[0, np.cumsum(m)]
    out.duals = [np.r_[alpha[ro[p]:ro[p + 1]], beta[co[p]:co[p + 1] - 1]] for p in range(P)]
    out.sweeps = int(r.sweeps)
    out.solve_ms = float(r.solve_ms)
    return out
