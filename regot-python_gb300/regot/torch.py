"""torch.autograd wrappers around the EROT solvers (no counterpart in the
reference, which has no derivatives).

ot_cost(M, a, b, reg)      regularised OT cost  a'alpha + b'beta - reg sum T
                           at the dual optimum (the negated dual objective of
                           sinkhorn_problem_obj.cpp:324-342); by the envelope
                           theorem dL/dM = g T*, dL/da = g alpha*, dL/db = g beta*
                           (duals centred, since sum a = sum b = 1 fixes them
                           only up to a constant).
ot_plan(M, a, b, reg)      the optimal plan T*; the backward of a loss on it is
                           the implicit adjoint: u = H^-1 dL/dgamma with the
                           exact dual Hessian H (one CG solve over the HVP
                           passes), dL/dM_ij = T_ij (u_i + u_j - W_ij) / reg,
                           dL/da = u_alpha, dL/db = (u_beta~, 0), W = dL/dT.
sqeuclid_ot_cost(x, y, a, b, reg, scale)
                           ot_cost with M_ij = |x_i - y_j|^2 / scale (formed by
                           the library's direct-difference kernel); the
                           backward dL/dx = 2 g (r o x - T y) / scale and
                           dL/dy = 2 g (c o y - T'x) / scale run the fused
                           contractions regot_erot_tyy / regot_erot_tty (no
                           n x m array; tensor cores for float32 points).
sqeuclid_plan_loss(x, y, a, b, reg, W, scale)
                           <T*, W> for that cost; dL/dx = 2 g (rG o x - G y) /
                           scale and dL/dy likewise with G = dL/dM of ot_plan,
                           through the same contractions with the adjoint u
                           and W; the loss and the adjoint right-hand side are
                           contractions too.

The solve runs on the GPU of the inputs through regot.Problem (float32 M:
mixed precision; float64: FP64). Forward tolerances are the caller's; the
gradients are exact for the returned solution up to the solve's residual.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _internal as I

__all__ = ["ot_cost", "ot_plan", "sqeuclid_ot_cost", "sqeuclid_plan_loss"]

_SOLVERS = ("sinkhorn_bcd", "sinkhorn_newton", "sinkhorn_ssns", "sinkhorn_lbfgs_dual")


def _np64(t):
    return np.ascontiguousarray(t.detach().to(torch.float64).cpu().numpy().ravel())


def _solve(M, a, b, reg, solver, tol, max_iter, kwargs):
    if solver not in _SOLVERS:
        raise ValueError(f"solver must be one of {_SOLVERS}")
    if not (M.is_cuda and M.dim() == 2):
        raise ValueError("M must be a 2-D CUDA tensor")
    Md = M.detach()
    if not Md.is_contiguous():
        Md = Md.contiguous()
    torch.cuda.current_stream(Md.device).synchronize()
    prob = I.Problem(Md, _np64(a), _np64(b), precision=kwargs.pop("precision", None),
                     device=Md.device.index or 0)
    r = getattr(prob, solver)(reg, tol=tol, max_iter=max_iter, plan=False, **kwargs)
    return prob, r


def _center(v):
    return v - v.mean()


def _dual_tensors(prob, gamma, device):
    n = prob.n
    g = torch.from_numpy(np.r_[gamma, 0.0]).to(device)  # beta_m = 0 appended
    return g[:n], g[n:]


class _OTCost(torch.autograd.Function):
    @staticmethod
    def forward(ctx, M, a, b, reg, solver, tol, max_iter, kwargs):
        prob, r = _solve(M, a, b, reg, solver, tol, max_iter, dict(kwargs))
        ctx.prob, ctx.gamma, ctx.reg = prob, r.dual, reg
        ctx.dtypes = (M.dtype, a.dtype, b.dtype)
        return torch.tensor(-r.obj_vals[-1], dtype=torch.float64, device=M.device)

    @staticmethod
    def backward(ctx, g):
        prob, gamma, reg = ctx.prob, ctx.gamma, ctx.reg
        dM = da = db = None
        if ctx.needs_input_grad[0]:
            T = torch.empty((prob.n, prob.m), dtype=torch.float64, device=g.device)
            prob.erot_plan(reg, gamma, out=T)
            dM = (g * T).to(ctx.dtypes[0])
        alpha, beta = _dual_tensors(prob, gamma, g.device)
        if ctx.needs_input_grad[1]:
            da = (g * _center(alpha)).to(ctx.dtypes[1])
        if ctx.needs_input_grad[2]:
            db = (g * _center(beta)).to(ctx.dtypes[2])
        return dM, da, db, None, None, None, None, None


def _cg_tol(prob, cg_tol):
    # FP32 Hessian products cannot take CG much below 1e-7 relative
    if cg_tol is not None:
        return cg_tol
    return 1e-12 if prob.precision == I.L.REGOT_PREC_FP64 else 1e-7


def _adjoint(prob, gamma, reg, T, W, cg_tol):
    """u = H^-1 dL/dgamma for a loss with dL/dT = W."""
    n, m = prob.n, prob.m
    WT = W * T / reg
    dgamma = torch.cat([WT.sum(1), WT.sum(0)[: m - 1]])
    u, _ = prob.erot_hess_solve(reg, gamma, dgamma.cpu().numpy(), tol=_cg_tol(prob, cg_tol))
    return u


class _OTPlan(torch.autograd.Function):
    @staticmethod
    def forward(ctx, M, a, b, reg, solver, tol, max_iter, cg_tol, kwargs):
        prob, r = _solve(M, a, b, reg, solver, tol, max_iter, dict(kwargs))
        T = torch.empty((prob.n, prob.m), dtype=torch.float64, device=M.device)
        prob.erot_plan(reg, r.dual, out=T)
        ctx.prob, ctx.gamma, ctx.reg, ctx.cg_tol = prob, r.dual, reg, cg_tol
        ctx.dtypes = (M.dtype, a.dtype, b.dtype)
        ctx.save_for_backward(T)
        return T

    @staticmethod
    def backward(ctx, W):
        (T,) = ctx.saved_tensors
        prob, gamma, reg = ctx.prob, ctx.gamma, ctx.reg
        n, m = prob.n, prob.m
        W = W.to(torch.float64).contiguous()
        u = _adjoint(prob, gamma, reg, T, W, ctx.cg_tol)
        ua = torch.from_numpy(u[:n].copy()).to(T.device)
        ub = torch.from_numpy(np.r_[u[n:], 0.0]).to(T.device)
        dM = da = db = None
        if ctx.needs_input_grad[0]:
            dM = (T / reg * (ua[:, None] + ub[None, :] - W)).to(ctx.dtypes[0])
        if ctx.needs_input_grad[1]:
            da = ua.to(ctx.dtypes[1])
        if ctx.needs_input_grad[2]:
            db = ub.to(ctx.dtypes[2])
        return dM, da, db, None, None, None, None, None, None


def _sqeuclid(x, y, scale):
    """M_ij = |x_i - y_j|^2 / scale by the library's direct-difference kernel
    (regot_sqeuclid_cost) in the points' precision (float32 or float64)."""
    import ctypes as C

    dt = torch.float64 if x.dtype == torch.float64 else torch.float32
    xd = x.detach().to(dt).contiguous()
    yd = y.detach().to(dt).contiguous()
    n, d = xd.shape
    m = yd.shape[0]
    if yd.shape[1] != d:
        raise ValueError("x and y must have the same number of columns")
    M = torch.empty((n, m), dtype=dt, device=x.device)
    ctx = I.L.context(x.device.index or 0)
    torch.cuda.current_stream(x.device).synchronize()
    ctx.check(ctx._lib.regot_sqeuclid_cost(
        ctx.handle, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n, m, d,
        1.0 / float(scale), I.L.REGOT_F64 if dt == torch.float64 else I.L.REGOT_F32,
        C.c_void_p(M.data_ptr()), m))
    return M


def _gamma_tensor(gamma, device):
    return torch.from_numpy(np.ascontiguousarray(gamma)).to(device)


class _SqEuclidCost(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, a, b, reg, scale, solver, tol, max_iter, kwargs):
        M = _sqeuclid(x, y, scale)
        prob, r = _solve(M, a, b, reg, solver, tol, max_iter, dict(kwargs))
        del M
        ctx.prob, ctx.gamma, ctx.reg, ctx.scale = prob, r.dual, reg, scale
        ctx.gam = _gamma_tensor(r.dual, x.device)
        ctx.save_for_backward(x, y)
        ctx.dtypes = (x.dtype, y.dtype, a.dtype, b.dtype)
        return torch.tensor(-r.obj_vals[-1], dtype=torch.float64, device=x.device)

    @staticmethod
    def backward(ctx, g):
        x, y = ctx.saved_tensors
        prob, gamma, reg, scale = ctx.prob, ctx.gamma, ctx.reg, ctx.scale
        dx = dy = da = db = None
        xd = x.detach().to(torch.float64).contiguous()
        yd = y.detach().to(torch.float64).contiguous()
        if ctx.needs_input_grad[0]:
            # dL/dx = 2 (rows o x - T y) / scale, T y on the tensor cores (FP32 storage)
            rows, TY = prob.erot_tyy(reg, ctx.gam, yd)
            dx = (g * 2.0 * (rows[:, None] * xd - TY) / scale).to(ctx.dtypes[0])
        if ctx.needs_input_grad[1]:
            # dL/dy = 2 (cols o y - T'x) / scale, the column-side contraction
            cols, TX = prob.erot_tty(reg, ctx.gam, xd)
            dy = (g * 2.0 * (cols[:, None] * yd - TX) / scale).to(ctx.dtypes[1])
        alpha, beta = _dual_tensors(prob, gamma, x.device)
        if ctx.needs_input_grad[2]:
            da = (g * _center(alpha)).to(ctx.dtypes[2])
        if ctx.needs_input_grad[3]:
            db = (g * _center(beta)).to(ctx.dtypes[3])
        return dx, dy, da, db, None, None, None, None, None, None


class _SqEuclidPlanLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, a, b, reg, W, scale, solver, tol, max_iter, cg_tol, kwargs):
        M = _sqeuclid(x, y, scale)
        prob, r = _solve(M, a, b, reg, solver, tol, max_iter, dict(kwargs))
        del M
        n, m = prob.n, prob.m
        W64 = W.detach().to(torch.float64).contiguous()
        gam = _gamma_tensor(r.dual, x.device)
        zero = torch.zeros(n + m - 1, dtype=torch.float64, device=x.device)
        # with u = 0 the contraction's G is -W o T / reg: its row and column
        # sums give the loss sum W o T and the adjoint right-hand side
        # dL/dgamma = (rows, cols~) of W o T / reg, without an n x m array
        e0 = torch.empty((n, 0), dtype=torch.float64, device=x.device)
        e1 = torch.empty((m, 0), dtype=torch.float64, device=x.device)
        rows0, _ = prob.erot_tyy(reg, gam, e1, u=zero, W=W64)
        cols0, _ = prob.erot_tty(reg, gam, e0, u=zero, W=W64)
        ctx.prob, ctx.gamma, ctx.reg, ctx.scale, ctx.cg_tol = prob, r.dual, reg, scale, cg_tol
        ctx.gam = gam
        ctx.dgamma = -torch.cat([rows0, cols0[: m - 1]])
        ctx.save_for_backward(x, y, W64)
        ctx.dtypes = (x.dtype, y.dtype, a.dtype, b.dtype)
        return -reg * rows0.sum()

    @staticmethod
    def backward(ctx, g):
        x, y, W = ctx.saved_tensors
        prob, gamma, reg, scale = ctx.prob, ctx.gamma, ctx.reg, ctx.scale
        n, m = prob.n, prob.m
        u, _ = prob.erot_hess_solve(reg, gamma, ctx.dgamma.cpu().numpy(),
                                    tol=_cg_tol(prob, ctx.cg_tol))
        ut = torch.from_numpy(u).to(x.device)
        xd = x.detach().to(torch.float64).contiguous()
        yd = y.detach().to(torch.float64).contiguous()
        dx = dy = da = db = None
        # G = T o (u_i + u_j - W_ij) / reg contracted on the fly (no n x m array)
        if ctx.needs_input_grad[0]:
            rows, GY = prob.erot_tyy(reg, ctx.gam, yd, u=ut, W=W)
            dx = (g * 2.0 * (rows[:, None] * xd - GY) / scale).to(ctx.dtypes[0])
        if ctx.needs_input_grad[1]:
            cols, GX = prob.erot_tty(reg, ctx.gam, xd, u=ut, W=W)
            dy = (g * 2.0 * (cols[:, None] * yd - GX) / scale).to(ctx.dtypes[1])
        ua = ut[:n]
        ub = torch.cat([ut[n:], ut.new_zeros(1)])
        if ctx.needs_input_grad[2]:
            da = (g * ua).to(ctx.dtypes[2])
        if ctx.needs_input_grad[3]:
            db = (g * ub).to(ctx.dtypes[3])
        return dx, dy, da, db, None, None, None, None, None, None, None, None


def ot_cost(M, a, b, reg, solver="sinkhorn_newton", tol=1e-10, max_iter=1000, **kwargs):
    """Regularised OT cost at the solution of `solver` (differentiable in M,
    a and b)."""
    return _OTCost.apply(M, a, b, float(reg), solver, float(tol), int(max_iter), kwargs)


def ot_plan(M, a, b, reg, solver="sinkhorn_newton", tol=1e-10, max_iter=1000, cg_tol=None,
            **kwargs):
    """Optimal plan T* (n x m, float64), differentiable through the implicit
    function of the dual optimality conditions."""
    return _OTPlan.apply(M, a, b, float(reg), solver, float(tol), int(max_iter), cg_tol, kwargs)


def sqeuclid_ot_cost(x, y, a, b, reg, scale=1.0, solver="sinkhorn_newton", tol=1e-10,
                     max_iter=1000, **kwargs):
    """ot_cost for M_ij = |x_i - y_j|^2 / scale, with the x-gradient from the
    fused weighted-plan contraction."""
    return _SqEuclidCost.apply(x, y, a, b, float(reg), float(scale), solver, float(tol),
                               int(max_iter), kwargs)


def sqeuclid_plan_loss(x, y, a, b, reg, W, scale=1.0, solver="sinkhorn_newton", tol=1e-10,
                       max_iter=1000, cg_tol=None, **kwargs):
    """<T*, W> for M_ij = |x_i - y_j|^2 / scale, with the implicit-adjoint
    x-gradient from the fused weighted-plan contraction (W is a constant)."""
    return _SqEuclidPlanLoss.apply(x, y, a, b, float(reg), W, float(scale), solver, float(tol),
                                   int(max_iter), cg_tol, kwargs)
