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
                           ot_cost with M_ij = |x_i - y_j|^2 / scale; the
                           backward dL/dx = 2 g (r o x - T y) / scale runs the
                           fused contraction regot_erot_tyy (no n x m array).
sqeuclid_plan_loss(x, y, a, b, reg, W, scale)
                           <T*, W> for that cost; dL/dx = 2 g (rG o x - G y) /
                           scale with G = dL/dM of ot_plan, again through
                           regot_erot_tyy with the adjoint u and W.

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
    n, m = prob.n, prob.m
    alpha = torch.from_numpy(gamma[:n].copy()).to(device)
    beta = torch.from_numpy(np.r_[gamma[n:], 0.0]).to(device)
    return alpha, beta


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
    return ((x * x).sum(1)[:, None] + (y * y).sum(1)[None, :] - 2.0 * x @ y.T).clamp_min(0) / scale


class _SqEuclidCost(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, a, b, reg, scale, solver, tol, max_iter, kwargs):
        with torch.no_grad():
            M = _sqeuclid(x, y, scale)
        prob, r = _solve(M, a, b, reg, solver, tol, max_iter, dict(kwargs))
        ctx.prob, ctx.gamma, ctx.reg, ctx.scale = prob, r.dual, reg, scale
        ctx.save_for_backward(x, y)
        ctx.dtypes = (x.dtype, y.dtype, a.dtype, b.dtype)
        return torch.tensor(-r.obj_vals[-1], dtype=torch.float64, device=x.device)

    @staticmethod
    def backward(ctx, g):
        x, y = ctx.saved_tensors
        prob, gamma, reg, scale = ctx.prob, ctx.gamma, ctx.reg, ctx.scale
        dx = dy = da = db = None
        if ctx.needs_input_grad[0]:
            gam = torch.from_numpy(gamma).to(x.device)
            Y = y.detach().to(torch.float64).contiguous()
            rows, TY = prob.erot_tyy(reg, gam, Y)
            xd = x.detach().to(torch.float64)
            dx = (g * 2.0 * (rows[:, None] * xd - TY) / scale).to(ctx.dtypes[0])
        if ctx.needs_input_grad[1]:
            T = torch.empty((prob.n, prob.m), dtype=torch.float64, device=y.device)
            prob.erot_plan(reg, gamma, out=T)
            yd = y.detach().to(torch.float64)
            xd = x.detach().to(torch.float64)
            dy = (g * 2.0 * (T.sum(0)[:, None] * yd - T.T @ xd) / scale).to(ctx.dtypes[1])
        alpha, beta = _dual_tensors(prob, gamma, x.device)
        if ctx.needs_input_grad[2]:
            da = (g * _center(alpha)).to(ctx.dtypes[2])
        if ctx.needs_input_grad[3]:
            db = (g * _center(beta)).to(ctx.dtypes[3])
        return dx, dy, da, db, None, None, None, None, None, None


class _SqEuclidPlanLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, a, b, reg, W, scale, solver, tol, max_iter, cg_tol, kwargs):
        with torch.no_grad():
            M = _sqeuclid(x, y, scale)
        prob, r = _solve(M, a, b, reg, solver, tol, max_iter, dict(kwargs))
        T = torch.empty((prob.n, prob.m), dtype=torch.float64, device=x.device)
        prob.erot_plan(reg, r.dual, out=T)
        W64 = W.detach().to(torch.float64).contiguous()
        ctx.prob, ctx.gamma, ctx.reg, ctx.scale, ctx.cg_tol = prob, r.dual, reg, scale, cg_tol
        ctx.save_for_backward(x, y, T, W64)
        ctx.dtypes = (x.dtype, y.dtype, a.dtype, b.dtype)
        return (W64 * T).sum()

    @staticmethod
    def backward(ctx, g):
        x, y, T, W = ctx.saved_tensors
        prob, gamma, reg, scale = ctx.prob, ctx.gamma, ctx.reg, ctx.scale
        n, m = prob.n, prob.m
        u = _adjoint(prob, gamma, reg, T, W, ctx.cg_tol)
        dx = dy = da = db = None
        if ctx.needs_input_grad[0]:
            # G = T o (u_i + u_j - W_ij) / reg contracted with y on the fly
            gam = torch.from_numpy(gamma).to(x.device)
            ut = torch.from_numpy(u).to(x.device)
            Y = y.detach().to(torch.float64).contiguous()
            rows, GY = prob.erot_tyy(reg, gam, Y, u=ut, W=W)
            xd = x.detach().to(torch.float64)
            dx = (g * 2.0 * (rows[:, None] * xd - GY) / scale).to(ctx.dtypes[0])
        ua = torch.from_numpy(u[:n].copy()).to(x.device)
        ub = torch.from_numpy(np.r_[u[n:], 0.0]).to(x.device)
        if ctx.needs_input_grad[1]:
            G = T / reg * (ua[:, None] + ub[None, :] - W)
            yd = y.detach().to(torch.float64)
            xd = x.detach().to(torch.float64)
            dy = (g * 2.0 * (G.sum(0)[:, None] * yd - G.T @ xd) / scale).to(ctx.dtypes[1])
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
