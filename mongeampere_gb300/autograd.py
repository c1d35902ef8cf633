"""torch.autograd binding of the Laguerre evaluation and its adjoint.

:func:`laguerre` returns the Kantorovich value ``sum_i (w_i m_i - int_{cell i} rho
|x - x_i|^2)``, the cell masses ``m`` and the first moments ``int_{cell i} rho x``
of the sites ``X`` (N x 2), the weights ``w`` (N) and the density's vertex values
``rho`` (V), all differentiable; :func:`centroids` divides the moments by the
masses.  The forward pass is ``ma_moments`` (one Laguerre evaluation), the backward
pass ``ma_kantorovich_vjp``, which recomputes the cells instead of storing them.
The reference (MongeAmpere++) has no derivatives beyond the Hessian in ``w``.
"""
from __future__ import annotations

import torch

from . import api


class _Laguerre(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, w, rho, dmesh, actx):
        dmesh.set_values(rho.detach())
        # the value from the evaluation (integrated about each site), the moments
        # from ma_moments
        v, _, _ = api.kantorovich(dmesh, X.detach(), w.detach(), hessian=False, ctx=actx)
        m, first = api.first_moment(dmesh, X.detach(), w.detach(), ctx=actx)
        value = torch.tensor(v, dtype=torch.float64, device=X.device)
        ctx.save_for_backward(X, w, rho)
        ctx.dmesh = dmesh
        ctx.actx = actx
        return value, m, first

    @staticmethod
    def backward(ctx, g_value, g_mass, g_first):
        X, w, rho = ctx.saved_tensors
        dmesh, actx = ctx.dmesh, ctx.actx
        dmesh.set_values(rho.detach())
        a = float(g_value) if g_value is not None else 0.0
        cm = g_mass.contiguous() if g_mass is not None else None
        cf = g_first.contiguous() if g_first is not None else None
        gX, gw, gr = api.kantorovich_vjp(dmesh, X.detach(), w.detach(), a, cm, cf, grad_rho=ctx.needs_input_grad[2],
                                         ctx=actx)
        return gX, gw, gr, None, None


def laguerre(X, w, rho, dmesh, ctx=None):
    """``(value, masses, first moments)`` of the Laguerre cells of ``(X, w)`` for the
    density ``rho`` (vertex values of ``dmesh``'s geometry); CUDA float64 tensors."""
    actx = ctx or api.default_context()
    return _Laguerre.apply(X, w, rho, dmesh, actx)


def centroids(X, w, rho, dmesh, ctx=None):
    """Cell centroids ``first / mass`` (differentiable) and the masses."""
    _, m, first = laguerre(X, w, rho, dmesh, ctx)
    return first / m.unsqueeze(1), m
