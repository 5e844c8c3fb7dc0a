"""Differentiation of the interpolant behind ``torch.autograd``.

``interpolate(ip, x, nodal_values)`` evaluates the mixed-precision form of a
built interpolant and registers a hand-written backward:

* dL/dx      -- G = g C^T on the tensor cores, then a reverse pass through the
                basis products per point (``smx_spectral_vjp_x``);
* dL/dvalues -- dL/dC = A(x)^T g on the tensor cores, the adjoint of the FP64
                coefficient transform (``smx_spectral_coefficients_adjoint``)
                and the chain rule through the plan's rows
                F[r] = zeta_s (fu[umap r] - fu[u0]) and its constant term.

The reference has no derivative with respect to the nodal values; its
derivative with respect to x is the dense Jacobian of ``gradient``
(interpolation.py:306-345), which the FP64 path reproduces.
"""
from __future__ import annotations

import torch


def _fu_gradient(ip, Fbar, dC_root):
    """Chain rule from dL/dF (plan rows) and dL/d(constant term) to dL/dfu."""
    P = ip._plan
    keep = P.keep
    fu = keep["fu"]
    dfu = torch.zeros_like(fu)
    R = P.c.n_entries
    if R == 0:
        return dfu
    eoff = keep["sum_eoff"]
    zrow = torch.repeat_interleave(keep["sum_zeta"].double(), (eoff[1:] - eoff[:-1]))
    zF = Fbar * zrow[:, None]
    dfu.index_add_(0, keep["umap"], zF)
    u0 = int(keep["umap"][0].item())
    zsum = float(keep["sum_zeta"].sum().item())
    # F = zeta (fu[umap] - c), offset = zeta0 fu[u0] + c sum(zeta), c = fu[u0]
    dfu[u0] += -zF.sum(0) + zsum * dC_root + float(keep["zeta0"]) * dC_root
    return dfu


class _SmolyakFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, fu, ip):
        ctx.ip = ip
        ctx.save_for_backward(x)
        return ip(x, precision="fp32")

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        ip = ctx.ip
        sp = ip.spectral_plan()
        need_x, need_fu = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        dx, dC = sp.vjp(x.contiguous(), g.contiguous(), need_x=need_x, need_coef=need_fu)
        dfu = None
        if need_fu:
            Fbar = sp.coefficient_adjoint(dC)
            dfu = _fu_gradient(ip, Fbar, dC[0])
        return (dx.to(x.dtype) if dx is not None else None), dfu, None


def interpolate(ip, x, nodal_values=None):
    """y = I[f](x) (FP32 orthogonal form) with gradients w.r.t. x and the nodal values.

    ``nodal_values`` defaults to ``ip.nodal_values``; pass a tensor with
    ``requires_grad=True`` to receive dL/d(nodal values).  A tensor with other
    values than the interpolant's is loaded with ``ip.set_nodal_values``."""
    fu = ip.nodal_values if nodal_values is None else nodal_values
    if fu is not ip.nodal_values and not torch.equal(fu.detach(), ip.nodal_values):
        ip.set_nodal_values(fu.detach())
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(x)
    x = x.to(device=fu.device, dtype=torch.float64)
    return _SmolyakFunction.apply(x, fu, ip)
