"""Envelope gradients for the GPU losses.

The reference differentiates ``sinkhorn2`` by unrolled autodiff through its
torch-backend iterations.  The GPU loop is one kernel, so gradients are set
at convergence instead, as ``ot.solve(..., grad='envelope')`` does
(``ot/solvers.py:489-498``): ``dL/dM = P``, ``dL/da = reg (log_u - mean)``,
``dL/db = reg (log_v - mean)``.
"""
import torch

from . import _lib


class _Envelope(torch.autograd.Function):
    @staticmethod
    def forward(ctx, loss, gM, ga, gb, M, a, b):
        ctx.save_for_backward(gM, ga, gb)
        ctx.shapes = (M.shape if M is not None else None, a.shape if a is not None else None,
                      b.shape if b is not None else None)
        return loss.clone()

    @staticmethod
    def backward(ctx, g):
        gM, ga, gb = ctx.saved_tensors
        sM, sa, sb = ctx.shapes
        return (None,
                None, None, None,
                (g * gM).reshape(sM).to(gM.dtype) if sM is not None else None,
                (g * ga).reshape(sa) if sa is not None else None,
                (g * gb).reshape(sb) if sb is not None else None)


def envelope_loss(loss, P, r, method, reg, a, b, M):
    if method == _lib.OTG_METHOD_KNOPP:
        lu, lv = torch.log(r.u), torch.log(r.v)
    else:
        lu, lv = r.u, r.v
    ga = reg * (lu - lu.mean())
    gb = reg * (lv - lv.mean())
    Mt = M if isinstance(M, torch.Tensor) and M.requires_grad else None
    at = a if isinstance(a, torch.Tensor) and a.requires_grad and a.numel() else None
    bt = b if isinstance(b, torch.Tensor) and b.requires_grad and b.numel() else None
    dev = loss.device
    gM = P if Mt is not None else torch.zeros(0, device=dev)
    if Mt is not None and Mt.device != dev:
        gM = gM.to(Mt.device)
    ga = ga.to(at.device) if at is not None else torch.zeros(0, device=dev)
    gb = gb.to(bt.device) if bt is not None else torch.zeros(0, device=dev)
    out = _Envelope.apply(loss, gM, ga, gb, Mt, at, bt)
    return out
