"""Gradients of the GPU losses.

``sinkhorn2`` (``ot/bregman/_sinkhorn.py:435-438``, loss ``sum(M * P)``): the
reference differentiates through its torch-backend iterations.  The GPU loop
is one kernel, so the same derivative is taken at the solution instead, by
implicit differentiation of the marginal constraints.  With
P_ij = exp((f_i + g_j - M_ij) / reg), r = (M o P) 1, c = (M o P)^T 1 and
H = [[diag(a), P], [P^T, diag(b)]], the pair (lam, mu) solving
H [lam; mu] = [r; c] gives

    dL/dM_ij = P_ij (1 + (lam_i + mu_j - M_ij) / reg),
    dL/da = lam + t,  dL/db = mu - t,

where t fixes the one free constant of (lam, mu) as the reference's iteration
does: its last update makes the rows exact, so a change of mass in b acts
like a rescaling of b, and b . dL/db = 0.  These are the reference's
unrolled-autodiff gradients at convergence (checked against its own
backward on recorded problems).  H is solved through its Schur complement
S = diag(b) - P^T diag(1/a) P (symmetric, positive semi-definite, null vector
1), shifted by the rank-one b b^T / sum(b) that selects the gauge b . mu = 0,
by conjugate gradients preconditioned with diag(b), in float64 on the device.

``ot.solve(..., grad='envelope')`` (``ot/solvers.py:489-498``) keeps the
envelope gradients of the regularised value: ``dL/dM = P``,
``dL/da = reg (log_u - mean)``, ``dL/db = reg (log_v - mean)``.
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


def implicit_grads(P, M, a, b, reg, rtol=1e-12, max_iter=None):
    """(dL/dM, dL/da, dL/db) of L = sum(M * P) at the Sinkhorn solution P of
    (a, b, M, reg), in float64 (see the module docstring)."""
    P = P.double()
    M = M.double()
    a = a.double()
    b = b.double()
    MP = M * P
    r, c = MP.sum(1), MP.sum(0)
    # bins of zero mass have zero rows / columns in P and drop out of the
    # system (their own gradient entries are then the gauge constant alone)
    ia = torch.where(a > 0, 1.0 / a, torch.zeros_like(a))
    ib = torch.where(b > 0, 1.0 / b, torch.zeros_like(b))
    beta = 1.0 / b.sum()

    # S + beta b b^T: the rank-one term lifts S's null direction (the constant
    # vector, only nearly null when the marginals are met to stopThr rather
    # than exactly: left in, conjugate gradients drift along it), and since
    # 1 . rhs = 0 its solution is the one with b . mu = 0, the reference's gauge
    def S(x):
        return b * x - P.t().mv(ia * P.mv(x)) + (beta * torch.dot(b, x)) * b

    rhs = c - P.t().mv(ia * r)
    mu = torch.zeros_like(b)
    res = rhs.clone()
    z = res * ib
    p = z.clone()
    rz = torch.dot(res, z)
    stop = (rtol * torch.linalg.vector_norm(rhs)) ** 2
    limit = max_iter or max(100, 4 * b.numel())
    for _ in range(limit):
        if float(torch.dot(res, res)) <= float(stop):
            break
        Sp = S(p)
        pSp = torch.dot(p, Sp)
        if not float(pSp) > 0.0:
            break
        alpha = rz / pSp
        mu = mu + alpha * p
        res = res - alpha * Sp
        z = res * ib
        rz_new = torch.dot(res, z)
        p = z + (rz_new / rz) * p
        rz = rz_new
    lam = (r - P.mv(mu)) * ia
    t = torch.dot(b, mu) / b.sum()
    gM = P * (1.0 + (lam[:, None] + mu[None, :] - M) / reg)
    return gM, lam + t, mu - t


class _Implicit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, loss, P, Md, ad, bd, reg, M, a, b):
        ctx.save_for_backward(P, Md, ad, bd)
        ctx.reg = reg
        ctx.meta = [None if x is None else (x.shape, x.dtype, x.device) for x in (M, a, b)]
        return loss.clone()

    @staticmethod
    def backward(ctx, g):
        P, Md, ad, bd = ctx.saved_tensors
        gM, ga, gb = implicit_grads(P, Md, ad, bd, ctx.reg)
        out = []
        for meta, gx in zip(ctx.meta, (gM, ga, gb)):
            if meta is None:
                out.append(None)
            else:
                shape, dtype, device = meta
                out.append((g.to(gx.dtype) * gx).to(device=device, dtype=dtype).reshape(shape))
        return (None, None, None, None, None, None) + tuple(out)


def implicit_loss(loss, P, Md, ad, bd, reg, a, b, M):
    """``loss`` with the implicit gradients attached for whichever of M, a, b
    are tensors that require them."""
    Mt = M if isinstance(M, torch.Tensor) and M.requires_grad else None
    at = a if isinstance(a, torch.Tensor) and a.requires_grad and a.numel() else None
    bt = b if isinstance(b, torch.Tensor) and b.requires_grad and b.numel() else None
    return _Implicit.apply(loss, P.detach(), Md.detach(), ad.detach(), bd.detach(), float(reg), Mt, at, bt)
