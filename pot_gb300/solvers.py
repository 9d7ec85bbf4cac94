"""GPU ``ot.solve`` and ``ot.solve_sample`` for their entropic branches.

``solve`` (``ot/solvers.py:57-604``): with ``reg > 0``, no unbalanced term
and ``reg_type`` in ``{"KL", "entropy"}`` the reference calls ``sinkhorn_log``
(``:428-494``, defaults ``max_iter = 1000``, ``tol = 1e-9``) and reports the
log scalings as potentials, ``value_linear = <M, P>`` and ``value`` with the
entropy or KL term.  Here the solve is the dense GPU kernel and the plan and
both values come from one pass of the batched plan kernel.

``solve_sample`` (``:1354-1877``): without ``lazy`` it builds the cost with
``dist`` and calls ``solve``; with ``lazy=True`` and ``reg > 0`` it runs the
online (lazy) Sinkhorn, whose cost is never stored, and returns
``value_linear``, the potentials, the lazy plan and the log (``:1857-1877``).

The other branches (exact OT, unbalanced, L2 or user regularisers, the
geomloss / factored / low-rank / Nystroem / Gaussian / 1-D methods) are not
on the GPU path and raise ``NotImplementedError``.
"""
import numpy as np
import torch

from . import bregman
from . import batch as pb
from . import empirical
from ._arrays import Boundary, is_empty
from .utils import OTResult, dist

LAZY_METHODS = ("1d", "gaussian", "lowrank", "nystroem", "factored", "geomloss", "geomloss_auto",
                "geomloss_tensorized", "geomloss_online", "geomloss_multiscale")


def _not_gpu(what):
    return NotImplementedError("pot_gb300: %s is not on the GPU path" % what)


def solve(M, a=None, b=None, reg=None, c=None, reg_type="KL", unbalanced=None, unbalanced_type="KL", method=None,
          n_threads=1, max_iter=None, plan_init=None, potentials_init=None, tol=None, verbose=False,
          grad="autodiff"):
    """GPU ``ot.solve``, entropic balanced branch (``ot/solvers.py:428-494``).

    ``grad``: 'autodiff' and 'envelope' attach the envelope gradients of
    ``value`` (dM = P, da = reg (log_u - mean), db = reg (log_v - mean)) --
    for 'autodiff' this stands in for differentiating through the
    iterations; 'detach' attaches none; 'last_step' runs ``max_iter - 1``
    GPU iterations and differentiates one last log-domain step."""
    if reg is None or reg == 0:
        raise _not_gpu("exact OT (reg=None or 0)")
    if unbalanced is not None:
        if isinstance(reg_type, tuple) or reg_type.lower() != "kl" or unbalanced_type.lower() != "kl":
            raise _not_gpu("unbalanced OT with reg_type=%r, unbalanced_type=%r" % (reg_type, unbalanced_type))
        return _solve_unbalanced(M, a, b, reg, c, unbalanced, potentials_init, max_iter, tol, verbose)
    if isinstance(reg_type, tuple) or reg_type.lower() not in ("kl", "entropy"):
        raise _not_gpu("reg_type=%r" % (reg_type,))
    if grad not in ("autodiff", "envelope", "last_step", "detach"):
        raise ValueError("Unknown grad mode '%s'" % grad)
    max_iter = 1000 if max_iter is None else max_iter
    tol = 1e-9 if tol is None else tol
    if grad == "last_step":
        if max_iter == 0:
            raise ValueError("The maximum number of iterations must be greater than 0 when using grad=last_step.")
        max_iter = max_iter - 1
    bd, Md, ad, bv = bregman._prep(a, b, M)
    if Md.dim() != 2:
        raise ValueError("M must be a 2-D cost matrix")
    r, _ = bregman._run_single(bd, ad, bv, Md, reg, bregman._lib.OTG_METHOD_LOG, max_iter, tol, verbose, True,
                               None, False)
    lu, lv = r.u, r.v
    kl = reg_type.lower() == "kl"
    if grad == "last_step":
        return _last_step(bd, M, a, b, Md, ad, bv, lu, lv, float(reg), kl, max_iter, r)
    layout, Mp = pb._uniform_batch(Md[None])
    reg_t = torch.full((1,), float(reg), dtype=torch.float64, device=Md.device)
    P, vals = pb.batched_plan(layout, Mp, lu, lv, ad, bv, reg_t, bregman._lib.OTG_METHOD_LOG, kl=kl)
    n, m = Md.shape
    P = P.view(n, int(layout.ldm_np[0]))[:, :m]
    value_linear = vals[0, 0].to(Md.dtype)
    value = (vals[0, 0] + float(reg) * vals[0, 1]).to(Md.dtype)
    if grad in ("autodiff", "envelope") and _needs_grad(M, a, b):
        from ._autograd import envelope_loss
        value = envelope_loss(value, P.contiguous(), r, bregman._lib.OTG_METHOD_LOG, float(reg), a, b, M)
    return OTResult(potentials=(bd.out(lu), bd.out(lv)), value=bd.scalar(value),
                    value_linear=bd.scalar(value_linear), plan=bd.out(P.contiguous()), backend=bd.kind)


def _solve_unbalanced(M, a, b, reg, c, reg_m, potentials_init, max_iter, tol, verbose):
    """``ot.solve`` with ``reg > 0`` and a KL marginal penalty
    (``ot/solvers.py:525-550``): ``sinkhorn_knopp_unbalanced`` with
    ``c = a b^T`` unless given, ``max_iter = 1000``, ``tol = 1e-9``; value =
    total cost, value_linear = linear cost, potentials = (logu, logv)."""
    from .unbalanced import sinkhorn_knopp_unbalanced
    P, lg = sinkhorn_knopp_unbalanced(a if a is not None else [], b if b is not None else [], M, reg, reg_m,
                                      "kl", c, potentials_init, numItermax=1000 if max_iter is None else max_iter,
                                      stopThr=1e-9 if tol is None else tol, verbose=verbose, log=True)
    return OTResult(potentials=(lg["logu"], lg["logv"]), value=lg["total_cost"], value_linear=lg["cost"], plan=P)


def _needs_grad(*xs):
    return any(isinstance(x, torch.Tensor) and x.requires_grad for x in xs)


def _last_step(bd, M0, a0, b0, Md, ad, bv, lu, lv, reg, kl, max_iter, r):
    """``grad='last_step'`` (``ot/solvers.py:462-476``): one more log-domain
    step on the caller's (differentiable) tensors after ``max_iter - 1``
    GPU iterations."""
    dev = Md.device
    Mt = M0 if isinstance(M0, torch.Tensor) else Md
    at = a0 if isinstance(a0, torch.Tensor) and not is_empty(a0) else ad
    bt = b0 if isinstance(b0, torch.Tensor) and not is_empty(b0) else bv
    Mt, at, bt = Mt.to(dev), at.to(dev), bt.to(dev)
    v = torch.log(bt) - torch.logsumexp(-Mt / reg + lu[:, None], 0)
    u = torch.log(at) - torch.logsumexp(-Mt / reg + v[None, :], 1)
    plan = torch.exp(-Mt / reg + u[:, None] + v[None, :])
    value_linear = torch.sum(Mt * plan)
    if kl:
        value = value_linear + reg * torch.sum(plan * torch.log(plan / (at[:, None] * bt[None, :]) + 1e-16))
    else:
        value = value_linear + reg * torch.sum(plan * torch.log(plan + 1e-16))
    if bd.kind == "numpy":
        return OTResult(potentials=(bd.out(u), bd.out(v)), value=bd.scalar(value), value_linear=bd.scalar(value_linear),
                        plan=bd.out(plan), backend=bd.kind)
    return OTResult(potentials=(u, v), value=value, value_linear=value_linear, plan=plan, backend=bd.kind)


def solve_sample(X_a, X_b, a=None, b=None, metric="sqeuclidean", reg=None, c=None, reg_type="KL", unbalanced=None,
                 unbalanced_type="KL", lazy=False, batch_size=None, method=None, n_threads=1, max_iter=None,
                 plan_init=None, rank=100, scaling=0.95, potentials_init=None, X_init=None, tol=None,
                 verbose=False, grad="autodiff"):
    """GPU ``ot.solve_sample``: the dense route through ``dist`` + ``solve``
    and the lazy entropic route (``ot/solvers.py:1743-1877``)."""
    if method is not None and method.lower() in LAZY_METHODS:
        raise _not_gpu("solve_sample method=%r" % method)
    if not lazy:
        M = dist(X_a, X_b, metric)
        return solve(M, a, b, reg, c, reg_type, unbalanced, unbalanced_type, method, n_threads, max_iter,
                     plan_init, potentials_init, tol, verbose, grad)
    if reg is None or reg == 0:
        raise NotImplementedError("Exact OT solver with lazy=True not implemented")
    if unbalanced is not None:
        raise NotImplementedError('Not implemented unbalanced_type="{}" with regularization'.format(unbalanced_type))
    max_iter = 1000 if max_iter is None else max_iter
    tol = 1e-9 if tol is None else tol
    batch_size = 100 if batch_size is None else batch_size
    value_linear, log = empirical_sinkhorn2(X_a, X_b, reg, a, b, metric=metric, numIterMax=max_iter, stopThr=tol,
                                            isLazy=True, batchSize=batch_size, verbose=verbose, log=True)
    return OTResult(potentials=(log["u"], log["v"]), value=None, value_linear=value_linear,
                    lazy_plan=log["lazy_plan"], plan=None, log=log)


def empirical_sinkhorn2(X_s, X_t, reg, a=None, b=None, metric="sqeuclidean", numIterMax=10000, stopThr=1e-9,
                        isLazy=False, batchSize=100, verbose=False, log=False, warn=True, warmstart=None, **kwargs):
    """GPU ``ot.bregman.empirical_sinkhorn2`` (``ot/bregman/_empirical.py:305-517``):
    lazy -- the online solve, then the loss of the lazy plan in one kernel
    (``otg_lazy_loss``); dense -- ``dist`` then ``sinkhorn2``."""
    if metric != "sqeuclidean":
        raise _not_gpu("empirical_sinkhorn2 metric '%s'" % metric)
    if not isLazy:
        M = dist(X_s, X_t, metric)
        bd = Boundary(X_s, X_t, a, b)
        ns, nt = np.shape(X_s)[0], np.shape(X_t)[0]
        aa = np.full(ns, 1.0 / ns) if a is None else a
        bb = np.full(nt, 1.0 / nt) if b is None else b
        if bd.kind != "numpy":
            Md = M
            aa = bd.to_dev(aa, Md.dtype) if not isinstance(aa, torch.Tensor) else aa
            bb = bd.to_dev(bb, Md.dtype) if not isinstance(bb, torch.Tensor) else bb
        return bregman.sinkhorn2(aa, bb, M, reg, numItermax=numIterMax, stopThr=stopThr, verbose=verbose, log=log,
                                 warn=warn, warmstart=warmstart, **kwargs)
    res = empirical.empirical_sinkhorn(X_s, X_t, reg, a, b, metric, numIterMax=numIterMax, stopThr=stopThr,
                                       isLazy=True, batchSize=batchSize, verbose=verbose, log=log, warn=warn,
                                       warmstart=warmstart)
    f, g = res[0], res[1]
    loss = empirical.lazy_loss(X_s, X_t, f, g, reg)
    return (loss, res[2]) if log else loss


def empirical_sinkhorn_divergence(X_s, X_t, reg, a=None, b=None, metric="sqeuclidean", numIterMax=10000,
                                  stopThr=1e-9, verbose=False, log=False, warn=True, warmstart=None, **kwargs):
    """GPU ``ot.bregman.empirical_sinkhorn_divergence``
    (``ot/bregman/_empirical.py:520-763``): ``W(a, b) - (W(a, a) + W(b, b)) / 2``
    from three ``empirical_sinkhorn2`` solves, clipped at zero; the warm
    start ``(u, v)`` seeds the cross solve and ``(u, u)``, ``(v, v)`` the
    two self solves."""
    ws_a = ws_b = None
    if warmstart is not None:
        u, v = warmstart
        ws_a, ws_b = (u, u), (v, v)
    kw = dict(metric=metric, numIterMax=numIterMax, stopThr=stopThr, verbose=verbose, log=log, warn=warn)
    ab = empirical_sinkhorn2(X_s, X_t, reg, a, b, warmstart=warmstart, **kw, **kwargs)
    aa = empirical_sinkhorn2(X_s, X_s, reg, a, a, warmstart=ws_a, **kw, **kwargs)
    bb = empirical_sinkhorn2(X_t, X_t, reg, b, b, warmstart=ws_b, **kw, **kwargs)
    if log:
        (lab, log_ab), (la, log_a), (lb, log_b) = ab, aa, bb
    else:
        lab, la, lb = ab, aa, bb
    div = lab - 0.5 * (la + lb)
    div = np.maximum(0, div) if not isinstance(div, torch.Tensor) else torch.clamp(div, min=0)
    if log:
        return div, {"sinkhorn_loss_ab": lab, "sinkhorn_loss_a": la, "sinkhorn_loss_b": lb,
                     "log_sinkhorn_ab": log_ab, "log_sinkhorn_a": log_a, "log_sinkhorn_b": log_b}
    return div
