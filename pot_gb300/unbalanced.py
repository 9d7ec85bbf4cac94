"""GPU unbalanced entropic OT with KL marginal penalties:
``ot.unbalanced.sinkhorn_unbalanced`` / ``sinkhorn_unbalanced2`` with
``method='sinkhorn'`` and ``sinkhorn_knopp_unbalanced``
(PythonOT/POT ``ot/unbalanced/_sinkhorn.py:19-249``, ``:252-562``,
``:565-818``), 1-D ``b``.

The iteration runs in the dense persistent kernel (``OTG_METHOD_UNB``): u
first, ``u = (a / K v)^fi1``, ``v = (b / K^T u)^fi2``, the relative
sup-norm change of ``(u, v)`` reduced grid-wide and checked every
iteration, the previous pair kept on a zero ``K^T u`` or a non-finite
scaling.  ``c = a b^T`` (``reg_type='kl'``) and ``c = 1``
(``reg_type='entropy'``) are applied inside the passes; a user ``c`` is
folded into the cost as ``M - reg log c``.  The plan and the costs of the
log (``cost``, ``total_cost``) come from the plan and marginal kernels.
"""
import ctypes
import warnings

import numpy as np
import torch

from . import _lib
from . import batch as pb
from .bregman import _prep, solve_dense, _errs_as


def _pair(reg_m):
    if isinstance(reg_m, (int, float)) or (hasattr(reg_m, "ndim") and np.ndim(reg_m) == 0):
        return float(reg_m), float(reg_m)
    return float(reg_m[0]), float(reg_m[1])


def _kl_vec(p, q):
    return float(torch.sum(p * torch.log(p / q + 1e-16)))


def sinkhorn_knopp_unbalanced(a, b, M, reg, reg_m, reg_type="kl", c=None, warmstart=None, numItermax=1000,
                              stopThr=1e-6, verbose=False, log=False, **kwargs):
    """GPU ``ot.unbalanced.sinkhorn_knopp_unbalanced`` (1-D ``b``)."""
    bd, Md, ad, bv = _prep(a, b, M)
    if bv.dim() > 1:
        raise NotImplementedError("pot_gb300 sinkhorn_knopp_unbalanced: several target histograms are not on the "
                                  "GPU path")
    rm1, rm2 = _pair(reg_m)
    reg = float(reg)
    c_ones = 0
    cd = None
    if reg_type.lower() == "entropy":
        warnings.warn("If reg_type = entropy, then the matrix c is overwritten by the one matrix.")
        c_ones = 1
    elif c is not None:
        cd = bd.to_dev(c, Md.dtype)
        Md = (Md - reg * torch.log(cd)).contiguous()
        c_ones = 1
    wu = wv = None
    if warmstart is not None:
        wu, wv = (bd.to_dev(warmstart[0], Md.dtype).contiguous(), bd.to_dev(warmstart[1], Md.dtype).contiguous())
    r = solve_dense(Md, ad, bv, reg, _lib.OTG_METHOD_UNB, numItermax, stopThr, wu, wv, check_period=1,
                    unbalanced=(rm1, rm2, c_ones))
    if r.status == _lib.STATUS_NUMERICAL:
        warnings.warn("Numerical errors at iteration %s" % r.niter)
    if verbose:
        for i, e in enumerate(r.errs):
            if i % 50 == 0:
                print("{:5s}|{:12s}".format("It.", "Err") + "\n" + "-" * 19)
            print("{:5d}|{:8e}|".format(i, e))
    u, v = r.u, r.v
    al = torch.ones_like(u) if c_ones else ad
    be = torch.ones_like(v) if c_ones else bv
    ut, vt = (al * u).contiguous(), (be * v).contiguous()
    n, m = Md.shape
    layout, Mp = pb._uniform_batch(Md[None])
    reg_t = torch.full((1,), reg, dtype=torch.float64, device=Md.device)
    P, vals = pb.batched_plan(layout, Mp, ut, vt, ad, bv, reg_t, _lib.OTG_METHOD_KNOPP, kl=not c_ones)
    P = P.view(n, int(layout.ldm_np[0]))[:, :m].contiguous()
    if not log:
        return bd.out(P)
    Morig = bd.to_dev(M, Md.dtype) if cd is not None else Md
    cost = float(vals[0, 0]) if cd is None else float(torch.sum(P * Morig))
    if cd is not None:
        reg_term = float(torch.sum(P * torch.log(P / cd + 1e-16)))
    else:
        reg_term = float(vals[0, 1])  # sum P log(P / c + 1e-16) for c = a b^T or c = 1
    total = cost + reg * reg_term
    if rm1 != float("inf") or rm2 != float("inf"):
        lib = _lib.load()
        rows = torch.empty(n, dtype=torch.float64, device=Md.device)
        cols = torch.empty(m, dtype=torch.float64, device=Md.device)
        lu, lv = torch.log(ut), torch.log(vt)
        _lib.check(lib.otg_dense_marginals(_lib.dtype_code(Md.dtype), ctypes.c_void_p(Md.data_ptr()), n, m,
                                           Md.stride(0), _lib.ptr(lu), _lib.ptr(lv), reg, _lib.ptr(rows),
                                           _lib.ptr(cols), _lib.stream_handle(Md.device)), "otg_dense_marginals")
        if rm1 != float("inf"):
            total += rm1 * _kl_vec(rows, ad.double())
        if rm2 != float("inf"):
            total += rm2 * _kl_vec(cols, bv.double())
    lg = {"err": _errs_as(bd, r.errs, Md), "logu": bd.out(torch.log(u + 1e-300)),
          "logv": bd.out(torch.log(v + 1e-300)),
          "cost": bd.scalar(torch.tensor(cost, dtype=Md.dtype, device=Md.device)),
          "total_cost": bd.scalar(torch.tensor(total, dtype=Md.dtype, device=Md.device))}
    return bd.out(P), lg


def sinkhorn_unbalanced(a, b, M, reg, reg_m, method="sinkhorn", reg_type="kl", c=None, warmstart=None,
                        numItermax=1000, stopThr=1e-6, verbose=False, log=False, **kwargs):
    """GPU ``ot.unbalanced.sinkhorn_unbalanced``: method dispatch of
    ``ot/unbalanced/_sinkhorn.py:160-249``."""
    meth = method.lower()
    if meth == "sinkhorn_reg_scaling":
        warnings.warn("Method not implemented yet. Using classic Sinkhorn-Knopp")
        meth = "sinkhorn"
    if meth == "sinkhorn":
        return sinkhorn_knopp_unbalanced(a, b, M, reg, reg_m, reg_type, c, warmstart, numItermax=numItermax,
                                         stopThr=stopThr, verbose=verbose, log=log, **kwargs)
    if meth in ("sinkhorn_stabilized", "sinkhorn_translation_invariant"):
        raise NotImplementedError("pot_gb300: unbalanced method='%s' is not on the GPU path" % method)
    raise ValueError("Unknown method '%s'." % method)


def sinkhorn_unbalanced2(a, b, M, reg, reg_m, method="sinkhorn", reg_type="kl", c=None, warmstart=None,
                         returnCost="linear", numItermax=1000, stopThr=1e-6, verbose=False, log=False, **kwargs):
    """GPU ``ot.unbalanced.sinkhorn_unbalanced2`` (1-D ``b``): the linear or
    total cost of the plan (``:490-502``)."""
    if returnCost not in ("linear", "total"):
        raise ValueError("Unknown returnCost = {}".format(returnCost))
    P, lg = sinkhorn_unbalanced(a, b, M, reg, reg_m, method, reg_type, c, warmstart, numItermax=numItermax,
                                stopThr=stopThr, verbose=verbose, log=True, **kwargs)
    cost = lg["cost"] if returnCost == "linear" else lg["total_cost"]
    return (cost, lg) if log else cost
