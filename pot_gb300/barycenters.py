"""GPU ``ot.bregman.barycenter`` (``ot/bregman/_barycenter.py:23-138``) for
the 'sinkhorn' (scaling, ``barycenter_sinkhorn`` :141-259) and
'sinkhorn_log' (``_barycenter_sinkhorn_log`` :403-473) methods.

The iteration loop runs natively behind ``otg_barycenter`` (``csrc/bary.cu``):
GEMMs for the scaling form, log-semiring row and column passes for the log
form, fused per-row updates, one synchronisation per error check
(``ii % 10 == 1``).  Signatures, defaults, the log (``err``, ``niter``) and
the non-convergence warning follow the reference.
"""
import ctypes
import warnings

import numpy as np
import torch

from . import _lib
from ._arrays import Boundary
from .bregman import NONCONV_MSG, _errs_as


def _run(A, M, reg, weights, method, numItermax, stopThr, verbose, log, warn):
    bd = Boundary(A, M, weights)
    Ad = bd.to_dev(A)
    Md = bd.to_dev(M, Ad.dtype)
    if Md.stride(1) != 1:
        Md = Md.contiguous()
    Ad = Ad.contiguous()
    dim, H = Ad.shape
    if Md.shape != (dim, dim):
        raise ValueError("M must be (dim, dim) for histograms of size dim")
    if weights is None:
        wd = torch.full((H,), 1.0 / H, dtype=Ad.dtype, device=Ad.device)
    else:
        if len(weights) != H:
            raise ValueError("weights has %d entries for %d histograms" % (len(weights), H))
        wd = bd.to_dev(weights, Ad.dtype).contiguous()
    lib = _lib.load()
    dt = _lib.dtype_code(Ad.dtype)
    wsb = lib.otg_barycenter_workspace_bytes(dt, method, dim, H)
    ws = torch.empty(wsb, dtype=torch.uint8, device=Ad.device)
    bar = torch.empty(dim, dtype=Ad.dtype, device=Ad.device)
    cap = max(2, numItermax // 10 + 2)
    hist = (ctypes.c_double * cap)()
    info = (ctypes.c_int32 * 3)()
    p = _lib.OtgBaryProblem(dtype=dt, method=method, M=Md.data_ptr(), dim=dim, ldm=Md.stride(0), A=Ad.data_ptr(),
                            n_hists=H, max_iter=int(numItermax), weights=wd.data_ptr(), reg=float(reg),
                            stop_thr=float(stopThr), out_bar=bar.data_ptr(), err_hist=hist, hist_cap=cap, info=info,
                            workspace=ws.data_ptr(), workspace_bytes=wsb)
    _lib.check(lib.otg_barycenter(ctypes.byref(p), _lib.stream_handle(Ad.device)), "otg_barycenter")
    errs = np.array([hist[k] for k in range(min(info[2], cap))])
    if verbose:
        for k, e in enumerate(errs[:-1] if info[0] == _lib.STATUS_CONVERGED else errs):
            ii = 10 * k + 1
            if ii % 200 == 0:
                print("{:5s}|{:12s}".format("It.", "Err") + "\n" + "-" * 19)
            print("{:5d}|{:8e}|".format(ii, e))
    if info[0] == _lib.STATUS_MAXITER and warn:
        warnings.warn(NONCONV_MSG)
    if log:
        return bd.out(bar), {"err": _errs_as(bd, errs, bar), "niter": int(info[1])}
    return bd.out(bar)


def barycenter_sinkhorn(A, M, reg, weights=None, numItermax=1000, stopThr=1e-4, verbose=False, log=False,
                        warn=True):
    """GPU ``ot.bregman.barycenter_sinkhorn`` (scaling form)."""
    return _run(A, M, reg, weights, _lib.OTG_METHOD_KNOPP, numItermax, stopThr, verbose, log, warn)


def barycenter_sinkhorn_log(A, M, reg, weights=None, numItermax=1000, stopThr=1e-4, verbose=False, log=False,
                            warn=True):
    """GPU ``ot.bregman._barycenter._barycenter_sinkhorn_log`` (log domain)."""
    return _run(A, M, reg, weights, _lib.OTG_METHOD_LOG, numItermax, stopThr, verbose, log, warn)


def barycenter(A, M, reg, weights=None, method="sinkhorn", numItermax=10000, stopThr=1e-4, verbose=False,
               log=False, warn=True, **kwargs):
    """GPU ``ot.bregman.barycenter``: dispatch on ``method`` (``:95-138``)."""
    meth = method.lower()
    if meth == "sinkhorn":
        return barycenter_sinkhorn(A, M, reg, weights=weights, numItermax=numItermax, stopThr=stopThr,
                                   verbose=verbose, log=log, warn=warn, **kwargs)
    if meth == "sinkhorn_log":
        return barycenter_sinkhorn_log(A, M, reg, weights=weights, numItermax=numItermax, stopThr=stopThr,
                                       verbose=verbose, log=log, warn=warn, **kwargs)
    if meth == "sinkhorn_stabilized":
        raise NotImplementedError("pot_gb300: barycenter method='sinkhorn_stabilized' is not on the GPU path")
    raise ValueError("Unknown method '%s'." % method)
