"""GPU ``ot.bregman.empirical_sinkhorn`` (``ot/bregman/_empirical.py:74-263``)
for the squared-Euclidean metric.

``isLazy=True`` runs the online kernel (``csrc/otg online``): the cost is
never stored; potentials f, g are dimensionless log-scalings as in the
reference, the L1 row-marginal error is checked after iterations with
``(i+1) % 10 == 0`` and compared with ``<=``.  The online path computes in
float32 (tensor-core dot products with a high/low half split); float64
inputs are solved in float32 and returned as float64.  ``isLazy=False``
builds the dense cost on the GPU and calls the dense scaling-form solver,
as the reference calls ``sinkhorn``.
"""
import ctypes
import warnings

import numpy as np
import torch

from . import _lib
from ._arrays import Boundary, check_shape, shape_of
from . import bregman
from . import batch as pb
from .gromov import pow2_scale

# statistics of the last online_sinkhorn call: fixup_units = row blocks that a
# fix-up pass recomputed (their shifted sums left the representable range)
LAST_STATS = {"fixup_units": 0}

NONCONV_MSG = bregman.NONCONV_MSG


class LazyPlan:
    """Plan entries exp(f_i + g_j - |x_i - y_j|^2 / reg) computed on demand
    (the ``lazy_plan`` of the reference's log, ``ot/utils.py:1425``)."""

    def __init__(self, X, Y, f, g, reg, out):
        self.X, self.Y, self.f, self.g, self.reg, self._out = X, Y, f, g, reg, out
        self.shape = (X.shape[0], Y.shape[0])

    def __getitem__(self, key):
        i, j = key if isinstance(key, tuple) else (key, slice(None))
        i = slice(i, i + 1) if isinstance(i, int) else i
        j = slice(j, j + 1) if isinstance(j, int) else j
        X, Y = self.X[i].double(), self.Y[j].double()
        C = ((X[:, None, :] - Y[None, :, :]) ** 2).sum(-1)
        P = torch.exp(self.f[i].double()[:, None] + self.g[j].double()[None, :] - C / self.reg)
        return self._out(P.to(self.f.dtype))


def online_sinkhorn(X, Y, reg, a, b, numIterMax, stopThr, warm_f=None, warm_g=None, sum_window_log2=0.0):
    """Device float32 tensors in; (f, g, status, niter, errs) out.
    ``sum_window_log2`` > 0 narrows the acceptance window of the folded
    passes' shifted sums (rows outside it go through the fix-up pass)."""
    lib = _lib.load()
    n, d = X.shape
    m = Y.shape[0]
    wsb = lib.otg_online_workspace_bytes(n, m, d)
    ws = torch.empty(wsb, dtype=torch.uint8, device=X.device)
    f = torch.empty(n, dtype=torch.float32, device=X.device)
    g = torch.empty(m, dtype=torch.float32, device=X.device)
    cap = max(2, numIterMax // 10 + 2)
    hist = (ctypes.c_double * cap)()
    info = (ctypes.c_int32 * 4)()
    p = _lib.OtgOnlineProblem(X=X.data_ptr(), Y=Y.data_ptr(), n=n, m=m, d=d, max_iter=int(numIterMax),
                              a=a.data_ptr(), b=b.data_ptr(),
                              warm_f=warm_f.data_ptr() if warm_f is not None else None,
                              warm_g=warm_g.data_ptr() if warm_g is not None else None, reg=float(reg),
                              stop_thr=float(stopThr), scale_x=pow2_scale(float(X.abs().max())),
                              scale_y=pow2_scale(float(Y.abs().max())), out_f=f.data_ptr(), out_g=g.data_ptr(),
                              err_hist=hist, hist_cap=cap, info=info, workspace=ws.data_ptr(),
                              workspace_bytes=wsb, timeout_ms=0, sum_window_log2=float(sum_window_log2))
    _lib.check(lib.otg_sinkhorn_online(ctypes.byref(p), _lib.stream_handle(X.device)), "otg_sinkhorn_online")
    if info[0] == _lib.STATUS_ABORTED:
        raise RuntimeError("pot_gb300: a device-side wait of the online kernel timed out")
    LAST_STATS["fixup_units"] = int(info[3])
    return f, g, info[0], info[1], [hist[k] for k in range(min(info[2], cap))]


def lazy_loss(X_s, X_t, f, g, reg):
    """``sum_ij C_ij exp(f_i + g_j - C_ij / reg)`` over squared distances,
    the loss of ``empirical_sinkhorn2(isLazy=True)``
    (``ot/bregman/_empirical.py:470-478``), in one kernel
    (``otg_lazy_loss``, fp64 accumulation)."""
    bd = Boundary(X_s, X_t, f, g)
    X = bd.to_dev(X_s)
    dt = X.dtype
    X = X.contiguous()
    Y = bd.to_dev(X_t, dt).contiguous()
    fd, gd = bd.to_dev(f, dt).contiguous(), bd.to_dev(g, dt).contiguous()
    out = torch.empty(1, dtype=torch.float64, device=X.device)
    lib = _lib.load()
    _lib.check(lib.otg_lazy_loss(_lib.dtype_code(dt), _lib.ptr(X), _lib.ptr(Y), X.shape[0], Y.shape[0], X.shape[1],
                                 _lib.ptr(fd), _lib.ptr(gd), float(reg), _lib.ptr(out), _lib.stream_handle(X.device)),
               "otg_lazy_loss")
    return bd.scalar(out[0].to(dt))


def empirical_sinkhorn(X_s, X_t, reg, a=None, b=None, metric="sqeuclidean", numIterMax=10000, stopThr=1e-9,
                       isLazy=False, batchSize=100, verbose=False, log=False, warn=True, warmstart=None, **kwargs):
    """GPU ``ot.bregman.empirical_sinkhorn`` (squared-Euclidean metric)."""
    if metric != "sqeuclidean":
        raise NotImplementedError("pot_gb300 empirical_sinkhorn: metric '%s' is not on the GPU path" % metric)
    if isLazy and not (isinstance(batchSize, int) or (isinstance(batchSize, tuple) and len(batchSize) == 2)):
        raise ValueError("Batch size must be in integer or a tuple of two integers")
    sX, sY = shape_of(X_s), shape_of(X_t)
    if len(sX) != 2 or len(sY) != 2 or sX[1] != sY[1]:
        raise ValueError("X_s and X_t must be point arrays (ns, d) and (nt, d), got %s and %s" % (sX, sY))
    check_shape("a", a, [(sX[0],)])
    check_shape("b", b, [(sY[0],)])
    if warmstart is not None:
        check_shape("warmstart[0]", warmstart[0], [(sX[0],)])
        check_shape("warmstart[1]", warmstart[1], [(sY[0],)])
    bd = Boundary(X_s, X_t, a, b)
    Xd = bd.to_dev(X_s)
    Yd = bd.to_dev(X_t, Xd.dtype)
    dt = Xd.dtype
    ns, nt = Xd.shape[0], Yd.shape[0]
    ad = torch.full((ns,), 1.0 / ns, dtype=dt, device=Xd.device) if a is None else bd.to_dev(a, dt)
    bv = torch.full((nt,), 1.0 / nt, dtype=dt, device=Xd.device) if b is None else bd.to_dev(b, dt)
    if not isLazy:
        layout = pb.RaggedLayout([ns], [nt], dt, Xd.device)
        Mp, _ = pb.batched_sqdist(layout, Xd.reshape(-1).contiguous(), Yd.reshape(-1).contiguous(), [0], [0],
                                  [Xd.shape[1]])
        M = Mp.view(ns, int(layout.ldm_np[0]))[:, :nt]
        return bregman.sinkhorn(ad, bv, M, reg, numItermax=numIterMax, stopThr=stopThr, verbose=verbose,
                                log=log, warn=warn, warmstart=warmstart) if bd.kind != "numpy" else \
            bregman.sinkhorn(ad.cpu().numpy(), bv.cpu().numpy(), M.cpu().numpy(), reg, numItermax=numIterMax,
                             stopThr=stopThr, verbose=verbose, log=log, warn=warn, warmstart=warmstart)
    X32, Y32 = Xd.float().contiguous(), Yd.float().contiguous()
    wf = wg = None
    if warmstart is not None:
        wf = bd.to_dev(warmstart[0], torch.float32).contiguous()
        wg = bd.to_dev(warmstart[1], torch.float32).contiguous()
    f, g, status, niter, errs = online_sinkhorn(X32, Y32, reg, ad.float().contiguous(), bv.float().contiguous(),
                                                numIterMax, stopThr, wf, wg)
    if verbose:
        for k, e in enumerate(errs):
            it = 10 * (k + 1)
            if it % 100 == 0:
                print("Error in marginal at iteration {} = {}".format(it, e))
    if status != _lib.STATUS_CONVERGED and warn:
        warnings.warn(NONCONV_MSG)
    f, g = f.to(dt), g.to(dt)
    if log:
        lg = {"err": [np.float64(e) for e in errs] if bd.kind == "numpy" else [torch.tensor(e) for e in errs],
              "u": bd.out(f), "v": bd.out(g), "niter": niter,
              "lazy_plan": LazyPlan(Xd, Yd, f, g, float(reg), bd.out)}
        return bd.out(f), bd.out(g), lg
    return bd.out(f), bd.out(g)
