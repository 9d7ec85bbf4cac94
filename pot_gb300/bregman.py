"""Drop-in replacements for ``ot.sinkhorn``, ``ot.sinkhorn2``,
``ot.bregman.sinkhorn_knopp``, ``ot.bregman.sinkhorn_log``,
``ot.bregman.sinkhorn_stabilized``, ``ot.bregman.sinkhorn_epsilon_scaling``
and ``ot.bregman.greenkhorn``.

Signatures, defaults, return values, log-dict keys and warnings follow
PythonOT/POT ``ot/bregman/_sinkhorn.py`` (``sinkhorn`` :21-234, ``sinkhorn2``
:237-484, ``sinkhorn_knopp`` :487-687, ``sinkhorn_log`` :690-918,
``sinkhorn_stabilized`` :1105-1368, ``sinkhorn_epsilon_scaling``
:1371-1575, ``greenkhorn`` :921-1102).  The
iteration loop runs on the GPU in one persistent kernel
(``csrc/dense.cu``); the host only reads the result block once per solve.
"""
import ctypes
import math
import warnings

import numpy as np
import torch

from . import _lib
from ._arrays import Boundary, is_empty

NONCONV_MSG = ("Sinkhorn did not converge. You might want to "
               "increase the number of iterations `numItermax` "
               "or the regularization parameter `reg`.")


def _hist_cap(max_iter):
    return max(2, max_iter // 10 + 2)


class DenseResult:
    __slots__ = ("u", "v", "status", "niter", "errs", "workspace", "layout", "nabs", "absorbed_last", "method", "K")


_SMS = {}


def _sm_count():
    dev = torch.cuda.current_device()
    if dev not in _SMS:
        _SMS[dev] = torch.cuda.get_device_properties(dev).multi_processor_count
    return _SMS[dev]


def default_grid(n, m, dtype=None):
    """CTAs for one dense solve: small problems use few CTAs so the grid
    barriers stay cheap; large ones fill every SM (0 = all co-resident CTAs).
    float64 passes are bound by FP64 throughput, so they spread over up to
    one CTA per SM already at small sizes (n = m = 1024: 152 CTAs, measured
    1.3-1.6x faster than 64)."""
    elems = n * m
    if elems >= (1 << 24):
        return 0
    if dtype == torch.float64:
        return max(4, min(_sm_count(), elems // 4096))
    return max(4, elems // 16384)


# largest Gibbs kernel (bytes) precomputed for a float64 scaling-form solve
GIBBS_MAX_BYTES = 16 << 30


def solve_dense(M, a, b, reg, method, max_iter, stop_thr, warm_u=None, warm_v=None, grid=None,
                timeout_ms=0, read_back=True, tau=0.0, check_period=10, unbalanced=None, gibbs=None):
    """Run one dense solve on device tensors (contiguous rows, same dtype).

    Returns a DenseResult whose ``u, v`` are scalings (knopp) or natural-log
    potentials (log).  With ``read_back`` the status, last loop index and
    error history are copied to the host (one synchronisation).  ``gibbs``
    (default: float64 scaling form) first stores K = exp(-M/reg) so the
    passes read it instead of exponentiating every cost entry each
    iteration (float64 exponentials bound the solve on this GPU); the
    iterates are bit-identical."""
    lib = _lib.load()
    n, m = M.shape
    if grid is None:
        grid = default_grid(n, m, M.dtype)
    dt = _lib.dtype_code(M.dtype)
    cap = max(2, max_iter // check_period + 2)
    wsb = lib.otg_dense_workspace_bytes(dt, n, m, cap, grid)
    ws = torch.empty(wsb, dtype=torch.uint8, device=M.device)
    out_u = torch.empty(n, dtype=M.dtype, device=M.device)
    out_v = torch.empty(m, dtype=M.dtype, device=M.device)
    p = _lib.OtgDenseProblem(
        dtype=dt, method=method, M=M.data_ptr(), n=n, m=m, ldm=M.stride(0),
        a=a.data_ptr(), b=b.data_ptr(),
        warm_u=warm_u.data_ptr() if warm_u is not None else None,
        warm_v=warm_v.data_ptr() if warm_v is not None else None,
        reg=float(reg), max_iter=int(max_iter), hist_cap=cap, stop_thr=float(stop_thr),
        out_u=out_u.data_ptr(), out_v=out_v.data_ptr(), workspace_bytes=wsb, grid=grid,
        timeout_ms=timeout_ms, tau=float(tau), check_period=int(check_period))
    if unbalanced is not None:
        p.reg_m1, p.reg_m2, p.c_ones = float(unbalanced[0]), float(unbalanced[1]), int(unbalanced[2])
    if gibbs is None:
        gibbs = (method == _lib.OTG_METHOD_KNOPP and unbalanced is None and M.dtype == torch.float64
                 and n * m * 8 <= GIBBS_MAX_BYTES)
    K = None
    if gibbs:
        K = torch.empty((n, m), dtype=M.dtype, device=M.device)
        _lib.check(lib.otg_gibbs_kernel(dt, ctypes.c_void_p(M.data_ptr()), n, m, M.stride(0), float(reg),
                                        _lib.ptr(K), m, _lib.stream_handle(M.device)), "otg_gibbs_kernel")
        p.K, p.ldk = K.data_ptr(), m
    _lib.check(lib.otg_sinkhorn_dense(ctypes.byref(p), ctypes.c_void_p(ws.data_ptr()),
                                      _lib.stream_handle(M.device)), "otg_sinkhorn_dense")
    r = DenseResult()
    r.u, r.v, r.workspace, r.K = out_u, out_v, ws, K
    r.status, r.niter, r.errs = None, None, None
    r.layout = (dt, n, m, cap, grid)
    r.method = method
    if read_back:
        read_result(r)
    return r


def read_result(r):
    lib = _lib.load()
    dt, n, m, cap, grid = r.layout
    off = lib.otg_dense_info_offset(dt, n, m, cap, grid)
    ctrl = (off + 8 * cap + 255) // 256 * 256
    blk = r.workspace[off:ctrl + 32].cpu().numpy()
    hist = blk[:8 * cap].view(np.float64)
    info = blk[ctrl - off:ctrl - off + 32].view(np.int32)
    r.status, r.niter = int(info[0]), int(info[1])
    nchk = int(info[2])
    r.nabs, r.absorbed_last = int(info[5]), bool(info[6])
    if int(info[3]) != 0:
        r.status = _lib.STATUS_ABORTED
    # the unbalanced form logs the errors themselves, the others squared norms
    r.errs = hist[:nchk].copy() if r.method == _lib.OTG_METHOD_UNB else np.sqrt(hist[:nchk])
    if r.status == _lib.STATUS_ABORTED:
        raise RuntimeError("pot_gb300: a device-side wait timed out; the solve was abandoned")
    return r


def _errs_as(bd, errs, like):
    if bd.kind == "numpy":
        return [np.float64(e) for e in errs]
    t = torch.as_tensor(np.asarray(errs, dtype=np.float64), dtype=like.dtype)
    if not bd.host_torch:
        t = t.to(like.device)
    return list(t.unbind()) if len(errs) else []


def _print_errs(errs, check_before_print):
    for k, e in enumerate(errs):
        ii = 10 * k
        if not check_before_print and k == len(errs) - 1:
            pass
        if ii % 200 == 0:
            print("{:5s}|{:12s}".format("It.", "Err") + "\n" + "-" * 19)
        print("{:5d}|{:8e}|".format(ii, e))


def _shape(x):
    return tuple(x.shape) if hasattr(x, "shape") else np.shape(x)


def _check_shapes(a, b, M):
    """Histogram lengths against the cost's sides, before any device work:
    the kernels read a[0..n) and b[0..m), so a short histogram is an error
    here (the reference fails in numpy broadcasting), not an out-of-bounds
    read on the GPU."""
    sM = _shape(M)
    if len(sM) != 2:
        raise ValueError("M must be a 2-D cost matrix")
    n, m = sM
    if not is_empty(a) and _shape(a)[:1] != (n,):
        raise ValueError("a has %s entries, M has %d rows" % (_shape(a)[:1] or "no", n))
    if not is_empty(b) and _shape(b)[:1] != (m,):
        raise ValueError("b has %s entries, M has %d columns" % (_shape(b)[:1] or "no", m))


def _prep(a, b, M):
    _check_shapes(a, b, M)
    bd = Boundary(M, a, b)
    Md = bd.to_dev(M)
    if Md.dim() != 2:
        raise ValueError("M must be a 2-D cost matrix")
    if Md.stride(1) != 1 or Md.stride(0) < Md.shape[1]:
        Md = Md.contiguous()
    n, m = Md.shape
    ad = torch.full((n,), 1.0 / n, dtype=Md.dtype, device=Md.device) if is_empty(a) else bd.to_dev(a, Md.dtype)
    bdv = torch.full((m,), 1.0 / m, dtype=Md.dtype, device=Md.device) if is_empty(b) else bd.to_dev(b, Md.dtype)
    return bd, Md, ad.contiguous(), bdv.contiguous()


def _warm(bd, warmstart, dtype, n=None, m=None):
    if warmstart is None:
        return None, None
    wu, wv = bd.to_dev(warmstart[0], dtype).contiguous(), bd.to_dev(warmstart[1], dtype).contiguous()
    if (n is not None and wu.shape[:1] != (n,)) or (m is not None and wv.shape[:1] != (m,)):
        raise ValueError("warmstart potentials of lengths %s, %s for a %s x %s problem"
                         % (tuple(wu.shape[:1]), tuple(wv.shape[:1]), n, m))
    return wu, wv


def _run_single(bd, a, b, M, reg, method, numItermax, stopThr, verbose, warn, warmstart, want_plan):
    wu, wv = _warm(bd, warmstart, M.dtype, M.shape[0], M.shape[1])
    r = solve_dense(M, a, b, reg, method, numItermax, stopThr, wu, wv)
    if r.status == _lib.STATUS_NUMERICAL:
        warnings.warn("Warning: numerical errors at iteration %d" % r.niter)
    if verbose:
        errs = r.errs
        if method == _lib.OTG_METHOD_KNOPP and r.status == _lib.STATUS_CONVERGED:
            errs = errs[:-1]  # the reference prints after its break test
        _print_errs(errs, method == _lib.OTG_METHOD_LOG)
    if r.status == _lib.STATUS_MAXITER and warn:
        warnings.warn(NONCONV_MSG)
    P = None
    lib = _lib.load()
    if want_plan:
        P = torch.empty_like(M)
        _lib.check(lib.otg_dense_plan(_lib.dtype_code(M.dtype), method, ctypes.c_void_p(M.data_ptr()),
                                      M.shape[0], M.shape[1], M.stride(0), _lib.ptr(r.u), _lib.ptr(r.v),
                                      float(reg), _lib.ptr(P), P.stride(0), None,
                                      _lib.stream_handle(M.device)), "otg_dense_plan")
    return r, P


def _loss(M, r, reg, method):
    lib = _lib.load()
    acc = torch.zeros(1, dtype=torch.float64, device=M.device)
    _lib.check(lib.otg_dense_plan(_lib.dtype_code(M.dtype), method, ctypes.c_void_p(M.data_ptr()),
                                  M.shape[0], M.shape[1], M.stride(0), _lib.ptr(r.u), _lib.ptr(r.v),
                                  float(reg), None, 0, _lib.ptr(acc), _lib.stream_handle(M.device)),
               "otg_dense_plan")
    return acc[0].to(M.dtype)


def sinkhorn_knopp(a, b, M, reg, numItermax=1000, stopThr=1e-9, verbose=False, log=False,
                   warn=True, warmstart=None, **kwargs):
    """Scaling-form Sinkhorn on the GPU; see ``ot.bregman.sinkhorn_knopp``."""
    bd, Md, ad, bdv = _prep(a, b, M)
    if bdv.dim() > 1:
        return _knopp_multi(bd, ad, bdv, Md, reg, numItermax, stopThr, verbose, log, warn, warmstart)
    r, P = _run_single(bd, ad, bdv, Md, reg, _lib.OTG_METHOD_KNOPP, numItermax, stopThr, verbose,
                       warn, warmstart, True)
    if log:
        lg = {"err": _errs_as(bd, r.errs, Md), "niter": r.niter, "u": bd.out(r.u), "v": bd.out(r.v)}
        return bd.out(P), lg
    return bd.out(P)


def sinkhorn_log(a, b, M, reg, numItermax=1000, stopThr=1e-9, verbose=False, log=False,
                 warn=True, warmstart=None, **kwargs):
    """Log-domain Sinkhorn on the GPU; see ``ot.bregman.sinkhorn_log``."""
    bd, Md, ad, bdv = _prep(a, b, M)
    if bdv.dim() > 1:
        return _log_multi(bd, ad, bdv, Md, reg, numItermax, stopThr, verbose, log, warmstart)
    r, P = _run_single(bd, ad, bdv, Md, reg, _lib.OTG_METHOD_LOG, numItermax, stopThr, verbose,
                       warn, warmstart, True)
    if log:
        lg = {"err": _errs_as(bd, r.errs, Md), "niter": r.niter, "log_u": bd.out(r.u),
              "log_v": bd.out(r.v), "u": bd.out(torch.exp(r.u)), "v": bd.out(torch.exp(r.v))}
        return bd.out(P), lg
    return bd.out(P)


def _log_multi(bd, a, B, M, reg, numItermax, stopThr, verbose, log, warmstart):
    """Several target histograms: every histogram is its own sinkhorn_log
    solve, as in the reference's recursion (``_sinkhorn.py:819-854``), all of
    them in one work-balanced launch of the batch kernel (the histograms
    share the cost block; each stops on its own test).  Returns the
    per-histogram losses and a log holding only the potentials.  With
    ``verbose`` the histograms are solved one after another (the error
    tables are printed per solve, as the reference does)."""
    H = B.shape[1]
    ws = warmstart if warmstart is not None else [None] * H
    if verbose:
        return _log_multi_sequential(bd, a, B, M, reg, numItermax, stopThr, verbose, log, ws)
    from . import batch as pb
    n, m = M.shape
    dt, dev = M.dtype, M.device
    lay = pb.RaggedLayout([n] * H, [m] * H, dt, dev)
    ld = int(lay.ldm_np[0])
    if ld == m and M.is_contiguous():
        Mp = M.reshape(-1)
    else:
        Mp = torch.full((n, ld), float("inf"), dtype=dt, device=dev)
        Mp[:, :m].copy_(M)
        Mp = Mp.reshape(-1)
    # one shared cost block: every histogram's problem reads it
    lay.m_off.zero_()
    lay.m_off_np = np.zeros(H, dtype=np.int64)
    a_p = a.repeat(H).contiguous()
    b_p = B.t().contiguous().reshape(-1)
    warm_u = None
    if warmstart is not None:
        warm_u = torch.cat([_warm(bd, ws[k], dt)[0] for k in range(H)]).contiguous()
    u, v, st, _, _, _ = pb.run_multi(lay, Mp, a_p, b_p, reg, numItermax, stopThr, warm_u=warm_u)
    U, V = u.view(H, n).t(), v.view(H, m).t()
    for k in range(H):
        if int(st[k]) == _lib.STATUS_MAXITER:
            warnings.warn(NONCONV_MSG)
    losses = []
    for k in range(H):
        r = DenseResult()
        r.u, r.v = U[:, k].contiguous(), V[:, k].contiguous()
        losses.append(_loss(M, r, reg, _lib.OTG_METHOD_LOG))
    res = torch.stack(losses)
    if log:
        lu, lv = U.contiguous(), V.contiguous()
        return bd.out(res), {"log_u": bd.out(lu), "log_v": bd.out(lv), "u": bd.out(torch.exp(lu)),
                             "v": bd.out(torch.exp(lv))}
    return bd.out(res)


def _log_multi_sequential(bd, a, B, M, reg, numItermax, stopThr, verbose, log, ws):
    H = B.shape[1]
    losses, lus, lvs = [], [], []
    for k in range(H):
        r, _ = _run_single(bd, a, B[:, k].contiguous(), M, reg, _lib.OTG_METHOD_LOG, numItermax,
                           stopThr, verbose, True, ws[k], False)
        losses.append(_loss(M, r, reg, _lib.OTG_METHOD_LOG))
        lus.append(r.u)
        lvs.append(r.v)
    res = torch.stack(losses)
    if log:
        lu, lv = torch.stack(lus, 1), torch.stack(lvs, 1)
        return bd.out(res), {"log_u": bd.out(lu), "log_v": bd.out(lv), "u": bd.out(torch.exp(lu)),
                             "v": bd.out(torch.exp(lv))}
    return bd.out(res)


def _knopp_multi(bd, a, B, M, reg, numItermax, stopThr, verbose, log, warn, warmstart):
    """Scaling form with several target histograms (``_sinkhorn.py:600-687``
    with ``n_hists``): the histograms evolve independently and interact only
    through the joint stop (Frobenius norm of all column-marginal errors) and
    the joint revert on numerical errors.  Each histogram is iterated on the
    GPU with its error history, first over a short horizon that grows four
    times until the joint stop (or a numerical error, or numItermax) falls
    inside it; every histogram is then re-run to exactly that index (a run
    that ended there already is kept)."""
    H = B.shape[1]
    wu = wv = None
    if warmstart is not None:
        wu = bd.to_dev(warmstart[0], M.dtype)
        wv = bd.to_dev(warmstart[1], M.dtype)
    warm = lambda k: (None, None) if wu is None else (wu[:, k].contiguous(), wv[:, k].contiguous())  # noqa: E731
    horizon = min(numItermax, 64)
    while True:
        runs = [solve_dense(M, a, B[:, k].contiguous(), reg, _lib.OTG_METHOD_KNOPP, horizon, 0.0, *warm(k))
                for k in range(H)]
        nan_at = min([r.niter for r in runs if r.status == _lib.STATUS_NUMERICAL], default=None)
        nchk = min(len(r.errs) for r in runs)
        joint = [float(np.sqrt(sum(r.errs[k] ** 2 for r in runs))) for k in range(nchk)]
        stop_ii, errs = None, []
        for k, e in enumerate(joint):
            ii = 10 * k
            if nan_at is not None and ii >= nan_at:
                break
            errs.append(e)
            if e < stopThr:
                stop_ii = ii
                break
        if stop_ii is not None or nan_at is not None or horizon == numItermax:
            break
        horizon = min(numItermax, 4 * horizon)
    if stop_ii is not None:
        final_iters, niter, status = stop_ii + 1, stop_ii, _lib.STATUS_CONVERGED
    elif nan_at is not None:
        final_iters, niter, status = nan_at, nan_at, _lib.STATUS_NUMERICAL
    else:
        final_iters, niter, status = numItermax, numItermax - 1, _lib.STATUS_MAXITER
    if final_iters == horizon and nan_at is None:
        final = runs
    else:
        final = [solve_dense(M, a, B[:, k].contiguous(), reg, _lib.OTG_METHOD_KNOPP, final_iters, 0.0, *warm(k))
                 for k in range(H)] if final_iters > 0 else None
    if final is None:  # numerical error in the first iteration: the initial scalings
        n, m = M.shape
        U = torch.full((n, H), 1.0 / n, dtype=M.dtype, device=M.device) if wu is None else torch.exp(wu)
        V = torch.full((m, H), 1.0 / m, dtype=M.dtype, device=M.device) if wv is None else torch.exp(wv)
        losses = []
        for k in range(H):
            r = DenseResult()
            r.u, r.v = U[:, k].contiguous(), V[:, k].contiguous()
            losses.append(_loss(M, r, reg, _lib.OTG_METHOD_KNOPP))
    else:
        U = torch.stack([r.u for r in final], 1)
        V = torch.stack([r.v for r in final], 1)
        losses = [_loss(M, r, reg, _lib.OTG_METHOD_KNOPP) for r in final]
    if status == _lib.STATUS_NUMERICAL:
        warnings.warn("Warning: numerical errors at iteration %d" % niter)
    if verbose:
        _print_errs(np.array(errs[:-1] if status == _lib.STATUS_CONVERGED else errs), False)
    if status == _lib.STATUS_MAXITER and warn:
        warnings.warn(NONCONV_MSG)
    res = torch.stack(losses)
    if log:
        return bd.out(res), {"err": _errs_as(bd, np.array(errs), M), "niter": niter, "u": bd.out(U),
                             "v": bd.out(V)}
    return bd.out(res)


def _stab_solve(bd, a, b, M, reg, numItermax, tau, stopThr, warmstart, print_period):
    """One stabilised solve (``OTG_METHOD_STAB``); returns the result and the
    reference's ``logu, logv`` (its gauge: shifted by the absorptions)."""
    wu = wv = None
    if warmstart is not None:
        al, be = _warm(bd, warmstart, M.dtype, M.shape[0], M.shape[1])
        wu, wv = (al / reg).contiguous(), (be / reg).contiguous()
    r = solve_dense(M, a, b, reg, _lib.OTG_METHOD_STAB, numItermax, stopThr, wu, wv, tau=tau,
                    check_period=print_period)
    n, m = M.shape
    k = r.nabs
    logu = r.u - k * math.log(n)
    logv = r.v + (((k - 1) * math.log(n) - math.log(m)) if r.absorbed_last else k * math.log(n))
    return r, logu, logv


def _plan_from_logs(M, logu, logv, reg):
    lib = _lib.load()
    P = torch.empty_like(M)
    _lib.check(lib.otg_dense_plan(_lib.dtype_code(M.dtype), _lib.OTG_METHOD_LOG, ctypes.c_void_p(M.data_ptr()),
                                  M.shape[0], M.shape[1], M.stride(0), _lib.ptr(logu), _lib.ptr(logv), float(reg),
                                  _lib.ptr(P), P.stride(0), None, _lib.stream_handle(M.device)), "otg_dense_plan")
    return P


def sinkhorn_stabilized(a, b, M, reg, numItermax=1000, tau=1e3, stopThr=1e-9, warmstart=None, verbose=False,
                        print_period=20, log=False, warn=True, **kwargs):
    """GPU ``ot.bregman.sinkhorn_stabilized`` (``_sinkhorn.py:1105-1368``),
    1-D ``b``.  ``warmstart`` is ``(alpha, beta)`` in cost units, as in the
    reference.  The iteration runs in the log domain on the GPU and
    reproduces the reference's absorptions, error history and stop index;
    the log holds ``err, n_iter, logu, logv, alpha, beta, warmstart``."""
    bd, Md, ad, bdv = _prep(a, b, M)
    if bdv.dim() > 1:
        raise NotImplementedError("pot_gb300 sinkhorn_stabilized: several target histograms are not on the GPU path")
    r, logu, logv, lg = _stabilized(bd, ad, bdv, Md, reg, numItermax, stopThr, warmstart, verbose, warn, log,
                                    tau, print_period)
    P = _plan_from_logs(Md, logu, logv, reg)
    return (bd.out(P), lg) if log else bd.out(P)


def _stabilized(bd, ad, bdv, Md, reg, numItermax, stopThr, warmstart, verbose, warn, log, tau=1e3,
                print_period=20):
    r, logu, logv = _stab_solve(bd, ad, bdv, Md, reg, numItermax, tau, stopThr, warmstart, print_period)
    if verbose:
        for k, e in enumerate(r.errs):
            ii = k * print_period
            if ii % (print_period * 20) == 0:
                print("{:5s}|{:12s}".format("It.", "Err") + "\n" + "-" * 19)
            print("{:5d}|{:8e}|".format(ii, e))
    if r.status == _lib.STATUS_NUMERICAL:
        warnings.warn("Numerical errors at iteration %d" % r.niter)
    elif r.status == _lib.STATUS_MAXITER and warn:
        warnings.warn(NONCONV_MSG)
    lg = None
    if log:
        alpha, beta = reg * logu, reg * logv
        lg = {"err": _errs_as(bd, r.errs, Md), "n_iter": r.niter, "logu": bd.out(logu), "logv": bd.out(logv),
              "alpha": bd.out(alpha), "beta": bd.out(beta), "warmstart": (bd.out(alpha), bd.out(beta))}
    return r, logu, logv, lg


def sinkhorn_epsilon_scaling(a, b, M, reg, numItermax=100, epsilon0=1e4, numInnerItermax=100, tau=1e3,
                             stopThr=1e-9, warmstart=None, verbose=False, print_period=10, log=False, warn=True,
                             **kwargs):
    """GPU ``ot.bregman.sinkhorn_epsilon_scaling`` (``_sinkhorn.py:1371-1575``):
    at least 35 outer steps with ``reg_k = (epsilon0 - reg) exp(-k) + reg``,
    each a stabilised GPU solve warm-started from the previous
    ``(alpha, beta)``; every ``print_period`` steps the squared marginal
    errors of the inner plan (``otg_dense_marginals``) are logged."""
    bd, Md, ad, bdv = _prep(a, b, M)
    lib = _lib.load()
    n, m = Md.shape
    numItermax = max(35, numItermax)
    ws = None if warmstart is None else _warm(bd, warmstart, Md.dtype, n, m)
    rows = torch.empty(n, dtype=torch.float64, device=Md.device)
    cols = torch.empty(m, dtype=torch.float64, device=Md.device)
    a64, b64 = ad.double(), bdv.double()
    errs = []
    err = 1.0
    stopped = False
    ii = 0
    logu = logv = regi = None
    for ii in range(numItermax):
        regi = (epsilon0 - reg) * math.exp(-ii) + reg
        r, logu, logv = _stab_solve(bd, ad, bdv, Md, regi, numInnerItermax, tau, stopThr, ws, 20)
        if r.status == _lib.STATUS_NUMERICAL:
            warnings.warn("Numerical errors at iteration %d" % r.niter)
        elif r.status == _lib.STATUS_MAXITER:
            warnings.warn(NONCONV_MSG)
        ws = (regi * logu, regi * logv)
        if ii % print_period == 0:
            _lib.check(lib.otg_dense_marginals(_lib.dtype_code(Md.dtype), ctypes.c_void_p(Md.data_ptr()), n, m,
                                               Md.stride(0), _lib.ptr(logu), _lib.ptr(logv), float(regi),
                                               _lib.ptr(rows), _lib.ptr(cols), _lib.stream_handle(Md.device)),
                       "otg_dense_marginals")
            err = float(torch.linalg.vector_norm(cols - b64) ** 2 + torch.linalg.vector_norm(rows - a64) ** 2)
            errs.append(err)
            if verbose:
                if ii % (print_period * 10) == 0:
                    print("{:5s}|{:12s}".format("It.", "Err") + "\n" + "-" * 19)
                print("{:5d}|{:8e}|".format(ii, err))
        if err <= stopThr and ii > 35:
            stopped = True
            break
    if not stopped and warn:
        warnings.warn(NONCONV_MSG)
    P = _plan_from_logs(Md, logu, logv, regi)
    if log:
        alpha, beta = bd.out(ws[0]), bd.out(ws[1])
        lg = {"err": _errs_as(bd, np.asarray(errs), Md), "alpha": alpha, "beta": beta, "warmstart": (alpha, beta),
              "niter": ii}
        return bd.out(P), lg
    return bd.out(P)


def greenkhorn(a, b, M, reg, numItermax=10000, stopThr=1e-9, verbose=False, log=False, warn=True,
               warmstart=None):
    """GPU ``ot.bregman.greenkhorn`` (``_sinkhorn.py:921-1102``): greedy
    coordinate steps, each rescaling the row or column with the largest
    marginal violation, run as one chain in a single CTA
    (``otg_greenkhorn``).  Returns the plan; with ``log=True`` also a dict
    with ``n_iter`` (last step index), ``u`` and ``v``.  ``warmstart`` is the
    pair of log-scalings, as in the reference."""
    bd, Md, ad, bdv = _prep(a, b, M)
    if bdv.dim() > 1:
        raise ValueError("greenkhorn takes one target histogram (1-D b)")
    n, m = Md.shape
    wu, wv = _warm(bd, warmstart, Md.dtype, n, m)
    lib = _lib.load()
    code = _lib.dtype_code(Md.dtype)
    dev = Md.device
    u = torch.empty(n, dtype=Md.dtype, device=dev)
    v = torch.empty(m, dtype=Md.dtype, device=dev)
    P = torch.empty((n, m), dtype=Md.dtype, device=dev)
    info = torch.zeros(2, dtype=torch.int32, device=dev)
    ws = torch.empty(lib.otg_greenkhorn_workspace_bytes(code, n, m), dtype=torch.uint8, device=dev)
    steps = min(max(0, int(numItermax)), 2 ** 31 - 1)
    _lib.check(lib.otg_greenkhorn(code, _lib.ptr(Md), n, m, Md.stride(0), _lib.ptr(ad), _lib.ptr(bdv), float(reg),
                                  _lib.ptr(wu), _lib.ptr(wv), steps, float(stopThr), _lib.ptr(P), P.stride(0),
                                  _lib.ptr(u), _lib.ptr(v), _lib.ptr(info), _lib.ptr(ws), ws.numel(),
                                  _lib.stream_handle(dev)), "otg_greenkhorn")
    niter, status = (int(x) for x in info.tolist())
    if status == _lib.STATUS_MAXITER and warn:
        warnings.warn(NONCONV_MSG)
    if log:
        return bd.out(P), {"n_iter": niter, "u": bd.out(u), "v": bd.out(v)}
    return bd.out(P)


def sinkhorn(a, b, M, reg, method="sinkhorn", numItermax=1000, stopThr=1e-9, verbose=False,
             log=False, warn=True, warmstart=None, **kwargs):
    """GPU ``ot.sinkhorn``: dispatch on ``method`` (``_sinkhorn.py:164-234``)."""
    meth = method.lower()
    if meth == "sinkhorn":
        return sinkhorn_knopp(a, b, M, reg, numItermax=numItermax, stopThr=stopThr, verbose=verbose,
                              log=log, warn=warn, warmstart=warmstart, **kwargs)
    if meth == "sinkhorn_log":
        return sinkhorn_log(a, b, M, reg, numItermax=numItermax, stopThr=stopThr, verbose=verbose,
                            log=log, warn=warn, warmstart=warmstart, **kwargs)
    if meth == "sinkhorn_stabilized":
        return sinkhorn_stabilized(a, b, M, reg, numItermax=numItermax, stopThr=stopThr, warmstart=warmstart,
                                   verbose=verbose, log=log, warn=warn, **kwargs)
    if meth == "sinkhorn_epsilon_scaling":
        return sinkhorn_epsilon_scaling(a, b, M, reg, numItermax=numItermax, stopThr=stopThr,
                                        warmstart=warmstart, verbose=verbose, log=log, warn=warn, **kwargs)
    if meth == "greenkhorn":
        return greenkhorn(a, b, M, reg, numItermax=numItermax, stopThr=stopThr, verbose=verbose, log=log,
                          warn=warn, warmstart=warmstart)
    raise ValueError("Unknown method '%s'." % method)


def sinkhorn2(a, b, M, reg, method="sinkhorn", numItermax=1000, stopThr=1e-9, verbose=False,
              log=False, warn=False, warmstart=None, **kwargs):
    """GPU ``ot.sinkhorn2``: the loss ``<P, M>`` (fp64 accumulation) for 1-D
    ``b``; the per-histogram losses for 2-D ``b`` (``_sinkhorn.py:435-484``).
    For torch inputs that require gradients (1-D ``b``, methods 'sinkhorn' and
    'sinkhorn_log') the loss carries the gradients the reference's autodiff
    through its iterations converges to, by implicit differentiation at the
    solution (``_autograd.implicit_grads``)."""
    meth = method.lower()
    if meth == "sinkhorn_stabilized":
        bd, Md, ad, bdv = _prep(a, b, M)
        if bdv.dim() > 1:
            raise NotImplementedError("pot_gb300 sinkhorn_stabilized: several target histograms are not on "
                                      "the GPU path")
        kw = {k: kwargs[k] for k in ("tau", "print_period") if k in kwargs}
        r, logu, logv, lg = _stabilized(bd, ad, bdv, Md, reg, numItermax, stopThr, warmstart, verbose, warn,
                                        log, **kw)
        rr = DenseResult()
        rr.u, rr.v = logu, logv
        out = bd.scalar(_loss(Md, rr, reg, _lib.OTG_METHOD_LOG))
        return (out, lg) if log else out
    if meth not in ("sinkhorn", "sinkhorn_log"):
        raise ValueError("Unknown method '%s'." % method)
    bd, Md, ad, bdv = _prep(a, b, M)
    code = _lib.OTG_METHOD_KNOPP if meth == "sinkhorn" else _lib.OTG_METHOD_LOG
    if bdv.dim() > 1:
        fn = sinkhorn_knopp if meth == "sinkhorn" else sinkhorn_log
        return fn(a, b, M, reg, numItermax=numItermax, stopThr=stopThr, verbose=verbose, log=log,
                  warn=warn, warmstart=warmstart)
    need_grad = any(isinstance(x, torch.Tensor) and x.requires_grad for x in (a, b, M))
    r, P = _run_single(bd, ad, bdv, Md, reg, code, numItermax, stopThr, verbose, warn, warmstart,
                       need_grad)
    loss = _loss(Md, r, reg, code)
    if need_grad:
        # the reference's autodiff through its iterations, taken at the
        # solution by implicit differentiation
        from ._autograd import implicit_loss
        loss = implicit_loss(loss, P, Md, ad, bdv, float(reg), a, b, M)
    out = bd.scalar(loss)
    if log:
        if code == _lib.OTG_METHOD_KNOPP:
            lg = {"err": _errs_as(bd, r.errs, Md), "niter": r.niter, "u": bd.out(r.u), "v": bd.out(r.v)}
        else:
            lg = {"err": _errs_as(bd, r.errs, Md), "niter": r.niter, "log_u": bd.out(r.u),
                  "log_v": bd.out(r.v), "u": bd.out(torch.exp(r.u)), "v": bd.out(torch.exp(r.v))}
        return out, lg
    return out
