"""GPU entropic Gromov-Wasserstein: drop-ins for
``ot.gromov.entropic_gromov_wasserstein`` / ``entropic_gromov_wasserstein2``
(PythonOT/POT ``ot/gromov/_bregman.py:25-253``, ``:256-400``) and the fused
variants ``entropic_fused_gromov_wasserstein`` / ``...2`` (``:997-1241``,
``:1244-1403``) with the square loss, plus the log-domain inner-solver
variant used for large problems.

Per outer iteration: the gradient ``2 (constC - C1 T (2 C2)^T)`` comes from
two GEMMs (``csrc/gw.cu``: tcgen05 tensor cores with a high/low half split
for float32 inputs; an fp64 CUDA-core GEMM for float64 inputs) whose last
epilogue writes the inner solver's cost directly; the inner Sinkhorn is the
dense persistent kernel.  Outer-loop semantics follow the reference: the
inner solve is the scaling-form Sinkhorn (``method='sinkhorn'``), the
warm start carries ``epsilon * log(u)`` as the next log-scaling (the
reference's own convention), ``||T - Tprev||_F`` is logged every 10th
iteration, and a mass check warns at the end.
"""
import ctypes
import warnings

import torch

from . import _lib
from ._arrays import Boundary, check_shape, shape_of
from . import bregman


def _pad(x, q):
    return (x + q - 1) // q * q


def pow2_scale(bound, target_log2=14):
    """Power of two that brings values bounded by `bound` to at most
    2^target_log2: high parts then sit in the normal half-precision range
    (max 65504) and low parts rarely underflow; the factor is undone exactly."""
    import math
    if not bound > 0 or not math.isfinite(bound):
        return 1.0
    return 2.0 ** (target_log2 - math.ceil(math.log2(bound)))


class _Planes:
    """High/low half planes of an operand, zero-padded to whole 128 tiles."""

    def __init__(self, rows, cols, device):
        self.rows, self.cols = _pad(rows, 128), _pad(cols, 128)
        self.hi = torch.zeros(self.rows, self.cols, dtype=torch.float16, device=device)
        self.lo = torch.zeros_like(self.hi)

    def fill(self, X, scale=1.0, transpose=False):
        lib = _lib.load()
        r, c = X.shape
        _lib.check(lib.otg_split_half(_lib.ptr(X), r, c, X.stride(0), float(scale), int(transpose),
                                      _lib.ptr(self.hi), _lib.ptr(self.lo), self.cols,
                                      _lib.stream_handle(X.device)), "otg_split_half")
        return self


class TensorProduct:
    """``G(T) = 2 constC - 2 C1 T hC2^T`` with hC2 = 2 C2 (square loss),
    i.e. gwggrad (``ot/gromov/_utils.py:323``); float32 inputs on the
    tensor cores, float64 on the fp64 GEMM."""

    def __init__(self, C1, C2, p, q):
        self.dtype, self.device = C1.dtype, C1.device
        self.n, self.m = C1.shape[0], C2.shape[0]
        # constC_ij = alpha_i + beta_j, alpha = C1^2 p, beta = C2^2 q  (_utils.py:233-239)
        self.alpha = ((C1 * C1) @ p).contiguous()
        self.beta = ((C2 * C2) @ q).contiguous()
        self.C1, self.hC2 = C1.contiguous(), (2.0 * C2).contiguous()
        self.lib = _lib.load()
        if self.dtype == torch.float32:
            n, m = self.n, self.m
            # exact power-of-two prescales: C1, hC2 from their maxima, T from
            # T_ij <= min(max p, max q), the product C1 T from sum_l T_lk = q_k
            c1max = float(self.C1.abs().max())
            self.s1 = pow2_scale(c1max)
            self.s2 = pow2_scale(float(self.hC2.abs().max()))
            tmax = min(float(p.max()), float(q.max()))
            self.sT = pow2_scale(tmax)
            self.e1 = pow2_scale(self.s1 * c1max * float(q.max()) * self.sT)
            self.A1 = _Planes(n, n, self.device).fill(self.C1, self.s1)
            self.B2 = _Planes(m, m, self.device).fill(self.hC2, self.s2)
            self.Tt = _Planes(m, n, self.device)
            self.P1 = _Planes(n, m, self.device)
            self.flag = torch.zeros(1, dtype=torch.int32, device=self.device)

    def grad(self, T, out=None, w=1.0, addend=None, s_add=0.0):
        """``w * 2 (constC - C1 T hC2^T) [+ s_add * addend]`` as an (n, m)
        tensor of the input dtype (``addend`` may be ``out``)."""
        n, m = self.n, self.m
        st = _lib.stream_handle(self.device)
        if out is None:
            out = torch.empty(n, m, dtype=self.dtype, device=self.device)
        if self.dtype == torch.float64:
            A1 = torch.empty(n, m, dtype=torch.float64, device=self.device)
            _lib.check(self.lib.otg_gemm_f64(0, 0, n, m, n, 1.0, _lib.ptr(self.C1), n, _lib.ptr(T), T.stride(0),
                                             0.0, _lib.ptr(A1), m, st), "otg_gemm_f64")
            base = (2.0 * w) * (self.alpha[:, None] + self.beta[None, :])
            if addend is not None:
                base = base + s_add * addend
            out.copy_(base)
            _lib.check(self.lib.otg_gemm_f64(0, 1, n, m, m, -2.0 * w, _lib.ptr(A1), m, _lib.ptr(self.hC2), m, 1.0,
                                             _lib.ptr(out), m, st), "otg_gemm_f64")
            return out
        Tc = T.contiguous()
        self.Tt.fill(Tc, self.sT, transpose=True)
        g1 = _lib.OtgSplitGemm(a_hi=_lib.ptr(self.A1.hi), a_lo=_lib.ptr(self.A1.lo), a_rows=self.A1.rows,
                               lda=self.A1.cols, b_hi=_lib.ptr(self.Tt.hi), b_lo=_lib.ptr(self.Tt.lo),
                               b_rows=self.Tt.rows, ldb=self.Tt.cols, k_alloc=self.A1.cols, mode=0, scale=self.e1,
                               s_acc=0.0, s_vec=0.0, out_hi=_lib.ptr(self.P1.hi), out_lo=_lib.ptr(self.P1.lo),
                               ld_h=self.P1.cols, out=None, ld_o=0, M=n, N=m, rowv=None, colv=None,
                               abort_flag=_lib.ptr(self.flag), timeout_ms=0)
        _lib.check(self.lib.otg_gemm_split3(ctypes.byref(g1), st), "otg_gemm_split3")
        g2 = _lib.OtgSplitGemm(a_hi=_lib.ptr(self.P1.hi), a_lo=_lib.ptr(self.P1.lo), a_rows=self.P1.rows,
                               lda=self.P1.cols, b_hi=_lib.ptr(self.B2.hi), b_lo=_lib.ptr(self.B2.lo),
                               b_rows=self.B2.rows, ldb=self.B2.cols, k_alloc=self.P1.cols, mode=1, scale=1.0,
                               s_acc=-2.0 * w / (self.s1 * self.sT * self.e1 * self.s2), s_vec=2.0 * w, out_hi=None,
                               out_lo=None, ld_h=0, out=_lib.ptr(out),
                               ld_o=out.stride(0), M=n, N=m, rowv=_lib.ptr(self.alpha), colv=_lib.ptr(self.beta),
                               abort_flag=_lib.ptr(self.flag), timeout_ms=0,
                               addend=_lib.ptr(addend) if addend is not None else None,
                               ld_add=addend.stride(0) if addend is not None else 0, s_add=float(s_add))
        _lib.check(self.lib.otg_gemm_split3(ctypes.byref(g2), st), "otg_gemm_split3")
        return out

    def check_abort(self):
        if self.dtype == torch.float32 and int(self.flag.item()) != 0:
            raise RuntimeError("pot_gb300: a device-side wait of the tensor-core GEMM timed out")


def _check_gw_shapes(C1, C2, p, q, G0=None, Mf=None):
    """Structure matrices square, marginals and (n, m) inputs of matching
    sizes, checked on the caller's arrays before any device work."""
    s1, s2 = shape_of(C1), shape_of(C2)
    if len(s1) != 2 or s1[0] != s1[1] or len(s2) != 2 or s2[0] != s2[1]:
        raise ValueError("C1 and C2 must be square matrices, got %s and %s" % (s1, s2))
    n, m = s1[0], s2[0]
    check_shape("p", p, [(n,)])
    check_shape("q", q, [(m,)])
    check_shape("G0", G0, [(n, m)])
    check_shape("M", Mf, [(n, m)])


def _validate(loss_fun, solver):
    if solver not in ["PGD", "PPA"]:
        raise ValueError("Unknown solver '%s'. Pick one in ['PGD', 'PPA']." % solver)
    if loss_fun not in ("square_loss", "kl_loss"):
        raise ValueError(f"Unknown `loss_fun='{loss_fun}'`. Use one of: {'square_loss', 'kl_loss'}.")
    if loss_fun == "kl_loss":
        raise NotImplementedError("pot_gb300: entropic GW implements loss_fun='square_loss' on the GPU path")


def entropic_gromov_wasserstein(C1, C2, p=None, q=None, loss_fun="square_loss", epsilon=0.1, symmetric=None,
                                G0=None, max_iter=1000, tol=1e-9, solver="PGD", warmstart=False, verbose=False,
                                log=False, **kwargs):
    """GPU ``ot.gromov.entropic_gromov_wasserstein`` (square loss)."""
    T, lg = _entropic_gw(None, C1, C2, p, q, loss_fun, epsilon, symmetric, 1.0, G0, max_iter, tol, solver,
                         warmstart, verbose, kwargs)
    if log:
        return T, {"err": lg["err"], "gw_dist": lg["dist"]}
    return T


def entropic_fused_gromov_wasserstein(M, C1, C2, p=None, q=None, loss_fun="square_loss", epsilon=0.1,
                                      symmetric=None, alpha=0.5, G0=None, max_iter=1000, tol=1e-9, solver="PGD",
                                      warmstart=False, verbose=False, log=False, **kwargs):
    """GPU ``ot.gromov.entropic_fused_gromov_wasserstein``
    (``ot/gromov/_bregman.py:997-1241``, square loss): the entropic GW loop
    with the inner cost ``alpha * gwggrad(T) + (1 - alpha) M``, the linear
    term added in the GEMM epilogue; ``log`` holds ``err`` and ``fgw_dist``."""
    T, lg = _entropic_gw(M, C1, C2, p, q, loss_fun, epsilon, symmetric, alpha, G0, max_iter, tol, solver,
                         warmstart, verbose, kwargs)
    if log:
        return T, {"err": lg["err"], "fgw_dist": lg["dist"]}
    return T


def entropic_fused_gromov_wasserstein2(M, C1, C2, p=None, q=None, loss_fun="square_loss", epsilon=0.1,
                                       symmetric=None, alpha=0.5, G0=None, max_iter=1000, tol=1e-9, solver="PGD",
                                       warmstart=False, verbose=False, log=False, **kwargs):
    """GPU ``ot.gromov.entropic_fused_gromov_wasserstein2``
    (``ot/gromov/_bregman.py:1244-1403``): the FGW loss; the log adds ``T``,
    ``quad_loss`` and ``lin_loss``."""
    T, lg = _entropic_gw(M, C1, C2, p, q, loss_fun, epsilon, symmetric, alpha, G0, max_iter, tol, solver,
                         warmstart, verbose, kwargs, keep_device=True)
    bd = lg["bd"]
    lin = lg["lin"]
    logv = {"err": lg["err"], "fgw_dist": lg["dist"], "T": bd.out(T),
            "quad_loss": bd.scalar(torch.tensor(lg["dist_f"] - (1 - alpha) * lin, dtype=T.dtype, device=T.device)),
            "lin_loss": bd.scalar(torch.tensor(lin * (1 - alpha), dtype=T.dtype, device=T.device))}
    if log:
        return logv["fgw_dist"], logv
    return logv["fgw_dist"]


def _entropic_gw(Mf, C1, C2, p, q, loss_fun, epsilon, symmetric, alpha, G0, max_iter, tol, solver, warmstart,
                 verbose, kwargs, keep_device=False):
    """Outer loop of ``ot/gromov/_bregman.py:150-253`` (GW) and
    ``:1140-1241`` (fused GW with ``Mf``): gradient by tensor-core GEMMs,
    scaling-form inner Sinkhorn, ``||T - Tprev||_F`` every 10th iteration."""
    _validate(loss_fun, solver)
    if "method" in kwargs:
        raise TypeError("sinkhorn() got multiple values for keyword argument 'method'")
    kwargs = dict(kwargs)
    _check_gw_shapes(C1, C2, p, q, G0, Mf)
    bd = Boundary(C1, C2, p, q, G0, Mf)
    C1d = bd.to_dev(C1)
    C2d = bd.to_dev(C2, C1d.dtype)
    dt, dev = C1d.dtype, C1d.device
    n, m = C1d.shape[0], C2d.shape[0]
    Mfd = None if Mf is None else bd.to_dev(Mf, dt).contiguous()
    pd = torch.full((n,), 1.0 / n, dtype=dt, device=dev) if p is None else bd.to_dev(p, dt)
    qd = torch.full((m,), 1.0 / m, dtype=dt, device=dev) if q is None else bd.to_dev(q, dt)
    T = torch.outer(pd, qd) if G0 is None else bd.to_dev(G0, dt).contiguous()
    if symmetric is None:
        symmetric = bool(torch.allclose(C1d, C1d.T, atol=1e-10) and torch.allclose(C2d, C2d.T, atol=1e-10))
    tp = TensorProduct(C1d, C2d, pd, qd)
    tpt = None if symmetric else TensorProduct(C1d.T.contiguous(), C2d.T.contiguous(), pd, qd)
    numItermax = kwargs.pop("numItermax", 1000)
    stopThr = kwargs.pop("stopThr", 1e-9)
    if warmstart:
        mu = torch.full((n,), -float(torch.log(torch.tensor(float(n)))), dtype=dt, device=dev)
        nu = torch.full((m,), -float(torch.log(torch.tensor(float(m)))), dtype=dt, device=dev)
    lin_w = 0.0 if Mfd is None else 1.0 - alpha
    cpt, err = 0, 1.0
    errs = []
    M = torch.empty(n, m, dtype=dt, device=dev)
    while err > tol and cpt < max_iter:
        Tprev = T
        if symmetric:
            tp.grad(T, M, w=alpha, addend=Mfd, s_add=lin_w)
        else:
            # alpha/2 (G(T) + G^t(T)) + (1 - alpha) Mf, the second GEMM adding onto the first
            tp.grad(T, M, w=0.5 * alpha, addend=Mfd, s_add=lin_w)
            tpt.grad(T, M, w=0.5 * alpha, addend=M, s_add=1.0)
        tens = M
        if solver == "PPA":
            tens = M - epsilon * torch.log(T)
        if warmstart:
            T, lg = bregman.sinkhorn_knopp(pd, qd, tens, epsilon, numItermax=numItermax, stopThr=stopThr, log=True,
                                           warmstart=(mu, nu), **kwargs)
            mu = epsilon * torch.log(lg["u"])
            nu = epsilon * torch.log(lg["v"])
        else:
            T = bregman.sinkhorn_knopp(pd, qd, tens, epsilon, numItermax=numItermax, stopThr=stopThr, **kwargs)
        if cpt % 10 == 0:
            err = float(torch.linalg.norm(T - Tprev))
            errs.append(err)
            if verbose:
                if cpt % 200 == 0:
                    print("{:5s}|{:12s}".format("It.", "Err") + "\n" + "-" * 19)
                print("{:5d}|{:8e}|".format(cpt, err))
        cpt += 1
    tp.check_abort()
    if abs(float(T.sum()) - 1) > 1e-5:
        warnings.warn("Solver failed to produce a transport plan. You might "
                      "want to increase the regularization parameter `epsilon`.")
    quad = 0.5 * float((tp.grad(T) * T).sum())
    lin = 0.0 if Mfd is None else float((Mfd * T).sum())
    dist = (1.0 - alpha) * lin + alpha * quad if Mfd is not None else quad
    out = {"err": [torch.tensor(e) for e in errs] if bd.kind == "torch" else errs,
           "dist": bd.scalar(torch.tensor(dist, dtype=dt, device=dev)), "dist_f": dist, "lin": lin, "bd": bd}
    return (T if keep_device else bd.out(T)), out


def entropic_gromov_wasserstein2(C1, C2, p=None, q=None, loss_fun="square_loss", epsilon=0.1, symmetric=None,
                                 G0=None, max_iter=1000, tol=1e-9, solver="PGD", warmstart=False, verbose=False,
                                 log=False, **kwargs):
    """GPU ``ot.gromov.entropic_gromov_wasserstein2``: the GW loss (and log
    with ``T``)."""
    T, logv = entropic_gromov_wasserstein(C1, C2, p, q, loss_fun, epsilon, symmetric, G0, max_iter, tol, solver,
                                          warmstart, verbose, log=True, **kwargs)
    logv["T"] = T
    if log:
        return logv["gw_dist"], logv
    return logv["gw_dist"]


def entropic_gromov_wasserstein_log(C1, C2, p=None, q=None, epsilon=5e-3, max_iter=50, tol=0.0,
                                    numItermax=100000, stopThr=1e-7, return_stats=False):
    """Entropic GW (square loss, PGD) with the log-domain inner solver warm
    started from the previous outer iteration's potentials: the same outer
    loop with ``sinkhorn_log`` inside.  Returns (T, log) with ``gw_dist``,
    ``err`` and the inner iteration counts."""
    _check_gw_shapes(C1, C2, p, q)
    bd = Boundary(C1, C2, p, q)
    C1d = bd.to_dev(C1)
    C2d = bd.to_dev(C2, C1d.dtype)
    dt, dev = C1d.dtype, C1d.device
    n, m = C1d.shape[0], C2d.shape[0]
    pd = torch.full((n,), 1.0 / n, dtype=dt, device=dev) if p is None else bd.to_dev(p, dt)
    qd = torch.full((m,), 1.0 / m, dtype=dt, device=dev) if q is None else bd.to_dev(q, dt)
    T = torch.outer(pd, qd)
    tp = TensorProduct(C1d, C2d, pd, qd)
    M = torch.empty(n, m, dtype=dt, device=dev)
    wu = wv = None
    cpt, err, errs, inner = 0, 1.0, [], []
    lib = _lib.load()
    while err > tol and cpt < max_iter:
        Tprev = T
        tp.grad(T, M)
        r = bregman.solve_dense(M, pd, qd, epsilon, _lib.OTG_METHOD_LOG, numItermax, stopThr, wu, wv)
        wu, wv = r.u, r.v
        inner.append(r.niter)
        T = torch.empty_like(M)
        _lib.check(lib.otg_dense_plan(_lib.dtype_code(dt), _lib.OTG_METHOD_LOG, _lib.ptr(M), n, m, m, _lib.ptr(r.u),
                                      _lib.ptr(r.v), float(epsilon), _lib.ptr(T), m, None,
                                      _lib.stream_handle(dev)), "otg_dense_plan")
        if cpt % 10 == 0:
            err = float(torch.linalg.norm(T - Tprev))
            errs.append(err)
        cpt += 1
    tp.check_abort()
    gw = 0.5 * float((tp.grad(T) * T).sum())
    return bd.out(T), {"gw_dist": gw, "err": errs, "inner_niter": inner, "log_u": bd.out(wu), "log_v": bd.out(wv)}
