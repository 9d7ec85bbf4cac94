"""Accelerated log-domain Sinkhorn iterations (TEST INFRASTRUCTURE ONLY).

No reference counterpart: these restate, in float64 numpy, the iterations the
GPU batch solver runs for the warm-start refinement, so that they can be
checked step for step.  Both keep the reference's stop test (the column
marginal of the iterate pair in L2, ``ot/bregman/_sinkhorn.py:884-899``) and,
with the acceleration switched off, are ``sinkhorn_log`` (``:880-899``).

- ``sinkhorn_log_relaxed``: over-relaxed updates ``v <- v + omega (v_new - v)``
  (from the second iteration on; the first v comes from u alone) and
  ``u <- u + omega (u_new - u)``, the stop test every ``check_period``
  iterations -- the iteration of ``otg_sinkhorn_multi`` with ``omega`` and
  ``check_period``.
- ``sinkhorn_log_anderson``: Anderson mixing (type II, window ``depth``) of
  the map ``G(u) = rowT(colT(u))``: ``u <- sum_k alpha_k G(u_k)`` over the last
  ``depth`` iterates, ``alpha`` minimising ``|sum_k alpha_k (G(u_k) - u_k)|``
  with ``sum alpha = 1`` (normal equations with a Tikhonov term
  ``lam * trace / depth``).  The stop test measures the pair (mixed u, last
  v), which is what the next column pass sees.
- ``sinkhorn_log_anderson_v``: the iteration of ``otg_sinkhorn_multi`` with
  ``anderson_depth``: Anderson mixing of the map ``F(v) = colT(rowT(v))``
  with ``u`` always the exact row update of the mixed ``v`` (so the stop
  test is the plain one on a pair with an exact row marginal), history in
  ``depth`` slots filled round-robin, the weights from the slot-ordered Gram
  matrix by Gaussian elimination with partial pivoting, a restart with the
  plain step when the solve fails or ``sum |alpha|`` exceeds 1e4.
"""
import numpy as np

from .entropic import _f64, _uniform_if_empty, logsumexp


def _setup(a, b, M, reg):
    M = _f64(M)
    a, b = _uniform_if_empty(a, b, M)
    with np.errstate(divide="ignore"):
        return -M / reg, np.log(a), np.log(b), b


def _col_err(Mr, u, v, b):
    return float(np.linalg.norm(np.sum(np.exp(Mr + u[:, None] + v[None, :]), 0) - b))


def sinkhorn_log_relaxed(a, b, M, reg, omega=1.0, numItermax=1000, stopThr=1e-9, warm_u=None, check_period=10):
    """Over-relaxed log-domain Sinkhorn; returns (log_u, log_v, niter, errs)
    with niter the last loop index (the reference's convention)."""
    Mr, la, lb, b = _setup(a, b, M, reg)
    u = np.zeros(Mr.shape[0]) if warm_u is None else _f64(warm_u).copy()
    v = None
    errs = []
    ii = 0
    for ii in range(numItermax):
        vn = lb - logsumexp(Mr + u[:, None], 0)
        v = vn if v is None else v + omega * (vn - v)
        un = la - logsumexp(Mr + v[None, :], 1)
        u = u + omega * (un - u)
        if ii % check_period == 0:
            errs.append(_col_err(Mr, u, v, b))
            if errs[-1] < stopThr:
                break
    return u, v, ii, errs


def sinkhorn_log_anderson(a, b, M, reg, depth=5, numItermax=1000, stopThr=1e-9, warm_u=None, lam=1e-10):
    """Anderson-accelerated log-domain Sinkhorn, stop test every iteration;
    returns (log_u, log_v, niter, errs) for the pair that met the test."""
    Mr, la, lb, b = _setup(a, b, M, reg)
    u = np.zeros(Mr.shape[0]) if warm_u is None else _f64(warm_u).copy()
    us, gs = [], []
    errs = []
    v = None
    ii = 0
    for ii in range(numItermax):
        L = logsumexp(Mr + u[:, None], 0)
        if v is not None:
            # column marginal of (u, v): the pair the last mixing produced
            errs.append(float(np.linalg.norm(np.exp(v + L) - b)))
            if errs[-1] < stopThr:
                return u, v, ii - 1, errs
        v = lb - L
        g = la - logsumexp(Mr + v[None, :], 1)
        us.append(u)
        gs.append(g)
        if len(us) > depth:
            us.pop(0)
            gs.pop(0)
        R = np.stack([gk - uk for uk, gk in zip(us, gs)], 1)
        k = R.shape[1]
        if k == 1:
            u = g
            continue
        A = R.T @ R
        A = A + lam * (np.trace(A) / k) * np.eye(k)
        w = np.linalg.solve(A, np.ones(k))
        u = np.stack(gs, 1) @ (w / w.sum())
    return u, v, ii, errs


AND_LAMBDA = 1e-10
AND_MAX_L1 = 1e4


def _anderson_weights(G, nh, s):
    """Mixing weights of the slot-ordered history (None: restart)."""
    if nh < 2:
        return None
    tr = float(np.trace(G[:nh, :nh]))
    if not tr > 0.0:
        return None
    A = G[:nh, :nh] + AND_LAMBDA * tr / nh * np.eye(nh)
    Mx = np.concatenate([A, np.ones((nh, 1))], 1)
    for c in range(nh):
        piv = c + int(np.argmax(np.abs(Mx[c:, c])))
        if not abs(Mx[piv, c]) > 0.0:
            return None
        Mx[[c, piv]] = Mx[[piv, c]]
        for i in range(c + 1, nh):
            Mx[i, c:] -= Mx[i, c] / Mx[c, c] * Mx[c, c:]
    w = np.zeros(nh)
    for i in range(nh - 1, -1, -1):
        w[i] = (Mx[i, nh] - Mx[i, i + 1:nh] @ w[i + 1:nh]) / Mx[i, i]
    w = w / w.sum()
    l1 = float(np.abs(w).sum())
    if not (np.isfinite(l1) and l1 < AND_MAX_L1):
        return None
    return w


def sinkhorn_log_anderson_v(a, b, M, reg, depth=5, numItermax=1000, stopThr=1e-9, warm_u=None, check_period=1):
    """Anderson-mixed log-domain Sinkhorn on v (``otg_sinkhorn_multi`` with
    ``anderson_depth``); returns (log_u, log_v, niter, errs) with niter the
    last loop index and (log_u, log_v) the pair that met the test."""
    Mr, la, lb, b = _setup(a, b, M, reg)
    m = Mr.shape[1]
    u = np.zeros(Mr.shape[0]) if warm_u is None else _f64(warm_u).copy()
    F = np.zeros((depth, m))
    R = np.zeros((depth, m))
    G = np.zeros((depth, depth))
    cnt = 0
    v = None
    errs = []
    prev_check = False
    for ii in range(numItermax + 1):
        L = logsumexp(Mr + u[:, None], 0)
        if prev_check:
            errs.append(float(np.linalg.norm(np.exp(v + L) - b)))
            if errs[-1] < stopThr:
                return u, v, ii - 1, errs
        if ii == numItermax:
            break
        f = lb - L
        if v is None:
            vn = f
        else:
            s = cnt % depth
            nh = min(cnt + 1, depth)
            F[s] = f
            R[s] = f - v
            for q in range(nh):
                G[s, q] = G[q, s] = float(R[s] @ R[q])
            w = _anderson_weights(G, nh, s)
            if w is None:
                vn = f
                cnt = cnt + 1 if nh == 1 else 0
            else:
                vn = w @ F[:nh]
                cnt += 1
        v = vn
        u = la - logsumexp(Mr + v[None, :], 1)
        prev_check = ii % check_period == 0
    return u, v, numItermax - 1, errs
