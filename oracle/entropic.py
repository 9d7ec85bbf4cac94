"""Float64 numpy restatement of the reference's entropic-OT algorithms.

TEST INFRASTRUCTURE ONLY: the checker that the CUDA path is compared with.
Product code never imports this module.

Each function names the reference lines (PythonOT/POT 0.9.7.dev0) whose
behaviour it restates: iteration order, the every-10th-iteration stopping
test, the error norm, the returned log keys and the warning events.  Warnings
are not raised here; they are recorded in ``log["_warnings"]`` so that tests
can compare them with the GPU path's warnings.
"""
import numpy as np

NONCONV = "Sinkhorn did not converge"
NUMERR = "numerical errors at iteration"
NUMERR_STAB = "Numerical errors at iteration %d"


def _f64(x):
    return np.asarray(x, dtype=np.float64)


def sqeuclidean(X, Y=None):
    """Squared Euclidean cost, ``ot/utils.py:270-305`` (``euclidean_distances``,
    squared=True): ``|x|^2 + |y|^2 - 2 x.y``, clamped at 0, zero diagonal when
    ``Y`` is ``X``."""
    same = Y is None or Y is X
    X = _f64(X)
    Y = X if same else _f64(Y)
    c = -2.0 * (X @ Y.T)
    c += np.einsum("ij,ij->i", X, X)[:, None]
    c += np.einsum("ij,ij->i", Y, Y)[None, :]
    c = np.maximum(c, 0.0)
    if same:
        np.fill_diagonal(c, 0.0)
    return c


def logsumexp(x, axis):
    """Max-shifted log-sum-exp with the conventions of
    ``scipy.special.logsumexp`` (what ``NumpyBackend.logsumexp``,
    ``ot/backend.py:1306``, calls): an all ``-inf`` slice gives ``-inf``."""
    mx = np.max(x, axis=axis, keepdims=True)
    shift = np.where(np.isfinite(mx), mx, 0.0)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        s = np.sum(np.exp(x - shift), axis=axis, keepdims=True)
        out = np.log(s) + shift
    return np.squeeze(out, axis=axis)


def _uniform_if_empty(a, b, M):
    """Empty weight lists mean uniform, ``ot/bregman/_sinkhorn.py:592-595``."""
    a = _f64(a)
    b = _f64(b)
    if a.size == 0:
        a = np.full(M.shape[0], 1.0 / M.shape[0])
    if b.size == 0:
        b = np.full(M.shape[1], 1.0 / M.shape[1])
    return a, b


def sinkhorn_knopp(a, b, M, reg, numItermax=1000, stopThr=1e-9, warmstart=None):
    """Scaling-form Sinkhorn, ``ot/bregman/_sinkhorn.py:487-687``.

    Per iteration: ``v = b / (K^T u)``, ``u = 1 / ((1/a) K v)`` (``:629-631``);
    zero / NaN / Inf in the new scalings reverts to the previous pair and
    stops (``:633-645``); every 10th iteration the column-marginal L2
    violation is logged and compared with ``stopThr`` (``:646-658``).
    Returns ``(plan, log)`` for 1-D ``b`` and ``(losses, log)`` for 2-D ``b``
    (``:676-687``).  ``log["niter"]`` is the last loop index.
    """
    M = _f64(M)
    a, b = _uniform_if_empty(a, b, M)
    n, m = M.shape
    n_hists = b.shape[1] if b.ndim > 1 else 0
    warns = []
    if warmstart is None:
        if n_hists:
            u = np.ones((n, n_hists)) / n
            v = np.ones((m, n_hists)) / m
        else:
            u = np.ones(n) / n
            v = np.ones(m) / m
    else:
        u, v = np.exp(_f64(warmstart[0])), np.exp(_f64(warmstart[1]))
    with np.errstate(all="ignore"):
        K = np.exp(M / (-reg))
        Kp = (1.0 / a).reshape(-1, 1) * K
    errs = []
    ii = 0
    converged_or_broke = False
    with np.errstate(all="ignore"):
        for ii in range(numItermax):
            uprev, vprev = u, v
            Ktu = K.T @ u
            v = b / Ktu
            u = 1.0 / (Kp @ v)
            if (np.any(Ktu == 0) or np.any(np.isnan(u)) or np.any(np.isnan(v))
                    or np.any(np.isinf(u)) or np.any(np.isinf(v))):
                warns.append("Warning: %s %d" % (NUMERR, ii))
                u, v = uprev, vprev
                converged_or_broke = True
                break
            if ii % 10 == 0:
                if n_hists:
                    col = np.einsum("ik,ij,jk->jk", u, K, v)
                else:
                    col = np.einsum("i,ij,j->j", u, K, v)
                err = float(np.linalg.norm(col - b))
                errs.append(err)
                if err < stopThr:
                    converged_or_broke = True
                    break
    if not converged_or_broke:
        warns.append(NONCONV)
    log = {"err": errs, "niter": ii, "u": u, "v": v, "_warnings": warns}
    with np.errstate(all="ignore"):
        if n_hists:
            return np.einsum("ik,ij,jk,ij->k", u, K, v, M), log
        return u.reshape(-1, 1) * K * v.reshape(1, -1), log


def sinkhorn_log(a, b, M, reg, numItermax=1000, stopThr=1e-9, warmstart=None):
    """Log-domain Sinkhorn, ``ot/bregman/_sinkhorn.py:690-918``.

    Per iteration ``v = log b - LSE_i(-M/reg + u)`` then
    ``u = log a - LSE_j(-M/reg + v)`` (``:881-882``); every 10th iteration the
    column marginal of ``exp(-M/reg + u + v)`` is compared with ``b`` in L2
    (``:884-899``).  2-D ``b`` recurses per histogram and returns the per
    histogram losses with a log holding only the potentials (``:819-854``).
    """
    M = _f64(M)
    a, b = _uniform_if_empty(a, b, M)
    n_hists = b.shape[1] if b.ndim > 1 else 0
    if n_hists:
        ws = warmstart if warmstart is not None else [None] * n_hists
        losses, lus, lvs, warns = [], [], [], []
        for k in range(n_hists):
            P, lg = sinkhorn_log(a, b[:, k], M, reg, numItermax, stopThr, ws[k])
            losses.append(float(np.sum(M * P)))
            lus.append(lg["log_u"])
            lvs.append(lg["log_v"])
            warns += lg["_warnings"]
        log_u = np.stack(lus, 1)
        log_v = np.stack(lvs, 1)
        return np.array(losses), {"log_u": log_u, "log_v": log_v,
                                  "u": np.exp(log_u), "v": np.exp(log_v),
                                  "_warnings": warns}
    Mr = -M / reg
    if warmstart is None:
        u = np.zeros(M.shape[0])
        v = np.zeros(M.shape[1])
    else:
        u, v = _f64(warmstart[0]).copy(), _f64(warmstart[1]).copy()
    with np.errstate(divide="ignore"):
        loga, logb = np.log(a), np.log(b)
    errs = []
    ii = 0
    stopped = False
    with np.errstate(all="ignore"):
        for ii in range(numItermax):
            v = logb - logsumexp(Mr + u[:, None], 0)
            u = loga - logsumexp(Mr + v[None, :], 1)
            if ii % 10 == 0:
                col = np.sum(np.exp(Mr + u[:, None] + v[None, :]), 0)
                err = float(np.linalg.norm(col - b))
                errs.append(err)
                if err < stopThr:
                    stopped = True
                    break
        P = np.exp(Mr + u[:, None] + v[None, :])
    warns = [] if stopped else [NONCONV]
    return P, {"err": errs, "niter": ii, "log_u": u, "log_v": v,
               "u": np.exp(u), "v": np.exp(v), "_warnings": warns}


def greenkhorn(a, b, M, reg, numItermax=10000, stopThr=1e-9, warmstart=None):
    """Greedy coordinate Sinkhorn, ``ot/bregman/_sinkhorn.py:1034-1102``.

    K = exp(-M / reg); u, v start at 1/n, 1/m (or exp of the warm start);
    each step picks the row and the column whose marginal violation is the
    largest in absolute value (first index on ties), rescales the row when
    its violation is strictly larger, else the column, updates both
    violation vectors incrementally, and stops after the step whose chosen
    maximum is <= stopThr.  Returns (plan, log) with log keys n_iter, u, v."""
    M = _f64(M)
    a, b = _uniform_if_empty(a, b, M)
    K = np.exp(-M / reg)
    if warmstart is None:
        u = np.full(M.shape[0], 1.0 / M.shape[0])
        v = np.full(M.shape[1], 1.0 / M.shape[1])
    else:
        u, v = np.exp(_f64(warmstart[0])), np.exp(_f64(warmstart[1]))
    G = u[:, None] * K * v[None, :]
    viol = G.sum(1) - a
    viol_2 = G.sum(0) - b
    warns = []
    ii = -1
    for ii in range(numItermax):
        i_1 = int(np.argmax(np.abs(viol)))
        i_2 = int(np.argmax(np.abs(viol_2)))
        m_viol_1 = abs(viol[i_1])
        m_viol_2 = abs(viol_2[i_2])
        stop_val = np.maximum(m_viol_1, m_viol_2)
        if m_viol_1 > m_viol_2:
            old_u = u[i_1]
            new_u = a[i_1] / np.dot(K[i_1, :], v)
            G[i_1, :] = new_u * K[i_1, :] * v
            viol[i_1] = np.dot(new_u * K[i_1, :], v) - a[i_1]
            viol_2 += K[i_1, :] * (new_u - old_u) * v
            u[i_1] = new_u
        else:
            old_v = v[i_2]
            dot = np.dot(K[:, i_2], u)
            new_v = b[i_2] / dot
            G[:, i_2] = u * K[:, i_2] * new_v
            viol += (-old_v + new_v) * K[:, i_2] * u
            viol_2[i_2] = new_v * dot - b[i_2]
            v[i_2] = new_v
        if stop_val <= stopThr:
            break
    else:
        warns.append(NONCONV)
    return G, {"n_iter": ii, "u": u, "v": v, "_warnings": warns}


def sinkhorn(a, b, M, reg, method="sinkhorn", **kw):
    """Method dispatch of ``ot/bregman/_sinkhorn.py:164-234``."""
    if method.lower() == "sinkhorn":
        return sinkhorn_knopp(a, b, M, reg, **kw)
    if method.lower() == "sinkhorn_log":
        return sinkhorn_log(a, b, M, reg, **kw)
    if method.lower() == "greenkhorn":
        kw.setdefault("numItermax", 1000)  # the dispatcher's default, not greenkhorn's
        return greenkhorn(a, b, M, reg, **kw)
    if method.lower() == "sinkhorn_stabilized":
        return sinkhorn_stabilized(a, b, M, reg, **kw)
    if method.lower() == "sinkhorn_epsilon_scaling":
        return sinkhorn_epsilon_scaling(a, b, M, reg, **kw)
    raise ValueError("Unknown method '%s'." % method)


def sinkhorn2(a, b, M, reg, method="sinkhorn", **kw):
    """Loss ``sum(M * plan)`` for 1-D ``b`` (``_sinkhorn.py:435-438``); the
    solver's per-histogram losses for 2-D ``b`` (``:440-484``)."""
    res, log = sinkhorn(a, b, M, reg, method=method, **kw)
    if _f64(b).ndim < 2:
        return float(np.sum(_f64(M) * res)), log
    return res, log


def sinkhorn_stabilized(a, b, M, reg, numItermax=1000, tau=1e3, stopThr=1e-9, warmstart=None,
                        print_period=20):
    """Log-stabilised scaling Sinkhorn, ``ot/bregman/_sinkhorn.py:1105-1368``
    (1-D ``b``).

    Scalings start at ``u = 1/n, v = 1/m`` (``:1250-1256``) over the absorbed
    potentials ``alpha, beta`` (zero or the warm start); per iteration
    ``v = b / K^T u`` then ``u = a / K v`` (``:1277-1279``) with
    ``K = exp(-(M - alpha - beta)/reg)``; when ``max |u|`` or ``max |v|``
    exceeds ``tau`` the scalings are absorbed (``alpha += reg log u``, ...)
    and reset to ``1/n, 1/m`` (``:1282-1296``); every ``print_period``
    iterations the L2 column-marginal violation of the current plan is
    recorded (``:1298-1310``) and the loop stops once it is ``<= stopThr``
    (``:1318``); a NaN scaling reverts to the previous pair (``:1321-1327``).
    """
    M = _f64(M)
    a, b = _uniform_if_empty(a, b, M)
    if b.ndim > 1:
        raise NotImplementedError("several target histograms")
    n, m = M.shape
    if warmstart is None:
        alpha, beta = np.zeros(n), np.zeros(m)
    else:
        alpha, beta = _f64(warmstart[0]).copy(), _f64(warmstart[1]).copy()
    u, v = np.full(n, 1.0 / n), np.full(m, 1.0 / m)

    def kernel(al, be):
        return np.exp(-(M - al[:, None] - be[None, :]) / reg)

    def gamma(al, be, uu, vv):
        return np.exp(-(M - al[:, None] - be[None, :]) / reg + np.log(uu)[:, None] + np.log(vv)[None, :])

    K = kernel(alpha, beta)
    errs, warns = [], []
    err = 1.0
    ii = 0
    stopped = False
    with np.errstate(all="ignore"):
        for ii in range(numItermax):
            uprev, vprev = u, v
            v = b / (K.T @ u)
            u = a / (K @ v)
            if np.max(np.abs(u)) > tau or np.max(np.abs(v)) > tau:
                alpha, beta = alpha + reg * np.log(u), beta + reg * np.log(v)
                u, v = np.full(n, 1.0 / n), np.full(m, 1.0 / m)
                K = kernel(alpha, beta)
            if ii % print_period == 0:
                err = float(np.linalg.norm(np.sum(gamma(alpha, beta, u, v), 0) - b))
                errs.append(err)
            if err <= stopThr:
                stopped = True
                break
            if np.any(np.isnan(u)) or np.any(np.isnan(v)):
                warns.append(NUMERR_STAB % ii)
                u, v = uprev, vprev
                stopped = True
                break
        P = gamma(alpha, beta, u, v)
        logu = alpha / reg + np.log(u)
        logv = beta / reg + np.log(v)
    if not stopped:
        warns.append(NONCONV)
    al, be = alpha + reg * np.log(u), beta + reg * np.log(v)
    return P, {"err": errs, "n_iter": ii, "logu": logu, "logv": logv, "alpha": al, "beta": be,
               "warmstart": (al, be), "_warnings": warns}


def sinkhorn_epsilon_scaling(a, b, M, reg, numItermax=100, epsilon0=1e4, numInnerItermax=100, tau=1e3,
                             stopThr=1e-9, warmstart=None, print_period=10):
    """Epsilon scaling over the stabilised solver,
    ``ot/bregman/_sinkhorn.py:1371-1575``: at least 35 outer steps
    (``:1495-1496``), ``reg_k = (epsilon0 - reg) exp(-k) + reg``, each a
    stabilised solve of ``numInnerItermax`` iterations warm-started from the
    previous ``(alpha, beta)`` (whose own non-convergence warnings are kept);
    every ``print_period`` steps ``|G^T 1 - b|^2 + |G 1 - a|^2`` is recorded
    and the loop stops once it is ``<= stopThr`` after step 35."""
    M = _f64(M)
    a, b = _uniform_if_empty(a, b, M)
    n, m = M.shape
    numItermin = 35
    numItermax = max(numItermin, numItermax)
    if warmstart is None:
        alpha, beta = np.zeros(n), np.zeros(m)
    else:
        alpha, beta = _f64(warmstart[0]).copy(), _f64(warmstart[1]).copy()
    errs, warns = [], []
    err = 1.0
    ii = 0
    stopped = False
    G = None
    for ii in range(numItermax):
        regi = (epsilon0 - reg) * np.exp(-ii) + reg
        G, lg = sinkhorn_stabilized(a, b, M, regi, numItermax=numInnerItermax, tau=tau, stopThr=stopThr,
                                    warmstart=(alpha, beta), print_period=20)
        warns += lg["_warnings"]
        alpha, beta = lg["alpha"], lg["beta"]
        if ii % print_period == 0:
            err = float(np.linalg.norm(G.sum(0) - b) ** 2 + np.linalg.norm(G.sum(1) - a) ** 2)
            errs.append(err)
        if err <= stopThr and ii > numItermin:
            stopped = True
            break
    if not stopped:
        warns.append(NONCONV)
    return G, {"err": errs, "alpha": alpha, "beta": beta, "warmstart": (alpha, beta), "niter": ii,
               "_warnings": warns}


def solve_entropic(M, a=None, b=None, reg=1.0, reg_type="KL", max_iter=None, tol=None):
    """The regularised balanced branch of ``ot.solve`` for ``reg_type`` in
    ``{"KL", "entropy"}`` (``ot/solvers.py:428-494``): ``sinkhorn_log`` with
    ``max_iter = 1000, tol = 1e-9`` by default; potentials are the log
    scalings; ``value_linear = <M, P>`` and ``value`` adds
    ``reg * sum P log(P + 1e-16)`` (entropy) or
    ``reg * sum P log(P / (a b^T) + 1e-16)`` (KL, ``ot/backend.py:1542``)."""
    M = _f64(M)
    n, m = M.shape
    a = np.full(n, 1.0 / n) if a is None else _f64(a)
    b = np.full(m, 1.0 / m) if b is None else _f64(b)
    P, lg = sinkhorn_log(a, b, M, reg, numItermax=1000 if max_iter is None else max_iter,
                         stopThr=1e-9 if tol is None else tol)
    vlin = float(np.sum(M * P))
    with np.errstate(divide="ignore", invalid="ignore"):
        if reg_type.lower() == "entropy":
            value = vlin + reg * float(np.sum(P * np.log(P + 1e-16)))
        else:
            value = vlin + reg * float(np.sum(P * np.log(P / (a[:, None] * b[None, :]) + 1e-16)))
    return {"plan": P, "value": value, "value_linear": vlin, "potentials": (lg["log_u"], lg["log_v"]),
            "log": lg}


def empirical_sinkhorn2_lazy(X, Y, reg, a=None, b=None, numIterMax=10000, stopThr=1e-9, batchSize=100,
                             warmstart=None):
    """``ot/bregman/_empirical.py:430-481`` with ``isLazy=True``: the lazy
    solve, then ``sum_ij C_ij exp(f_i + g_j - C_ij/reg)`` accumulated over row
    blocks of ``batchSize``."""
    f, g, lg = empirical_sinkhorn_lazy(X, Y, reg, a, b, numIterMax, stopThr, batchSize, warmstart)
    X, Y = _f64(X), _f64(Y)
    bs = batchSize if isinstance(batchSize, int) else batchSize[0]
    loss = 0.0
    for i in range(0, X.shape[0], bs):
        C = sqeuclidean(X[i:i + bs], Y)
        loss += float(np.sum(C * np.exp(f[i:i + bs, None] + g[None, :] - C / reg)))
    return loss, lg


def barycenter_sinkhorn(A, M, reg, weights=None, numItermax=1000, stopThr=1e-4):
    """Entropic Wasserstein barycenter, scaling form,
    ``ot/bregman/_barycenter.py:141-259``: ``K = exp(-M/reg)``;
    ``UKv = K (A^T / K^T 1)^T``, ``u = geomMean(UKv) / UKv``; per iteration
    ``UKv = u * K^T (A / K u)``, ``u = u * geomBar(w, UKv) / UKv``; at
    ``ii % 10 == 1`` the error ``sum_i std_k UKv_ik`` stops the loop when
    ``< stopThr``.  Returns ``geomBar(w, UKv)`` and ``{"err", "niter"}``."""
    A, M = _f64(A), _f64(M)
    dim, H = A.shape
    w = np.full(H, 1.0 / H) if weights is None else _f64(weights)
    K = np.exp(-M / reg)
    UKv = K @ (A.T / np.sum(K, axis=0)).T
    u = (np.exp(np.mean(np.log(UKv), axis=1)) / UKv.T).T
    errs, warns = [], []
    ii = 0
    stopped = False
    for ii in range(numItermax):
        UKv = u * (K.T @ (A / (K @ u)))
        u = (u.T * np.exp(np.log(UKv) @ w)).T / UKv
        if ii % 10 == 1:
            err = float(np.sum(np.std(UKv, axis=1)))
            errs.append(err)
            if err < stopThr:
                stopped = True
                break
    if not stopped:
        warns.append(NONCONV)
    return np.exp(np.log(UKv) @ w), {"err": errs, "niter": ii, "_warnings": warns}


def barycenter_sinkhorn_log(A, M, reg, weights=None, numItermax=1000, stopThr=1e-4):
    """Entropic Wasserstein barycenter, log domain,
    ``ot/bregman/_barycenter.py:403-473``: per iteration and histogram
    ``f_k = log A_k - LSE_j(-M/reg + G_k)``, ``log KU_k = LSE_i(-M/reg + f_k)``,
    ``log bar = sum_k w_k log KU_k``; at ``ii % 10 == 1`` the error
    ``sum_i std_k exp(G + log KU)``; then ``G = log bar - log KU``."""
    A, M = _f64(A), _f64(M)
    dim, H = A.shape
    w = np.full(H, 1.0 / H) if weights is None else _f64(weights)
    Mr = -M / reg
    logA = np.log(A + 1e-16)
    log_KU = np.zeros_like(logA)
    G = np.zeros_like(logA)
    errs, warns = [], []
    ii = 0
    stopped = False
    log_bar = np.zeros(dim)
    for ii in range(numItermax):
        log_bar = np.zeros(dim)
        for k in range(H):
            f = logA[:, k] - logsumexp(Mr + G[None, :, k], 1)
            log_KU[:, k] = logsumexp(Mr + f[:, None], 0)
            log_bar = log_bar + w[k] * log_KU[:, k]
        if ii % 10 == 1:
            err = float(np.exp(G + log_KU).std(axis=1).sum())
            errs.append(err)
            if err < stopThr:
                stopped = True
                break
        G = log_bar[:, None] - log_KU
    if not stopped:
        warns.append(NONCONV)
    return np.exp(log_bar), {"err": errs, "niter": ii, "_warnings": warns}


def sinkhorn_knopp_unbalanced(a, b, M, reg, reg_m, reg_type="kl", c=None, warmstart=None, numItermax=1000,
                              stopThr=1e-6):
    """Unbalanced scaling Sinkhorn with KL marginal penalties,
    ``ot/unbalanced/_sinkhorn.py:565-818`` (1-D ``b``):
    ``K = exp(-M/reg) * c`` with ``c = a b^T`` (or ones for
    ``reg_type='entropy'``); per iteration ``u = (a / K v)^fi1`` then
    ``v = (b / K^T u)^fi2`` with ``fi = reg_m / (reg_m + reg)`` (1 for an
    infinite ``reg_m``); a zero ``K^T u`` or a non-finite scaling reverts to
    the previous pair; the error ``0.5 (|du|_inf / max(|u|_inf, |uprev|_inf, 1)
    + same for v)`` is logged every iteration and stops the loop when
    ``< stopThr``.  The log holds ``err, logu, logv, cost, total_cost``."""
    M = _f64(M)
    a, b = _uniform_if_empty(a, b, M)
    n, m = M.shape
    rm1, rm2 = (float(reg_m), float(reg_m)) if np.isscalar(reg_m) else (float(reg_m[0]), float(reg_m[1]))
    if warmstart is None:
        u, v = np.ones(n), np.ones(m)
    else:
        u, v = np.exp(_f64(warmstart[0])), np.exp(_f64(warmstart[1]))
    warns = []
    if reg_type.lower() == "entropy":
        warns.append("If reg_type = entropy, then the matrix c is overwritten by the one matrix.")
        c = np.ones((n, m))
    c = np.outer(a, b) if c is None else _f64(c)
    K = np.exp(-M / reg) * c
    fi1 = rm1 / (rm1 + reg) if rm1 != float("inf") else 1
    fi2 = rm2 / (rm2 + reg) if rm2 != float("inf") else 1
    errs = []
    i = 0
    with np.errstate(all="ignore"):
        for i in range(numItermax):
            uprev, vprev = u, v
            u = (a / (K @ v)) ** fi1
            Ktu = K.T @ u
            v = (b / Ktu) ** fi2
            if (np.any(Ktu == 0.0) or np.any(np.isnan(u)) or np.any(np.isnan(v)) or np.any(np.isinf(u))
                    or np.any(np.isinf(v))):
                warns.append("Numerical errors at iteration %s" % i)
                u, v = uprev, vprev
                break
            err_u = np.max(np.abs(u - uprev)) / max(np.max(np.abs(u)), np.max(np.abs(uprev)), 1.0)
            err_v = np.max(np.abs(v - vprev)) / max(np.max(np.abs(v)), np.max(np.abs(vprev)), 1.0)
            err = 0.5 * (err_u + err_v)
            errs.append(float(err))
            if err < stopThr:
                break
        plan = u[:, None] * K * v[None, :]
        cost = float(np.sum(plan * M))

        def kl(p, q):
            return float(np.sum(p * np.log(p / q + 1e-16)))
        total = cost + reg * kl(plan, c)
        if rm1 != float("inf"):
            total += rm1 * kl(plan.sum(1), a)
        if rm2 != float("inf"):
            total += rm2 * kl(plan.sum(0), b)
    return plan, {"err": errs, "logu": np.log(u + 1e-300), "logv": np.log(v + 1e-300), "cost": cost,
                  "total_cost": total, "niter": i, "_warnings": warns}


def log_projection_batch(K, a=None, b=None, max_iter=10000, tol=1e-5):
    """Batched log-domain Bregman projection, ``ot/batch/_utils.py:165-290``.

    ``K`` is ``-M/reg`` with shape (B, n, m).  The update order is u first,
    then v (``:268-270``); every 10th iteration the largest L2 violation of
    the ROW marginal over the batch is compared with ``tol`` (``:273-278``).
    """
    K = _f64(K)
    B, n, m = K.shape
    a = np.ones((B, n)) / n if a is None else _f64(a)
    b = np.ones((B, m)) / m if b is None else _f64(b)
    u = np.zeros((B, n))
    v = np.zeros((B, m))
    with np.errstate(divide="ignore"):
        loga, logb = np.log(a), np.log(b)
    it = 0
    with np.errstate(all="ignore"):
        for it in range(max_iter):
            u = loga - logsumexp(K + v[:, None, :], 2)
            v = logb - logsumexp(K + u[:, :, None], 1)
            if it % 10 == 0:
                T = np.exp(K + u[:, :, None] + v[:, None, :])
                err = np.max(np.sqrt(np.sum((T.sum(2) - a) ** 2, 1)))
                if err < tol:
                    break
        logT = K + u[:, :, None] + v[:, None, :]
        T = np.exp(logT)
    return {"T": T, "log_T": logT, "n_iters": it, "potentials": (u, v)}


def scaling_projection_batch(K, a=None, b=None, max_iter=10000, tol=1e-5):
    """Batched scaling-form Bregman projection, ``ot/batch/_utils.py:46-162``:
    ``f = a / (K g)``, ``g = b / (K^T f)`` from ``f = g = 1``, same stopping
    rule as the log form."""
    K = _f64(K)
    B, n, m = K.shape
    a = np.ones((B, n)) / n if a is None else _f64(a)
    b = np.ones((B, m)) / m if b is None else _f64(b)
    f = np.ones((B, n))
    g = np.ones((B, m))
    it = 0
    with np.errstate(all="ignore"):
        for it in range(max_iter):
            f = a / np.sum(K * g[:, None, :], 2)
            g = b / np.sum(K * f[:, :, None], 1)
            if it % 10 == 0:
                T = K * f[:, :, None] * g[:, None, :]
                err = np.max(np.sqrt(np.sum((T.sum(2) - a) ** 2, 1)))
                if err < tol:
                    break
        T = K * f[:, :, None] * g[:, None, :]
    return {"T": T, "n_iters": it, "potentials": (f, g)}


def solve_batch(M, reg, a=None, b=None, max_iter=1000, tol=1e-5,
                solver="log_sinkhorn", reg_type="entropy"):
    """``ot/batch/_linear.py:236-357``: projection, then
    ``value_linear = sum(M*T)`` and ``value = value_linear + reg * R(T)`` with
    ``R = sum T log(T + 1e-16)`` (entropy) or ``sum T log(T/(a b^T) + 1e-16)``
    (KL).  Returns a dict with the OTResult fields."""
    M = _f64(M)
    B, n, m = M.shape
    a = np.ones((B, n)) / n if a is None else _f64(a)
    b = np.ones((B, m)) / m if b is None else _f64(b)
    if solver == "log_sinkhorn":
        out = log_projection_batch(-M / reg, a, b, max_iter, tol)
    elif solver == "sinkhorn":
        with np.errstate(all="ignore"):
            out = scaling_projection_batch(np.exp(-M / reg), a, b, max_iter, tol)
    else:
        raise ValueError("Unknown solver: %s" % solver)
    T = out["T"]
    value_linear = np.sum(M * T, axis=(1, 2))
    with np.errstate(all="ignore"):
        if reg_type.lower() == "entropy":
            value = value_linear + reg * np.sum(T * np.log(T + 1e-16), axis=(1, 2))
        else:
            ref = np.einsum("bi,bj->bij", a, b)
            value = value_linear + reg * np.sum(T * np.log(T / ref + 1e-16), axis=(1, 2))
    return {"plan": T, "value": value, "value_linear": value_linear,
            "potentials": out["potentials"], "n_iter": out["n_iters"]}


def init_matrix_square_loss(C1, C2, p, q):
    """``ot/gromov/_utils.py:153-241`` with the square-loss transforms of
    ``:114-126``: ``constC = C1^2 p 1^T + 1 q^T (C2^2)^T``, ``hC1 = C1``,
    ``hC2 = 2 C2``."""
    C1, C2, p, q = _f64(C1), _f64(C2), _f64(p), _f64(q)
    constC = np.outer((C1 ** 2) @ p, np.ones(len(q))) + np.outer(np.ones(len(p)), q @ (C2 ** 2).T)
    return constC, C1, 2.0 * C2


def tensor_product(constC, hC1, hC2, T):
    """``ot/gromov/_utils.py:244-280``: ``constC - hC1 T hC2^T``."""
    return constC - hC1 @ T @ hC2.T


def entropic_gromov_wasserstein(C1, C2, p=None, q=None, epsilon=0.1, symmetric=None,
                                G0=None, max_iter=1000, tol=1e-9, solver="PGD",
                                warmstart=False, numItermax=1000, stopThr=1e-9):
    """Entropic GW with square loss, ``ot/gromov/_bregman.py:25-253``.

    Outer loop ``:198-242``: ``tens = 2 (constC - hC1 T hC2^T)`` (averaged
    with the transposed problem when not symmetric, minus ``eps log T`` for
    PPA), then ``T = sinkhorn(p, q, tens, eps, method='sinkhorn')``.  With
    ``warmstart`` the scalings are carried as ``eps * log(u)`` and handed back
    as the warm start of the next call (``:213-224``), which the Knopp solver
    reads as ``log u``.  Every 10th outer iteration logs ``||T - Tprev||_F``.
    Returns ``(T, log)`` with ``log = {"err", "gw_dist"}``.
    """
    T, lg = _entropic_gw(None, C1, C2, p, q, epsilon, symmetric, 1.0, G0, max_iter, tol, solver, warmstart,
                         numItermax, stopThr)
    lg["gw_dist"] = lg.pop("dist")
    return T, lg


def entropic_fused_gromov_wasserstein(M, C1, C2, p=None, q=None, epsilon=0.1, symmetric=None, alpha=0.5,
                                      G0=None, max_iter=1000, tol=1e-9, solver="PGD", warmstart=False,
                                      numItermax=1000, stopThr=1e-9):
    """Entropic fused GW with square loss, ``ot/gromov/_bregman.py:997-1241``:
    the loop above with ``tens = alpha gwggrad(T) + (1 - alpha) M``
    (``:1184-1192``) and ``fgw_dist = (1 - alpha) <M, T> + alpha gwloss(T)``
    (``:1235-1238``)."""
    T, lg = _entropic_gw(M, C1, C2, p, q, epsilon, symmetric, alpha, G0, max_iter, tol, solver, warmstart,
                         numItermax, stopThr)
    lg["fgw_dist"] = lg.pop("dist")
    return T, lg


def _entropic_gw(M, C1, C2, p, q, epsilon, symmetric, alpha, G0, max_iter, tol, solver, warmstart, numItermax,
                 stopThr):
    C1, C2 = _f64(C1), _f64(C2)
    n1, n2 = C1.shape[0], C2.shape[0]
    p = np.full(n1, 1.0 / n1) if p is None else _f64(p)
    q = np.full(n2, 1.0 / n2) if q is None else _f64(q)
    T = np.outer(p, q) if G0 is None else _f64(G0)
    constC, hC1, hC2 = init_matrix_square_loss(C1, C2, p, q)
    if symmetric is None:
        symmetric = np.allclose(C1, C1.T, atol=1e-10) and np.allclose(C2, C2.T, atol=1e-10)
    if not symmetric:
        constCt, hC1t, hC2t = init_matrix_square_loss(C1.T, C2.T, p, q)
    if warmstart:
        mu = np.zeros(n1) - np.log(n1)
        nu = np.zeros(n2) - np.log(n2)
    cpt, err, errs, warns = 0, 1.0, [], []
    while err > tol and cpt < max_iter:
        Tprev = T
        if symmetric:
            tens = 2.0 * tensor_product(constC, hC1, hC2, T)
        else:
            tens = 0.5 * (2.0 * tensor_product(constC, hC1, hC2, T)
                          + 2.0 * tensor_product(constCt, hC1t, hC2t, T))
        if M is not None:
            tens = alpha * tens + (1 - alpha) * _f64(M)
        if solver == "PPA":
            with np.errstate(divide="ignore"):
                tens = tens - epsilon * np.log(T)
        if warmstart:
            T, lg = sinkhorn_knopp(p, q, tens, epsilon, numItermax, stopThr, (mu, nu))
            with np.errstate(divide="ignore"):
                mu = epsilon * np.log(lg["u"])
                nu = epsilon * np.log(lg["v"])
        else:
            T, lg = sinkhorn_knopp(p, q, tens, epsilon, numItermax, stopThr)
        warns += lg["_warnings"]
        if cpt % 10 == 0:
            err = float(np.linalg.norm(T - Tprev))
            errs.append(err)
        cpt += 1
    if abs(np.sum(T) - 1) > 1e-5:
        warns.append("Solver failed to produce a transport plan")
    gw = float(np.sum(tensor_product(constC, hC1, hC2, T) * T))
    dist = gw if M is None else (1 - alpha) * float(np.sum(_f64(M) * T)) + alpha * gw
    return T, {"err": errs, "dist": dist, "_warnings": warns, "n_outer": cpt}


def entropic_gw_log_inner(C1, C2, p=None, q=None, epsilon=0.1, max_iter=50, tol=0.0,
                          numItermax=1000, stopThr=1e-7):
    """The entropic-GW outer loop of ``ot/gromov/_bregman.py:198-242``
    (symmetric square loss, PGD) with the inner solve replaced by
    ``sinkhorn_log`` (``_sinkhorn.py:690``) warm-started from the previous
    outer iteration's ``(log_u, log_v)``.  The reference hard-codes the Knopp
    inner solver; this variant is the log-domain restatement used for the
    large entropic-GW workload."""
    C1, C2 = _f64(C1), _f64(C2)
    n1, n2 = C1.shape[0], C2.shape[0]
    p = np.full(n1, 1.0 / n1) if p is None else _f64(p)
    q = np.full(n2, 1.0 / n2) if q is None else _f64(q)
    T = np.outer(p, q)
    constC, hC1, hC2 = init_matrix_square_loss(C1, C2, p, q)
    ws = None
    cpt, err, errs, inner_iters = 0, 1.0, [], []
    while err > tol and cpt < max_iter:
        Tprev = T
        tens = 2.0 * tensor_product(constC, hC1, hC2, T)
        T, lg = sinkhorn_log(p, q, tens, epsilon, numItermax, stopThr, ws)
        ws = (lg["log_u"], lg["log_v"])
        inner_iters.append(lg["niter"])
        if cpt % 10 == 0:
            err = float(np.linalg.norm(T - Tprev))
            errs.append(err)
        cpt += 1
    gw = float(np.sum(tensor_product(constC, hC1, hC2, T) * T))
    return T, {"err": errs, "gw_dist": gw, "inner_niter": inner_iters,
               "log_u": ws[0], "log_v": ws[1]}


def empirical_sinkhorn_lazy(X, Y, reg, a=None, b=None, numIterMax=10000, stopThr=1e-9,
                            batchSize=100, warmstart=None):
    """Blockwise ("lazy") log-domain Sinkhorn on point clouds,
    ``ot/bregman/_empirical.py:190-263``.

    The cost ``sqeuclidean(X_blk, Y)`` is recomputed per block; per iteration
    ``f = log a - LSE_j(g - C/reg)`` then ``g = log b - LSE_i(f - C/reg)``;
    at every 10th iteration counted from one (``(i+1) % 10 == 0``) the L1
    violation of the ROW marginal is compared with ``stopThr`` using ``<=``.
    Returns ``(f, g, log)`` with ``log = {"err", "u": f, "v": g, "niter"}``.
    """
    X, Y = _f64(X), _f64(Y)
    ns, nt = X.shape[0], Y.shape[0]
    a = np.full(ns, 1.0 / ns) if a is None else _f64(a)
    b = np.full(nt, 1.0 / nt) if b is None else _f64(b)
    bs, bt = (batchSize, batchSize) if isinstance(batchSize, int) else batchSize
    f = np.zeros(ns) if warmstart is None else _f64(warmstart[0]).copy()
    g = np.zeros(nt) if warmstart is None else _f64(warmstart[1]).copy()
    loga, logb = np.log(a), np.log(b)
    errs, warns = [], []
    i_ot = 0
    stopped = False
    for i_ot in range(numIterMax):
        f = loga - np.concatenate([logsumexp(g[None, :] - sqeuclidean(X[i:i + bs], Y) / reg, 1)
                                   for i in range(0, ns, bs)])
        g = logb - np.concatenate([logsumexp(f[:, None] - sqeuclidean(X, Y[j:j + bt]) / reg, 0)
                                   for j in range(0, nt, bt)])
        if (i_ot + 1) % 10 == 0:
            m1 = np.concatenate([np.sum(np.exp(f[i:i + bs, None] + g[None, :]
                                               - sqeuclidean(X[i:i + bs], Y) / reg), 1)
                                 for i in range(0, ns, bs)])
            err = float(np.sum(np.abs(m1 - a)))
            errs.append(err)
            if err <= stopThr:
                stopped = True
                break
    if not stopped:
        warns.append(NONCONV)
    return f, g, {"err": errs, "u": f, "v": g, "niter": i_ot, "_warnings": warns}


def solve_gromov_batch(C1, C2, reg=1e-2, a=None, b=None, symmetric=None, M=None, alpha=None, T_init=None,
                       max_iter=50, tol=1e-5, max_iter_inner=50, tol_inner=1e-5, per_problem_inner=False):
    """Batched proximal (fused) Gromov-Wasserstein, squared loss, scalar costs:
    ``ot/batch/_quadratic.py:269-498`` with ``tensor_batch`` (:17, hC1 = 2 C1,
    hC2 = C2, f = square; non-symmetric inputs symmetrise f), the outer step
    ``Mk = (1-alpha) M + 2 alpha (constC - hC1 T hC2^T)`` (averaged with the
    transposed product when not symmetric), ``K = -Mk/reg + log T`` projected by
    the batched log Sinkhorn (:458-471), stop on ``max_b mean|T - Tprev| <
    tol``.  ``per_problem_inner`` runs the inner projection one problem at a
    time (each problem stops on its own error)."""
    C1, C2 = _f64(C1), _f64(C2)
    B, n, m = C1.shape[0], C1.shape[1], C2.shape[1]
    a = np.ones((B, n)) / n if a is None else _f64(a)
    b = np.ones((B, m)) / m if b is None else _f64(b)
    tr = lambda X: np.transpose(X, (0, 2, 1))  # noqa: E731
    if symmetric is None:
        symmetric = np.allclose(C1, tr(C1), atol=1e-10) and np.allclose(C2, tr(C2), atol=1e-10)
    fC1, fC2 = C1 ** 2, C2 ** 2
    if not symmetric:
        fC1, fC2 = 0.5 * (fC1 + tr(fC1)), 0.5 * (fC2 + tr(fC2))
    hC1, hC2 = 2.0 * C1, C2
    constC = np.einsum("bij,bj->bi", fC1, a)[:, :, None] + np.einsum("bij,bj->bi", fC2, b)[:, None, :]
    if M is None and alpha is None:
        M, alpha = np.zeros((B, n, m)), 1.0
    elif M is None or alpha is None:
        raise ValueError("M and alpha go together for the fused problem")
    M = _f64(M)

    def dot(T):
        d = hC1 @ T @ tr(hC2)
        if not symmetric:
            d = 0.5 * (d + tr(hC1) @ T @ hC2)
        return d

    if T_init is None:
        const = np.sqrt(a.sum(1) * b.sum(1))
        T = np.einsum("bi,bj->bij", a, b) / const[:, None, None]
    else:
        T = _f64(T_init)
    with np.errstate(divide="ignore"):
        log_T = np.log(T + 1e-15)
    it = 0
    out = None
    for it in range(max_iter):
        T_prev = T
        Mk = (1 - alpha) * M + 2 * alpha * (constC - dot(T))
        K = -Mk / reg + log_T
        if per_problem_inner:
            parts = [log_projection_batch(K[k:k + 1], a[k:k + 1], b[k:k + 1], max_iter_inner, tol_inner)
                     for k in range(B)]
            out = {"T": np.concatenate([p["T"] for p in parts]), "log_T": np.concatenate([p["log_T"] for p in parts]),
                   "potentials": (np.concatenate([p["potentials"][0] for p in parts]),
                                  np.concatenate([p["potentials"][1] for p in parts]))}
        else:
            out = log_projection_batch(K, a, b, max_iter_inner, tol_inner)
        T, log_T = out["T"], out["log_T"]
        if np.max(np.mean(np.abs(T_prev - T), axis=(1, 2))) < tol:
            break
    vl = np.sum(M * T, axis=(1, 2))
    const_rec = np.einsum("bij,bj->bi", fC1, T.sum(2))[:, :, None] + np.einsum("bij,bj->bi", fC2, T.sum(1))[:, None, :]
    vq = np.sum((const_rec - dot(T)) * T, axis=(1, 2))
    return {"plan": T, "value": (1 - alpha) * vl + alpha * vq, "value_linear": (1 - alpha) * vl,
            "value_quad": alpha * vq, "potentials": out["potentials"], "n_iter": it}
