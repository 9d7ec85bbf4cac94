"""Generate the golden fixtures in this folder by running the REFERENCE.

Run in a container that holds the reference source tree (it is imported
through ``ref_import.py``); the GPU machine never runs this script, it only reads
the ``.npz`` files it writes.  Every case records its inputs, the reference's
outputs and, where the reference warns, the warnings it raised.

    POT_REFERENCE_SRC=<reference tree> python tests/golden/gen_golden.py        # every section
    POT_REFERENCE_SRC=<reference tree> python tests/golden/gen_golden.py next   # one section
"""
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from ref_import import import_ot  # noqa: E402

ot = import_ot()


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print("wrote", name, os.path.getsize(path), "bytes")


def call_warn(fn, *a, **k):
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        out = fn(*a, **k)
    return out, [str(x.message) for x in w]


def dense_case(name, a, b, M, reg, numItermax=1000, stopThr=1e-9):
    """sinkhorn (Knopp) and sinkhorn_log on one dense problem."""
    out = dict(a=a, b=b, M=M, reg=reg, numItermax=numItermax, stopThr=stopThr)
    for method, tag in (("sinkhorn", "knopp"), ("sinkhorn_log", "log")):
        (P, lg), w = call_warn(ot.sinkhorn, a, b, M, reg, method=method, numItermax=numItermax,
                               stopThr=stopThr, log=True)
        out[tag + "_plan"] = P
        out[tag + "_loss"] = float(np.sum(M * P))
        out[tag + "_niter"] = lg["niter"]
        out[tag + "_err"] = np.array(lg["err"], dtype=np.float64)
        out[tag + "_u"] = lg["u"]
        out[tag + "_v"] = lg["v"]
        out[tag + "_nwarn"] = len(w)
        out[tag + "_warn_nonconv"] = int(any("did not converge" in s for s in w))
        out[tag + "_warn_numerr"] = int(any("numerical errors" in s for s in w))
    save(name, **out)


def core():
    # 1. reference doctest (ot/bregman/_sinkhorn.py:123-129, 342-347)
    a = np.array([0.5, 0.5])
    M = np.array([[0.0, 1.0], [1.0, 0.0]])
    P = ot.sinkhorn(a, a, M, 1)
    loss = ot.sinkhorn2(a, a, M, 1)
    save("doctest_2x2", a=a, b=a, M=M, plan=P, loss=loss)

    # 2. the plain dense CPU workload: 1024 points in R^2, N(0,I) vs N((1,1),0.5I)
    rng = np.random.default_rng(20240601)
    n = 1024
    x = rng.standard_normal((n, 2))
    y = rng.standard_normal((n, 2)) * np.sqrt(0.5) + 1.0
    M = ot.dist(x, y)
    M /= M.max()
    u = ot.unif(n)
    dense_case("dense_1024_gauss2d", u, u, M, 0.05, 1000, 1e-9)
    # store the points too: tests rebuild M with the oracle's cost
    d = dict(np.load(os.path.join(HERE, "dense_1024_gauss2d.npz")))
    d.pop("M")
    d.pop("knopp_plan")
    d.pop("log_plan")
    save("dense_1024_gauss2d", x=x, y=y, **d)

    # 3. small and ragged shapes, random weights, two regularisations
    rng = np.random.default_rng(7)
    for (n, m) in [(1, 1), (2, 3), (3, 2), (31, 33), (127, 129), (100, 100), (5, 300)]:
        for reg in (0.05, 0.5):
            M = rng.random((n, m))
            a = rng.dirichlet(np.ones(n)) if n > 1 else np.ones(1)
            b = rng.dirichlet(np.ones(m)) if m > 1 else np.ones(1)
            dense_case("dense_%dx%d_reg%g" % (n, m, reg), a, b, M, reg, 2000, 1e-9)

    # 4. failure paths: non-convergence at numItermax=1, reg=0 numerical error
    n = 100
    a1 = ot.datasets.make_1D_gauss(n, m=30, s=10)
    a2 = ot.datasets.make_1D_gauss(n, m=40, s=10)
    M = ot.utils.dist0(n)
    dense_case("fail_maxiter1", a1, a2, M, 1.0, 1, 0.0)
    (P, lg), w = call_warn(ot.sinkhorn, a1, a2, M, 0.0, method="sinkhorn", log=True, warn=False)
    save("fail_reg0_knopp", a=a1, b=a2, M=M, niter=lg["niter"], u=lg["u"], v=lg["v"],
         warn_numerr=int(any("numerical errors" in s for s in w)))

    # 5. several target histograms (2-D b), both methods
    rng = np.random.default_rng(11)
    n = 31
    x = rng.standard_normal((n, 2))
    M = ot.dist(x, x)
    a = ot.unif(n)
    B = np.stack([rng.dirichlet(np.ones(n)) for _ in range(3)], 1)
    out = dict(a=a, b=B, M=M, reg=1.0)
    for method, tag in (("sinkhorn", "knopp"), ("sinkhorn_log", "log")):
        loss, lg = ot.sinkhorn2(a, B, M, 1.0, method=method, log=True, stopThr=1e-10)
        out[tag + "_loss"] = np.asarray(loss)
        out[tag + "_u"] = lg["u"]
        out[tag + "_v"] = lg["v"]
    save("multib_31x3", **out)

    # 6. batch solvers (test/batch/test_solve_batch.py:28-62 setting)
    rng = np.random.RandomState(0)
    M = rng.rand(4, 16, 16)
    out = dict(M=M, reg=0.1, tol=1e-5, max_iter=10000)
    for solver in ("log_sinkhorn", "sinkhorn"):
        for reg_type in ("entropy", "kl"):
            res = ot.batch.solve_batch(M, 0.1, max_iter=10000, tol=1e-5, solver=solver,
                                       reg_type=reg_type, grad="detach")
            tag = "%s_%s" % (solver, reg_type)
            out[tag + "_plan"] = res.plan
            out[tag + "_value"] = res.value
            out[tag + "_value_linear"] = res.value_linear
            out[tag + "_pot_u"] = res.potentials[0]
            out[tag + "_pot_v"] = res.potentials[1]
            out[tag + "_n_iter"] = res.log["n_iter"]
    save("batch_4x16", **out)
    # ragged batch through zero-weight padding (uneven n, m in one padded batch)
    rng = np.random.default_rng(5)
    sizes = [(12, 9), (7, 16), (16, 16), (3, 5)]
    Bn, Bm = 16, 16
    M = rng.random((4, Bn, Bm))
    A = np.zeros((4, Bn))
    Bw = np.zeros((4, Bm))
    for k, (n, m) in enumerate(sizes):
        A[k, :n] = rng.dirichlet(np.ones(n))
        Bw[k, :m] = rng.dirichlet(np.ones(m))
    with np.errstate(all="ignore"), warnings.catch_warnings():
        warnings.simplefilter("ignore")
        res = ot.batch.solve_batch(M, 0.05, a=A, b=Bw, max_iter=20000, tol=1e-9, grad="detach")
    save("batch_ragged_padded", M=M, a=A, b=Bw, sizes=np.array(sizes), reg=0.05,
         plan=res.plan, value_linear=res.value_linear, n_iter=res.log["n_iter"])
    # solve_sample_batch on point clouds
    rng = np.random.default_rng(9)
    X = rng.standard_normal((3, 20, 3))
    Y = rng.standard_normal((3, 25, 3)) + 0.5
    res = ot.batch.solve_sample_batch(X, Y, 0.5, max_iter=5000, tol=1e-7, grad="detach")
    save("batch_sample_3x20x25", X=X, Y=Y, reg=0.5, plan=res.plan, value=res.value,
         value_linear=res.value_linear, n_iter=res.log["n_iter"])

    # 7. entropic GW (test/gromov/test_bregman.py:25-78 setting and variants)
    xs = ot.datasets.make_2D_samples_gauss(10, np.array([0, 0]), np.eye(2), random_state=42)
    xt = xs[::-1].copy()
    C1 = ot.dist(xs, xs)
    C2 = ot.dist(xt, xt)
    C1 /= C1.max()
    C2 /= C2.max()
    p = ot.unif(10)
    out = dict(C1=C1, C2=C2, p=p, q=p)
    for tag, kw in (("pgd", {}), ("pgd_warm", {"warmstart": True}), ("ppa", {"solver": "PPA"})):
        G, lg = ot.gromov.entropic_gromov_wasserstein(C1, C2, p, p, "square_loss", epsilon=1e-2,
                                                      max_iter=10, log=True, **kw)
        out[tag + "_T"] = G
        out[tag + "_gw"] = lg["gw_dist"]
        out[tag + "_err"] = np.array(lg["err"])
    save("egw_10", **out)
    rng = np.random.default_rng(3)
    xs = rng.standard_normal((48, 3))
    xt = rng.standard_normal((40, 8))
    C1 = ot.dist(xs, xs)
    C2 = ot.dist(xt, xt)
    C1 /= C1.max()
    C2 /= C2.max()
    G, lg = ot.gromov.entropic_gromov_wasserstein(C1, C2, None, None, "square_loss", epsilon=5e-2,
                                                  max_iter=20, tol=1e-9, log=True,
                                                  numItermax=2000, stopThr=1e-9)
    gw2 = ot.gromov.entropic_gromov_wasserstein2(C1, C2, None, None, "square_loss", epsilon=5e-2,
                                                 max_iter=20, tol=1e-9, numItermax=2000,
                                                 stopThr=1e-9)
    save("egw_48x40", C1=C1, C2=C2, T=G, gw=lg["gw_dist"], err=np.array(lg["err"]), gw2=gw2,
         epsilon=5e-2)
    # asymmetric input
    C1a = C1 + 0.05 * rng.random(C1.shape)
    G, lg = ot.gromov.entropic_gromov_wasserstein(C1a, C2, None, None, "square_loss", epsilon=5e-2,
                                                  max_iter=10, log=True)
    save("egw_asym_48x40", C1=C1a, C2=C2, T=G, gw=lg["gw_dist"], err=np.array(lg["err"]))

    # 7b. batched (fused) Gromov-Wasserstein (test/batch/test_solve_gromov_batch.py:19 setting)
    rng = np.random.RandomState(0)
    X1 = rng.randn(2, 8, 2)
    C1 = rng.randn(2, 8, 8)
    perm = np.random.RandomState(1).permutation(8)
    X2 = X1[:, perm, :] + 0.01 * rng.randn(2, 8, 2)
    C2 = C1[:, perm, :][:, :, perm] + 0.01 * rng.randn(2, 8, 8)
    Mb = ot.batch.dist_batch(X1, X2)
    res = ot.batch.solve_gromov_batch(C1, C2, reg=0.01, M=Mb, alpha=0.5, max_iter=1000, tol=1e-5,
                                      max_iter_inner=10000, tol_inner=1e-5, symmetric=False)
    save("gromov_batch_fused", C1=C1, C2=C2, M=Mb, plan=res.plan, value=res.value,
         value_linear=res.value_linear, value_quad=res.value_quad, n_iter=res.log["n_iter"])
    rng = np.random.default_rng(8)
    xs = rng.standard_normal((3, 12, 2))
    xt = rng.standard_normal((3, 10, 3))
    C1 = np.stack([ot.dist(x, x) for x in xs])
    C2 = np.stack([ot.dist(x, x) for x in xt])
    C1 /= C1.max(axis=(1, 2), keepdims=True)
    C2 /= C2.max(axis=(1, 2), keepdims=True)
    res = ot.batch.solve_gromov_batch(C1, C2, reg=0.05, max_iter=50, tol=1e-7, max_iter_inner=2000, tol_inner=1e-9)
    save("gromov_batch_sym", C1=C1, C2=C2, plan=res.plan, value=res.value, value_quad=res.value_quad,
         n_iter=res.log["n_iter"])

    # 8. lazy empirical Sinkhorn (ot/bregman/_empirical.py:190-263)
    rng = np.random.default_rng(21)
    X = rng.standard_normal((60, 3))
    Y = rng.standard_normal((50, 3)) + 1.0
    f, g, lg = ot.bregman.empirical_sinkhorn(X, Y, 1.0, isLazy=True, batchSize=7, numIterMax=500,
                                             stopThr=1e-9, log=True)
    save("lazy_60x50", X=X, Y=Y, reg=1.0, f=f, g=g, err=np.array(lg["err"]), niter=lg["niter"])


def stab_case(name, a, b, x, y, reg, **kw):
    """sinkhorn_stabilized (ot/bregman/_sinkhorn.py:1105) on one dense problem
    with M = dist(x, y) / max; M and the plan are stored for small cases."""
    M = ot.dist(x, y)
    M /= M.max()
    (P, lg), w = call_warn(ot.bregman.sinkhorn_stabilized, a, b, M, reg, log=True, **kw)
    out = dict(a=a, b=b, x=x, y=y, reg=reg, loss=float(np.sum(M * P)), n_iter=lg["n_iter"],
               err=np.array(lg["err"], dtype=np.float64), logu=lg["logu"], logv=lg["logv"],
               alpha=lg["alpha"], beta=lg["beta"],
               warn_nonconv=int(any("did not converge" in x for x in w)),
               warn_numerr=int(any("Numerical errors" in x for x in w)),
               **{"kw_" + k: v for k, v in kw.items() if k != "warmstart"})
    if "warmstart" in kw:
        out["ws_alpha"], out["ws_beta"] = kw["warmstart"]
    if M.size <= 5000:
        out["M"] = M
        out["plan"] = P
    save(name, **out)


def next_rows():
    # 9. stabilised Sinkhorn (ot/bregman/_sinkhorn.py:1105-1368): absorptions,
    # warm start, an exit at numItermax right after an absorption
    rng = np.random.default_rng(31)
    for (n, m) in [(31, 33), (127, 129)]:
        x = rng.standard_normal((n, 2))
        y = rng.standard_normal((m, 2)) + 0.5
        a = rng.random(n) + 0.1
        a /= a.sum()
        b = rng.random(m) + 0.1
        b /= b.sum()
        for reg in (0.5, 0.02, 0.002):
            stab_case("stab_%dx%d_reg%g" % (n, m, reg), a, b, x, y, reg, numItermax=2000)
    rng = np.random.default_rng(32)
    x = rng.standard_normal((40, 3))
    y = rng.standard_normal((50, 3))
    a, b = ot.unif(40), ot.unif(50)
    stab_case("stab_warm_40x50", a, b, x, y, 0.01,
              warmstart=(rng.standard_normal(40) * 0.01, rng.standard_normal(50) * 0.01), numItermax=3000)
    stab_case("stab_maxiter1_40x50", a, b, x, y, 0.01, numItermax=1)
    stab_case("stab_tau10_40x50", a, b, x, y, 0.05, tau=10.0, print_period=7, stopThr=1e-11)
    g = dict(np.load(os.path.join(HERE, "dense_1024_gauss2d.npz")))
    stab_case("stab_1024_gauss2d", g["a"], g["b"], g["x"], g["y"], 0.01, numItermax=1000)

    # 10. epsilon scaling (ot/bregman/_sinkhorn.py:1371-1575)
    rng = np.random.default_rng(33)
    x = rng.standard_normal((31, 2))
    y = rng.standard_normal((33, 2)) + 0.5
    M = ot.dist(x, y)
    M /= M.max()
    a, b = ot.unif(31), ot.unif(33)
    for reg, kw in ((0.01, {}), (0.05, dict(numItermax=60, epsilon0=10.0, numInnerItermax=30, print_period=5))):
        (G, lg), w = call_warn(ot.bregman.sinkhorn_epsilon_scaling, a, b, M, reg, log=True, **kw)
        save("epsscale_31x33_reg%g" % reg, a=a, b=b, M=M, reg=reg, plan=G, alpha=lg["alpha"], beta=lg["beta"],
             err=np.array(lg["err"], dtype=np.float64), niter=lg["niter"], nwarn=len(w),
             warn_nonconv=sum("did not converge" in x for x in w),
             **{"kw_" + k: v for k, v in kw.items()})

    # 11. ot.solve / ot.solve_sample entropic branches (ot/solvers.py:428-494, 1765-1877)
    rng = np.random.default_rng(34)
    x = rng.standard_normal((40, 3))
    y = rng.standard_normal((30, 3)) + 0.3
    a = rng.random(40) + 0.2
    a /= a.sum()
    b = rng.random(30) + 0.2
    b /= b.sum()
    M = ot.dist(x, y)
    for reg_type in ("KL", "entropy"):
        res = ot.solve(M, a, b, reg=0.5, reg_type=reg_type)
        save("solve_40x30_%s" % reg_type, x=x, y=y, a=a, b=b, M=M, reg=0.5, plan=res.plan, value=res.value,
             value_linear=res.value_linear, pa=res.potentials[0], pb=res.potentials[1])
    res = ot.solve(M, a, b, reg=0.5, max_iter=7, tol=0.0)
    save("solve_40x30_iter7", M=M, a=a, b=b, reg=0.5, plan=res.plan, value=res.value,
         value_linear=res.value_linear, pa=res.potentials[0], pb=res.potentials[1])
    res = ot.solve_sample(x, y, a, b, reg=0.5)
    save("solve_sample_40x30", x=x, y=y, a=a, b=b, reg=0.5, plan=res.plan, value=res.value,
         value_linear=res.value_linear, pa=res.potentials[0], pb=res.potentials[1])
    res = ot.solve_sample(x, y, a, b, reg=0.5, lazy=True, batch_size=7, tol=1e-10)
    save("solve_sample_lazy_40x30", x=x, y=y, a=a, b=b, reg=0.5, value_linear=res.value_linear,
         pa=res.potentials[0], pb=res.potentials[1], err=np.array(res.log["err"]), niter=res.log["niter"])
    loss, lg = ot.bregman.empirical_sinkhorn2(x, y, 0.5, a, b, isLazy=True, batchSize=11, numIterMax=300,
                                              stopThr=1e-9, log=True)
    save("emp2_lazy_40x30", x=x, y=y, a=a, b=b, reg=0.5, loss=float(loss), f=lg["u"], g=lg["v"],
         niter=lg["niter"], err=np.array(lg["err"]))
    div = ot.bregman.empirical_sinkhorn_divergence(x, y, 0.5, a, b)
    div_lazy = ot.bregman.empirical_sinkhorn_divergence(x, y, 0.5, a, b, isLazy=True, batchSize=9, stopThr=1e-9)
    save("emp_div_40x30", x=x, y=y, a=a, b=b, reg=0.5, div=float(div), div_lazy=float(div_lazy))


def fused_gw():
    # 12. entropic fused GW (ot/gromov/_bregman.py:997-1241, :1244-1403)
    rng = np.random.default_rng(41)
    xs = rng.standard_normal((30, 2))
    xt = rng.standard_normal((24, 3))
    C1, C2 = ot.dist(xs, xs), ot.dist(xt, xt)
    C1 /= C1.max()
    C2 /= C2.max()
    Fs = rng.standard_normal((30, 4))
    Ft = rng.standard_normal((24, 4)) + 0.5
    M = ot.dist(Fs, Ft)
    M /= M.max()
    p = ot.unif(30)
    q = rng.random(24) + 0.5
    q /= q.sum()
    out = dict(C1=C1, C2=C2, M=M, p=p, q=q)
    for tag, kw in (("pgd", dict(alpha=0.5)), ("pgd_a02_warm", dict(alpha=0.2, warmstart=True)),
                    ("ppa", dict(alpha=0.7, solver="PPA"))):
        (T, lg), w = call_warn(ot.gromov.entropic_fused_gromov_wasserstein, M, C1, C2, p, q, epsilon=0.05,
                               max_iter=200, tol=1e-9, log=True, **kw)
        out[tag + "_T"] = T
        out[tag + "_err"] = np.array(lg["err"], dtype=np.float64)
        out[tag + "_fgw"] = lg["fgw_dist"]
    val, lg2 = ot.gromov.entropic_fused_gromov_wasserstein2(M, C1, C2, p, q, epsilon=0.05, alpha=0.5, max_iter=200,
                                                           tol=1e-9, log=True)
    out["fgw2"] = val
    out["fgw2_quad"] = lg2["quad_loss"]
    out["fgw2_lin"] = lg2["lin_loss"]
    save("fgw_30x24", **out)
    C1a = C1 + 0.3 * rng.random((30, 30))
    (T, lg), w = call_warn(ot.gromov.entropic_fused_gromov_wasserstein, M, C1a, C2, p, q, epsilon=0.05, alpha=0.6,
                           max_iter=200, tol=1e-9, log=True)
    save("fgw_asym_30x24", C1=C1a, C2=C2, M=M, p=p, q=q, T=T, err=np.array(lg["err"]), fgw=lg["fgw_dist"])


def barycenters():
    # 13. entropic barycenters (ot/bregman/_barycenter.py:141-259, :403-473)
    x = np.arange(60, dtype=np.float64)
    M = ot.dist(x.reshape(-1, 1), x.reshape(-1, 1))
    M /= M.max()
    A = np.stack([np.exp(-(x - c) ** 2 / (2 * s ** 2)) for c, s in ((15, 4), (40, 6), (30, 10))], 1)
    A /= A.sum(0, keepdims=True)
    w = np.array([0.2, 0.5, 0.3])
    out = dict(A=A, M=M, w=w)
    for tag, method, reg in (("sk", "sinkhorn", 0.01), ("log", "sinkhorn_log", 0.01), ("log_small", "sinkhorn_log",
                                                                                        1e-3)):
        (bar, lg), wn = call_warn(ot.bregman.barycenter, A, M, reg, weights=w, method=method, numItermax=2000,
                                  stopThr=1e-8, log=True)
        out[tag + "_bar"] = bar
        out[tag + "_err"] = np.array(lg["err"], dtype=np.float64)
        out[tag + "_niter"] = lg["niter"]
        out[tag + "_nonconv"] = int(any("did not converge" in m for m in wn))
    bar = ot.bregman.barycenter(A, M, 0.05)
    out["default_bar"] = bar
    save("bary_60x3", **out)
    rng = np.random.default_rng(51)
    X = rng.standard_normal((300, 2))
    M = ot.dist(X, X)
    M /= M.max()
    A = rng.random((300, 5)) ** 3
    A /= A.sum(0, keepdims=True)
    (bar, lg), wn = call_warn(ot.bregman.barycenter_sinkhorn, A, M, 0.02, numItermax=300, stopThr=1e-9, log=True)
    (bar2, lg2), wn2 = call_warn(ot.bregman.barycenter, A, M, 0.02, method="sinkhorn_log", numItermax=300,
                                 stopThr=1e-9, log=True)
    save("bary_300x5", A=A, x=X, sk_bar=bar, sk_err=np.array(lg["err"]), sk_niter=lg["niter"], log_bar=bar2,
         log_err=np.array(lg2["err"]), log_niter=lg2["niter"])


def unbalanced():
    # 14. unbalanced scaling Sinkhorn (ot/unbalanced/_sinkhorn.py:565-818)
    rng = np.random.default_rng(61)
    x = rng.standard_normal((50, 2))
    y = rng.standard_normal((40, 2)) + 0.7
    M = ot.dist(x, y)
    M /= M.max()
    a = rng.random(50) + 0.1
    a /= a.sum()
    b = 1.5 * (rng.random(40) + 0.1) / 40
    out = dict(x=x, y=y, a=a, b=b, M=M)
    cases = (("kl", dict(reg=0.05, reg_m=1.0)), ("kl_pair", dict(reg=0.05, reg_m=(0.5, float("inf")))),
             ("ent", dict(reg=0.1, reg_m=2.0, reg_type="entropy")), ("kl_small", dict(reg=0.005, reg_m=0.3)),
             ("warm", dict(reg=0.05, reg_m=1.0, warmstart=(rng.standard_normal(50) * 0.1,
                                                           rng.standard_normal(40) * 0.1))),
             ("iter5", dict(reg=0.05, reg_m=1.0, numItermax=5)))
    for tag, kw in cases:
        kw = dict(kw)
        reg, reg_m = kw.pop("reg"), kw.pop("reg_m")
        (P, lg), w = call_warn(ot.unbalanced.sinkhorn_unbalanced, a, b, M, reg, reg_m, log=True, **kw)
        out[tag + "_plan"] = P
        out[tag + "_err"] = np.array(lg["err"], dtype=np.float64)
        out[tag + "_logu"] = lg["logu"]
        out[tag + "_logv"] = lg["logv"]
        out[tag + "_cost"] = lg["cost"]
        out[tag + "_total"] = lg["total_cost"]
        if "warmstart" in kw:
            out["warm_wu"], out["warm_wv"] = kw["warmstart"]
    res = ot.solve(M, a, b, reg=0.05, unbalanced=1.0)
    out["solve_plan"], out["solve_value"], out["solve_value_linear"] = res.plan, res.value, res.value_linear
    out["solve_pa"], out["solve_pb"] = res.potentials
    out["u2_linear"] = ot.unbalanced.sinkhorn_unbalanced2(a, b, M, 0.05, 1.0)
    out["u2_total"] = ot.unbalanced.sinkhorn_unbalanced2(a, b, M, 0.05, 1.0, returnCost="total")
    save("unbal_50x40", **out)


SECTIONS = {"core": core, "next": next_rows, "fgw": fused_gw, "bary": barycenters, "unbal": unbalanced}


def greenkhorn():
    # 12. greedy coordinate Sinkhorn (ot/bregman/_sinkhorn.py:921-1102): the
    # doctest, a symmetric uniform problem (ties between rows and columns), a
    # rectangular weighted one, a warm start, a short budget, empty weights
    def case(name, a, b, M, reg, **kw):
        (G, lg), w = call_warn(ot.sinkhorn, a, b, M, reg, method="greenkhorn", log=True, **kw)
        out = dict(a=a, b=b, M=M, reg=reg, plan=G, n_iter=lg["n_iter"], u=lg["u"], v=lg["v"],
                   warn_nonconv=int(any("did not converge" in s for s in w)))
        for k, val in kw.items():
            if k == "warmstart":
                out["ws_u"], out["ws_v"] = val
            else:
                out["kw_" + k] = val
        save(name, **out)

    a = np.array([0.5, 0.5])
    case("green_doctest_2x2", a, a, np.array([[0.0, 1.0], [1.0, 0.0]]), 1.0)
    rng = np.random.default_rng(41)
    x = rng.standard_normal((100, 2))
    M = ot.dist(x, x)
    u = ot.unif(100)
    case("green_sym_100", u, u, M, 1.0, stopThr=1e-10)
    x = rng.standard_normal((31, 2))
    y = rng.standard_normal((33, 2)) + 0.5
    M = ot.dist(x, y)
    M /= M.max()
    a = rng.random(31) + 0.1
    a /= a.sum()
    b = rng.random(33) + 0.1
    b /= b.sum()
    case("green_31x33_reg0.1", a, b, M, 0.1, stopThr=1e-9)
    case("green_31x33_warm", a, b, M, 0.1, stopThr=1e-9,
         warmstart=(rng.standard_normal(31) * 0.1 - np.log(31), rng.standard_normal(33) * 0.1 - np.log(33)))
    case("green_31x33_iter25", a, b, M, 0.05, numItermax=25)
    case("green_empty_40x50", np.array([]), np.array([]), ot.dist(rng.standard_normal((40, 3)),
                                                                rng.standard_normal((50, 3))), 1.0,
         stopThr=1e-10)


SECTIONS["green"] = greenkhorn


def sinkhorn2_grads():
    # 13. gradients of sinkhorn2 by the reference's own autodiff through its
    # torch-backend iterations (ot/bregman/_sinkhorn.py:435-438; the scenario
    # of test/test_bregman.py:203-225 with values recorded)
    import torch

    def case(name, a, b, M, reg, method, **kw):
        a1 = torch.tensor(a, requires_grad=True)
        b1 = torch.tensor(b, requires_grad=True)
        M1 = torch.tensor(M, requires_grad=True)
        val = ot.sinkhorn2(a1, b1, M1, reg, method=method, **kw)
        val.backward()
        save(name, a=a, b=b, M=M, reg=reg, method=method, loss=float(val.detach()), grad_a=a1.grad.numpy(),
             grad_b=b1.grad.numpy(), grad_M=M1.grad.numpy(), **{"kw_" + k: v for k, v in kw.items()})

    rng = np.random.default_rng(51)
    x = rng.standard_normal((30, 2))
    y = rng.standard_normal((40, 2)) + 0.5
    M = ot.dist(x, y)
    M /= M.max()
    a = rng.random(30) + 0.2
    a /= a.sum()
    b = rng.random(40) + 0.2
    b /= b.sum()
    case("grad2_30x40_knopp", a, b, M, 0.1, "sinkhorn", stopThr=1e-12, numItermax=100000)
    case("grad2_30x40_log", a, b, M, 0.1, "sinkhorn_log", stopThr=1e-12, numItermax=100000)
    x = rng.standard_normal((100, 2))
    y = rng.standard_normal((100, 2))
    u = ot.unif(100)
    case("grad2_100_reg1", u, u, ot.dist(x, y), 1.0, "sinkhorn")


SECTIONS["grad"] = sinkhorn2_grads


def main(names):
    for k in names or list(SECTIONS):
        SECTIONS[k]()


if __name__ == "__main__":
    main(sys.argv[1:])
