"""Pin the CPU oracle to the reference: every golden vector the reference
produced (tests/golden/gen_golden.py) and its own doctest values."""
import numpy as np
import pytest

import oracle
from conftest import golden, golden_names

DENSE = golden_names("dense_") + ["fail_maxiter1"]


def _M(g):
    if "M" in g:
        return g["M"]
    M = oracle.sqeuclidean(g["x"], g["y"])
    return M / M.max()


def test_doctest_values():
    g = golden("doctest_2x2")
    P, _ = oracle.sinkhorn(g["a"], g["b"], g["M"], 1.0)
    np.testing.assert_allclose(P, [[0.36552929, 0.13447071], [0.13447071, 0.36552929]], atol=1e-8)
    loss, _ = oracle.sinkhorn2(g["a"], g["b"], g["M"], 1.0)
    assert abs(loss - 0.26894142136999516) < 1e-15
    np.testing.assert_allclose(P, g["plan"], rtol=1e-14)


@pytest.mark.parametrize("name", DENSE)
@pytest.mark.parametrize("tag", ["knopp", "log"])
def test_dense_against_reference(name, tag):
    g = golden(name)
    M = _M(g)
    fn = oracle.sinkhorn_knopp if tag == "knopp" else oracle.sinkhorn_log
    P, lg = fn(g["a"], g["b"], M, float(g["reg"]), int(g["numItermax"]), float(g["stopThr"]))
    assert lg["niter"] == int(g[tag + "_niter"])
    np.testing.assert_allclose(lg["err"], g[tag + "_err"], rtol=1e-7, atol=1e-15)
    np.testing.assert_allclose(lg["u"], g[tag + "_u"], rtol=1e-9)
    np.testing.assert_allclose(lg["v"], g[tag + "_v"], rtol=1e-9)
    assert abs(float(np.sum(M * P)) - float(g[tag + "_loss"])) <= 1e-10 * abs(float(g[tag + "_loss"])) + 1e-300
    if tag + "_plan" in g:
        np.testing.assert_allclose(P, g[tag + "_plan"], rtol=1e-8, atol=1e-300)
    assert int(any("did not converge" in w for w in lg["_warnings"])) == int(g[tag + "_warn_nonconv"])


def test_reg0_numerical_error_reverts():
    g = golden("fail_reg0_knopp")
    _, lg = oracle.sinkhorn_knopp(g["a"], g["b"], g["M"], 0.0)
    assert lg["niter"] == int(g["niter"])
    assert any("numerical errors" in w for w in lg["_warnings"]) == bool(g["warn_numerr"])
    np.testing.assert_allclose(lg["u"], g["u"])
    np.testing.assert_allclose(lg["v"], g["v"])


@pytest.mark.parametrize("tag", ["knopp", "log"])
def test_multi_histogram(tag):
    g = golden("multib_31x3")
    method = "sinkhorn" if tag == "knopp" else "sinkhorn_log"
    loss, lg = oracle.sinkhorn2(g["a"], g["b"], g["M"], 1.0, method=method, stopThr=1e-10)
    np.testing.assert_allclose(loss, g[tag + "_loss"], rtol=1e-10)
    np.testing.assert_allclose(lg["u"], g[tag + "_u"], rtol=1e-8)
    np.testing.assert_allclose(lg["v"], g[tag + "_v"], rtol=1e-8)


@pytest.mark.parametrize("solver", ["log_sinkhorn", "sinkhorn"])
@pytest.mark.parametrize("reg_type", ["entropy", "kl"])
def test_batch(solver, reg_type):
    g = golden("batch_4x16")
    r = oracle.solve_batch(g["M"], 0.1, max_iter=10000, tol=1e-5, solver=solver, reg_type=reg_type)
    tag = "%s_%s" % (solver, reg_type)
    assert r["n_iter"] == int(g[tag + "_n_iter"])
    np.testing.assert_allclose(r["plan"], g[tag + "_plan"], rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(r["value"], g[tag + "_value"], rtol=1e-9)
    np.testing.assert_allclose(r["value_linear"], g[tag + "_value_linear"], rtol=1e-9)
    np.testing.assert_allclose(r["potentials"][0], g[tag + "_pot_u"], rtol=1e-9)


def test_batch_padded_ragged():
    g = golden("batch_ragged_padded")
    r = oracle.solve_batch(g["M"], float(g["reg"]), g["a"], g["b"], max_iter=20000, tol=1e-9)
    assert r["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(r["plan"], g["plan"], rtol=1e-8, atol=1e-300)


def test_batch_sample():
    g = golden("batch_sample_3x20x25")
    X, Y = g["X"], g["Y"]
    M = np.stack([oracle.sqeuclidean(X[k], Y[k]) for k in range(X.shape[0])])
    r = oracle.solve_batch(M, float(g["reg"]), max_iter=5000, tol=1e-7)
    assert r["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(r["plan"], g["plan"], rtol=1e-7, atol=1e-14)


@pytest.mark.parametrize("tag,kw", [("pgd", {}), ("pgd_warm", {"warmstart": True}), ("ppa", {"solver": "PPA"})])
def test_egw_small(tag, kw):
    g = golden("egw_10")
    T, lg = oracle.entropic_gromov_wasserstein(g["C1"], g["C2"], g["p"], g["q"], 1e-2, max_iter=10, **kw)
    np.testing.assert_allclose(T, g[tag + "_T"], rtol=1e-8, atol=1e-14)
    assert abs(lg["gw_dist"] - float(g[tag + "_gw"])) < 1e-10
    np.testing.assert_allclose(lg["err"], g[tag + "_err"], rtol=1e-6, atol=1e-14)


@pytest.mark.parametrize("name", ["egw_48x40", "egw_asym_48x40"])
def test_egw_medium(name):
    g = golden(name)
    kw = dict(max_iter=20, tol=1e-9, numItermax=2000, stopThr=1e-9) if name == "egw_48x40" else dict(max_iter=10)
    T, lg = oracle.entropic_gromov_wasserstein(g["C1"], g["C2"], epsilon=5e-2, **kw)
    np.testing.assert_allclose(T, g["T"], rtol=1e-7, atol=1e-13)
    assert abs(lg["gw_dist"] - float(g["gw"])) < 1e-9


def test_lazy():
    g = golden("lazy_60x50")
    f, gg, lg = oracle.empirical_sinkhorn_lazy(g["X"], g["Y"], 1.0, batchSize=7, numIterMax=500, stopThr=1e-9)
    assert lg["niter"] == int(g["niter"])
    np.testing.assert_allclose(f, g["f"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(gg, g["g"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(lg["err"], g["err"], rtol=1e-6, atol=1e-15)


def test_warmstart_net_gradients_match_finite_differences():
    """Pins the network oracle: analytic gradients vs central differences."""
    from oracle import warmstart_net as wn
    from pot_gb300.warmstart.net import init_params
    rng = np.random.default_rng(0)
    d = 3
    params = {k: v.astype(np.float64) for k, v in init_params(d, seed=1, h1=6, h2=5, h3=7).items()}
    for k in params:
        if k.startswith("b"):
            params[k] = rng.standard_normal(params[k].shape) * 0.1
    X = rng.standard_normal((2, 9, d))
    Y = rng.standard_normal((2, 8, d))
    t = rng.standard_normal((2, 9))
    t -= t.mean(1, keepdims=True)
    loss, g, _ = wn.loss_and_grads(params, X, Y, t)
    h = 1e-6
    for name in params:
        flat = params[name].reshape(-1)
        for idx in rng.choice(flat.size, size=min(4, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + h
            lp, _, _ = wn.loss_and_grads(params, X, Y, t)
            flat[idx] = old - h
            lm, _, _ = wn.loss_and_grads(params, X, Y, t)
            flat[idx] = old
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[name].reshape(-1)[idx]) <= 1e-6 + 1e-5 * abs(fd), (name, idx, fd, g[name].reshape(-1)[idx])


@pytest.mark.parametrize("name", ["gromov_batch_fused", "gromov_batch_sym"])
def test_gromov_batch(name):
    g = golden(name)
    if name == "gromov_batch_fused":
        r = oracle.solve_gromov_batch(g["C1"], g["C2"], reg=0.01, M=g["M"], alpha=0.5, max_iter=1000, tol=1e-5,
                                      max_iter_inner=10000, tol_inner=1e-5, symmetric=False)
        np.testing.assert_allclose(r["value_linear"], g["value_linear"], rtol=1e-8)
    else:
        r = oracle.solve_gromov_batch(g["C1"], g["C2"], reg=0.05, max_iter=50, tol=1e-7, max_iter_inner=2000,
                                      tol_inner=1e-9)
    assert r["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(r["plan"], g["plan"], rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(r["value"], g["value"], rtol=1e-8)
    np.testing.assert_allclose(r["value_quad"], g["value_quad"], rtol=1e-8)


STAB = golden_names("stab_")


def _stab_kw(g):
    kw = {k[3:]: (int(v) if k in ("kw_numItermax", "kw_print_period") else float(v))
          for k, v in g.items() if k.startswith("kw_")}
    if "ws_alpha" in g:
        kw["warmstart"] = (g["ws_alpha"], g["ws_beta"])
    return kw


@pytest.mark.parametrize("name", STAB)
def test_stabilized(name):
    g = golden(name)
    M = _M(g)
    P, lg = oracle.sinkhorn_stabilized(g["a"], g["b"], M, float(g["reg"]), **_stab_kw(g))
    assert lg["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(lg["err"], g["err"], rtol=1e-7, atol=1e-15)
    np.testing.assert_allclose(lg["logu"], g["logu"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(lg["logv"], g["logv"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(lg["alpha"], g["alpha"], rtol=1e-9, atol=1e-12)
    assert abs(float(np.sum(M * P)) - float(g["loss"])) <= 1e-9 * abs(float(g["loss"]))
    if "plan" in g:
        np.testing.assert_allclose(P, g["plan"], rtol=1e-8, atol=1e-300)
    assert (oracle.NONCONV in lg["_warnings"]) == bool(g["warn_nonconv"])


@pytest.mark.parametrize("name", golden_names("epsscale_"))
def test_epsilon_scaling(name):
    g = golden(name)
    kw = {k[3:]: (float(v) if k == "kw_epsilon0" else int(v)) for k, v in g.items() if k.startswith("kw_")}
    G, lg = oracle.sinkhorn_epsilon_scaling(g["a"], g["b"], g["M"], float(g["reg"]), **kw)
    assert lg["niter"] == int(g["niter"])
    np.testing.assert_allclose(lg["err"], g["err"], rtol=1e-6, atol=1e-20)
    np.testing.assert_allclose(G, g["plan"], rtol=1e-7, atol=1e-300)
    np.testing.assert_allclose(lg["alpha"], g["alpha"], rtol=1e-8, atol=1e-12)
    assert sum(w == oracle.NONCONV for w in lg["_warnings"]) == int(g["warn_nonconv"])


@pytest.mark.parametrize("name", ["solve_40x30_KL", "solve_40x30_entropy", "solve_40x30_iter7"])
def test_solve_entropic(name):
    g = golden(name)
    kw = dict(max_iter=7, tol=0.0) if name.endswith("iter7") else {}
    r = oracle.solve_entropic(g["M"], g["a"], g["b"], float(g["reg"]),
                              reg_type="entropy" if name.endswith("entropy") else "KL", **kw)
    np.testing.assert_allclose(r["plan"], g["plan"], rtol=1e-10)
    assert abs(r["value"] - float(g["value"])) <= 1e-10 * abs(float(g["value"]))
    assert abs(r["value_linear"] - float(g["value_linear"])) <= 1e-10 * abs(float(g["value_linear"]))
    np.testing.assert_allclose(r["potentials"][0], g["pa"], rtol=1e-10)


def test_empirical_sinkhorn2_lazy():
    g = golden("emp2_lazy_40x30")
    loss, lg = oracle.empirical_sinkhorn2_lazy(g["x"], g["y"], float(g["reg"]), g["a"], g["b"], numIterMax=300,
                                               stopThr=1e-9, batchSize=11)
    assert lg["niter"] == int(g["niter"])
    assert abs(loss - float(g["loss"])) <= 1e-10 * abs(float(g["loss"]))
    np.testing.assert_allclose(lg["u"], g["f"], rtol=1e-10)
    g = golden("solve_sample_lazy_40x30")
    loss, lg = oracle.empirical_sinkhorn2_lazy(g["x"], g["y"], float(g["reg"]), g["a"], g["b"], numIterMax=1000,
                                               stopThr=1e-10, batchSize=7)
    assert lg["niter"] == int(g["niter"])
    assert abs(loss - float(g["value_linear"])) <= 1e-10 * abs(loss)
    np.testing.assert_allclose(lg["u"], g["pa"], rtol=1e-10)


@pytest.mark.parametrize("tag,kw", [("pgd", dict(alpha=0.5)), ("pgd_a02_warm", dict(alpha=0.2, warmstart=True)),
                                    ("ppa", dict(alpha=0.7, solver="PPA"))])
def test_fused_gw(tag, kw):
    g = golden("fgw_30x24")
    T, lg = oracle.entropic_fused_gromov_wasserstein(g["M"], g["C1"], g["C2"], g["p"], g["q"], epsilon=0.05,
                                                     max_iter=200, tol=1e-9, **kw)
    np.testing.assert_allclose(T, g[tag + "_T"], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(lg["err"], g[tag + "_err"], rtol=1e-7, atol=1e-15)
    assert abs(lg["fgw_dist"] - float(g[tag + "_fgw"])) <= 1e-10 * abs(float(g[tag + "_fgw"]))


def test_fused_gw_asymmetric():
    g = golden("fgw_asym_30x24")
    T, lg = oracle.entropic_fused_gromov_wasserstein(g["M"], g["C1"], g["C2"], g["p"], g["q"], epsilon=0.05,
                                                     alpha=0.6, max_iter=200, tol=1e-9)
    np.testing.assert_allclose(T, g["T"], rtol=1e-9, atol=1e-15)
    assert abs(lg["fgw_dist"] - float(g["fgw"])) <= 1e-10 * abs(float(g["fgw"]))


@pytest.mark.parametrize("tag,reg", [("sk", 0.01), ("log", 0.01), ("log_small", 1e-3)])
def test_barycenter(tag, reg):
    g = golden("bary_60x3")
    fn = oracle.barycenter_sinkhorn if tag == "sk" else oracle.barycenter_sinkhorn_log
    bar, lg = fn(g["A"], g["M"], reg, g["w"], numItermax=2000, stopThr=1e-8)
    assert lg["niter"] == int(g[tag + "_niter"])
    np.testing.assert_allclose(lg["err"], g[tag + "_err"], rtol=1e-6, atol=1e-16)
    np.testing.assert_allclose(bar, g[tag + "_bar"], rtol=1e-9, atol=1e-300)
    assert (oracle.NONCONV in lg["_warnings"]) == bool(g[tag + "_nonconv"])
    bar, _ = oracle.barycenter_sinkhorn(g["A"], g["M"], 0.05)
    np.testing.assert_allclose(bar, g["default_bar"], rtol=1e-9)


def test_barycenter_300():
    g = golden("bary_300x5")
    M = oracle.sqeuclidean(g["x"])
    M /= M.max()
    for tag, fn in (("sk", oracle.barycenter_sinkhorn), ("log", oracle.barycenter_sinkhorn_log)):
        bar, lg = fn(g["A"], M, 0.02, numItermax=300, stopThr=1e-9)
        assert lg["niter"] == int(g[tag + "_niter"])
        np.testing.assert_allclose(bar, g[tag + "_bar"], rtol=1e-8, atol=1e-300)


UNBAL = [("kl", dict(reg=0.05, reg_m=1.0)), ("kl_pair", dict(reg=0.05, reg_m=(0.5, float("inf")))),
         ("ent", dict(reg=0.1, reg_m=2.0, reg_type="entropy")), ("kl_small", dict(reg=0.005, reg_m=0.3)),
         ("warm", dict(reg=0.05, reg_m=1.0)), ("iter5", dict(reg=0.05, reg_m=1.0, numItermax=5))]


@pytest.mark.parametrize("tag,kw", UNBAL)
def test_unbalanced(tag, kw):
    g = golden("unbal_50x40")
    kw = dict(kw)
    reg, reg_m = kw.pop("reg"), kw.pop("reg_m")
    if tag == "warm":
        kw["warmstart"] = (g["warm_wu"], g["warm_wv"])
    P, lg = oracle.sinkhorn_knopp_unbalanced(g["a"], g["b"], g["M"], reg, reg_m, **kw)
    assert len(lg["err"]) == len(g[tag + "_err"])
    np.testing.assert_allclose(lg["err"], g[tag + "_err"], rtol=1e-7, atol=1e-15)
    np.testing.assert_allclose(P, g[tag + "_plan"], rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(lg["logu"], g[tag + "_logu"], rtol=1e-9, atol=1e-12)
    assert abs(lg["total_cost"] - float(g[tag + "_total"])) <= 1e-9 * abs(float(g[tag + "_total"]))


def test_accelerated_oracles_reach_the_solution_faster():
    """The over-relaxed and Anderson-accelerated restatements (the checkers of
    the warm-start refinement) are sinkhorn_log with the acceleration off, and
    reach the same solution in fewer iterations with it on."""
    from oracle import accelerated as acc
    rng = np.random.default_rng(5)
    n, m = 120, 100
    X = rng.standard_normal((n, 4))
    Y = rng.standard_normal((m, 4)) * 0.7 + 0.5
    M = oracle.sqeuclidean(X, Y)
    M /= M.max()
    a, b = rng.dirichlet(np.ones(n) * 3), rng.dirichlet(np.ones(m) * 3)
    reg = 0.02
    _, lg = oracle.sinkhorn_log(a, b, M, reg, numItermax=20000, stopThr=1e-9)
    u1, v1, it1, _ = acc.sinkhorn_log_relaxed(a, b, M, reg, omega=1.0, numItermax=20000, stopThr=1e-9)
    assert it1 == lg["niter"]
    np.testing.assert_allclose(u1, lg["log_u"], rtol=1e-12, atol=1e-12)
    ur, vr, itr, _ = acc.sinkhorn_log_relaxed(a, b, M, reg, omega=1.5, numItermax=20000, stopThr=1e-9,
                                              check_period=1)
    ua, va, ita, errs = acc.sinkhorn_log_anderson(a, b, M, reg, depth=5, numItermax=20000, stopThr=1e-9)
    assert errs[-1] < 1e-9 and itr < it1 and ita < itr
    for u, v in ((ur, vr), (ua, va)):
        P = np.exp(-M / reg + u[:, None] + v[None, :])
        P0 = np.exp(-M / reg + lg["log_u"][:, None] + lg["log_v"][None, :])
        assert np.abs(P - P0).sum() / P0.sum() < 1e-6


def _green_kw(g):
    kw = {k[3:]: g[k].item() for k in g if k.startswith("kw_")}
    if "ws_u" in g:
        kw["warmstart"] = (g["ws_u"], g["ws_v"])
    return kw


@pytest.mark.parametrize("name", golden_names("green_"))
def test_greenkhorn(name):
    """The greedy coordinate restatement follows the reference step by step:
    same choices, so the same plan, scalings and last index, bit for bit."""
    g = golden(name)
    P, lg = oracle.sinkhorn(g["a"], g["b"], g["M"], float(g["reg"]), method="greenkhorn", **_green_kw(g))
    assert lg["n_iter"] == int(g["n_iter"])
    np.testing.assert_array_equal(P, g["plan"])
    np.testing.assert_array_equal(lg["u"], g["u"])
    np.testing.assert_array_equal(lg["v"], g["v"])
    assert (oracle.NONCONV in lg["_warnings"]) == bool(g["warn_nonconv"])


def test_greenkhorn_doctest():
    """ot/bregman/_sinkhorn.py:995-1001."""
    P, _ = oracle.greenkhorn([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0)
    np.testing.assert_allclose(P, [[0.36552929, 0.13447071], [0.13447071, 0.36552929]], atol=1e-8)
