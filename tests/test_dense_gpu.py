"""Parity of the dense GPU Sinkhorn (both forms) with the oracle and with the
reference's golden vectors.

Tolerances:
  float64 inputs  -> potentials rtol 1e-8, plan relative L1 1e-9, identical
                     niter and error history (rtol 1e-6) as the reference.
  float32 inputs  -> plan relative L1 <= 1e-5 against the float64 oracle and
                     float64 marginal violation of the returned plan <= 2x
                     stopThr (the GPU stops on its own fp32 error estimate).
"""
import warnings

import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from conftest import golden, golden_names

pytestmark = pytest.mark.gpu

DENSE = golden_names("dense_")


def _M(g):
    if "M" in g:
        return g["M"]
    M = oracle.sqeuclidean(g["x"], g["y"])
    return M / M.max()


def rel_l1(P, Q):
    return float(np.abs(P - Q).sum() / max(np.abs(Q).sum(), 1e-300))


def test_doctest_values(cuda):
    a = [0.5, 0.5]
    M = [[0.0, 1.0], [1.0, 0.0]]
    P = pg.sinkhorn(a, a, M, 1)
    np.testing.assert_allclose(P, [[0.36552929, 0.13447071], [0.13447071, 0.36552929]], atol=1e-8)
    loss = pg.sinkhorn2(a, a, M, 1)
    assert abs(float(loss) - 0.26894142136999516) < 1e-14


@pytest.mark.parametrize("name", DENSE)
@pytest.mark.parametrize("tag", ["knopp", "log"])
def test_dense_f64_golden(cuda, name, tag):
    g = golden(name)
    M = _M(g)
    method = "sinkhorn" if tag == "knopp" else "sinkhorn_log"
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        P, lg = pg.sinkhorn(g["a"], g["b"], M, float(g["reg"]), method=method,
                            numItermax=int(g["numItermax"]), stopThr=float(g["stopThr"]), log=True)
    assert lg["niter"] == int(g[tag + "_niter"])
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), g[tag + "_err"], rtol=1e-6, atol=1e-14)
    np.testing.assert_allclose(lg["u"], g[tag + "_u"], rtol=1e-8)
    np.testing.assert_allclose(lg["v"], g[tag + "_v"], rtol=1e-8)
    Pref, _ = oracle.sinkhorn(g["a"], g["b"], M, float(g["reg"]), method=method,
                              numItermax=int(g["numItermax"]), stopThr=float(g["stopThr"]))
    assert rel_l1(P, Pref) < 1e-9
    loss = pg.sinkhorn2(g["a"], g["b"], M, float(g["reg"]), method=method,
                        numItermax=int(g["numItermax"]), stopThr=float(g["stopThr"]))
    assert abs(float(loss) - float(g[tag + "_loss"])) <= 1e-9 * abs(float(g[tag + "_loss"])) + 1e-15
    nonconv = any("did not converge" in str(x.message) for x in w)
    assert nonconv == bool(g[tag + "_warn_nonconv"])


@pytest.mark.parametrize("name", ["dense_1024_gauss2d", "dense_127x129_reg0.05", "dense_5x300_reg0.5",
                                  "dense_31x33_reg0.5"])
@pytest.mark.parametrize("method", ["sinkhorn", "sinkhorn_log"])
def test_dense_f32_vs_oracle(cuda, name, method):
    g = golden(name)
    M = _M(g)
    stop = 1e-6
    Pref, _ = oracle.sinkhorn(g["a"], g["b"], M, float(g["reg"]), method=method, numItermax=5000,
                              stopThr=1e-12)
    Mt = torch.tensor(M, dtype=torch.float32, device=cuda)
    at = torch.tensor(g["a"], dtype=torch.float32, device=cuda)
    bt = torch.tensor(g["b"], dtype=torch.float32, device=cuda)
    P = pg.sinkhorn(at, bt, Mt, float(g["reg"]), method=method, numItermax=5000, stopThr=stop)
    assert P.dtype == torch.float32 and P.device.type == "cuda"
    P = P.double().cpu().numpy()
    assert rel_l1(P, Pref) <= 1e-5
    viol = np.linalg.norm(P.sum(0) - g["b"])
    assert viol <= 2 * stop


def test_failure_maxiter_warns(cuda):
    g = golden("fail_maxiter1")
    for method in ("sinkhorn", "sinkhorn_log"):
        with pytest.warns(UserWarning, match="did not converge"):
            pg.sinkhorn(g["a"], g["b"], g["M"], 1.0, method=method, stopThr=0, numItermax=1)
        with warnings.catch_warnings():
            warnings.simplefilter("error")
            pg.sinkhorn2(g["a"], g["b"], g["M"], 1.0, method=method, stopThr=0, numItermax=1, warn=False)


def test_reg0_numerical_error_reverts(cuda):
    g = golden("fail_reg0_knopp")
    with pytest.warns(UserWarning, match="numerical errors"):
        _, lg = pg.sinkhorn(g["a"], g["b"], g["M"], 0.0, method="sinkhorn", warn=False, log=True)
    assert lg["niter"] == int(g["niter"])
    np.testing.assert_allclose(lg["u"], g["u"])
    np.testing.assert_allclose(lg["v"], g["v"])


def test_empty_weights_mean_uniform(cuda):
    rng = np.random.default_rng(1)
    M = rng.random((20, 30))
    P1 = pg.sinkhorn([], [], M, 0.5, method="sinkhorn_log")
    P2 = pg.sinkhorn(np.full(20, 1 / 20), np.full(30, 1 / 30), M, 0.5, method="sinkhorn_log")
    np.testing.assert_allclose(P1, P2, rtol=1e-12)


def test_warmstart_matches_oracle(cuda):
    g = golden("dense_100x100_reg0.05")
    rng = np.random.default_rng(2)
    wu = rng.standard_normal(100) * 0.1
    wv = rng.standard_normal(100) * 0.1
    for method in ("sinkhorn", "sinkhorn_log"):
        Pref, lref = oracle.sinkhorn(g["a"], g["b"], g["M"], 0.05, method=method, warmstart=(wu, wv))
        P, lg = pg.sinkhorn(g["a"], g["b"], g["M"], 0.05, method=method, warmstart=(wu, wv), log=True)
        assert lg["niter"] == lref["niter"]
        assert rel_l1(P, Pref) < 1e-9


def test_torch_cuda_in_torch_cuda_out(cuda):
    M = torch.rand(33, 17, dtype=torch.float64, device=cuda)
    a = torch.full((33,), 1 / 33, dtype=torch.float64, device=cuda)
    b = torch.full((17,), 1 / 17, dtype=torch.float64, device=cuda)
    for method in ("sinkhorn", "sinkhorn_log"):
        P, lg = pg.sinkhorn(a, b, M, 0.2, method=method, log=True)
        assert P.device == M.device and P.dtype == M.dtype
        assert isinstance(lg["err"][0], torch.Tensor)
        loss = pg.sinkhorn2(a, b, M, 0.2, method=method)
        assert loss.dim() == 0 and loss.device == M.device
        Pref, _ = oracle.sinkhorn(a.cpu().numpy(), b.cpu().numpy(), M.cpu().numpy(), 0.2, method=method)
        assert rel_l1(P.cpu().numpy(), Pref) < 1e-9


@pytest.mark.parametrize("method", ["sinkhorn", "sinkhorn_log"])
def test_sinkhorn2_gradients_shapes(cuda, method):
    n = 20
    rng = np.random.default_rng(0)
    x = rng.standard_normal((n, 2))
    M = torch.tensor(oracle.sqeuclidean(x, x), device=cuda, requires_grad=True)
    a = torch.full((n,), 1 / n, dtype=torch.float64, device=cuda, requires_grad=True)
    b = torch.full((n,), 1 / n, dtype=torch.float64, device=cuda, requires_grad=True)
    loss = pg.sinkhorn2(a, b, M, 1.0, method=method)
    loss.backward()
    assert M.grad.shape == M.shape and a.grad.shape == a.shape and b.grad.shape == b.shape


def test_log_multi_histogram(cuda):
    g = golden("multib_31x3")
    loss, lg = pg.sinkhorn2(g["a"], g["b"], g["M"], 1.0, method="sinkhorn_log", log=True, stopThr=1e-10)
    np.testing.assert_allclose(loss, g["log_loss"], rtol=1e-9)
    np.testing.assert_allclose(lg["u"], g["log_u"], rtol=1e-7)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_log_multi_histogram_matches_single_solves(cuda, dtype):
    """Several histograms in one batch launch: every histogram exactly as its
    own sinkhorn_log solve (the reference's recursion), warm starts per
    histogram included; float32 with 7 columns exercises the padded block."""
    rng = np.random.default_rng(5)
    n, m, H = 90, 7 if dtype == np.float32 else 40, 4
    M = rng.random((n, m)).astype(dtype)
    a = np.full(n, 1.0 / n, dtype=dtype)
    B = rng.dirichlet(np.ones(m), size=H).T.astype(dtype)
    ws = [(rng.standard_normal(n).astype(dtype) * 0.1, np.zeros(m, dtype=dtype)) for _ in range(H)]
    thr = 1e-9 if dtype == np.float64 else 1e-6
    loss, lg = pg.sinkhorn2(a, B, M, 0.2, method="sinkhorn_log", log=True, stopThr=thr, warmstart=ws)
    for k in range(H):
        lk, lgk = pg.sinkhorn2(a, B[:, k], M, 0.2, method="sinkhorn_log", log=True, stopThr=thr, warmstart=ws[k])
        tol = 1e-12 if dtype == np.float64 else 2e-5
        np.testing.assert_allclose(loss[k], lk, rtol=tol)
        np.testing.assert_allclose(lg["log_u"][:, k], lgk["log_u"], rtol=tol, atol=tol)
        np.testing.assert_allclose(lg["log_v"][:, k], lgk["log_v"], rtol=tol, atol=tol)


def test_knopp_multi_histogram(cuda):
    g = golden("multib_31x3")
    loss, lg = pg.sinkhorn2(g["a"], g["b"], g["M"], 1.0, method="sinkhorn", log=True, stopThr=1e-10)
    np.testing.assert_allclose(loss, g["knopp_loss"], rtol=1e-9)
    np.testing.assert_allclose(lg["u"], g["knopp_u"], rtol=1e-8)
    np.testing.assert_allclose(lg["v"], g["knopp_v"], rtol=1e-8)
    lref, lgr = oracle.sinkhorn_knopp(g["a"], g["b"], g["M"], 1.0, stopThr=1e-10)
    assert lg["niter"] == lgr["niter"]
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), lgr["err"], rtol=1e-6)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("shape", [(300, 256), (127, 129)])
def test_precomputed_gibbs_kernel_is_bit_identical(cuda, dtype, shape):
    """The scaling form over a stored K = exp(-M/reg) (otg_gibbs_kernel, the
    float64 default) runs the same iterates as exponentiating every entry
    in the passes: identical potentials, stop index and error history."""
    from pot_gb300 import bregman, _lib
    n, m = shape
    rng = np.random.default_rng(3)
    M = oracle.sqeuclidean(rng.normal(size=(n, 2)), rng.normal(size=(m, 2)) + 1.0)
    M = torch.tensor(M / M.max(), dtype=dtype, device=cuda)
    a = torch.tensor(rng.dirichlet(np.ones(n)), dtype=dtype, device=cuda)
    b = torch.tensor(rng.dirichlet(np.ones(m)), dtype=dtype, device=cuda)
    r0 = bregman.solve_dense(M, a, b, 0.05, _lib.OTG_METHOD_KNOPP, 1000, 1e-9, gibbs=False)
    r1 = bregman.solve_dense(M, a, b, 0.05, _lib.OTG_METHOD_KNOPP, 1000, 1e-9, gibbs=True)
    assert r1.K is not None and r0.K is None
    assert r0.niter == r1.niter and r0.status == r1.status
    np.testing.assert_array_equal(r0.errs, r1.errs)
    np.testing.assert_array_equal(r0.u.cpu().numpy(), r1.u.cpu().numpy())
    np.testing.assert_array_equal(r0.v.cpu().numpy(), r1.v.cpu().numpy())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("method", ["sinkhorn", "sinkhorn_log"])
def test_error_history_is_reproducible(cuda, dtype, method):
    """The squared marginal error of a check is summed over fixed slots in a
    fixed order (which CTA merges a slab varies from run to run, the order
    of the sum does not): ten solves give bit-identical error histories,
    stop indices and potentials."""
    from pot_gb300 import bregman, _lib
    n, m = 700, 3000
    rng = np.random.default_rng(11)
    M = oracle.sqeuclidean(rng.normal(size=(n, 2)), rng.normal(size=(m, 2)) + 1.0)
    M = torch.tensor(M / M.max(), dtype=dtype, device=cuda)
    a = torch.tensor(rng.dirichlet(np.ones(n)), dtype=dtype, device=cuda)
    b = torch.tensor(rng.dirichlet(np.ones(m)), dtype=dtype, device=cuda)
    code = _lib.OTG_METHOD_LOG if method == "sinkhorn_log" else _lib.OTG_METHOD_KNOPP
    stop = 1e-9 if dtype == torch.float64 else 1e-6
    runs = [bregman.solve_dense(M, a, b, 0.02, code, 2000, stop, gibbs=False) for _ in range(10)]
    for r in runs[1:]:
        assert r.niter == runs[0].niter and r.status == runs[0].status
        np.testing.assert_array_equal(r.errs, runs[0].errs)
        assert torch.equal(r.u, runs[0].u) and torch.equal(r.v, runs[0].v)
