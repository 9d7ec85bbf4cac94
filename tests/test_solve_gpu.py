"""Parity of the entropic branches of ``solve`` / ``solve_sample``, of
``empirical_sinkhorn2`` and of ``dist`` with the reference's golden vectors.

Tolerances: dense float64 paths -- plan relative L1 1e-9, values rtol 1e-9,
potentials rtol 1e-8 (the GPU cost is formed from coordinate differences,
the reference's from |x|^2 + |y|^2 - 2 x.y, which differ by rounding);
lazy paths solve in float32 with tensor-core dot products -- plan relative
L1 1e-5 and loss rtol 1e-5 against the float64 golden."""
import warnings

import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from conftest import golden

pytestmark = pytest.mark.gpu


def rel_l1(P, Q):
    return float(np.abs(P - Q).sum() / max(np.abs(Q).sum(), 1e-300))


@pytest.mark.parametrize("name", ["solve_40x30_KL", "solve_40x30_entropy", "solve_40x30_iter7"])
def test_solve_golden(cuda, name):
    g = golden(name)
    kw = dict(max_iter=7, tol=0.0) if name.endswith("iter7") else {}
    reg_type = "entropy" if name.endswith("entropy") else "KL"
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        res = pg.solve(g["M"], g["a"], g["b"], reg=float(g["reg"]), reg_type=reg_type, **kw)
    assert rel_l1(res.plan, g["plan"]) < 1e-9
    assert abs(float(res.value) - float(g["value"])) <= 1e-9 * abs(float(g["value"]))
    assert abs(float(res.value_linear) - float(g["value_linear"])) <= 1e-9 * abs(float(g["value_linear"]))
    np.testing.assert_allclose(res.potentials[0], g["pa"], rtol=1e-8)
    np.testing.assert_allclose(res.potential_b, g["pb"], rtol=1e-8)
    assert any("did not converge" in str(x.message) for x in w) == name.endswith("iter7")


def test_solve_sample_dense_golden(cuda):
    g = golden("solve_sample_40x30")
    res = pg.solve_sample(g["x"], g["y"], g["a"], g["b"], reg=float(g["reg"]))
    assert rel_l1(res.plan, g["plan"]) < 1e-9
    assert abs(float(res.value) - float(g["value"])) <= 1e-9 * abs(float(g["value"]))
    np.testing.assert_allclose(res.potentials[0], g["pa"], rtol=1e-8)


def _lazy_plan(x, y, f, g, reg):
    C = oracle.sqeuclidean(x, y)
    return np.exp(f[:, None] + g[None, :] - C / reg)


def test_solve_sample_lazy_golden(cuda):
    g = golden("solve_sample_lazy_40x30")
    res = pg.solve_sample(g["x"], g["y"], g["a"], g["b"], reg=float(g["reg"]), lazy=True, batch_size=7, tol=1e-6)
    assert res.plan is None and res.value is None
    P = _lazy_plan(g["x"], g["y"], res.potentials[0], res.potentials[1], float(g["reg"]))
    Pref = _lazy_plan(g["x"], g["y"], g["pa"], g["pb"], float(g["reg"]))
    assert rel_l1(P, Pref) <= 1e-5
    assert abs(float(res.value_linear) - float(g["value_linear"])) <= 1e-5 * abs(float(g["value_linear"]))
    assert res.lazy_plan[:2, :3].shape == (2, 3)
    assert res.log["niter"] % 10 == 9


def test_empirical_sinkhorn2_lazy_golden(cuda):
    g = golden("emp2_lazy_40x30")
    loss, lg = pg.empirical_sinkhorn2(g["x"], g["y"], float(g["reg"]), g["a"], g["b"], isLazy=True, batchSize=11,
                                      numIterMax=300, stopThr=1e-6, log=True)
    assert abs(float(loss) - float(g["loss"])) <= 1e-5 * abs(float(g["loss"]))
    # the loss kernel against the same sum in float64 on the returned potentials
    ref = float(np.sum(oracle.sqeuclidean(g["x"], g["y"]) *
                       _lazy_plan(g["x"], g["y"], lg["u"], lg["v"], float(g["reg"]))))
    assert abs(float(loss) - ref) <= 1e-12 * abs(ref)


def test_empirical_sinkhorn2_dense_matches_sinkhorn2(cuda):
    g = golden("emp2_lazy_40x30")
    loss = pg.empirical_sinkhorn2(g["x"], g["y"], float(g["reg"]), g["a"], g["b"], numIterMax=300, stopThr=1e-9)
    M = oracle.sqeuclidean(g["x"], g["y"])
    ref, _ = oracle.sinkhorn2(g["a"], g["b"], M, float(g["reg"]), numItermax=300, stopThr=1e-9)
    assert abs(float(loss) - ref) <= 1e-9 * abs(ref)


def test_dist(cuda):
    rng = np.random.default_rng(5)
    x = rng.standard_normal((37, 5))
    y = rng.standard_normal((23, 5))
    np.testing.assert_allclose(pg.dist(x, y), oracle.sqeuclidean(x, y), rtol=1e-12, atol=1e-12)
    D = pg.dist(x)
    assert np.all(np.diag(D) == 0.0)
    np.testing.assert_allclose(D, oracle.sqeuclidean(x), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(pg.dist(x, y, metric="euclidean"), np.sqrt(oracle.sqeuclidean(x, y)), rtol=1e-12,
                               atol=1e-12)
    xt = torch.tensor(x, dtype=torch.float32, device=cuda)
    assert pg.dist(xt, xt).device.type == "cuda"
    with pytest.raises(NotImplementedError):
        pg.dist(x, y, metric="cityblock")


@pytest.mark.parametrize("grad", ["envelope", "autodiff", "last_step", "detach"])
def test_solve_grad_modes(cuda, grad):
    g = golden("solve_40x30_KL")
    M = torch.tensor(g["M"], device=cuda, requires_grad=True)
    a = torch.tensor(g["a"], device=cuda, requires_grad=True)
    b = torch.tensor(g["b"], device=cuda, requires_grad=True)
    res = pg.solve(M, a, b, reg=float(g["reg"]), grad=grad)
    assert abs(float(res.value.detach()) - float(g["value"])) <= 1e-8 * abs(float(g["value"]))
    if grad == "detach":
        assert not res.value.requires_grad
        return
    res.value.backward()
    assert M.grad.shape == M.shape and a.grad.shape == a.shape and b.grad.shape == b.shape
    if grad in ("envelope", "autodiff"):
        np.testing.assert_allclose(M.grad.cpu().numpy(), g["plan"], rtol=1e-8, atol=1e-14)


def test_solve_not_on_gpu_path(cuda):
    M = np.random.default_rng(0).random((4, 5))
    for kw in (dict(reg=None), dict(reg=1.0, unbalanced=1.0, unbalanced_type="L2"), dict(reg=1.0, reg_type="L2")):
        with pytest.raises(NotImplementedError):
            pg.solve(M, **kw)


def test_solve_f32(cuda):
    g = golden("solve_40x30_KL")
    f = lambda x: torch.tensor(x, dtype=torch.float32, device=cuda)  # noqa: E731
    res = pg.solve(f(g["M"]), f(g["a"]), f(g["b"]), reg=float(g["reg"]), tol=1e-6)
    assert res.plan.dtype == torch.float32
    assert rel_l1(res.plan.double().cpu().numpy(), g["plan"]) <= 1e-5
    assert abs(float(res.value) - float(g["value"])) <= 1e-5 * abs(float(g["value"]))


def test_empirical_sinkhorn_divergence(cuda):
    g = golden("emp_div_40x30")
    d = pg.empirical_sinkhorn_divergence(g["x"], g["y"], float(g["reg"]), g["a"], g["b"])
    assert abs(float(d) - float(g["div"])) <= 1e-8 * abs(float(g["div"]))
    dl = pg.empirical_sinkhorn_divergence(g["x"], g["y"], float(g["reg"]), g["a"], g["b"], isLazy=True, batchSize=9,
                                          stopThr=1e-6)
    assert abs(float(dl) - float(g["div_lazy"])) <= 1e-4 * abs(float(g["div_lazy"]))
