"""Greenkhorn on the GPU (``otg_greenkhorn``) against the reference's golden
runs and the float64 oracle.

The GPU chain sums its dot products in another order than numpy's BLAS, so
its violations differ from the reference's in the last bits.  Unless two
candidate violations come within that rounding of each other, it makes the
reference's choices step for step: same last index, plan and scalings to
rounding.  A symmetric problem with a == b (rows and columns tie at the
start) gets the reference's own cross-method tolerance on the plan.
"""
import warnings

import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from conftest import golden, golden_names

pytestmark = pytest.mark.gpu

TIED = {"green_sym_100"}  # a == b and M symmetric: the first step is an exact row/column tie


def _kw(g):
    kw = {k[3:]: g[k].item() for k in g if k.startswith("kw_")}
    if "ws_u" in g:
        kw["warmstart"] = (g["ws_u"], g["ws_v"])
    return kw


def _run(g, **extra):
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        P, lg = pg.sinkhorn(g["a"], g["b"], g["M"], float(g["reg"]), method="greenkhorn", log=True,
                            **_kw(g), **extra)
    return P, lg, [str(x.message) for x in w]


@pytest.mark.parametrize("name", golden_names("green_"))
def test_golden(cuda, name):
    g = golden(name)
    P, lg, w = _run(g)
    assert isinstance(P, np.ndarray) and P.dtype == np.float64
    assert any("did not converge" in s for s in w) == bool(g["warn_nonconv"])
    if name in TIED:
        # both chains ran the full budget; the plans agree as the reference's
        # own variants test asks (test/test_bregman.py:284, atol 1e-5)
        assert lg["n_iter"] == int(g["n_iter"])
        np.testing.assert_allclose(P, g["plan"], atol=1e-5)
        return
    assert lg["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(P, g["plan"], rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(lg["u"], g["u"], rtol=1e-9)
    np.testing.assert_allclose(lg["v"], g["v"], rtol=1e-9)


def test_doctest(cuda):
    """ot/bregman/_sinkhorn.py:995-1001."""
    P = pg.greenkhorn([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1)
    np.testing.assert_allclose(P, [[0.36552929, 0.13447071], [0.13447071, 0.36552929]], atol=1e-8)


def test_bit_identical_runs(cuda):
    g = golden("green_31x33_reg0.1")
    M = torch.tensor(g["M"], device=cuda)
    a = torch.tensor(g["a"], device=cuda)
    b = torch.tensor(g["b"], device=cuda)
    P1, l1 = pg.greenkhorn(a, b, M, 0.1, stopThr=1e-12, numItermax=3000, log=True, warn=False)
    P2, l2 = pg.greenkhorn(a, b, M, 0.1, stopThr=1e-12, numItermax=3000, log=True, warn=False)
    assert P1.is_cuda and P1.dtype == torch.float64
    assert l1["n_iter"] == l2["n_iter"]
    assert torch.equal(P1, P2) and torch.equal(l1["u"], l2["u"]) and torch.equal(l1["v"], l2["v"])


def test_larger_against_oracle(cuda):
    rng = np.random.default_rng(42)
    n, m = 600, 700
    x = rng.standard_normal((n, 3))
    y = rng.standard_normal((m, 3)) + 0.3
    M = oracle.sqeuclidean(x, y)
    M /= M.max()
    a = rng.dirichlet(np.ones(n) * 5)
    b = rng.dirichlet(np.ones(m) * 5)
    Po, lo = oracle.greenkhorn(a, b, M, 0.03, numItermax=200000, stopThr=1e-9)
    assert not lo["_warnings"]
    P, lg = pg.greenkhorn(a, b, M, 0.03, numItermax=200000, stopThr=1e-9, log=True)
    # both stop at a violation <= 1e-9; the step counts may part after a near tie
    assert abs(lg["n_iter"] - lo["n_iter"]) <= 0.05 * lo["n_iter"]
    assert np.abs(P.sum(1) - a).max() <= 2e-9 and np.abs(P.sum(0) - b).max() <= 2e-9
    np.testing.assert_allclose(P, Po, rtol=0, atol=1e-8)


def test_float32_against_oracle(cuda):
    g = golden("green_31x33_reg0.1")
    Po, _ = oracle.greenkhorn(g["a"], g["b"], g["M"], 0.1, stopThr=1e-7)
    M = torch.tensor(g["M"], dtype=torch.float32, device=cuda)
    a = torch.tensor(g["a"], dtype=torch.float32, device=cuda)
    b = torch.tensor(g["b"], dtype=torch.float32, device=cuda)
    P = pg.greenkhorn(a, b, M, 0.1, stopThr=1e-7)
    assert P.dtype == torch.float32 and P.is_cuda
    P = P.double().cpu().numpy()
    assert np.abs(P - Po).sum() / np.abs(Po).sum() <= 1e-4


def test_zero_budget_returns_the_start(cuda):
    g = golden("green_31x33_reg0.1")
    Po, lo = oracle.greenkhorn(g["a"], g["b"], g["M"], 0.1, numItermax=0)
    with pytest.warns(UserWarning, match="did not converge"):
        P, lg = pg.greenkhorn(g["a"], g["b"], g["M"], 0.1, numItermax=0, log=True)
    assert lg["n_iter"] == lo["n_iter"] == -1
    np.testing.assert_allclose(P, Po, rtol=1e-15)


def test_two_target_histograms_rejected(cuda):
    g = golden("green_31x33_reg0.1")
    with pytest.raises(ValueError):
        pg.greenkhorn(g["a"], np.stack([g["b"], g["b"]], 1), g["M"], 0.1)
