"""Parity of the stabilised Sinkhorn (``OTG_METHOD_STAB``) and of epsilon
scaling with the reference's golden vectors and the oracle.

Tolerances (float64 inputs): identical stop index and absorption-affected
error history (rtol 1e-6), logu/logv/alpha rtol 1e-8 (atol 1e-8 on values
that carry absorption shifts of k log n), plan relative L1 1e-9.  Float32:
plan relative L1 1e-5 against the float64 oracle."""
import warnings

import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from conftest import golden, golden_names

pytestmark = pytest.mark.gpu

STAB = golden_names("stab_")


def _M(g):
    if "M" in g:
        return g["M"]
    M = oracle.sqeuclidean(g["x"], g["y"])
    return M / M.max()


def _kw(g):
    kw = {k[3:]: (int(v) if k in ("kw_numItermax", "kw_print_period") else float(v))
          for k, v in g.items() if k.startswith("kw_")}
    if "ws_alpha" in g:
        kw["warmstart"] = (g["ws_alpha"], g["ws_beta"])
    return kw


def rel_l1(P, Q):
    return float(np.abs(P - Q).sum() / max(np.abs(Q).sum(), 1e-300))


@pytest.mark.parametrize("name", STAB)
def test_stabilized_f64_golden(cuda, name):
    g = golden(name)
    M = _M(g)
    kw = _kw(g)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        P, lg = pg.sinkhorn_stabilized(g["a"], g["b"], M, float(g["reg"]), log=True, **kw)
    assert lg["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), g["err"], rtol=1e-6, atol=1e-14)
    np.testing.assert_allclose(lg["logu"], g["logu"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(lg["logv"], g["logv"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(lg["alpha"], g["alpha"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(lg["beta"], g["beta"], rtol=1e-8, atol=1e-10)
    Pref, _ = oracle.sinkhorn_stabilized(g["a"], g["b"], M, float(g["reg"]), **kw)
    assert rel_l1(P, Pref) < 1e-9
    assert abs(float(np.sum(M * P)) - float(g["loss"])) <= 1e-9 * abs(float(g["loss"]))
    assert any("did not converge" in str(x.message) for x in w) == bool(g["warn_nonconv"])


@pytest.mark.parametrize("name", ["stab_31x33_reg0.02", "stab_127x129_reg0.002", "stab_warm_40x50"])
def test_stabilized_dispatch_and_loss(cuda, name):
    g = golden(name)
    M = _M(g)
    kw = _kw(g)
    ws = kw.pop("warmstart", None)
    P = pg.sinkhorn(g["a"], g["b"], M, float(g["reg"]), method="sinkhorn_stabilized", warmstart=ws,
                    warn=False, **kw)
    Pref, _ = oracle.sinkhorn_stabilized(g["a"], g["b"], M, float(g["reg"]), warmstart=ws, **kw)
    assert rel_l1(P, Pref) < 1e-9
    loss = pg.sinkhorn2(g["a"], g["b"], M, float(g["reg"]), method="sinkhorn_stabilized", warmstart=ws, **kw)
    assert abs(float(loss) - float(g["loss"])) <= 1e-9 * abs(float(g["loss"]))


@pytest.mark.parametrize("name", ["stab_31x33_reg0.02", "stab_127x129_reg0.02"])
def test_stabilized_f32(cuda, name):
    g = golden(name)
    M = _M(g)
    Pref, _ = oracle.sinkhorn_stabilized(g["a"], g["b"], M, float(g["reg"]), numItermax=5000, stopThr=1e-12)
    dev = torch.device("cuda")
    P = pg.sinkhorn_stabilized(torch.tensor(g["a"], dtype=torch.float32, device=dev),
                               torch.tensor(g["b"], dtype=torch.float32, device=dev),
                               torch.tensor(M, dtype=torch.float32, device=dev), float(g["reg"]),
                               numItermax=5000, stopThr=1e-6, warn=False)
    assert P.dtype == torch.float32 and P.device.type == "cuda"
    assert rel_l1(P.double().cpu().numpy(), Pref) <= 1e-5


@pytest.mark.parametrize("name", golden_names("epsscale_"))
def test_epsilon_scaling_golden(cuda, name):
    g = golden(name)
    kw = {k[3:]: (float(v) if k == "kw_epsilon0" else int(v)) for k, v in g.items() if k.startswith("kw_")}
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        G, lg = pg.sinkhorn(g["a"], g["b"], g["M"], float(g["reg"]), method="sinkhorn_epsilon_scaling",
                            log=True, **kw)
    assert lg["niter"] == int(g["niter"])
    assert len(lg["err"]) == len(g["err"])
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), g["err"], rtol=1e-3, atol=1e-15)
    assert rel_l1(G, g["plan"]) < 1e-9
    np.testing.assert_allclose(lg["alpha"], g["alpha"], rtol=1e-8, atol=1e-10)
    assert sum("did not converge" in str(x.message) for x in w) == int(g["warn_nonconv"])
