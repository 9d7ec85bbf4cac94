"""Parity of the GPU unbalanced Sinkhorn (``OTG_METHOD_UNB``) with the
reference's golden vectors: identical per-iteration error history (rtol
1e-6) and stop index, plan relative L1 1e-9, log scalings rtol 1e-8, costs
rtol 1e-9 (float64); float32 against the float64 oracle within relative L1
1e-4."""
import warnings

import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from conftest import golden

pytestmark = pytest.mark.gpu

CASES = [("kl", dict(reg=0.05, reg_m=1.0)), ("kl_pair", dict(reg=0.05, reg_m=(0.5, float("inf")))),
         ("ent", dict(reg=0.1, reg_m=2.0, reg_type="entropy")), ("kl_small", dict(reg=0.005, reg_m=0.3)),
         ("warm", dict(reg=0.05, reg_m=1.0)), ("iter5", dict(reg=0.05, reg_m=1.0, numItermax=5))]


def rel_l1(P, Q):
    return float(np.abs(P - Q).sum() / np.abs(Q).sum())


@pytest.mark.parametrize("tag,kw", CASES)
def test_unbalanced_f64_golden(cuda, tag, kw):
    g = golden("unbal_50x40")
    kw = dict(kw)
    reg, reg_m = kw.pop("reg"), kw.pop("reg_m")
    if tag == "warm":
        kw["warmstart"] = (g["warm_wu"], g["warm_wv"])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        P, lg = pg.sinkhorn_unbalanced(g["a"], g["b"], g["M"], reg, reg_m, log=True, **kw)
    assert len(lg["err"]) == len(g[tag + "_err"])
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), g[tag + "_err"], rtol=1e-6, atol=1e-14)
    assert rel_l1(P, g[tag + "_plan"]) < 1e-9
    np.testing.assert_allclose(lg["logu"], g[tag + "_logu"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(lg["logv"], g[tag + "_logv"], rtol=1e-8, atol=1e-10)
    assert abs(float(lg["cost"]) - float(g[tag + "_cost"])) <= 1e-9 * abs(float(g[tag + "_cost"]))
    assert abs(float(lg["total_cost"]) - float(g[tag + "_total"])) <= 1e-9 * abs(float(g[tag + "_total"]))


def test_unbalanced2_and_user_c(cuda):
    g = golden("unbal_50x40")
    lin = pg.sinkhorn_unbalanced2(g["a"], g["b"], g["M"], 0.05, 1.0)
    tot = pg.sinkhorn_unbalanced2(g["a"], g["b"], g["M"], 0.05, 1.0, returnCost="total")
    assert abs(float(lin) - float(g["u2_linear"])) <= 1e-9 * abs(float(g["u2_linear"]))
    assert abs(float(tot) - float(g["u2_total"])) <= 1e-9 * abs(float(g["u2_total"]))
    # an explicit c equal to a b^T gives the default problem
    c = np.outer(g["a"], g["b"])
    P, lg = pg.sinkhorn_knopp_unbalanced(g["a"], g["b"], g["M"], 0.05, 1.0, c=c, log=True)
    assert rel_l1(P, g["kl_plan"]) < 1e-9
    assert abs(float(lg["total_cost"]) - float(g["kl_total"])) <= 1e-9 * abs(float(g["kl_total"]))


def test_unbalanced_f32(cuda):
    g = golden("unbal_50x40")
    Pref, _ = oracle.sinkhorn_knopp_unbalanced(g["a"], g["b"], g["M"], 0.05, 1.0, stopThr=1e-9)
    f = lambda x: torch.tensor(x, dtype=torch.float32, device=cuda)  # noqa: E731
    P = pg.sinkhorn_unbalanced(f(g["a"]), f(g["b"]), f(g["M"]), 0.05, 1.0, stopThr=1e-6)
    assert P.dtype == torch.float32 and P.device.type == "cuda"
    assert rel_l1(P.double().cpu().numpy(), Pref) <= 1e-4


def test_solve_unbalanced_golden(cuda):
    g = golden("unbal_50x40")
    res = pg.solve(g["M"], g["a"], g["b"], reg=0.05, unbalanced=1.0)
    assert rel_l1(res.plan, g["solve_plan"]) < 1e-9
    # the total cost nearly cancels here (about 1e-9): compare with an absolute floor
    assert abs(float(res.value) - float(g["solve_value"])) <= 1e-9 * abs(float(g["solve_value"])) + 1e-14
    assert abs(float(res.value_linear) - float(g["solve_value_linear"])) <= 1e-9 * abs(float(g["solve_value_linear"]))
    np.testing.assert_allclose(res.potentials[0], g["solve_pa"], rtol=1e-8, atol=1e-10)
