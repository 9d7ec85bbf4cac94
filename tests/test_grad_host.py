"""Implicit gradients of sinkhorn2 (pot_gb300._autograd.implicit_grads) on the
host, at the float64 oracle's plan, against the reference's own autodiff
through its iterations (tests/golden/gen_golden.py, section ``grad``)."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from pot_gb300._autograd import implicit_grads


def _grads(g):
    kw = {k[3:]: g[k].item() for k in g if k.startswith("kw_")}
    P, _ = oracle.sinkhorn(g["a"], g["b"], g["M"], float(g["reg"]), method=str(g["method"]), **kw)
    t = lambda x: torch.tensor(x, dtype=torch.float64)  # noqa: E731
    return [x.numpy() for x in implicit_grads(t(P), t(g["M"]), t(g["a"]), t(g["b"]), float(g["reg"]))]


def _rel(x, ref):
    return np.abs(x - ref).max() / np.abs(ref).max()


@pytest.mark.parametrize("name", ["grad2_30x40_knopp", "grad2_30x40_log"])
def test_converged_gradients_equal_reference_autodiff(name):
    """Solved to 1e-12, the reference's unrolled derivative has converged:
    M, a and b gradients agree to 1e-10 relative (measured ~2e-13)."""
    g = golden(name)
    gM, ga, gb = _grads(g)
    assert _rel(gM, g["grad_M"]) < 1e-10
    assert _rel(ga, g["grad_a"]) < 1e-10
    assert _rel(gb, g["grad_b"]) < 1e-10
    assert abs(float(np.dot(g["b"], gb))) < 1e-14  # the gauge of the reference's last (row) update


def test_reference_scenario_default_threshold():
    """test/test_bregman.py:203-225's setting (n = 100, reg = 1) at the default
    stopThr = 1e-9 (40 iterations): 1e-6 relative (measured 2.5e-8 on M,
    6e-8 on a, 3e-8 on b)."""
    g = golden("grad2_100_reg1")
    gM, ga, gb = _grads(g)
    assert _rel(gM, g["grad_M"]) < 1e-6
    assert _rel(ga, g["grad_a"]) < 1e-6
    assert _rel(gb, g["grad_b"]) < 1e-6


def test_short_solve_keeps_the_gauge_direction_out():
    """Marginals met only to 1e-8 (31 scaling iterations): the near-null
    direction of the Schur complement must not leak into the gradient (the
    rank-one shift keeps conjugate gradients off it): still 1e-6 against the
    reference's converged backward."""
    g = golden("grad2_100_reg1")
    P, _ = oracle.sinkhorn_knopp(g["a"], g["b"], g["M"], 1.0, numItermax=31, stopThr=0.0)
    t = lambda x: torch.tensor(x, dtype=torch.float64)  # noqa: E731
    gM, ga, gb = [x.numpy() for x in implicit_grads(t(P), t(g["M"]), t(g["a"]), t(g["b"]), 1.0)]
    assert _rel(gM, g["grad_M"]) < 1e-6
    assert _rel(gb, g["grad_b"]) < 1e-6


def test_zero_mass_bins_stay_finite():
    """Histograms with empty bins: the gradients stay finite, and the M
    gradient of the occupied block is unchanged by appending empty bins."""
    g = golden("grad2_30x40_knopp")
    a0 = np.concatenate([g["a"], [0.0]])
    b0 = np.concatenate([g["b"], [0.0, 0.0]])
    M0 = np.pad(g["M"], ((0, 1), (0, 2)), constant_values=0.5)
    P, lg = oracle.sinkhorn_log(a0, b0, M0, 0.1, stopThr=1e-12, numItermax=100000)
    assert not lg["_warnings"] and P[30].max() == 0.0 and P[:, 40:].max() == 0.0
    t = lambda x: torch.tensor(x, dtype=torch.float64)  # noqa: E731
    gM, ga, gb = [x.numpy() for x in implicit_grads(t(P), t(M0), t(a0), t(b0), 0.1)]
    assert np.all(np.isfinite(gM)) and np.all(np.isfinite(ga)) and np.all(np.isfinite(gb))
    assert _rel(gM[:30, :40], g["grad_M"]) < 1e-8
