"""Gradient values of sinkhorn2 on the GPU: the reference's own backward
through its iterations (recorded in tests/golden, section ``grad``) against
the implicit gradients at the GPU solution (pot_gb300._autograd)."""
import numpy as np
import pytest
import torch

import pot_gb300 as pg
from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["grad2_30x40_knopp", "grad2_30x40_log", "grad2_100_reg1"])
def test_sinkhorn2_gradients_match_reference_autodiff(cuda, name):
    """Gradient values, not only shapes.  Solved to 1e-12 the two agree to
    1e-8 relative; at the default stopThr of the reference's own gradient
    test (test_bregman.py:203, n = 100, reg = 1) to 1e-5 (measured on the
    host at the float64 oracle's plan: 6e-8)."""
    g = golden(name)
    kw = {k[3:]: g[k].item() for k in g if k.startswith("kw_")}
    M = torch.tensor(g["M"], device=cuda, requires_grad=True)
    a = torch.tensor(g["a"], device=cuda, requires_grad=True)
    b = torch.tensor(g["b"], device=cuda, requires_grad=True)
    loss = pg.sinkhorn2(a, b, M, float(g["reg"]), method=str(g["method"]), **kw)
    assert loss.requires_grad and loss.is_cuda
    assert abs(float(loss.detach()) - float(g["loss"])) <= 1e-9 * abs(float(g["loss"]))
    (2.0 * loss).backward()
    tol = 1e-8 if kw.get("stopThr", 1e-9) <= 1e-12 else 1e-5
    for x, ref in ((M, g["grad_M"]), (a, g["grad_a"]), (b, g["grad_b"])):
        got = x.grad.cpu().numpy() / 2.0
        assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def test_sinkhorn2_gradients_float32(cuda):
    """float32 inputs get float32 gradients, computed in float64 from the
    float32 plan: within 1e-3 relative of the float64 gradients."""
    g = golden("grad2_30x40_log")
    out = {}
    for dt in (torch.float32, torch.float64):
        M = torch.tensor(g["M"], dtype=dt, device=cuda, requires_grad=True)
        a = torch.tensor(g["a"], dtype=dt, device=cuda, requires_grad=True)
        b = torch.tensor(g["b"], dtype=dt, device=cuda, requires_grad=True)
        pg.sinkhorn2(a, b, M, 0.1, method="sinkhorn_log", stopThr=1e-7).backward()
        assert M.grad.dtype == dt and a.grad.dtype == dt
        out[dt] = [x.grad.double().cpu().numpy() for x in (M, a, b)]
    for g32, g64 in zip(out[torch.float32], out[torch.float64]):
        assert np.abs(g32 - g64).max() <= 1e-3 * np.abs(g64).max()
