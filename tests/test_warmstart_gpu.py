"""Learned warm start: GPU forward/backward against the float64 oracle, the
AdamW step against its formula, and the gain of a trained network over the
zero-initialised solver on held-out pairs.

Tolerances: forward relative 1e-5, gradients relative (norm per tensor)
1e-4 (fp32 kernels vs fp64 oracle).
"""
import numpy as np
import pytest
import torch

from oracle import warmstart_net as wn
from pot_gb300.warmstart import net as wsn
from pot_gb300.warmstart import pipeline as wp

pytestmark = pytest.mark.gpu


def test_forward_backward_match_oracle(cuda):
    rng = np.random.default_rng(0)
    d, P, n, m, K = 5, 3, 37, 29, 4
    params = wsn.init_params(d, seed=2, h1=16, h2=12, h3=20, dz=d + K)
    for k in params:
        if k.startswith("b"):
            params[k] = (rng.standard_normal(params[k].shape) * 0.1).astype(np.float32)
    X = rng.standard_normal((P, n, d)).astype(np.float32)
    Y = rng.standard_normal((P, m, d)).astype(np.float32)
    Z = np.concatenate([X, rng.standard_normal((P, n, K)).astype(np.float32)], 2)
    t = rng.standard_normal((P, n)).astype(np.float32)
    t -= t.mean(1, keepdims=True)
    loss_ref, g_ref, f_ref = wn.loss_and_grads(params, X, Y, t, Z)
    net = wsn.WarmStartNet(d, params=params, device=cuda, h1=16, h2=12, h3=20, dz=d + K)
    f = net.forward(torch.tensor(X, device=cuda).view(P * n, d), torch.tensor(Y, device=cuda).view(P * m, d),
                    P, n, m, Z=torch.tensor(Z, device=cuda).view(P * n, d + K), keep=True)
    np.testing.assert_allclose(f.view(P, n).cpu().numpy(), f_ref, rtol=1e-5, atol=1e-5)
    loss, df = net.loss_and_grad(f, torch.tensor(t, device=cuda).view(-1), P, n)
    assert abs(loss.item() - loss_ref) <= 1e-5 * abs(loss_ref)
    net.backward(df)
    gmax = max(np.abs(v).max() for v in g_ref.values())
    for name, _ in net.shapes:
        g = net.G(name).cpu().numpy().astype(np.float64)
        r = g_ref[name].reshape(g.shape)
        # the output bias has an exactly zero gradient (the loss ignores a
        # constant shift): compare it with an absolute floor
        assert np.linalg.norm(g - r) <= 1e-4 * np.linalg.norm(r) + 1e-6 * gmax, name


def test_adamw_step_matches_formula(cuda):
    net = wsn.WarmStartNet(4, device=cuda, seed=3, h1=8, h2=8, h3=8)
    w0 = net.flat.clone()
    g = torch.randn_like(w0)
    net.grad.copy_(g)
    net.adamw(1e-2, b1=0.9, b2=0.999, eps=1e-8, wd=0.1)
    m = 0.1 * g
    v = 0.001 * g * g
    ref = w0 - 1e-2 * ((m / 0.1) / (torch.sqrt(v / 0.001) + 1e-8) + 0.1 * w0)
    torch.testing.assert_close(net.flat, ref, rtol=1e-5, atol=1e-6)


def test_trained_network_reduces_iterations(cuda):
    """A network trained briefly on solver-generated targets cuts the
    iterations to 1e-6 on held-out pairs relative to zero initialisation,
    and every warm solve still meets the same marginal tolerance."""
    n, d = 512, 16
    X, Y = wp.gen_pairs(11, 512, n, d, cuda)
    T, Ft, maxc, _ = wp.targets(X, Y, 0.02, 1e-7)
    net = wp.new_net(d, device=cuda, seed=0)
    wp.train(net, X, Y, T, Ft, maxc, steps=600, pairs_per_step=16, lr=2e-3, verbose=False)
    Xe, Ye = wp.gen_pairs(99_000, 64, n, d, cuda)
    ps = wp.PairSolver(Xe, Ye)
    _, _, st0, nit0, err0 = ps.solve(0.02, 1e-6)
    _, _, st1, nit1, err1 = ps.solve(0.02, 1e-6, warm_u=wp.warm_potential(net, Xe, Ye, ps))
    assert (st0 == 0).all() and (st1 == 0).all()
    assert (err1 < 1e-6).all() and (err0 < 1e-6).all()
    assert nit1.float().mean() < nit0.float().mean()
