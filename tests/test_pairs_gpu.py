"""Batched cloud-pair solves with the cost rebuilt on the tensor cores
(otg_sinkhorn_pairs): against the float64 oracle and the stored-cost batch
solver on the same problems.

The cost tiles carry about 22 bits (fp16 hi/lo x3) instead of the stored
float32 cost's 24, so iterates agree to float32 precision, not bit for bit:
plans within 1e-5 (relative L1) of the float64 oracle stopped at the same
threshold, stop indices within one check of the stored-cost solver's, and
the exact-cost column-marginal violation of every returned pair below 2 x
stopThr.  The max-only pass gives each pair's largest cost to 1e-6.
"""
import numpy as np
import pytest
import torch

import oracle
from pot_gb300 import batch as pb
from pot_gb300.warmstart import pipeline as wp

pytestmark = pytest.mark.gpu


def _clouds(seed, P, n, m, d, cuda):
    g = torch.Generator(device="cpu").manual_seed(seed)
    X = torch.randn(P, n, d, generator=g) * 0.7
    Y = torch.randn(P, m, d, generator=g) * 0.5 + 0.3
    return X.to(cuda), Y.to(cuda)


@pytest.mark.parametrize("n,m,d", [(200, 333, 3), (256, 128, 16), (130, 300, 64)])
def test_max_cost_matches_float64(cuda, n, m, d):
    X, Y = _clouds(1, 5, n, m, d, cuda)
    mx = pb.pairs_max_cost(X, Y).cpu().numpy()
    for p in range(5):
        C = oracle.sqeuclidean(X[p].double().cpu().numpy(), Y[p].double().cpu().numpy())
        assert abs(mx[p] - C.max()) <= 1e-6 * C.max(), (p, mx[p], C.max())


@pytest.mark.parametrize("n,m,d", [(200, 333, 3), (256, 128, 16)])
@pytest.mark.parametrize("anderson", [0, 5])
def test_pairs_vs_oracle(cuda, n, m, d, anderson):
    P, reg_rel, tol = 4, 0.05, 1e-6
    X, Y = _clouds(2 + d, P, n, m, d, cuda)
    g = torch.Generator(device="cpu").manual_seed(9)
    a = torch.distributions.Dirichlet(torch.ones(n)).sample((P,)).float().to(cuda)
    b = torch.distributions.Dirichlet(torch.ones(m)).sample((P,)).float().to(cuda)
    regs = []
    for p in range(P):
        C = oracle.sqeuclidean(X[p].double().cpu().numpy(), Y[p].double().cpu().numpy())
        regs.append(reg_rel * C.max())
    u, v, st, nit, err = pb.run_pairs(X, Y, regs, a, b, 20000, tol, check_period=1, anderson=anderson)
    assert (st == 0).all()
    for p in range(P):
        Xp, Yp = X[p].double().cpu().numpy(), Y[p].double().cpu().numpy()
        ap, bp = a[p].double().cpu().numpy(), b[p].double().cpu().numpy()
        C = oracle.sqeuclidean(Xp, Yp)
        Pg = np.exp(u[p].double().cpu().numpy()[:, None] - C / regs[p] + v[p].double().cpu().numpy()[None, :])
        assert np.linalg.norm(Pg.sum(0) - bp) < 2 * tol, p
        assert np.abs(Pg.sum(1) - ap).sum() < 1e-5, p
        Pref, lg = oracle.sinkhorn_log(ap, bp, C, regs[p], numItermax=20000, stopThr=1e-9)
        assert np.abs(Pg - Pref).sum() / Pref.sum() < 1e-4, p


def test_pairs_far_start(cuda):
    """A warm start far from the solution (random potentials of size 400 in
    natural-log units): the first passes keep the running max, the later ones
    sum under shifts taken from them, and every pair still reaches the float64
    oracle's plan."""
    P, n, m, d, tol = 4, 256, 384, 16, 1e-6
    X, Y = _clouds(31, P, n, m, d, cuda)
    regs = []
    for p in range(P):
        C = oracle.sqeuclidean(X[p].double().cpu().numpy(), Y[p].double().cpu().numpy())
        regs.append(0.05 * C.max())
    g = torch.Generator(device="cpu").manual_seed(4)
    far = (torch.randn(P, n, generator=g) * 400.0).to(cuda)  # natural-log units, far from any solution
    u, v, st, nit, err = pb.run_pairs(X, Y, regs, None, None, 20000, tol, warm_u=far, check_period=1)
    assert (st == 0).all() and (err < tol).all()
    for p in range(P):
        Xp, Yp = X[p].double().cpu().numpy(), Y[p].double().cpu().numpy()
        C = oracle.sqeuclidean(Xp, Yp)
        Pg = np.exp(u[p].double().cpu().numpy()[:, None] - C / regs[p] + v[p].double().cpu().numpy()[None, :])
        Pref, _ = oracle.sinkhorn_log(np.full(n, 1 / n), np.full(m, 1 / m), C, regs[p], numItermax=20000,
                                      stopThr=1e-9)
        assert np.abs(Pg - Pref).sum() / Pref.sum() < 1e-4, p


def test_pairs_fixup_path(cuda):
    """A narrow acceptance window for the shifted sums sends most row blocks
    of the early passes through the fix-up launch (explicit unit lists over
    the pairs); the result is the default run's."""
    P, n, m, d, tol = 4, 256, 384, 16, 1e-6
    X, Y = _clouds(33, P, n, m, d, cuda)
    mx = pb.pairs_max_cost(X, Y)
    regs = mx.double() * 0.05
    u0, v0, st0, nit0, _ = pb.run_pairs(X, Y, regs, None, None, 20000, tol, check_period=1)
    u1, v1, st1, nit1, _ = pb.run_pairs(X, Y, regs, None, None, 20000, tol, check_period=1, sum_window_log2=0.5)
    assert (st0 == 0).all() and (st1 == 0).all()
    assert (nit1 - nit0).abs().max() <= 2
    for p in range(P):
        C = oracle.sqeuclidean(X[p].double().cpu().numpy(), Y[p].double().cpu().numpy())
        r = float(regs[p])
        Pa = np.exp(u0[p].double().cpu().numpy()[:, None] - C / r + v0[p].double().cpu().numpy()[None, :])
        Pb = np.exp(u1[p].double().cpu().numpy()[:, None] - C / r + v1[p].double().cpu().numpy()[None, :])
        assert np.abs(Pb - Pa).sum() / Pa.sum() < 1e-5, p


def test_pairs_match_the_stored_cost_solver(cuda):
    """The same pairs through both engines of the pair solver: stop indices
    within one check, potentials to float32 precision."""
    X, Y = _clouds(7, 8, 256, 256, 16, cuda)
    ps_m = wp.PairSolver(X, Y)
    ps_o = wp.PairSolver(X, Y, maxc=ps_m.maxc, engine="online")
    for per in (1, 10):
        um, vm, sm, nm, em = ps_m.solve(0.02, 1e-6, check_period=per)
        uo, vo, so, no, eo = ps_o.solve(0.02, 1e-6, check_period=per)
        assert (sm == 0).all() and (so == 0).all()
        assert (nm - no).abs().max().item() <= per
        du = (uo - uo.mean(1, keepdim=True)) - (um - um.mean(1, keepdim=True))
        assert du.abs().max().item() < 2e-3 * (1 + um.abs().max().item())


def test_pairs_max_iter_and_warm_start(cuda):
    X, Y = _clouds(11, 3, 128, 200, 8, cuda)
    mx = pb.pairs_max_cost(X, Y)
    reg = 0.003 * mx
    u, v, st, nit, err = pb.run_pairs(X, Y, reg, max_iter=25, tol=1e-12)
    assert (st == 1).all() and (nit == 24).all()
    for p in range(3):
        C = oracle.sqeuclidean(X[p].double().cpu().numpy(), Y[p].double().cpu().numpy())
        _, lg = oracle.sinkhorn_log([], [], C, float(reg[p]), numItermax=25, stopThr=1e-12)
        uu = u[p].double().cpu().numpy()
        ref = lg["log_u"]
        assert np.abs((uu - uu.mean()) - (ref - ref.mean())).max() < 2e-3 * (1 + np.abs(ref).max())
    # a converged start stops at the first check
    u2, v2, st2, nit2, _ = pb.run_pairs(X, Y, reg, max_iter=20000, tol=1e-6, check_period=1)
    u3, v3, st3, nit3, _ = pb.run_pairs(X, Y, reg, max_iter=20000, tol=1e-6, warm_u=u2, check_period=1)
    assert (st3 == 0).all() and (nit3 <= 1).all()


def test_warm_pipeline_on_the_online_engine(cuda):
    """The headline pipeline (multiscale prior + Anderson) on the online engine:
    every pair converges with the plain test, in fewer iterations than zero
    start."""
    X, Y = wp.gen_pairs(40_000_000, 32, 512, 16, cuda)
    ps = wp.PairSolver(X, Y, engine="online")
    wu = wp.prior_potential(X, Y, ps, 0.02)
    _, _, s1, n1, e1 = ps.solve(0.02, 1e-6, warm_u=wu, check_period=1, anderson=8)
    _, _, s0, n0, e0 = ps.solve(0.02, 1e-6, check_period=1)
    assert (s1 == 0).all() and (s0 == 0).all() and (e1 < 1e-6).all()
    assert n1.double().mean() < n0.double().mean()
