"""Parity at the benchmark configurations, against the float64 oracle.

- online-cost workload (8-component Gaussian mixture in R^64, Dirichlet(50)
  weights, reg = 0.01 x median cost) on its 4096-point subsample: the float32
  online solver (tensor-core cost tiles, fp16 hi/lo x3) against the
  oracle's converged sinkhorn_log (stored fixture,
  tests/golden/gen_config_fixtures.py): plan relative L1 <= 1e-5.  The loss
  and the exact-cost marginals are within 1e-5 (relative / L1), not 1e-6, and
  the solver's own float32 L1 error estimate levels off at 1.3e-6, so it is
  run to stopThr 2e-6: at this regularisation the exponent arguments are
  ~100 in magnitude, where one float32 ulp is 7.6e-6, which bounds the
  accuracy of every float32 potential;
- entropic Gromov-Wasserstein (C1, C2 from N(0, I3) / N(0, I8) points, each
  divided by its maximum, epsilon = 5e-3) at n = m = 1024, five outer
  iterations: the float32 tensor-core path against the float64 oracle run
  here;
- the uneven-batch workload (n, m ~ U{32..1024}, d in {3, 16}, Dirichlet(1)
  weights, reg down to 1e-3 x max cost), float32 with the reference's stop
  rule per problem at 1e-6: every problem's exact-cost column-marginal
  violation below 2 x stopThr and its plan within 1e-4 (relative L1) of the
  oracle's at the same stop threshold.
"""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from pot_gb300 import batch as pb
from pot_gb300 import gromov as pgw
from pot_gb300.empirical import online_sinkhorn

pytestmark = pytest.mark.gpu


def test_online_config_subsample_vs_converged_oracle(cuda):
    g = golden("online_gmm4096_d64")
    X, Y, a, b, reg = g["X"], g["Y"], g["a"], g["b"], float(g["reg"])
    C = oracle.sqeuclidean(X.astype(np.float64), Y.astype(np.float64))
    Pref = np.exp(g["conv_log_u"][:, None] - C / reg + g["conv_log_v"][None, :])
    f32 = lambda z: torch.tensor(z, dtype=torch.float32, device=cuda)  # noqa: E731
    f, gg, st, nit, errs = online_sinkhorn(f32(X), f32(Y), reg, f32(a), f32(b), 5000, 2e-6)
    P = np.exp(f.double().cpu().numpy()[:, None] - C / reg + gg.double().cpu().numpy()[None, :])
    rel = np.abs(P - Pref).sum() / Pref.sum()
    loss, loss_ref = float((P * C).sum()), float((Pref * C).sum())
    row_l1 = np.abs(P.sum(1) - a).sum()
    col_l2 = np.linalg.norm(P.sum(0) - b)
    print("online 4096 d=64 reg=0.01 median: status %d niter %d (oracle %d at 1e-6), plan rel L1 %.2e, "
          "loss rel %.2e, row L1 %.2e, col L2 %.2e, last errors %s"
          % (st, nit, int(g["niter"]), rel, abs(loss - loss_ref) / loss_ref, row_l1, col_l2, errs[-3:]))
    assert st == 0 and errs[-1] <= 2e-6
    assert rel <= 1e-5
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    assert row_l1 <= 1e-5 and col_l2 <= 1e-5


def test_gw_config_n1024_vs_oracle(cuda):
    rng = np.random.default_rng(5)
    n = 1024
    xs = rng.standard_normal((n, 3))
    xt = rng.standard_normal((n, 8))
    C1, C2 = oracle.sqeuclidean(xs, xs), oracle.sqeuclidean(xt, xt)
    C1 /= C1.max()
    C2 /= C2.max()
    kw = dict(epsilon=5e-3, max_iter=5, numItermax=100000, stopThr=1e-7)
    Tref, lref = oracle.entropic_gw_log_inner(C1, C2, **kw)
    T, lg = pgw.entropic_gromov_wasserstein_log(torch.tensor(C1, dtype=torch.float32, device=cuda),
                                                torch.tensor(C2, dtype=torch.float32, device=cuda), **kw)
    T = T.double().cpu().numpy()
    rel = np.abs(T - Tref).sum() / Tref.sum()
    grel = abs(lg["gw_dist"] - lref["gw_dist"]) / abs(lref["gw_dist"])
    print("gw n=1024 eps=5e-3, 5 outer: plan rel L1 %.2e, gw_dist rel %.2e, inner %s vs %s"
          % (rel, grel, lg["inner_niter"], lref.get("inner_niter")))
    assert rel <= 1e-4
    assert grel <= 1e-5


def test_ragged_config_sample_float32(cuda):
    g = golden("ragged_cfg3")
    sizes, rels = g["sizes"], g["reg_rel"]
    B = len(sizes)
    Xs = [g["X%d" % k] for k in range(B)]
    Ys = [g["Y%d" % k] for k in range(B)]
    As = [g["a%d" % k] for k in range(B)]
    Bs = [g["b%d" % k] for k in range(B)]
    # the oracle's regularisations (rel x max cost of the float32 points, in float64)
    regs = [float(rels[k] * oracle.sqeuclidean(Xs[k].astype(np.float64), Ys[k].astype(np.float64)).max())
            for k in range(B)]
    res = pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, max_iter=100000, tol=1e-6, dtype=torch.float32)
    st = res.status.cpu().numpy()
    nit = res.niter.cpu().numpy()
    worst = 0.0
    for k in range(B):
        C = oracle.sqeuclidean(Xs[k].astype(np.float64), Ys[k].astype(np.float64))
        u, v = (t.double().cpu().numpy() for t in res.potentials(k))
        P = np.exp(u[:, None] - C / regs[k] + v[None, :])
        Pref = np.exp(g["log_u%d" % k][:, None] - C / regs[k] + g["log_v%d" % k][None, :])
        rel = np.abs(P - Pref).sum() / Pref.sum()
        worst = max(worst, rel)
        assert st[k] == 0, k
        assert np.linalg.norm(P.sum(0) - Bs[k]) < 2e-6, k
        assert np.abs(P.sum(1) - As[k]).sum() < 1e-4, k
        assert rel <= 1e-4, (k, rel, int(nit[k]), int(g["niter%d" % k]))
    print("ragged sample (24 problems, float32): worst plan rel L1 %.2e" % worst)
