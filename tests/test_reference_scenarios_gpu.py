"""The reference's own hot-path test scenarios, restated against the GPU
drop-ins with CUDA (and numpy) inputs.

Each test takes the inputs, calls and tolerances of one test in the
reference's suite (the reference itself is not available where the GPU tests
run, so its scenarios are restated here in this project's code):

- ``test/test_bregman.py:284`` test_sinkhorn_variants: the 'sinkhorn',
  'sinkhorn_log', 'sinkhorn_stabilized', 'sinkhorn_epsilon_scaling' and
  'greenkhorn' plans agree to 1e-5;
- ``test/test_bregman.py:1197`` test_lazy_empirical_sinkhorn (squared
  Euclidean parts): marginals of the lazy plans against ``sinkhorn`` to
  1e-5, ``empirical_sinkhorn2`` against ``sinkhorn2`` to 1e-5, the lazy plan
  against the log plan to 1e-5;
- ``test/batch/test_solve_batch.py:28`` test_solve_batch: ``solve_batch``
  against ``solve`` problem by problem (plan 1e-5, linear value 1e-4), and
  ``:64`` test_bregman_batch (scaling vs log projection, 1e-3);
- ``test/gromov/test_bregman.py:25`` test_entropic_gromov (square loss):
  numpy inputs with G0 given against CUDA inputs with symmetric=True and
  G0 None, to 1e-6, marginals to 1e-4.
"""
import numpy as np
import pytest
import torch

import pot_gb300 as pg
from pot_gb300 import batch as pb
from pot_gb300 import gromov as pgw

pytestmark = pytest.mark.gpu


def _cuda(*xs):
    return [torch.tensor(x, dtype=torch.float64, device="cuda") for x in xs]


def test_sinkhorn_variants(cuda):
    n = 100
    rng = np.random.RandomState(0)
    x = rng.randn(n, 2)
    u = np.full(n, 1.0 / n)
    M = pg.dist(x, x)
    ub, Mb = _cuda(u, M)
    G = pg.sinkhorn(u, u, M, 1, method="sinkhorn", stopThr=1e-10)
    Gl = pg.sinkhorn(ub, ub, Mb, 1, method="sinkhorn_log", stopThr=1e-10).cpu().numpy()
    G0 = pg.sinkhorn(ub, ub, Mb, 1, method="sinkhorn", stopThr=1e-10).cpu().numpy()
    Gs = pg.sinkhorn(ub, ub, Mb, 1, method="sinkhorn_stabilized", stopThr=1e-10).cpu().numpy()
    Ges = pg.sinkhorn(ub, ub, Mb, 1, method="sinkhorn_epsilon_scaling", stopThr=1e-10).cpu().numpy()
    G_green = pg.sinkhorn(ub, ub, Mb, 1, method="greenkhorn", stopThr=1e-10).cpu().numpy()
    np.testing.assert_allclose(G, G0, atol=1e-05)
    np.testing.assert_allclose(G, Gl, atol=1e-05)
    np.testing.assert_allclose(G0, Gs, atol=1e-05)
    np.testing.assert_allclose(G0, Ges, atol=1e-05)
    np.testing.assert_allclose(G0, G_green, atol=1e-5)


def test_lazy_empirical_sinkhorn(cuda):
    n = 10
    a = np.full(n, 1.0 / n)
    X_s = np.reshape(np.arange(n, dtype=np.float64), (n, 1))
    X_t = np.reshape(np.arange(0, n, dtype=np.float64), (n, 1))
    M = pg.dist(X_s, X_t)
    ab, X_sb, X_tb, Mb = _cuda(a, X_s, X_t, M)
    f, g = pg.empirical_sinkhorn(X_sb, X_tb, 1, numIterMax=1000, isLazy=True, batchSize=(1, 3))
    f, g = f.cpu().numpy(), g.cpu().numpy()
    G_sqe = np.exp(f[:, None] + g[None, :] - M / 1)
    sinkhorn_sqe = pg.sinkhorn(ab, ab, Mb, 1).cpu().numpy()
    f, g, _ = pg.empirical_sinkhorn(X_sb, X_tb, 1, numIterMax=1000, isLazy=True, batchSize=5, log=True)
    f, g = f.cpu().numpy(), g.cpu().numpy()
    G_log = np.exp(f[:, None] + g[None, :] - M / 1)
    sinkhorn_log, _ = pg.sinkhorn(ab, ab, Mb, 1, log=True)
    sinkhorn_log = sinkhorn_log.cpu().numpy()
    loss_emp, log = pg.empirical_sinkhorn2(X_sb, X_tb, 1, numIterMax=1000, isLazy=True, batchSize=5, log=True)
    G_lazy = log["lazy_plan"][:].cpu().numpy()
    loss_sinkhorn = pg.sinkhorn2(ab, ab, Mb, 1).cpu().numpy()
    np.testing.assert_allclose(G_sqe[1, 1], G_lazy[1, 1], atol=1e-03)
    np.testing.assert_allclose(sinkhorn_sqe.sum(1), G_sqe.sum(1), atol=1e-05)
    np.testing.assert_allclose(sinkhorn_sqe.sum(0), G_sqe.sum(0), atol=1e-05)
    np.testing.assert_allclose(sinkhorn_log.sum(1), G_log.sum(1), atol=1e-05)
    np.testing.assert_allclose(sinkhorn_log.sum(0), G_log.sum(0), atol=1e-05)
    np.testing.assert_allclose(loss_emp.cpu().numpy(), loss_sinkhorn, atol=1e-05)
    np.testing.assert_allclose(G_log, G_lazy, atol=1e-05)


@pytest.mark.parametrize("solver", ["sinkhorn", "log_sinkhorn"])
@pytest.mark.parametrize("reg_type", ["kl", "entropy"])
def test_solve_batch(cuda, solver, reg_type):
    batchsize, n = 4, 16
    rng = np.random.RandomState(0)
    M = rng.rand(batchsize, n, n)
    res = pb.solve_batch(M, a=None, b=None, reg=0.1, max_iter=10000, tol=1e-5, solver=solver, reg_type=reg_type,
                         grad="detach")
    for i in range(batchsize):
        res_i = pg.solve(M[i], a=None, b=None, reg=0.1, max_iter=10000, tol=1e-5, reg_type=reg_type)
        np.testing.assert_allclose(res_i.plan, res.plan[i], atol=1e-05)
        np.testing.assert_allclose(res_i.value_linear, res.value_linear[i], atol=1e-4)


def test_bregman_batch(cuda):
    batchsize, d, n = 4, 2, 4
    rng = np.random.RandomState(0)
    X = rng.rand(batchsize, n, d)
    M = pb.dist_batch(X, X)
    K = np.exp(-M / 0.01)
    res = pb.bregman_projection_batch(K, max_iter=50, tol=1e-10)
    res_log = pb.bregman_log_projection_batch(-M / 0.01, max_iter=50, tol=1e-10)
    np.testing.assert_allclose(res["T"], res_log["T"], atol=1e-3)


def test_entropic_gromov_square_loss(cuda):
    n = 10
    rng = np.random.RandomState(42)
    xs = rng.randn(n, 2)
    xt = xs[::-1].copy()
    p = np.full(n, 1.0 / n)
    q = np.full(n, 1.0 / n)
    G0 = p[:, None] * q[None, :]
    C1, C2 = pg.dist(xs, xs), pg.dist(xt, xt)
    C1 /= C1.max()
    C2 /= C2.max()
    C1b, C2b, pb_ = _cuda(C1, C2, p)
    G, log = pgw.entropic_gromov_wasserstein(C1, C2, None, q, "square_loss", symmetric=None, G0=G0, epsilon=1e-2,
                                             max_iter=10, log=True)
    Gb = pgw.entropic_gromov_wasserstein(C1b, C2b, pb_, None, "square_loss", symmetric=True, G0=None, epsilon=1e-2,
                                         max_iter=10, log=False).cpu().numpy()
    np.testing.assert_allclose(G, Gb, atol=1e-06)
    np.testing.assert_allclose(p, Gb.sum(1), atol=1e-04)
    np.testing.assert_allclose(q, Gb.sum(0), atol=1e-04)
