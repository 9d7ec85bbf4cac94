"""Dense solves replayed from a CUDA graph (pot_gb300.graphs.SinkhornGraph)
give the results of the direct calls and of the oracle on every replay:
same stop index, plan relative L1 <= 1e-9 and loss relative <= 1e-9 in
float64, for both forms."""
import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from pot_gb300.graphs import SinkhornGraph

pytestmark = pytest.mark.gpu


def _problem(seed, n, m):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 2))
    y = rng.normal(size=(m, 2)) * np.sqrt(0.5) + 1.0
    M = oracle.sqeuclidean(x, y)
    M /= M.max()
    a = rng.dirichlet(np.ones(n) * 5)
    b = rng.dirichlet(np.ones(m) * 5)
    return a, b, M


@pytest.mark.parametrize("method", ["sinkhorn", "sinkhorn_log"])
def test_graph_replays_match_oracle(cuda, method):
    n, m, reg = 200, 170, 0.05
    g = SinkhornGraph(n, m, reg, method=method, numItermax=1000, stopThr=1e-9, dtype=torch.float64, device=cuda)
    ref_fn = oracle.sinkhorn_knopp if method == "sinkhorn" else oracle.sinkhorn_log
    for seed in range(3):
        a, b, M = _problem(seed, n, m)
        ad, bd, Md = (torch.tensor(t, device=cuda) for t in (a, b, M))
        P, lg = g(ad, bd, Md, log=True)
        P = P.cpu().numpy()
        Po, lo = ref_fn(a, b, M, reg, numItermax=1000, stopThr=1e-9)
        assert lg["niter"] == lo["niter"], (seed, lg["niter"], lo["niter"])
        assert np.abs(P - Po).sum() / Po.sum() < 1e-9
        loss = float((M * Po).sum())
        assert abs(lg["loss"] - loss) <= 1e-9 * abs(loss)
        np.testing.assert_allclose(lg["err"], lo["err"], rtol=1e-6, atol=1e-15)
        # the direct call runs the same kernels
        Pd = pg.sinkhorn(ad, bd, Md, reg, method=method, stopThr=1e-9).cpu().numpy()
        np.testing.assert_allclose(P, Pd, rtol=1e-12, atol=1e-300)


def test_graph_rejects_other_shapes(cuda):
    g = SinkhornGraph(64, 48, 0.1, device=cuda)
    a, b, M = _problem(0, 64, 40)
    with pytest.raises(ValueError):
        g(torch.tensor(a, device=cuda), torch.tensor(b, device=cuda), torch.tensor(M, device=cuda))
    with pytest.raises(ValueError):
        SinkhornGraph(8, 8, 0.1, method="greenkhorn", device=cuda)
