"""Parity of the GPU entropic barycenters (scaling and log forms) with the
reference's golden vectors: identical stop index, error history rtol 1e-6,
barycenter rtol 1e-8 (float64); float32 against the float64 oracle within
relative L1 1e-4."""
import warnings

import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tag,method,reg", [("sk", "sinkhorn", 0.01), ("log", "sinkhorn_log", 0.01),
                                            ("log_small", "sinkhorn_log", 1e-3)])
def test_barycenter_f64_golden(cuda, tag, method, reg):
    g = golden("bary_60x3")
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        bar, lg = pg.barycenter(g["A"], g["M"], reg, weights=g["w"], method=method, numItermax=2000, stopThr=1e-8,
                                log=True)
    assert lg["niter"] == int(g[tag + "_niter"])
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), g[tag + "_err"], rtol=1e-6, atol=1e-15)
    np.testing.assert_allclose(bar, g[tag + "_bar"], rtol=1e-8, atol=1e-300)
    assert any("did not converge" in str(x.message) for x in w) == bool(g[tag + "_nonconv"])


def test_barycenter_default_and_300(cuda):
    g = golden("bary_60x3")
    np.testing.assert_allclose(pg.barycenter(g["A"], g["M"], 0.05), g["default_bar"], rtol=1e-8)
    g = golden("bary_300x5")
    M = oracle.sqeuclidean(g["x"])
    M /= M.max()
    for tag, method in (("sk", "sinkhorn"), ("log", "sinkhorn_log")):
        bar, lg = pg.barycenter(g["A"], M, 0.02, method=method, numItermax=300, stopThr=1e-9, log=True)
        assert lg["niter"] == int(g[tag + "_niter"])
        np.testing.assert_allclose(bar, g[tag + "_bar"], rtol=1e-7, atol=1e-300)


@pytest.mark.parametrize("method", ["sinkhorn", "sinkhorn_log"])
def test_barycenter_f32(cuda, method):
    g = golden("bary_60x3")
    fn = oracle.barycenter_sinkhorn if method == "sinkhorn" else oracle.barycenter_sinkhorn_log
    ref, _ = fn(g["A"], g["M"], 0.05, g["w"], numItermax=2000, stopThr=1e-6)
    f = lambda x: torch.tensor(x, dtype=torch.float32, device=cuda)  # noqa: E731
    bar = pg.barycenter(f(g["A"]), f(g["M"]), 0.05, weights=f(g["w"]), method=method, numItermax=2000, stopThr=1e-6)
    assert bar.dtype == torch.float32 and bar.device.type == "cuda"
    bar = bar.double().cpu().numpy()
    assert np.abs(bar - ref).sum() / ref.sum() <= 1e-4
