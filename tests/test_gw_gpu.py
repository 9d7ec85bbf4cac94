"""Entropic Gromov-Wasserstein on the GPU.

- The tcgen05 split GEMM against an fp64 product: relative Frobenius error
  <= 3e-6 (three half-precision passes carry about 22 bits).
- float64 inputs (fp64 GEMM + fp64 inner Sinkhorn) against the reference's
  golden plans: rtol 1e-8.
- float32 inputs (tensor-core products, fp32 inner Sinkhorn) against the
  float64 oracle: plan relative L1 <= 1e-3, gw_dist relative <= 1e-4.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from pot_gb300 import _lib
from pot_gb300 import gromov as pgw

pytestmark = pytest.mark.gpu


def _split_gemm(A, B, mode=1):
    lib = _lib.load()
    dev = A.device
    sa = pgw.pow2_scale(float(A.abs().max()))
    sb = pgw.pow2_scale(float(B.abs().max()))
    Ap = pgw._Planes(A.shape[0], A.shape[1], dev).fill(A, sa)
    Bp = pgw._Planes(B.shape[0], B.shape[1], dev).fill(B, sb)
    out = torch.zeros(A.shape[0], B.shape[0], dtype=torch.float32, device=dev)
    zr = torch.zeros(A.shape[0], dtype=torch.float32, device=dev)
    zc = torch.zeros(B.shape[0], dtype=torch.float32, device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    g = _lib.OtgSplitGemm(a_hi=_lib.ptr(Ap.hi), a_lo=_lib.ptr(Ap.lo), a_rows=Ap.rows, lda=Ap.cols,
                          b_hi=_lib.ptr(Bp.hi), b_lo=_lib.ptr(Bp.lo), b_rows=Bp.rows, ldb=Bp.cols, k_alloc=Ap.cols,
                          mode=1, scale=1.0, s_acc=1.0 / (sa * sb), s_vec=0.0, out_hi=None, out_lo=None, ld_h=0,
                          out=_lib.ptr(out), ld_o=out.stride(0), M=A.shape[0], N=B.shape[0], rowv=_lib.ptr(zr),
                          colv=_lib.ptr(zc), abort_flag=_lib.ptr(flag), timeout_ms=0)
    assert lib.otg_gemm_split3(ctypes.byref(g), _lib.stream_handle(dev)) == 0
    torch.cuda.synchronize()
    assert int(flag.item()) == 0
    return out


@pytest.mark.parametrize("shape", [(128, 128, 64), (300, 500, 700), (1024, 256, 2048)])
def test_split_gemm_matches_fp64(cuda, shape):
    M, N, K = shape
    g = torch.Generator(device="cpu").manual_seed(0)
    A = torch.rand(M, K, generator=g, dtype=torch.float64)
    B = torch.rand(N, K, generator=g, dtype=torch.float64)
    ref = A @ B.T
    out = _split_gemm(A.float().to(cuda), B.float().to(cuda)).double().cpu()
    # the fp32 inputs themselves carry 2^-24 relative rounding
    Af, Bf = A.float().double(), B.float().double()
    ref32 = Af @ Bf.T
    rel = float(torch.linalg.norm(out - ref32) / torch.linalg.norm(ref32))
    assert rel <= 3e-6, rel
    assert float(torch.linalg.norm(out - ref) / torch.linalg.norm(ref)) <= 3e-6


@pytest.mark.parametrize("tag,kw", [("pgd", {}), ("pgd_warm", {"warmstart": True}), ("ppa", {"solver": "PPA"})])
def test_egw_f64_golden(cuda, tag, kw):
    g = golden("egw_10")
    T, lg = pgw.entropic_gromov_wasserstein(g["C1"], g["C2"], g["p"], g["q"], "square_loss", epsilon=1e-2,
                                            max_iter=10, log=True, **kw)
    np.testing.assert_allclose(T, g[tag + "_T"], rtol=1e-8, atol=1e-13)
    assert abs(float(lg["gw_dist"]) - float(g[tag + "_gw"])) < 1e-10
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), g[tag + "_err"], rtol=1e-6, atol=1e-14)


@pytest.mark.parametrize("name", ["egw_48x40", "egw_asym_48x40"])
def test_egw_f64_medium_golden(cuda, name):
    g = golden(name)
    if name == "egw_48x40":
        kw = dict(max_iter=20, tol=1e-9, numItermax=2000, stopThr=1e-9)
    else:
        kw = dict(max_iter=10)
    T, lg = pgw.entropic_gromov_wasserstein(g["C1"], g["C2"], None, None, "square_loss", epsilon=5e-2, log=True, **kw)
    np.testing.assert_allclose(T, g["T"], rtol=1e-7, atol=1e-13)
    assert abs(float(lg["gw_dist"]) - float(g["gw"])) < 1e-9
    if name == "egw_48x40":
        gw2 = pgw.entropic_gromov_wasserstein2(g["C1"], g["C2"], None, None, "square_loss", epsilon=5e-2, **kw)
        assert abs(float(gw2) - float(g["gw2"])) < 1e-9


def test_egw_f32_tensor_cores_vs_oracle(cuda):
    g = golden("egw_48x40")
    kw = dict(max_iter=20, tol=1e-9, numItermax=2000, stopThr=1e-9)
    Tref, lref = oracle.entropic_gromov_wasserstein(g["C1"], g["C2"], epsilon=5e-2, **kw)
    C1 = torch.tensor(g["C1"], dtype=torch.float32, device=cuda)
    C2 = torch.tensor(g["C2"], dtype=torch.float32, device=cuda)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # fp32 inner solves stop at numItermax before 1e-9
        T, lg = pgw.entropic_gromov_wasserstein(C1, C2, None, None, "square_loss", epsilon=5e-2, log=True, **kw)
    T = T.double().cpu().numpy()
    assert np.abs(T - Tref).sum() / Tref.sum() <= 1e-3
    assert abs(float(lg["gw_dist"]) - lref["gw_dist"]) <= 1e-4 * abs(lref["gw_dist"])


def test_egw_log_inner_vs_oracle(cuda):
    rng = np.random.default_rng(5)
    n = 200
    xs = rng.standard_normal((n, 3))
    xt = rng.standard_normal((n, 8))
    C1 = oracle.sqeuclidean(xs, xs)
    C2 = oracle.sqeuclidean(xt, xt)
    C1 /= C1.max()
    C2 /= C2.max()
    Tref, lref = oracle.entropic_gw_log_inner(C1, C2, epsilon=2e-2, max_iter=6, numItermax=5000, stopThr=1e-7)
    for dt, tol_t, tol_g in ((torch.float64, 1e-7, 1e-9), (torch.float32, 2e-3, 2e-4)):
        T, lg = pgw.entropic_gromov_wasserstein_log(torch.tensor(C1, dtype=dt, device=cuda),
                                                    torch.tensor(C2, dtype=dt, device=cuda), epsilon=2e-2,
                                                    max_iter=6, numItermax=5000, stopThr=1e-7)
        T = T.double().cpu().numpy()
        assert np.abs(T - Tref).sum() / Tref.sum() <= tol_t, dt
        assert abs(lg["gw_dist"] - lref["gw_dist"]) <= tol_g * abs(lref["gw_dist"]), dt


@pytest.mark.parametrize("tag,kw", [("pgd", dict(alpha=0.5)), ("pgd_a02_warm", dict(alpha=0.2, warmstart=True)),
                                    ("ppa", dict(alpha=0.7, solver="PPA"))])
def test_fused_egw_f64_golden(cuda, tag, kw):
    g = golden("fgw_30x24")
    T, lg = pgw.entropic_fused_gromov_wasserstein(g["M"], g["C1"], g["C2"], g["p"], g["q"], epsilon=0.05,
                                                  max_iter=200, tol=1e-9, log=True, **kw)
    np.testing.assert_allclose(T, g[tag + "_T"], rtol=1e-7, atol=1e-13)
    np.testing.assert_allclose(np.array(lg["err"], dtype=float), g[tag + "_err"], rtol=1e-6, atol=1e-13)
    assert abs(float(lg["fgw_dist"]) - float(g[tag + "_fgw"])) <= 1e-9 * abs(float(g[tag + "_fgw"]))


def test_fused_egw2_and_asymmetric_f64_golden(cuda):
    g = golden("fgw_30x24")
    val, lg = pgw.entropic_fused_gromov_wasserstein2(g["M"], g["C1"], g["C2"], g["p"], g["q"], epsilon=0.05,
                                                     alpha=0.5, max_iter=200, tol=1e-9, log=True)
    assert abs(float(val) - float(g["fgw2"])) <= 1e-9 * abs(float(g["fgw2"]))
    assert abs(float(lg["quad_loss"]) - float(g["fgw2_quad"])) <= 1e-9 * abs(float(g["fgw2_quad"]))
    assert abs(float(lg["lin_loss"]) - float(g["fgw2_lin"])) <= 1e-9 * abs(float(g["fgw2_lin"]))
    g = golden("fgw_asym_30x24")
    T, lg = pgw.entropic_fused_gromov_wasserstein(g["M"], g["C1"], g["C2"], g["p"], g["q"], epsilon=0.05,
                                                  alpha=0.6, max_iter=200, tol=1e-9, log=True)
    np.testing.assert_allclose(T, g["T"], rtol=1e-7, atol=1e-13)
    assert abs(float(lg["fgw_dist"]) - float(g["fgw"])) <= 1e-9 * abs(float(g["fgw"]))


@pytest.mark.parametrize("name", ["fgw_30x24", "fgw_asym_30x24"])
def test_fused_egw_f32_tensor_cores_vs_oracle(cuda, name):
    g = golden(name)
    alpha = 0.5 if name == "fgw_30x24" else 0.6
    Tref, lref = oracle.entropic_fused_gromov_wasserstein(g["M"], g["C1"], g["C2"], g["p"], g["q"], epsilon=0.05,
                                                          alpha=alpha, max_iter=200, tol=1e-9)
    f = lambda x: torch.tensor(x, dtype=torch.float32, device=cuda)  # noqa: E731
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        T, lg = pgw.entropic_fused_gromov_wasserstein(f(g["M"]), f(g["C1"]), f(g["C2"]), f(g["p"]), f(g["q"]),
                                                      epsilon=0.05, alpha=alpha, max_iter=200, tol=1e-9, log=True)
    T = T.double().cpu().numpy()
    assert np.abs(T - Tref).sum() / Tref.sum() <= 1e-3
    assert abs(float(lg["fgw_dist"]) - lref["fgw_dist"]) <= 1e-4 * abs(lref["fgw_dist"])
