"""Parity of the batched GPU solver with the oracle and the reference goldens.

The ``ot.batch`` drop-ins stop the whole batch on its largest error, as the
reference does: float64 results equal the reference's own outputs (golden
fixtures) to rtol 1e-9 with the reference's ``n_iter``, in both the log and
the scaling form.  With ``per_problem=True`` every problem stops on its own
error; the exact oracle for that is the batch projection run one problem at
a time (same stop index, 1e-9).  float32 ragged batches: plan relative L1 <=
1e-5 against the float64 oracle and a float64 column-marginal violation of at
most 2x stopThr.
"""
import numpy as np
import pytest
import torch

import oracle
import pot_gb300 as pg
from conftest import golden
from pot_gb300 import batch as pb

pytestmark = pytest.mark.gpu


def per_problem_oracle(M, reg, a, b, max_iter, tol, solver):
    out = []
    for k in range(M.shape[0]):
        r = oracle.solve_batch(M[k:k + 1], reg, a[k:k + 1], b[k:k + 1], max_iter, tol, solver)
        out.append(r)
    return out


@pytest.mark.parametrize("solver", ["log_sinkhorn", "sinkhorn"])
@pytest.mark.parametrize("reg_type", ["entropy", "kl"])
def test_solve_batch_f64_equals_reference(cuda, solver, reg_type):
    """The reference's whole-batch stop (test/batch/test_solve_batch.py:28
    setting): plans, values and potentials of the reference to 1e-9, its
    n_iter exactly."""
    g = golden("batch_4x16")
    res = pb.solve_batch(g["M"], 0.1, max_iter=10000, tol=1e-5, solver=solver, reg_type=reg_type)
    tag = "%s_%s" % (solver, reg_type)
    assert res.log["n_iter"] == int(g[tag + "_n_iter"])
    np.testing.assert_allclose(res.plan, g[tag + "_plan"], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(res.value, g[tag + "_value"], rtol=1e-9)
    np.testing.assert_allclose(res.value_linear, g[tag + "_value_linear"], rtol=1e-9)
    np.testing.assert_allclose(res.potentials[0], g[tag + "_pot_u"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(res.potentials[1], g[tag + "_pot_v"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("solver", ["log_sinkhorn", "sinkhorn"])
def test_solve_batch_per_problem_stop(cuda, solver):
    """per_problem=True: every problem stops on its own error, exactly as the
    batch projection run one problem at a time."""
    g = golden("batch_4x16")
    M = g["M"]
    B, n, m = M.shape
    a = np.full((B, n), 1 / n)
    b = np.full((B, m), 1 / m)
    res = pb.solve_batch(M, 0.1, max_iter=10000, tol=1e-5, solver=solver, per_problem=True)
    ref = per_problem_oracle(M, 0.1, a, b, 10000, 1e-5, solver)
    for k in range(B):
        np.testing.assert_allclose(res.plan[k], ref[k]["plan"][0], rtol=1e-9, atol=1e-15)
        np.testing.assert_allclose(res.value[k], ref[k]["value"][0], rtol=1e-9)
        np.testing.assert_allclose(res.potentials[0][k], ref[k]["potentials"][0][0], rtol=1e-8, atol=1e-12)
    assert res.log["n_iter"] == max(r["n_iter"] for r in ref)
    assert res.log["n_iter"] <= int(g["%s_entropy_n_iter" % solver])


def test_solve_batch_padded_ragged(cuda):
    g = golden("batch_ragged_padded")
    res = pb.solve_batch(g["M"], float(g["reg"]), a=g["a"], b=g["b"], max_iter=20000, tol=1e-9)
    assert not np.isnan(res.plan).any()
    assert res.log["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(res.plan, g["plan"], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(res.value_linear, g["value_linear"], rtol=1e-9)


def test_solve_sample_batch(cuda):
    g = golden("batch_sample_3x20x25")
    res = pb.solve_sample_batch(g["X"], g["Y"], float(g["reg"]), max_iter=5000, tol=1e-7)
    assert res.log["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(res.plan, g["plan"], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(res.value, g["value"], rtol=1e-9)
    np.testing.assert_allclose(res.value_linear, g["value_linear"], rtol=1e-9)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_stop_is_reproducible(cuda, dtype):
    """The per-column errors are summed in a fixed order: ten runs of a batch
    give bit-identical potentials, errors and stop indices (float32 with the
    cluster tail handoff)."""
    Xs, Ys, As, Bs, regs = _ragged_case(5, 64, 20, 400)
    tol = 1e-9 if dtype == torch.float64 else 1e-6
    runs = [pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=20000, tol=tol,
                                   dtype=dtype) for _ in range(10)]
    for r in runs[1:]:
        assert torch.equal(r.niter, runs[0].niter)
        assert torch.equal(r.err, runs[0].err)
        assert torch.equal(r.u, runs[0].u) and torch.equal(r.v, runs[0].v)


def test_dist_batch_matches_oracle(cuda):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((3, 17, 5))
    Y = rng.standard_normal((3, 22, 5))
    M = pb.dist_batch(X, Y)
    for k in range(3):
        np.testing.assert_allclose(M[k], oracle.sqeuclidean(X[k], Y[k]), rtol=1e-12, atol=1e-12)


def test_projection_functions(cuda):
    rng = np.random.default_rng(1)
    M = rng.random((3, 10, 12))
    out = pb.bregman_log_projection_batch(-M / 0.2, max_iter=10000, tol=1e-9)
    assert out["T"].shape == (3, 10, 12) and out["log_T"].shape == (3, 10, 12)
    np.testing.assert_allclose(out["T"].sum(2), np.full((3, 10), 0.1), atol=1e-8)
    out2 = pb.bregman_projection_batch(np.exp(-M / 0.2), max_iter=10000, tol=1e-9)
    np.testing.assert_allclose(out2["T"], out["T"], atol=1e-8)


def _ragged_case(seed, B, lo, hi, dims=(3, 16)):
    rng = np.random.default_rng(seed)
    Xs, Ys, As, Bs, regs = [], [], [], [], []
    for k in range(B):
        n, m = rng.integers(lo, hi + 1, size=2)
        d = dims[k % len(dims)]
        Xs.append(rng.random((n, d)))
        Ys.append(rng.random((m, d)))
        As.append(rng.dirichlet(np.ones(n)))
        Bs.append(rng.dirichlet(np.ones(m)))
        regs.append(10 ** rng.uniform(-2, -1))
    return Xs, Ys, As, Bs, regs


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_ragged_vs_oracle(cuda, dtype):
    Xs, Ys, As, Bs, regs = _ragged_case(3, 24, 2, 300)
    tol = 1e-9 if dtype == torch.float64 else 1e-6
    res = pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=50000, tol=tol, dtype=dtype)
    torch.cuda.synchronize()
    st = res.status.cpu().numpy()
    nit = res.niter.cpu().numpy()
    for k in range(len(Xs)):
        M = oracle.sqeuclidean(Xs[k], Ys[k])
        reg = regs[k] * M.max()
        P, lg = oracle.sinkhorn_log(As[k], Bs[k], M, reg, numItermax=50000, stopThr=tol if dtype == torch.float64 else 1e-12)
        u, v = (t.double().cpu().numpy() for t in res.potentials(k))
        Pg = np.exp(-M / reg + u[:, None] + v[None, :])
        assert st[k] == 0, (k, st[k])
        if dtype == torch.float64:
            assert nit[k] == lg["niter"], (k, nit[k], lg["niter"])
            assert np.abs(Pg - P).sum() / P.sum() < 1e-9
        else:
            assert np.abs(Pg - P).sum() / P.sum() < 1e-5, k
            assert np.linalg.norm(Pg.sum(0) - Bs[k]) < 2 * tol


def test_ragged_sizes_at_the_limits(cuda):
    # 1x1, thin, wide and the largest column count the kernel takes in one pass
    rng = np.random.default_rng(4)
    shapes = [(1, 1), (1, 37), (37, 1), (3, 1024), (1024, 3), (5, 2048), (2048, 7)]
    Xs = [rng.random((n, 3)) for n, _ in shapes]
    Ys = [rng.random((m, 3)) for _, m in shapes]
    res = pb.solve_sample_ragged(Xs, Ys, 0.1, reg_relative=True, max_iter=20000, tol=1e-9, dtype=torch.float64)
    for k, (n, m) in enumerate(shapes):
        M = oracle.sqeuclidean(Xs[k], Ys[k])
        reg = 0.1 * M.max() if M.max() > 0 else 0.1
        if M.max() == 0:
            continue
        P, lg = oracle.sinkhorn_log([], [], M, reg, numItermax=20000, stopThr=1e-9)
        u, v = (t.cpu().numpy() for t in res.potentials(k))
        Pg = np.exp(-M / reg + u[:, None] + v[None, :])
        assert np.abs(Pg - P).sum() / P.sum() < 1e-9, (n, m)


def test_multi_and_per_cta_engines_agree(cuda):
    """The work-balanced engine and the CTA-per-problem engine run the same
    per-problem iteration: identical stop index, potentials to 1e-9."""
    Xs, Ys, As, Bs, regs = _ragged_case(8, 40, 1, 400)
    r1 = pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=20000, tol=1e-9,
                                dtype=torch.float64, engine="multi")
    r2 = pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=20000, tol=1e-9,
                                dtype=torch.float64, engine="cta")
    np.testing.assert_array_equal(r1.niter.cpu().numpy(), r2.niter.cpu().numpy())
    np.testing.assert_array_equal(r1.status.cpu().numpy(), r2.status.cpu().numpy())
    for k in range(len(Xs)):
        u1, v1 = (t.cpu().numpy() for t in r1.potentials(k))
        u2, v2 = (t.cpu().numpy() for t in r2.potentials(k))
        np.testing.assert_allclose(u1, u2, rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(v1, v2, rtol=1e-9, atol=1e-9)


def test_multi_engine_max_iter_and_single_problem(cuda):
    rng = np.random.default_rng(12)
    X = rng.random((700, 3))
    Y = rng.random((650, 3))
    r = pb.solve_sample_ragged([X], [Y], 0.003, reg_relative=True, max_iter=25, tol=1e-12, dtype=torch.float64)
    M = oracle.sqeuclidean(X, Y)
    P, lg = oracle.sinkhorn_log([], [], M, 0.003 * M.max(), numItermax=25, stopThr=1e-12)
    assert int(r.status[0]) == 1 and int(r.niter[0]) == lg["niter"] == 24
    u, v = (t.cpu().numpy() for t in r.potentials(0))
    np.testing.assert_allclose(u, lg["log_u"], rtol=1e-9, atol=1e-9)


def _gromov_kw(name, g):
    if name == "gromov_batch_fused":
        return dict(reg=0.01, M=g["M"], alpha=0.5, max_iter=1000, tol=1e-5, max_iter_inner=10000, tol_inner=1e-5,
                    symmetric=False)
    return dict(reg=0.05, max_iter=50, tol=1e-7, max_iter_inner=2000, tol_inner=1e-9)


@pytest.mark.parametrize("name", ["gromov_batch_fused", "gromov_batch_sym"])
def test_solve_gromov_batch(cuda, name):
    """float64, the reference's rules (inner whole-batch stop, outer stop on
    the largest mean plan change): the reference's own outputs to rtol 1e-8
    and its n_iter."""
    g = golden(name)
    res = pb.solve_gromov_batch(g["C1"], g["C2"], **_gromov_kw(name, g))
    assert res.log["n_iter"] == int(g["n_iter"])
    np.testing.assert_allclose(res.plan, g["plan"], rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(res.value, g["value"], rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(res.value_quad, g["value_quad"], rtol=1e-8, atol=1e-14)


@pytest.mark.parametrize("name", ["gromov_batch_fused", "gromov_batch_sym"])
def test_solve_gromov_batch_per_problem_inner(cuda, name):
    """per_problem=True: inner solves stop per problem, exactly as the oracle
    run with per-problem inner stops."""
    g = golden(name)
    kw = _gromov_kw(name, g)
    res = pb.solve_gromov_batch(g["C1"], g["C2"], per_problem=True, **kw)
    ref = oracle.solve_gromov_batch(g["C1"], g["C2"], per_problem_inner=True, **kw)
    assert res.log["n_iter"] == ref["n_iter"]
    np.testing.assert_allclose(res.plan, ref["plan"], rtol=1e-7, atol=1e-13)
    np.testing.assert_allclose(res.value_quad, ref["value_quad"], rtol=1e-7, atol=1e-13)


@pytest.mark.parametrize("sym", [True, False])
def test_solve_gromov_batch_f32_tensor_cores(cuda, sym):
    """float32 batches take the tcgen05 split-GEMM tensor product (both
    GEMMs of every problem in one launch each): against the float64 path on
    the same inputs, 5 outer steps (measured: plan L1 1.4e-6, values 6e-6)."""
    rng = np.random.default_rng(11)
    B, n, m = 6, 200, 150
    xs, xt = rng.standard_normal((B, n, 3)), rng.standard_normal((B, m, 8))
    C1 = ((xs[:, :, None] - xs[:, None]) ** 2).sum(-1)
    C2 = ((xt[:, :, None] - xt[:, None]) ** 2).sum(-1)
    if not sym:
        C1 = C1 + 0.3 * rng.random(C1.shape)
        C2 = C2 * (1 + 0.2 * rng.random(C2.shape))
    C1 /= C1.max(axis=(1, 2), keepdims=True)
    C2 /= C2.max(axis=(1, 2), keepdims=True)
    kw = dict(reg=0.05, max_iter=5, tol=1e-9, max_iter_inner=500, tol_inner=1e-6)
    r64 = pb.solve_gromov_batch(torch.tensor(C1, device=cuda), torch.tensor(C2, device=cuda), **kw)
    r32 = pb.solve_gromov_batch(torch.tensor(C1, dtype=torch.float32, device=cuda),
                                torch.tensor(C2, dtype=torch.float32, device=cuda), **kw)
    assert r32.log["n_iter"] == r64.log["n_iter"]
    p32, p64 = r32.plan.double().cpu().numpy(), r64.plan.cpu().numpy()
    assert np.abs(p32 - p64).sum() / np.abs(p64).sum() < 1e-5
    np.testing.assert_allclose(r32.value.double().cpu().numpy(), r64.value.cpu().numpy(), rtol=5e-5)


def test_solve_gromov_batch_f32_golden(cuda):
    """float32 on the reference's symmetric batch against the float64 oracle
    at the same inner tolerance (measured: plan L1 9.3e-6, value 1.1e-6)."""
    g = golden("gromov_batch_sym")
    kw = dict(reg=0.05, max_iter=50, tol=1e-7, max_iter_inner=2000, tol_inner=1e-6)
    res = pb.solve_gromov_batch(torch.tensor(g["C1"], dtype=torch.float32, device=cuda),
                                torch.tensor(g["C2"], dtype=torch.float32, device=cuda), **kw)
    ref = oracle.solve_gromov_batch(g["C1"], g["C2"], **kw)
    plan = res.plan.double().cpu().numpy()
    assert np.abs(plan - ref["plan"]).sum() / np.abs(ref["plan"]).sum() < 2e-5
    np.testing.assert_allclose(res.value.double().cpu().numpy(), ref["value"], rtol=1e-5)


@pytest.mark.parametrize("d", [2, 3, 8, 16, 5])
def test_cost_blocks_register_tiled(cuda, d):
    """float32 cost blocks of a ragged batch with a shared dimension (the
    register-tiled kernel for d in {2, 3, 8, 16}, the generic one for 5):
    sum_k (x_k - y_k)^2 against float64, +inf padding, per-problem maxima."""
    rng = np.random.default_rng(d)
    rows, cols = [1, 63, 64, 65, 300, 2048], [1, 255, 257, 64, 1000, 2048]
    X = [rng.standard_normal((n, d)) for n in rows]
    Y = [rng.standard_normal((m, d)) + 0.5 for m in cols]
    layout = pb.RaggedLayout(rows, cols, torch.float32, cuda)
    xo = np.concatenate([[0], np.cumsum([n * d for n in rows])[:-1]])
    yo = np.concatenate([[0], np.cumsum([m * d for m in cols])[:-1]])
    Xp = torch.tensor(np.concatenate([x.ravel() for x in X]), dtype=torch.float32, device=cuda)
    Yp = torch.tensor(np.concatenate([y.ravel() for y in Y]), dtype=torch.float32, device=cuda)
    M, mx = pb.batched_sqdist(layout, Xp, Yp, xo, yo, [d] * len(rows), want_max=True)
    M = M.cpu().numpy()
    mx = mx.cpu().numpy()
    for p, (n, m) in enumerate(zip(rows, cols)):
        ld = int(layout.ldm_np[p])
        blk = M[int(layout.m_off_np[p]):int(layout.m_off_np[p]) + n * ld].reshape(n, ld)
        x32 = X[p].astype(np.float32).astype(np.float64)
        y32 = Y[p].astype(np.float32).astype(np.float64)
        ref = ((x32[:, None, :] - y32[None, :, :]) ** 2).sum(-1)
        np.testing.assert_allclose(blk[:, :m], ref, rtol=2e-6, atol=1e-6)
        assert np.all(np.isinf(blk[:, m:]))
        assert abs(mx[p] - ref.max()) <= 2e-6 * ref.max()



def test_multi_over_relaxed_reaches_the_same_solution(cuda):
    """omega != 1 over-relaxes the updates (warm-start refinement): the stop
    test is the same exact marginal error, so the result is the plain solve's
    solution to within the tolerance, reached in fewer iterations."""
    rng = np.random.default_rng(9)
    B = 6
    rows = rng.integers(40, 120, B)
    cols = rng.integers(40, 120, B)
    layout = pb.RaggedLayout(rows, cols, torch.float64, cuda)
    Ms = []
    for n, m in zip(rows, cols):
        M = oracle.sqeuclidean(rng.random((n, 3)), rng.random((m, 3)))
        Ms.append(torch.tensor(M / M.max(), device=cuda))
    Mp = pb.pack_dense(layout, Ms)
    a = torch.cat([torch.full((int(n),), 1.0 / n, dtype=torch.float64, device=cuda) for n in rows])
    b = torch.cat([torch.full((int(m),), 1.0 / m, dtype=torch.float64, device=cuda) for m in cols])
    reg = 0.02
    plain = pb.run_multi(layout, Mp, a, b, reg, 20000, 1e-12)
    relax = pb.run_multi(layout, Mp, a, b, reg, 20000, 1e-12, omega=1.5)
    assert (relax[2] == 0).all() and (plain[2] == 0).all()
    assert relax[3].sum() < plain[3].sum()
    for p in range(B):
        r0, n = int(layout.r_off_np[p]), int(rows[p])
        up, ur = plain[0][r0:r0 + n], relax[0][r0:r0 + n]
        # potentials are defined up to a constant shared by u and -v
        np.testing.assert_allclose((ur - ur.mean()).cpu().numpy(), (up - up.mean()).cpu().numpy(), atol=1e-6)


def test_multi_stop_test_every_iteration(cuda):
    """check_period=1 applies the reference's stop criterion (column-marginal
    L2 error of the iterate below stopThr) at every iteration: each problem
    stops at the first iteration that meets it, with the potentials of the
    oracle's sinkhorn_log run for exactly that many iterations."""
    rng = np.random.default_rng(21)
    B = 5
    rows = rng.integers(30, 90, B)
    cols = rng.integers(30, 90, B)
    layout = pb.RaggedLayout(rows, cols, torch.float64, cuda)
    Ms = []
    for n, m in zip(rows, cols):
        M = oracle.sqeuclidean(rng.random((n, 3)), rng.random((m, 3)))
        Ms.append(M / M.max())
    Mp = pb.pack_dense(layout, [torch.tensor(M, device=cuda) for M in Ms])
    a = torch.cat([torch.full((int(n),), 1.0 / n, dtype=torch.float64, device=cuda) for n in rows])
    b = torch.cat([torch.full((int(m),), 1.0 / m, dtype=torch.float64, device=cuda) for m in cols])
    reg, tol = 0.03, 1e-9
    every = pb.run_multi(layout, Mp, a, b, reg, 20000, tol, check_period=1)
    tenth = pb.run_multi(layout, Mp, a, b, reg, 20000, tol)
    assert (every[2] == 0).all() and (tenth[2] == 0).all()
    n1, n10 = every[3].cpu().numpy(), tenth[3].cpu().numpy()
    assert (n10 % 10 == 0).all() and (n1 <= n10).all() and (n1 % 10 != 0).any()

    def col_err(M, n, m, it):
        _, lg = oracle.sinkhorn_log(np.full(n, 1.0 / n), np.full(m, 1.0 / m), M, reg, numItermax=it, stopThr=0.0)
        P = np.exp(lg["log_u"][:, None] - M / reg + lg["log_v"][None, :])
        return np.linalg.norm(P.sum(0) - 1.0 / m), lg

    for p in range(B):
        n, m, k = int(rows[p]), int(cols[p]), int(n1[p])
        e, lg = col_err(Ms[p], n, m, k + 1)
        assert e < tol and col_err(Ms[p], n, m, k)[0] >= tol, (p, k)
        assert abs(float(every[4][p]) - e) <= 1e-6 * tol + 1e-3 * e
        r0 = int(layout.r_off_np[p])
        np.testing.assert_allclose(every[0][r0:r0 + n].cpu().numpy(), lg["log_u"], rtol=1e-9, atol=1e-9)


def test_schedules_divide_work_without_changing_results(cuda, tmp_path, monkeypatch):
    """Every schedule the autotuner may pick (CTAs per SM, units per warp,
    row-split caps) runs the same per-problem iteration: float64 stop indices
    identical, potentials to 1e-9; tune_multi picks one of them and caches it."""
    from pot_gb300 import tune
    monkeypatch.setenv("POT_GB300_TUNE_CACHE", str(tmp_path / "sched.json"))
    monkeypatch.setattr(tune, "_TUNER", None)
    Xs, Ys, As, Bs, regs = _ragged_case(17, 30, 2, 700)
    base = pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=20000, tol=1e-9,
                                  dtype=torch.float64)
    L = base.layout
    ap = torch.cat([torch.as_tensor(a, dtype=torch.float64) for a in As]).to(cuda)
    bp = torch.cat([torch.as_tensor(b, dtype=torch.float64) for b in Bs]).to(cuda)
    for s in [tune.Schedule(1, 4, 8, 16), tune.Schedule(2, 16, 32, 32), tune.Schedule(1, 8, 16, 64)]:
        u, v, st, nit, err, _ = pb.run_multi(L, base.M, ap, bp, base.reg, 20000, 1e-9, schedule=s)
        np.testing.assert_array_equal(nit.cpu().numpy(), base.niter.cpu().numpy())
        np.testing.assert_allclose(u.cpu().numpy(), base.u.cpu().numpy(), rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(v.cpu().numpy(), base.v.cpu().numpy(), rtol=1e-9, atol=1e-9)
    best = tune.tune_multi(L, base.M, ap, bp, base.reg, iters=10, reps=1)
    assert best.ctas_per_sm in tune.SPACE["ctas_per_sm"]["f64"]
    assert tune.lookup(L) == best
    assert len(tune.tuner().trials) == 1
    r = pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=20000, tol=1e-9,
                               dtype=torch.float64, autotune=True)
    np.testing.assert_array_equal(r.niter.cpu().numpy(), base.niter.cpu().numpy())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_tail_clusters_continue_the_batch_iteration(cuda, dtype):
    """When few problems remain and each fits a cluster's shared memory, one
    thread-block cluster per problem finishes them: same stop indices
    (float64) and potentials as the batch kernel run to the end alone."""
    rng = np.random.default_rng(31)
    B = 12
    rows = np.concatenate([rng.integers(20, 60, B - 3), [301, 177, 5]])
    cols = np.concatenate([rng.integers(20, 60, B - 3), [190, 333, 700]])
    Ms = []
    for n, m in zip(rows, cols):
        M = oracle.sqeuclidean(rng.random((n, 3)), rng.random((m, 3)))
        Ms.append(torch.tensor(M / M.max(), dtype=dtype, device=cuda))
    # small reg on the three large problems: they run long after the others stop
    reg = torch.tensor([0.05] * (B - 3) + [0.004, 0.004, 0.01], dtype=torch.float64, device=cuda)
    tol = 1e-9 if dtype == torch.float64 else 1e-6
    cl, ncl, tile, err = pb.multi_tail_config(dtype)
    assert cl in (8, 16) and ncl >= 1 and tile >= 64 * 1024, (cl, ncl, tile, err)
    # (iterations, problems, handoff threshold): the whole batch from the start
    # (more problems than resident clusters: a queue), a late handoff of the
    # last four problems, and a handoff of problems that end at max_iter
    for max_iter, sub, tp in ((20000, slice(0, B), 0), (20000, slice(0, B), 4), (37, slice(B - 4, B), 0)):
        lay = pb.RaggedLayout(rows[sub], cols[sub], dtype, cuda)
        Mq = pb.pack_dense(lay, Ms[sub])
        aq = torch.cat([torch.full((int(n),), 1.0 / n, dtype=dtype, device=cuda) for n in rows[sub]])
        bq = torch.cat([torch.full((int(m),), 1.0 / m, dtype=dtype, device=cuda) for m in cols[sub]])
        info = {}
        off = pb.run_multi(lay, Mq, aq, bq, reg[sub], max_iter, tol, tail_problems=-1, info=info)
        assert info["handoff_ii"] == -1
        # float64 hands over only on request (its passes are FP64-bound)
        tp_on = tp if (tp > 0 or dtype == torch.float32) else 3 * ncl
        on = pb.run_multi(lay, Mq, aq, bq, reg[sub], max_iter, tol, tail_problems=tp_on, info=info)
        nb = lay.B
        limit = tp_on if tp_on > 0 else 3 * ncl
        assert info["handoff_ii"] >= 1 and 1 <= info["handoff_problems"] <= min(nb, limit)
        assert (info["handoff_ii"] == 1) == (nb <= limit)
        np.testing.assert_array_equal(on[2].cpu().numpy(), off[2].cpu().numpy())
        if dtype == torch.float64:
            np.testing.assert_array_equal(on[3].cpu().numpy(), off[3].cpu().numpy())
            np.testing.assert_allclose(on[0].cpu().numpy(), off[0].cpu().numpy(), rtol=1e-9, atol=1e-9)
            np.testing.assert_allclose(on[1].cpu().numpy(), off[1].cpu().numpy(), rtol=1e-9, atol=1e-9)
            np.testing.assert_allclose(on[4].cpu().numpy(), off[4].cpu().numpy(), rtol=1e-6, atol=1e-15)
        else:
            assert np.abs(on[3].cpu().numpy() - off[3].cpu().numpy()).max() <= 10
            for p in range(nb):
                r0, n = int(lay.r_off_np[p]), int(lay.rows_np[p])
                uo, uf = on[0][r0:r0 + n].double(), off[0][r0:r0 + n].double()
                np.testing.assert_allclose((uo - uo.mean()).cpu().numpy(), (uf - uf.mean()).cpu().numpy(),
                                           atol=2e-3 * max(1.0, float(uf.abs().max())))


def test_float64_batches_keep_every_sm_by_default(cuda):
    """float64 passes are bound by FP64 throughput: the batch kernel keeps its
    last problems on every SM unless a handoff is requested."""
    rng = np.random.default_rng(2)
    rows, cols = np.array([40, 50]), np.array([45, 30])
    layout = pb.RaggedLayout(rows, cols, torch.float64, cuda)
    Ms = [torch.tensor(oracle.sqeuclidean(rng.random((n, 3)), rng.random((m, 3))), device=cuda)
          for n, m in zip(rows, cols)]
    Mp = pb.pack_dense(layout, Ms)
    a = torch.cat([torch.full((int(n),), 1.0 / n, dtype=torch.float64, device=cuda) for n in rows])
    b = torch.cat([torch.full((int(m),), 1.0 / m, dtype=torch.float64, device=cuda) for m in cols])
    info = {}
    pb.run_multi(layout, Mp, a, b, 0.05, 1000, 1e-9, info=info)
    assert info["handoff_ii"] == -1
    pb.run_multi(layout, Mp, a, b, 0.05, 1000, 1e-9, tail_problems=4, info=info)
    assert info["handoff_ii"] == 1


def _small_batch(seed, B, lo, hi, dtype, cuda):
    rng = np.random.default_rng(seed)
    rows = rng.integers(lo, hi, B)
    cols = rng.integers(lo, hi, B)
    layout = pb.RaggedLayout(rows, cols, dtype, cuda)
    Ms = []
    for n, m in zip(rows, cols):
        M = oracle.sqeuclidean(rng.random((n, 3)), rng.random((m, 3)))
        Ms.append(M / M.max())
    Mp = pb.pack_dense(layout, [torch.tensor(M, dtype=dtype, device=cuda) for M in Ms])
    a = torch.cat([torch.full((int(n),), 1.0 / n, dtype=dtype, device=cuda) for n in rows])
    b = torch.cat([torch.full((int(m),), 1.0 / m, dtype=dtype, device=cuda) for m in cols])
    return layout, Ms, Mp, a, b, rows, cols


@pytest.mark.parametrize("depth", [3, 5, 8])
def test_multi_anderson_matches_oracle(cuda, depth):
    """Anderson mixing of the v update (anderson_depth): float64 stop indices
    equal to the oracle's restatement of the same iteration, potentials to
    1e-8; the stop test is the plain one (column marginal below tol, row
    marginal exact), reached in fewer iterations than the plain solve."""
    from oracle import accelerated as acc
    layout, Ms, Mp, a, b, rows, cols = _small_batch(41, 6, 30, 160, torch.float64, cuda)
    reg, tol = 0.02, 1e-9
    res = pb.run_multi(layout, Mp, a, b, reg, 20000, tol, check_period=1, anderson=depth)
    plain = pb.run_multi(layout, Mp, a, b, reg, 20000, tol, check_period=1)
    assert (res[2] == 0).all()
    assert res[3].sum() < plain[3].sum()
    for p in range(layout.B):
        n, m = int(rows[p]), int(cols[p])
        u, v, it, errs = acc.sinkhorn_log_anderson_v(np.full(n, 1 / n), np.full(m, 1 / m), Ms[p], reg, depth=depth,
                                                     numItermax=20000, stopThr=tol, check_period=1)
        assert int(res[3][p]) == it, (p, int(res[3][p]), it)
        r0, c0 = int(layout.r_off_np[p]), int(layout.c_off_np[p])
        np.testing.assert_allclose(res[0][r0:r0 + n].cpu().numpy(), u, rtol=1e-8, atol=1e-8)
        np.testing.assert_allclose(res[1][c0:c0 + m].cpu().numpy(), v, rtol=1e-8, atol=1e-8)
        P = np.exp(u[:, None] - Ms[p] / reg + v[None, :])
        assert np.linalg.norm(P.sum(0) - 1 / m) < tol
        assert np.abs(P.sum(1) - 1 / n).max() < 1e-14


def test_multi_anderson_float32_meets_the_plain_test(cuda):
    """float32 with Anderson mixing: every problem converges with its float64
    column-marginal error below 2 tol, and its plan is within 1e-4 (relative
    L1) of the converged float64 solution (a stop at tol = 1e-6 itself leaves
    1e-5 to 4e-5 there, for the plain iteration as well)."""
    layout, Ms, Mp, a, b, rows, cols = _small_batch(43, 8, 100, 700, torch.float32, cuda)
    reg, tol = 0.02, 1e-6
    res = pb.run_multi(layout, Mp, a, b, reg, 20000, tol, check_period=1, anderson=5)
    assert (res[2] == 0).all()
    for p in range(layout.B):
        n, m = int(rows[p]), int(cols[p])
        Pref, _ = oracle.sinkhorn_log(np.full(n, 1 / n), np.full(m, 1 / m), Ms[p], reg, numItermax=20000,
                                      stopThr=1e-12)
        r0, c0 = int(layout.r_off_np[p]), int(layout.c_off_np[p])
        u = res[0][r0:r0 + n].double().cpu().numpy()
        v = res[1][c0:c0 + m].double().cpu().numpy()
        P = np.exp(u[:, None] - Ms[p] / reg + v[None, :])
        assert np.linalg.norm(P.sum(0) - 1 / m) < 2 * tol
        assert np.abs(P - Pref).sum() / Pref.sum() < 1e-4
