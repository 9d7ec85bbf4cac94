"""Property tests of host-side logic (no GPU): the packed layout of ragged
batches and the schedule search."""
import numpy as np
import pytest
import torch

from pot_gb300 import batch as pb
from pot_gb300 import tune

hypothesis = pytest.importorskip("hypothesis")
st = hypothesis.strategies


@hypothesis.given(st.lists(st.tuples(st.integers(1, 300), st.integers(1, 300)), min_size=1, max_size=12),
                  st.sampled_from([torch.float32, torch.float64]))
@hypothesis.settings(max_examples=60, deadline=None)
def test_ragged_layout_blocks_are_aligned_and_disjoint(shapes, dtype):
    rows = [r for r, _ in shapes]
    cols = [c for _, c in shapes]
    L = pb.RaggedLayout(rows, cols, dtype, torch.device("cpu"))
    es = 4 if dtype == torch.float32 else 8
    assert (L.ldm_np >= L.cols_np).all() and ((L.ldm_np * es) % 16 == 0).all()
    assert ((L.m_off_np * es) % 16 == 0).all()
    ends = L.m_off_np + L.rows_np * L.ldm_np
    assert (L.m_off_np[1:] == ends[:-1]).all() and int(ends[-1]) == L.total_m
    assert L.total_r == sum(rows) and L.total_c == sum(cols)
    # the largest-work-first order is a permutation
    assert sorted(L.order.tolist()) == list(range(len(shapes)))


@hypothesis.given(st.lists(st.floats(0.1, 10.0), min_size=5, max_size=5), st.floats(0.1, 10.0))
@hypothesis.settings(max_examples=40, deadline=None)
def test_schedule_search_returns_a_candidate_no_slower_than_the_start(weights, tail_w):
    t = tune.Tuner("")

    def cost(s):  # a separable convex cost with its optimum somewhere in the space
        return (weights[0] * abs(s.ctas_per_sm - 3) + weights[1] * abs(np.log2(s.units_per_warp) - 3)
                + weights[2] * abs(np.log2(s.cap_fill) - 4) + 0.01 * weights[3])

    best = t.search("k", "f32", cost, lambda s: tail_w * abs(np.log2(s.cap_tail) - 5), reps=1)
    assert best.ctas_per_sm in tune.SPACE["ctas_per_sm"]["f32"]
    assert best.units_per_warp in tune.SPACE["units_per_warp"]
    assert best.cap_fill in tune.SPACE["cap_fill"] and best.cap_tail in tune.SPACE["cap_tail"]
    start = tune.DEFAULT._replace(ctas_per_sm=max(tune.SPACE["ctas_per_sm"]["f32"]))
    assert cost(best) <= cost(start)
    assert t.get("k") == best


@hypothesis.given(st.integers(2, 30), st.integers(2, 30), st.floats(0.05, 1.0), st.integers(0, 10_000))
@hypothesis.settings(max_examples=30, deadline=None)
def test_oracle_forms_agree(n, m, reg, seed):
    """The oracle's scaling and log forms run the same iteration: the same
    stop index and plans equal to rounding (the reference's own
    test_sinkhorn_variants compares them within 1e-5); the stabilised form
    without absorptions equals them too."""
    import oracle
    rng = np.random.default_rng(seed)
    M = oracle.sqeuclidean(rng.random((n, 2)), rng.random((m, 2)))
    M /= max(M.max(), 1e-12)
    a, b = rng.dirichlet(np.ones(n)), rng.dirichlet(np.ones(m))
    P1, l1 = oracle.sinkhorn_knopp(a, b, M, reg, stopThr=1e-10)
    P2, l2 = oracle.sinkhorn_log(a, b, M, reg, stopThr=1e-10)
    P3, l3 = oracle.sinkhorn_stabilized(a, b, M, reg, stopThr=1e-10, tau=1e300)
    assert l1["niter"] == l2["niter"]
    np.testing.assert_allclose(P1, P2, rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(P3, P2, rtol=1e-8, atol=1e-14)
    # the returned plan meets the stop test (column-marginal L2 error below stopThr)
    # unless the iteration cap ended the solve
    if l2["niter"] < 999:
        assert np.linalg.norm(P2.sum(0) - b) < 1e-10
