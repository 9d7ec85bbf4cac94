"""Host-side logic that needs no GPU."""
import numpy as np
import pytest
import torch

import pot_gb300 as pg
from pot_gb300._arrays import Boundary, is_empty


def test_no_cpu_fallback():
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        pg.sinkhorn([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0)


def test_unknown_method_raises_before_any_device_work():
    with pytest.raises(ValueError):
        pg.sinkhorn([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0, method="new_method")
    with pytest.raises(ValueError):
        pg.sinkhorn2([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0, method="new_method")


def test_histogram_lengths_checked_before_device_work():
    """A histogram whose length does not match the cost's side is a ValueError
    on the host (the kernels would otherwise read past it); 2-D b (several
    histograms) and empty weights pass the check."""
    from pot_gb300.bregman import _check_shapes
    M = np.zeros((4, 3))
    with pytest.raises(ValueError):
        pg.sinkhorn(np.full(3, 1 / 3), np.full(3, 1 / 3), M, 1.0)
    with pytest.raises(ValueError):
        pg.sinkhorn2(np.full(4, 0.25), [0.5, 0.5], M, 1.0)
    with pytest.raises(ValueError):
        pg.greenkhorn(np.full(4, 0.25), np.full(4, 0.25), M, 1.0)
    with pytest.raises(ValueError):
        _check_shapes([], [], np.zeros(5))
    _check_shapes(np.full(4, 0.25), np.full((3, 2), 1 / 3), M)
    _check_shapes([], None, [[0.0, 1.0], [1.0, 0.0]])
    _check_shapes(torch.full((4,), 0.25), torch.full((3,), 1 / 3), torch.zeros(4, 3))


def test_point_gw_and_batch_shapes_checked_before_device_work():
    """The point-cloud, GW and batch drop-ins check their weights and side
    inputs against the problem sizes on the host; shapes the reference
    accepts pass the check (and then need the GPU)."""
    from pot_gb300 import batch as pb
    from pot_gb300 import gromov as pgw
    X, Y = np.zeros((5, 2)), np.zeros((4, 2))
    with pytest.raises(ValueError):
        pg.empirical_sinkhorn(X, Y, 1.0, a=np.full(4, 0.25))
    with pytest.raises(ValueError):
        pg.empirical_sinkhorn(X, np.zeros((4, 3)), 1.0)
    C1, C2 = np.zeros((5, 5)), np.zeros((4, 4))
    with pytest.raises(ValueError):
        pgw.entropic_gromov_wasserstein(C1, C2, np.full(4, 0.25), None)
    with pytest.raises(ValueError):
        pgw.entropic_gromov_wasserstein(np.zeros((5, 4)), C2)
    with pytest.raises(ValueError):
        pgw.entropic_fused_gromov_wasserstein(np.zeros((4, 5)), C1, C2)
    M = np.zeros((3, 5, 4))
    with pytest.raises(ValueError):
        pb.solve_batch(M, 0.1, a=np.full((3, 4), 0.25))
    with pytest.raises(ValueError):
        pb.bregman_log_projection_batch(M, b=np.full((2, 4), 0.25))
    with pytest.raises(ValueError):
        pb.solve_gromov_batch(np.zeros((3, 5, 5)), np.zeros((3, 4, 4)), b=np.full((3, 5), 0.2))
    if not torch.cuda.is_available():
        # shapes the reference accepts get past the check, to the device
        for call in (lambda: pb.solve_batch(M, 0.1, a=np.full(5, 0.2), b=np.full((3, 4), 0.25)),
                     lambda: pg.empirical_sinkhorn(X, Y, 1.0, a=np.full(5, 0.2)),
                     lambda: pgw.entropic_gromov_wasserstein(C1, C2, np.full(5, 0.2), np.full(4, 0.25))):
            with pytest.raises(RuntimeError, match="CUDA"):
                call()


def test_one_histogram_methods_have_no_loss_form():
    """test/test_bregman.py:1404-1407: sinkhorn2 accepts neither 'greenkhorn'
    nor 'sinkhorn_epsilon_scaling' (ValueError, before any device work)."""
    for method in ("greenkhorn", "sinkhorn_epsilon_scaling"):
        with pytest.raises(ValueError):
            pg.sinkhorn2([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0, method=method)


def test_greenkhorn_without_gpu_raises():
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        pg.sinkhorn([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0, method="greenkhorn")


def test_is_empty():
    assert is_empty([]) and is_empty(np.array([])) and is_empty(torch.tensor([]))
    assert not is_empty([1.0])


def test_patch_rebinds_every_importing_module(tmp_path, monkeypatch):
    """patch_pot replaces the names in all modules that bound them at import
    (a fake package tree stands in for POT)."""
    import sys
    import types
    from pot_gb300 import patch as pp
    root = types.ModuleType("fakeot")
    root.__path__ = []
    sys.modules["fakeot"] = root
    made = {}
    for suffix, names in pp.MODULES.items():
        if suffix == "":
            mod = root
        else:
            mod = types.ModuleType("fakeot" + suffix)
            sys.modules["fakeot" + suffix] = mod
        for nm in names:
            setattr(mod, nm, ("orig", suffix, nm))
        made[suffix] = mod
    try:
        done = pp.patch_pot(root)
        assert len(done) == sum(len(v) for v in pp.MODULES.values())
        for suffix, names in pp.MODULES.items():
            for nm in names:
                assert getattr(made[suffix], nm) is pp.GPU[nm]
        pp.unpatch_pot(root)
        for suffix, names in pp.MODULES.items():
            for nm in names:
                assert getattr(made[suffix], nm) == ("orig", suffix, nm)
    finally:
        for k in list(sys.modules):
            if k == "fakeot" or k.startswith("fakeot."):
                del sys.modules[k]


def test_otresult_fields_and_marginals():
    """OTResult (the container of ot.solve / ot.batch results, ot/utils.py:1127)
    exposes the reference's field names; marginals sum the plan over its last
    two axes (batched plans keep their batch axis)."""
    import numpy as np
    from pot_gb300.utils import OTResult
    P = np.arange(24, dtype=float).reshape(2, 3, 4)
    r = OTResult(potentials=("u", "v"), value=1.5, value_linear=1.0, plan=P, log={"n_iter": 3}, status=0)
    assert r.potential_a == "u" and r.potential_b == "v" and r.value == 1.5 and r.value_linear == 1.0
    np.testing.assert_array_equal(r.marginal_a, P.sum(-1))
    np.testing.assert_array_equal(r.marginal_b, P.sum(-2))
    assert r.log["n_iter"] == 3 and r.status == 0
    assert "value=1.5" in repr(r) and "shape=(2, 3, 4)" in repr(r)
    empty = OTResult()
    assert empty.marginals == (None, None) and empty.potential_a is None and repr(empty) == "OTResult()"
