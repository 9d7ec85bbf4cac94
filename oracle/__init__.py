"""CPU oracle for the entropic-OT hot path (TEST INFRASTRUCTURE ONLY).

This package restates, in float64 numpy, the reference algorithms that the
GPU kernels of ``pot_gb300`` replace.  It exists to check results: only the
tests, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl
reference`` legs of ``bench.py`` may import it.  The product path never calls
into it and has no CPU fallback.

Parity pin: every function here is checked against golden vectors produced by
the reference itself (PythonOT/POT 0.9.7.dev0, imported in the build container
by ``tests/golden/gen_golden.py``) and against the reference's own doctest
values; see ``tests/test_oracle.py``.
"""
from .entropic import NONCONV, NUMERR, NUMERR_STAB  # noqa: F401
from .entropic import (  # noqa: F401
    sqeuclidean,
    logsumexp,
    sinkhorn_knopp,
    sinkhorn_log,
    greenkhorn,
    sinkhorn,
    sinkhorn2,
    sinkhorn_stabilized,
    sinkhorn_epsilon_scaling,
    barycenter_sinkhorn,
    barycenter_sinkhorn_log,
    sinkhorn_knopp_unbalanced,
    solve_entropic,
    empirical_sinkhorn2_lazy,
    log_projection_batch,
    scaling_projection_batch,
    solve_batch,
    init_matrix_square_loss,
    tensor_product,
    entropic_gromov_wasserstein,
    entropic_fused_gromov_wasserstein,
    entropic_gw_log_inner,
    empirical_sinkhorn_lazy,
    solve_gromov_batch,
)
