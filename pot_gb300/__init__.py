"""pot_gb300 — GB300-native entropic optimal transport.

Drop-in GPU implementations of PythonOT/POT's entropic-OT hot path:
``sinkhorn`` / ``sinkhorn2`` (methods 'sinkhorn', 'sinkhorn_log',
'sinkhorn_stabilized', 'sinkhorn_epsilon_scaling', 'greenkhorn'), the ``ot.batch`` solvers,
entropic Gromov-Wasserstein, the lazy empirical Sinkhorn, and the entropic
branches of ``solve`` / ``solve_sample``.  All arithmetic runs in hand-written
CUDA kernels for sm_103a (``pot_gb300/csrc``) behind the C ABI of
``include/pot_gb300.h``; there is no CPU fallback.
"""
from .bregman import sinkhorn, sinkhorn2, sinkhorn_knopp, sinkhorn_log  # noqa: F401
from .bregman import sinkhorn_stabilized, sinkhorn_epsilon_scaling, greenkhorn  # noqa: F401
from . import batch  # noqa: F401
from .batch import solve_batch, solve_sample_batch, dist_batch  # noqa: F401
from . import gromov  # noqa: F401
from . import graphs, tune  # noqa: F401
from .empirical import empirical_sinkhorn  # noqa: F401
from .solvers import solve, solve_sample, empirical_sinkhorn2, empirical_sinkhorn_divergence  # noqa: F401
from .barycenters import barycenter, barycenter_sinkhorn  # noqa: F401
from .unbalanced import sinkhorn_unbalanced, sinkhorn_unbalanced2, sinkhorn_knopp_unbalanced  # noqa: F401
from .utils import dist, OTResult  # noqa: F401
from .patch import patch_pot, unpatch_pot  # noqa: F401

__version__ = "0.1.0"
