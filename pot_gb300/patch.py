"""Route an installed POT (``import ot``) through the GPU implementations.

POT binds the solver functions by name at import time in several modules,
so rebinding ``ot.sinkhorn`` alone is not enough.  ``patch_pot(ot)``
replaces the hot-path names in every module that imported them:

    ot/__init__.py:56            sinkhorn, sinkhorn2
    ot/bregman/__init__.py:13    sinkhorn, sinkhorn2, sinkhorn_knopp, sinkhorn_log, sinkhorn_stabilized,
                                 sinkhorn_epsilon_scaling, greenkhorn, empirical_sinkhorn, empirical_sinkhorn2,
                                 barycenter, barycenter_sinkhorn
    ot/bregman/_sinkhorn.py      sinkhorn_knopp, sinkhorn_log, sinkhorn_stabilized,
                                 sinkhorn_epsilon_scaling, greenkhorn (the dispatcher's callees)
    ot/bregman/_empirical.py:18  sinkhorn, sinkhorn2
    ot/gromov/_bregman.py:17     sinkhorn
    ot/gromov/__init__.py        entropic_gromov_wasserstein(2), entropic_fused_gromov_wasserstein(2)
    ot/batch/__init__.py         solve_batch, solve_sample_batch, dist_batch,
                                 bregman_log_projection_batch, bregman_projection_batch
    ot/batch/_linear.py          the same (module-level callers)
    ot/batch/_quadratic.py:14    bregman_log_projection_batch
    ot/solvers.py:13-14          sinkhorn_log, empirical_sinkhorn2, sinkhorn_knopp_unbalanced (the
                                 entropic branches of ot.solve / ot.solve_sample)
    ot/unbalanced/__init__.py    sinkhorn_unbalanced(2), sinkhorn_knopp_unbalanced
    ot/unbalanced/_sinkhorn.py   sinkhorn_knopp_unbalanced (the dispatcher's callee)
    ot/bregman/_barycenter.py:20, ot/da.py:19, ot/optim.py:14, ot/lowrank.py:13, ot/factored.py:12,
    ot/coot.py:14, ot/gromov/_estimators.py:14
                                 sinkhorn (consumers that bound it at import)

Calls the GPU path does not cover (other methods, metrics or losses) raise
NotImplementedError from the GPU function; ``unpatch_pot`` restores the
original bindings.
"""
import importlib

from . import bregman, batch, gromov, empirical, solvers, barycenters, unbalanced

GPU = {
    "sinkhorn": bregman.sinkhorn,
    "sinkhorn2": bregman.sinkhorn2,
    "sinkhorn_knopp": bregman.sinkhorn_knopp,
    "sinkhorn_log": bregman.sinkhorn_log,
    "sinkhorn_stabilized": bregman.sinkhorn_stabilized,
    "sinkhorn_epsilon_scaling": bregman.sinkhorn_epsilon_scaling,
    "greenkhorn": bregman.greenkhorn,
    "empirical_sinkhorn2": solvers.empirical_sinkhorn2,
    "empirical_sinkhorn_divergence": solvers.empirical_sinkhorn_divergence,
    "barycenter": barycenters.barycenter,
    "barycenter_sinkhorn": barycenters.barycenter_sinkhorn,
    "sinkhorn_unbalanced": unbalanced.sinkhorn_unbalanced,
    "sinkhorn_unbalanced2": unbalanced.sinkhorn_unbalanced2,
    "sinkhorn_knopp_unbalanced": unbalanced.sinkhorn_knopp_unbalanced,
    "empirical_sinkhorn": empirical.empirical_sinkhorn,
    "entropic_gromov_wasserstein": gromov.entropic_gromov_wasserstein,
    "entropic_gromov_wasserstein2": gromov.entropic_gromov_wasserstein2,
    "entropic_fused_gromov_wasserstein": gromov.entropic_fused_gromov_wasserstein,
    "entropic_fused_gromov_wasserstein2": gromov.entropic_fused_gromov_wasserstein2,
    "solve_batch": batch.solve_batch,
    "solve_sample_batch": batch.solve_sample_batch,
    "dist_batch": batch.dist_batch,
    "bregman_log_projection_batch": batch.bregman_log_projection_batch,
    "bregman_projection_batch": batch.bregman_projection_batch,
}

MODULES = {
    "": ["sinkhorn", "sinkhorn2"],
    ".bregman": ["sinkhorn", "sinkhorn2", "sinkhorn_knopp", "sinkhorn_log", "sinkhorn_stabilized",
                 "sinkhorn_epsilon_scaling", "greenkhorn", "empirical_sinkhorn", "empirical_sinkhorn2", "barycenter",
                 "barycenter_sinkhorn", "empirical_sinkhorn_divergence"],
    ".bregman._sinkhorn": ["sinkhorn_knopp", "sinkhorn_log", "sinkhorn_stabilized", "sinkhorn_epsilon_scaling",
                           "greenkhorn"],
    ".bregman._empirical": ["sinkhorn", "sinkhorn2"],
    ".gromov": ["entropic_gromov_wasserstein", "entropic_gromov_wasserstein2", "entropic_fused_gromov_wasserstein",
                "entropic_fused_gromov_wasserstein2"],
    ".gromov._bregman": ["sinkhorn"],
    ".batch": ["solve_batch", "solve_sample_batch", "dist_batch", "bregman_log_projection_batch",
               "bregman_projection_batch"],
    ".batch._linear": ["solve_batch", "dist_batch", "bregman_log_projection_batch", "bregman_projection_batch"],
    ".batch._quadratic": ["bregman_log_projection_batch"],
    ".solvers": ["sinkhorn_log", "empirical_sinkhorn2", "sinkhorn_knopp_unbalanced"],
    ".unbalanced": ["sinkhorn_unbalanced", "sinkhorn_unbalanced2", "sinkhorn_knopp_unbalanced"],
    ".unbalanced._sinkhorn": ["sinkhorn_knopp_unbalanced"],
    # consumers that bind `sinkhorn` at import (their Sinkhorn calls then run on the GPU)
    ".bregman._barycenter": ["sinkhorn"],
    ".da": ["sinkhorn"],
    ".optim": ["sinkhorn"],
    ".lowrank": ["sinkhorn"],
    ".factored": ["sinkhorn"],
    ".coot": ["sinkhorn"],
    ".gromov._estimators": ["sinkhorn"],
}

_saved = {}


def _module(root, suffix):
    name = root.__name__ + suffix
    try:
        return importlib.import_module(name)
    except ImportError:
        return None


def patch_pot(ot_module):
    """Rebind POT's hot-path names to the GPU implementations; returns the
    list of (module, name) pairs that were replaced."""
    done = []
    for suffix, names in MODULES.items():
        mod = _module(ot_module, suffix)
        if mod is None:
            continue
        for name in names:
            if hasattr(mod, name):
                key = (mod.__name__, name)
                if key not in _saved:
                    _saved[key] = getattr(mod, name)
                setattr(mod, name, GPU[name])
                done.append(key)
    return done


def unpatch_pot(ot_module):
    """Restore the bindings replaced by ``patch_pot``."""
    for (modname, name), fn in list(_saved.items()):
        mod = importlib.import_module(modname)
        setattr(mod, name, fn)
        del _saved[(modname, name)]
