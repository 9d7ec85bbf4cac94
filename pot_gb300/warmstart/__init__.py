"""Learned warm start for Sinkhorn: a point-cloud network predicts the
source potential, the solver's first half-step (the c-transform) gives the
target potential.  No counterpart in the reference; it feeds the existing
``warmstart=(log_u, log_v)`` argument of ``sinkhorn_log``
(ot/bregman/_sinkhorn.py:864-868)."""
