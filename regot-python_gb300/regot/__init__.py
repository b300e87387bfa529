"""regot: GPU (GB300, sm_103a) implementation of RegOT's dense solvers.

Drop-in for the reference package's ``regot`` module for the solvers
sinkhorn_bcd, sinkhorn_newton, sinkhorn_ssns, qrot_lbfgs_dual and qrot_assn
(reference: regot/__init__.py:1 re-exports regot._internal).
"""
from ._internal import *  # noqa: F401,F403
from ._internal import Problem  # noqa: F401

__version__ = "0.1.0"
