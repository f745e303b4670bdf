"""gbnuts: NUTS (diag_e, adaptive) sampling on GB300 for logistic / Poisson GLMs
and non-centred hierarchical normal / logistic models.

    from stan_gb300 import Model, services, sampler, callbacks, analyze, workloads
"""
from . import analyze, callbacks, workloads  # noqa: F401
from .model import Model  # noqa: F401
from . import sampler, services  # noqa: F401
