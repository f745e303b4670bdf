"""The oracle's log densities pinned to an independent restatement.

No reference test pins logistic, Poisson or hierarchical-normal log p values
(those live in Stan Math, absent here).  tests/logdensity_exact.py restates
each density from its distributions' definitions, with Stan's propto and
Jacobian semantics (the call sites src/stan/model/log_prob_grad.hpp:40-44,
79-83 and log_prob_propto.hpp:43-46), in extended precision.  The oracle
(compensated FP64 sums) must agree to 1e-13 relative in lp and in the
gradient's 2-norm: at seeded points of every family with all four
propto / jacobian settings, and at the full sizes of the benchmark workloads
(logistic N = 1000 K = 25 and N = 1e5 K = 100, hierarchical normal J = 2000,
Poisson N = 262144 K = 512).  The device's FP64 form is checked against the
same restatement through tests/golden/logdensity_exact.npz
(tests/test_gpu_loglik.py).
"""
import os

import numpy as np
import pytest

from tests import logdensity_exact as exact
from tests.datasets import logistic_laplace_draws, make_dataset

TOL = 1e-13


def _check(ds, th, propto=True, jacobian=True, tol=TOL):
    om = ds.oracle_model()
    lp_x, g_x = exact.for_dataset(ds, th, propto, jacobian)
    lp_o, g_o = om.log_prob_grad(th, propto, jacobian)
    assert abs(lp_o - lp_x) <= tol * abs(lp_x), (lp_o, lp_x)
    assert np.linalg.norm(g_o - g_x) <= tol * np.linalg.norm(g_x)
    assert om.log_prob(th, propto, jacobian) == lp_o


@pytest.mark.parametrize("kind", ["logistic", "poisson", "hier_normal", "hier_logistic"])
@pytest.mark.parametrize("propto,jacobian", [(True, True), (True, False), (False, True),
                                             (False, False)])
def test_oracle_matches_exact_restatement(kind, propto, jacobian):
    ds = make_dataset(kind, small=True, seed=21)
    rng = np.random.default_rng(22)
    for _ in range(3):
        _check(ds, rng.normal(size=ds.D) * 0.4, propto, jacobian)


@pytest.mark.parametrize("kind,scale", [("logistic", 0.3), ("logistic_100k", 0.05),
                                        ("hier_normal", 0.2), ("poisson", 0.05)])
def test_oracle_matches_exact_restatement_full_size(kind, scale):
    ds = make_dataset(kind, small=False, seed=1)
    th = np.random.default_rng(23).normal(size=ds.D) * scale
    _check(ds, th)


def test_oracle_at_a_posterior_point_full_size():
    """Near the posterior the gradient is a heavily cancelling sum of 1e5
    terms: the compensated oracle still holds 1e-13 of its 2-norm."""
    ds = make_dataset("logistic_100k", small=False, seed=1)
    th = logistic_laplace_draws(ds, 1, seed=3)[0]
    _check(ds, th)


def test_golden_fixture_is_the_exact_restatement():
    """The committed fixture the GPU test reads holds the restatement's values
    for its own datasets (recomputed here)."""
    path = os.path.join(os.path.dirname(__file__), "golden", "logdensity_exact.npz")
    f = np.load(path)
    for name in [k[:-3] for k in f.files if k.endswith("__X")]:
        kind = int(f[name + "__kind"])
        X, y = f[name + "__X"], f[name + "__y"]
        group = f[name + "__group"] if name + "__group" in f.files else None
        J = int(f[name + "__J"])
        hp = tuple(f[name + "__hp"])
        intercept = bool(f[name + "__intercept"])
        th = f[name + "__theta"]
        for v, (propto, jac) in enumerate([(1, 1), (1, 0), (0, 1), (0, 0)]):
            for i in range(th.shape[0]):
                lp, g = exact.lp_grad(kind, X, y, th[i], group, J, hp, intercept, propto, jac)
                assert lp == f[name + "__lp"][v, i]
                assert np.array_equal(g, f[name + "__grad"][v, i])
