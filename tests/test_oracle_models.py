"""Oracle log densities: analytic gradients against central finite differences
(the idea of src/stan/model/test_gradients.hpp:40), propto semantics, and
compensated vs plain sums."""
import math

import numpy as np
import pytest

import oracle
from tests.datasets import make_dataset


def _fd_grad(m, th, h=1e-6):
    g = np.zeros_like(th)
    for i in range(th.size):
        e = np.zeros_like(th)
        e[i] = h
        g[i] = (m.log_prob(th + e) - m.log_prob(th - e)) / (2 * h)
    return g


@pytest.mark.parametrize("kind", ["logistic", "poisson", "hier_normal", "hier_logistic"])
def test_gradient_matches_finite_differences(kind):
    ds = make_dataset(kind, small=True, seed=3)
    m = ds.oracle_model()
    rng = np.random.default_rng(5)
    for _ in range(3):
        th = rng.normal(size=m.D) * 0.3
        lp, g = m.log_prob_grad(th)
        assert lp == pytest.approx(m.log_prob(th), rel=1e-14)
        fd = _fd_grad(m, th)
        assert np.max(np.abs(g - fd)) <= 1e-5 * max(1.0, np.max(np.abs(g)))


@pytest.mark.parametrize("kind", ["logistic", "poisson", "hier_normal", "hier_logistic"])
def test_propto_drops_only_constants(kind):
    ds = make_dataset(kind, small=True, seed=4)
    m = ds.oracle_model()
    rng = np.random.default_rng(6)
    a, b = rng.normal(size=m.D) * 0.2, rng.normal(size=m.D) * 0.2
    da = m.log_prob(a, propto=False) - m.log_prob(a, propto=True)
    db = m.log_prob(b, propto=False) - m.log_prob(b, propto=True)
    assert da == pytest.approx(db, rel=1e-12, abs=1e-9)
    assert abs(da) > 0


def test_plain_and_compensated_sums_agree():
    ds = make_dataset("logistic", small=False, seed=1)
    mc = ds.oracle_model(compensated=True)
    mp = ds.oracle_model(compensated=False)
    th = np.random.default_rng(2).normal(size=mc.D) * 0.1
    lc, gc = mc.log_prob_grad(th)
    lpl, gp = mp.log_prob_grad(th)
    assert lpl == pytest.approx(lc, rel=1e-12)
    assert np.max(np.abs(gp - gc)) <= 1e-10 * np.max(np.abs(gc))


def test_jacobian_term_hier():
    ds = make_dataset("hier_normal", small=True, seed=8)
    m = ds.oracle_model()
    th = np.random.default_rng(0).normal(size=m.D) * 0.2
    assert m.log_prob(th, jacobian=True) - m.log_prob(th, jacobian=False) == pytest.approx(th[1] + th[2])
    c = m.write_array(th)
    assert c[1] == pytest.approx(math.exp(th[1])) and c[2] == pytest.approx(math.exp(th[2]))


def test_oracle_sampler_recovers_logistic_posterior():
    ds = make_dataset("logistic", small=True, seed=11)
    m = ds.oracle_model(compensated=False)
    r = m.sample(num_chains=4, num_warmup=300, num_samples=300, seed=7)
    assert np.all(r["return_code"] == 0)
    draws = r["rows"][:, :, 7:]
    mean = draws.reshape(-1, m.D).mean(0)
    sd = draws.reshape(-1, m.D).std(0)
    # truth within 4 posterior sd for every coordinate
    assert np.all(np.abs(mean - ds.truth) < 4 * sd + 1e-9)
    assert 0.6 < r["rows"][:, :, 1].mean() < 0.98
