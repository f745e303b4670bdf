"""The oracle's dense_e restatement pinned to the reference's unit tests:
covar_adaptation_test.cpp:5-29 (exact values), dense_e_metric_test.cpp:10-60
(sample_p covariance within 5 sigma) and :62-120 (dtau_dp against finite
differences of tau), and validate_dense_inv_metric's cases; plus a dense run
with the identity metric and adaptation off, which must equal the diag_e run
with unit metric draw for draw (T, dtau_dp and sample_p coincide exactly)."""
import numpy as np
import pytest

import oracle
from tests.datasets import make_dataset


def test_covar_adaptation_golden():
    # covar_adaptation_test.cpp: 10 zero draws with window params (50, 0, 0, 10)
    n = 10
    rc, covar, upd = oracle.covar_adaptation(50, 0, 0, n, np.zeros((n, n)), np.zeros((n, n)))
    assert rc == 0
    target = np.eye(n) * (1e-3 * 5.0 / (n + 5.0))
    assert np.array_equal(covar, target)
    assert upd[-1] == 1 and upd[:-1].sum() == 0


def test_covar_adaptation_matches_numpy():
    rng = np.random.default_rng(1)
    d, n = 4, 40
    q = rng.normal(size=(n, d)) @ np.array([[1, 0, 0, 0], [0.5, 1, 0, 0], [0, 0.3, 2, 0],
                                            [0.1, 0, 0, 0.5]])
    rc, covar, upd = oracle.covar_adaptation(100, 0, 0, n, q, np.eye(d))
    assert rc == 0 and upd[n - 1] == 1
    c = np.cov(q.T)
    want = (n / (n + 5.0)) * c + 1e-3 * (5.0 / (n + 5.0)) * np.eye(d)
    assert np.allclose(covar, want, rtol=1e-12, atol=1e-15)


def test_covar_adaptation_overflow():
    q = np.zeros((10, 2))
    q[3, 0] = np.inf
    rc, _, _ = oracle.covar_adaptation(50, 0, 0, 10, q, np.eye(2))
    assert rc == 1


def test_dense_sample_p_covariance():
    # dense_e_metric_test.cpp sample_p: 1000 momenta, covariance within 5 sigma of m
    m = np.array([[3.0, -2.0], [-2.0, 4.0]])
    _, _, p = oracle.dense_metric(np.linalg.inv(m), n=1000, seed=0, chain=0)
    n = p.shape[0]
    cov = p.T @ p / n
    var = np.array([[2 * m[0, 0], m[0, 1] ** 2 + m[1, 1] * m[0, 0]],
                    [m[1, 0] ** 2 + m[1, 1] * m[0, 0], 2 * m[1, 1]]])
    assert np.all(np.abs(m - cov) < 5.0 * np.sqrt(var / n))


def test_dense_dtau_dp_is_gradient_of_tau():
    rng = np.random.default_rng(2)
    d = 11
    b = rng.normal(size=(d, d))
    a = b @ b.T / d + np.eye(d)
    p = np.ones(d)
    T, dt, _ = oracle.dense_metric(a, p)
    assert T == pytest.approx(0.5 * p @ a @ p, rel=1e-13)
    eps = 1e-6
    for i in range(d):
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (oracle.dense_metric(a, pp)[0] - oracle.dense_metric(a, pm)[0]) / (2 * eps)
        assert fd == pytest.approx(dt[i], abs=eps)


def test_dense_metric_validation():
    assert oracle.dense_metric(np.array([[1.0, 0.5], [0.4, 1.0]])) is None   # not symmetric
    assert oracle.dense_metric(np.array([[1.0, 2.0], [2.0, 1.0]])) is None   # not PD
    assert oracle.dense_metric(np.array([[np.nan, 0.0], [0.0, 1.0]])) is None
    assert oracle.dense_metric(np.array([[2.0, 1e-9], [0.0, 1.0]])) is not None  # within 1e-8


def test_dense_identity_equals_diag_unit():
    ds = make_dataset("logistic", small=True, seed=5)
    om = ds.oracle_model()
    kw = dict(num_chains=2, num_warmup=30, num_samples=40, adapt=False, stepsize=0.2, seed=3,
              num_threads=2)
    a = om.sample(**kw)
    D = om.D
    b = om.sample(dense=True, inv_metrics=np.tile(np.eye(D), (2, 1, 1)), **kw)
    assert np.array_equal(a["rows"], b["rows"])
    assert np.array_equal(b["inv_metric"], np.tile(np.eye(D), (2, 1, 1)))


def test_dense_adaptive_run_posterior():
    """adapt_dense_e_nuts on a small logistic posterior: posterior means within
    4 MCSE of the diag_e run's, and the adapted metric symmetric positive definite."""
    from stan_gb300 import analyze
    ds = make_dataset("logistic", small=True, seed=7)
    om = ds.oracle_model()
    kw = dict(num_chains=4, num_warmup=300, num_samples=400, seed=11, num_threads=4)
    a = om.sample(**kw)
    b = om.sample(dense=True, **kw)
    assert np.all(a["return_code"] == 0) and np.all(b["return_code"] == 0)
    for k in range(7, a["rows"].shape[2]):
        xa = a["rows"][:, :, k].T
        xb = b["rows"][:, :, k].T
        se = np.hypot(analyze.mcse_mean(xa), analyze.mcse_mean(xb))
        assert abs(xa.mean() - xb.mean()) < 4 * se, k
    for c in range(4):
        m = b["inv_metric"][c]
        assert np.allclose(m, m.T, atol=1e-12) and np.all(np.linalg.eigvalsh(m) > 0)
