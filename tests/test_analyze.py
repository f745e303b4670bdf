"""ESS / MCSE restatement pinned to the reference's golden values.

Fixture: tests/golden/bern_draws.npz, extracted from the reference's
src/test/unit/analyze/mcmc/test_csv_files/bern{1..4}.csv by
tests/golden/make_bern_fixture.py.
"""
import os

import numpy as np
import pytest

from stan_gb300 import analyze as A

FIX = os.path.join(os.path.dirname(__file__), "golden", "bern_draws.npz")


@pytest.fixture(scope="module")
def bern():
    return np.load(FIX)


def test_bulk_tail_ess(bern):
    # split_rank_normalized_ess_test.cpp:37-53 (computed by R posterior; 1e-4)
    lp = A.split_rank_normalized_ess(bern["lp"])
    th = A.split_rank_normalized_ess(bern["theta"])
    assert lp[0] == pytest.approx(1512.7684, abs=1e-4)
    assert lp[1] == pytest.approx(1591.9707, abs=1e-4)
    assert th[0] == pytest.approx(1407.5124, abs=1e-4)
    assert th[1] == pytest.approx(1291.7131, abs=1e-4)


def test_basic_ess(bern):
    # ess_basic_test.cpp:45-52 (cmdstan 2.35.0 stansummary; 1e-8)
    assert A.ess(bern["lp"]) == pytest.approx(1335.41366787, abs=1e-8)
    assert A.ess(bern["theta"]) == pytest.approx(1377.5030282, abs=1e-8)


def test_mcse(bern):
    # mcse_test.cpp:39-49 (1e-4)
    assert A.mcse_mean(bern["lp"]) == pytest.approx(0.02016, abs=1e-4)
    assert A.mcse_mean(bern["theta"]) == pytest.approx(0.00323, abs=1e-4)
    assert A.mcse_sd(bern["lp"]) == pytest.approx(0.03553, abs=1e-4)
    assert A.mcse_sd(bern["theta"]) == pytest.approx(0.00216, abs=1e-4)


def test_failure_cases(bern):
    # split_rank_normalized_ess_test.cpp:55-73, mcse_test.cpp:51-73
    assert all(np.isnan(A.split_rank_normalized_ess(bern["divergent"])))
    th = bern["theta"].copy()
    th[0, 0] = np.inf
    assert all(np.isnan(A.split_rank_normalized_ess(th)))
    assert np.isnan(A.mcse_mean(th)) and np.isnan(A.mcse_sd(th))
    short = bern["theta"][:3]
    assert all(np.isnan(A.split_rank_normalized_ess(short)))
    assert np.isnan(A.mcse_mean(short))


def test_min_bulk_ess(bern):
    d = np.stack([bern["lp"], bern["theta"]], axis=2)
    v, name = A.min_bulk_ess(d, ["lp__", "theta"])
    assert name == "theta" and v == pytest.approx(1407.5124, abs=1e-4)


def test_split_rank_normalized_rhat(bern):
    # split_rank_normalized_rhat_test.cpp:40-52 (computed by R posterior; 1e-5)
    lp = A.split_rank_normalized_rhat(bern["lp"])
    th = A.split_rank_normalized_rhat(bern["theta"])
    assert max(lp) == pytest.approx(1.00073, abs=1e-5)
    assert max(th) == pytest.approx(1.006789, abs=1e-5)
    # split_rank_normalized_rhat_test.cpp:54-66
    assert all(np.isnan(A.split_rank_normalized_rhat(bern["divergent"])))
    bad = bern["theta"].copy()
    bad[0, 0] = np.inf
    assert all(np.isnan(A.split_rank_normalized_rhat(bad)))


def test_rhat_identical_chains_is_below_one():
    # rhat of chains with equal means: B = 0, so sqrt((n - 1) / n)
    x = np.tile(np.arange(10.0)[:, None], (1, 3))
    assert A.rhat(x) == pytest.approx(np.sqrt(9 / 10), abs=1e-15)
