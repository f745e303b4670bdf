"""The fit pool: a fit's results are the same alone and in any mix.

Each fit is run once through gbnuts_sample_run on its own and once inside a
pool next to fits of other families, sizes, chain counts and schedules; the
draws, chain status, adapted step size and metric, inits and gradient counts
must be bit-identical.
"""
import numpy as np
import pytest

from stan_gb300 import workloads
from tests.datasets import make_dataset

pytestmark = pytest.mark.gpu

FIELDS = ["draws", "n_rows", "n_warmup_rows", "status", "stepsize", "inv_metric", "init", "n_grad"]


def _fits():
    """(dataset, run kwargs) of a mixed set of small fits."""
    base = dict(num_warmup=150, num_samples=100, init_buffer=20, term_buffer=10, window=10,
                max_depth=8)
    return [
        (make_dataset("logistic", small=True, seed=2), dict(base, num_chains=4, random_seed=11)),
        (make_dataset("hier_normal", small=True, seed=3), dict(base, num_chains=6, random_seed=12)),
        (make_dataset("hier_logistic", small=True, seed=4), dict(base, num_chains=3, random_seed=13)),
        (make_dataset("poisson", small=True, seed=5),
         dict(base, num_chains=5, random_seed=14, num_warmup=80, save_warmup=True)),
        (workloads.hier_logistic(15000, 8, seed=7),  # D = 310: two warps per chain
         dict(base, num_chains=2, random_seed=16, num_warmup=60, num_samples=40)),
        (make_dataset("logistic_100k", small=True, seed=6),
         dict(num_chains=2, random_seed=15, adapt=False, num_warmup=0, num_samples=60,
              stepsize=0.2, max_depth=6)),
    ]


def _alone(ds, kw, x_dtype, precision):
    from stan_gb300 import Model, sampler
    m = Model.from_dataset(ds, x_dtype=x_dtype)
    return sampler.run(m, precision=precision, **kw)


def _same(a, b):
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


@pytest.mark.parametrize("precision,x_dtype", [("fp64", "f64"), ("fp32", "f32")])
def test_pool_fits_match_alone_runs(precision, x_dtype):
    from stan_gb300.serving import Pool
    fits = _fits()
    alone = [_alone(ds, kw, x_dtype, precision) for ds, kw in fits]
    pool = Pool(precision=precision, x_dtype=x_dtype, max_fits=8, reserve_bytes=0)
    ids = [pool.submit(ds, **kw) for ds, kw in fits]
    pool.run_all(n_steps=16)
    for i, fid in enumerate(ids):
        _same(pool.pop(fid), alone[i])
    pool.close()


def test_pool_admits_as_chains_free_up():
    """A chain budget of 8 admits the fits in waves; fits submitted while
    others run start later and still give their alone results."""
    from stan_gb300.serving import Pool, DONE, QUEUED
    fits = _fits()
    alone = [_alone(ds, kw, "f32", "fp32") for ds, kw in fits]
    pool = Pool(precision="fp32", x_dtype="f32", max_fits=3, max_chains=8, reserve_bytes=0)
    ids = [pool.submit(ds, **kw) for ds, kw in fits[:2]]
    running, queued = pool.step(5)
    assert running == 1 and queued == 1  # 4 + 6 chains exceed the budget of 8
    ids += [pool.submit(ds, **kw) for ds, kw in fits[2:]]
    assert pool.status(ids[-1])[0] == QUEUED
    max_chains = 0
    while True:
        running, queued = pool.step(7)
        max_chains = max(max_chains, pool.stats()[1])
        if running == 0 and queued == 0:
            break
    assert max_chains <= 8
    for i, fid in enumerate(ids):
        assert pool.status(fid)[0] == DONE
        _same(pool.pop(fid), alone[i])
    pool.close()


def test_pool_bad_fit_fails_alone():
    """A fit whose metric is not positive definite finishes with CONFIG
    (validate_diag_inv_metric.hpp:18-27); its neighbours are unaffected."""
    from stan_gb300 import _lib
    from stan_gb300.serving import Pool
    fits = _fits()[:2]
    ds, kw = fits[0]
    bad = -np.ones((kw["num_chains"], ds.D))
    pool = Pool(precision="fp64", x_dtype="f64", reserve_bytes=0)
    good_id = pool.submit(*fits[1][:1], **fits[1][1])
    bad_id = pool.submit(ds, inv_metrics=bad, **kw)
    pool.run_all()
    assert pool.status(bad_id) == (2, _lib.CONFIG)
    _same(pool.pop(good_id), _alone(fits[1][0], fits[1][1], "f64", "fp64"))
    pool.close()


def test_serve_poisson_arrivals():
    from stan_gb300.serving import Pool, poisson_arrivals, serve
    fits = _fits()
    datasets = [ds for ds, _ in fits[:3]] * 2
    arrivals = poisson_arrivals(rate=20.0, n=len(datasets), seed=3)
    pool = Pool(precision="fp32", x_dtype="f32", reserve_bytes=0)
    got = {}
    rep = serve(pool, datasets, arrivals, steps_per_call=16,
                run_kwargs=dict(num_chains=4, num_warmup=100, num_samples=50, random_seed=7),
                on_done=lambda i, r: got.__setitem__(i, r))
    assert sorted(got) == list(range(len(datasets)))
    assert np.all(rep.latencies > 0)
    s = rep.summary()
    assert s["n"] == len(datasets) and s["p99"] >= s["p50"] > 0
    # the same dataset and seed give the same draws whenever it arrives
    for i in range(3):
        assert np.array_equal(got[i].draws, got[i + 3].draws)
    pool.close()
