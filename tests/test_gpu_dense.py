"""Dense-metric NUTS (dense_e, covariance adaptation) on the device against the
oracle's restatement of dense_e_metric / covar_adaptation / adapt_dense_e_nuts:
the same draw stream in the reference's order, so transitions replay to
round-off; plus the identity metric equal to diag_e with unit metric draw for
draw, the services' dense protocol and the validation of dense metrics."""
import io

import numpy as np
import pytest

from tests.datasets import make_dataset
from tests.test_gpu_nuts_parity import _compare

pytestmark = pytest.mark.gpu


def _spd(D, C, seed, scale=0.3):
    rng = np.random.default_rng(seed)
    out = np.zeros((C, D, D))
    for c in range(C):
        b = rng.normal(size=(D, D)) * scale / np.sqrt(D)
        a = b @ b.T + np.diag(np.exp(rng.normal(size=D) * 0.3))
        out[c] = 0.5 * (a + a.T)
    return out


@pytest.mark.parametrize("kind", ["logistic", "hier_normal"])
def test_dense_transitions_replay(kind):
    from stan_gb300 import Model, sampler
    ds = make_dataset(kind, small=True, seed=2)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 4
    inits = np.random.default_rng(0).normal(size=(C, m.D)) * 0.2
    invm = _spd(m.D, C, 1)
    kw = dict(num_chains=C, adapt=False, num_warmup=0, num_samples=8, stepsize=0.12,
              inits=inits, inv_metrics=invm, max_depth=8)
    r = sampler.run(m, random_seed=5, metric="dense", **kw)
    o = om.sample(seed=5, dense=True, **kw)
    assert np.all(r.status == 0) and np.all(o["return_code"] == 0)
    _compare(r, o, 8)
    assert np.array_equal(r.inv_metric, invm)


def test_dense_identity_equals_diag_unit():
    from stan_gb300 import Model, sampler
    ds = make_dataset("logistic", small=True, seed=3)
    m = Model.from_dataset(ds)
    C = 4
    kw = dict(num_chains=C, adapt=False, num_warmup=20, num_samples=40, stepsize=0.2,
              random_seed=9)
    a = sampler.run(m, **kw)
    b = sampler.run(m, metric="dense", **kw)
    assert np.array_equal(a.draws, b.draws)


def test_dense_adaptive_run_replays_oracle():
    """adapt_dense_e_nuts with a short schedule: the first iterations replay
    exactly.  Later, a chain whose trajectory crosses a U-turn or acceptance
    decision under round-off (the gradient sums and the dot products are
    ordered differently) parts from the oracle's and adapts from a different
    trajectory, so: every chain's adapted step size within 10 %, and the chains
    that still track the oracle (step size to 1e-6; at least one) with the
    adapted dense metric equal to 1e-6 (of its largest entry)."""
    from stan_gb300 import Model, sampler
    ds = make_dataset("logistic", small=True, seed=4)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 4
    kw = dict(num_chains=C, adapt=True, num_warmup=150, num_samples=50, save_warmup=True,
              init_buffer=30, term_buffer=20, window=20, stepsize=1.0)
    r = sampler.run(m, random_seed=8, init_radius=2.0, metric="dense", **kw)
    o = om.sample(seed=8, init_radius=2.0, dense=True, **kw)
    assert np.all(r.status == 0) and np.all(o["return_code"] == 0)
    _compare(r, o, 40)
    rel = np.abs(r.stepsize - o["stepsize"]) / o["stepsize"]
    assert np.all(rel < 0.1), rel
    track = rel < 1e-6
    assert track.any(), rel
    # entries near zero (cross covariances) carry the round-off at the
    # matrix's scale
    scale = np.abs(o["inv_metric"][track]).max()
    assert np.allclose(r.inv_metric[track], o["inv_metric"][track], rtol=1e-6, atol=1e-6 * scale)


def test_dense_posterior_matches_diag():
    """A dense-metric fit and a diag fit of the same logistic posterior agree in
    posterior means within 4 MCSE; the adapted metrics are positive definite."""
    from stan_gb300 import Model, analyze, sampler
    ds = make_dataset("logistic", small=True, seed=12)
    m = Model.from_dataset(ds)
    kw = dict(num_chains=8, num_warmup=300, num_samples=400, random_seed=3)
    a = sampler.run(m, **kw)
    b = sampler.run(m, metric="dense", **kw)
    assert np.all(a.status == 0) and np.all(b.status == 0)
    da, db = a.sampling_draws(), b.sampling_draws()
    for k in range(7, da.shape[2]):
        se = np.hypot(analyze.mcse_mean(da[:, :, k]), analyze.mcse_mean(db[:, :, k]))
        assert abs(da[:, :, k].mean() - db[:, :, k].mean()) < 4 * se, k
    for c in range(8):
        assert np.all(np.linalg.eigvalsh(0.5 * (b.inv_metric[c] + b.inv_metric[c].T)) > 0)


def test_dense_service_protocol_and_validation():
    from stan_gb300 import Model, _lib, services
    from stan_gb300.callbacks import StreamWriter, StructuredWriter
    ds = make_dataset("logistic", small=True, seed=5)
    m = Model.from_dataset(ds)
    D, C = m.D, 2
    sample = [StreamWriter(io.StringIO()) for _ in range(C)]
    metric = [StructuredWriter() for _ in range(C)]
    kw = dict(init=None, random_seed=1, init_chain_id=1, init_radius=2.0, num_warmup=100,
              num_samples=20, num_thin=1, save_warmup=False, refresh=0, stepsize=1.0,
              stepsize_jitter=0.0, max_depth=10, delta=0.8, gamma=0.05, kappa=0.75, t0=10.0,
              init_buffer=20, term_buffer=10, window=20)
    rc = services.hmc_nuts_dense_e_adapt(m, C, init_inv_metric=None, sample_writer=sample,
                                         metric_writer=metric, **kw)
    assert rc == 0
    lines = sample[0].stream.getvalue().split("\n")
    assert lines[1] == "# Adaptation terminated"
    assert lines[3] == "# Elements of inverse mass matrix:"
    rows = [ln[2:].split(", ") for ln in lines[4:4 + D]]
    assert all(len(r) == D for r in rows)
    assert lines[4 + D].count(",") == 6 + D  # first draw
    rec = metric[0].records[0]
    assert rec["metric_type"] == "dense_e" and len(rec["inv_metric"]) == D
    assert all(len(r) == D for r in rec["inv_metric"])
    # a metric that is not positive definite is refused before sampling
    bad = np.eye(D)
    bad[0, 1] = bad[1, 0] = 2.0
    rc = services.hmc_nuts_dense_e_adapt(m, C, init_inv_metric=bad, **kw)
    assert rc == _lib.CONFIG
    # the pool runs diag_e fits only
    from stan_gb300.serving import Pool
    pool = Pool(reserve_bytes=0)
    with pytest.raises(_lib.GbnutsError):
        pool.submit(ds, num_chains=2, num_warmup=10, num_samples=10, metric="dense")
    pool.close()
