"""Device NUTS against the oracle's recursive restatement of base_nuts.

Both consume the same draw stream (include/gbnuts_draw_stream.h) in the
reference's order, so with equal inits, step size and metric the discrete
outputs of every transition (tree depth, n_leapfrog, divergence) must be equal
and the continuous ones equal to round-off (1e-9 relative here; the gradient
sums differ only in summation order).
"""
import numpy as np
import pytest

from tests.datasets import make_dataset

pytestmark = pytest.mark.gpu


def _compare(r, o, n, rtol=1e-9):
    gd = r.draws[:, :n]
    od = o["rows"][:, :n]
    assert np.array_equal(gd[:, :, 3:6], od[:, :, 3:6]), "treedepth / n_leapfrog / divergent differ"
    assert np.allclose(gd[:, :, 7:], od[:, :, 7:], rtol=rtol, atol=1e-10)
    assert np.allclose(gd[:, :, 0], od[:, :, 0], rtol=rtol, atol=1e-9)   # lp__
    assert np.allclose(gd[:, :, 1], od[:, :, 1], rtol=1e-7, atol=1e-9)  # accept_stat__
    assert np.allclose(gd[:, :, 6], od[:, :, 6], rtol=rtol, atol=1e-9)   # energy__


@pytest.mark.parametrize("kind", ["logistic", "poisson", "hier_normal", "hier_logistic"])
def test_single_transitions_replay(kind):
    from stan_gb300 import Model, sampler
    ds = make_dataset(kind, small=True, seed=2)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 4
    inits = np.random.default_rng(0).normal(size=(C, m.D)) * 0.2
    invm = np.exp(np.random.default_rng(1).normal(size=(C, m.D)) * 0.3)
    kw = dict(num_chains=C, adapt=False, num_warmup=0, num_samples=1, stepsize=0.15,
              inits=inits, inv_metrics=invm, max_depth=8)
    r = sampler.run(m, random_seed=5, **kw)
    o = om.sample(seed=5, **{k: v for k, v in kw.items() if k != "num_chains"}, num_chains=C)
    assert np.all(r.status == 0) and np.all(o["return_code"] == 0)
    _compare(r, o, 1)


def test_many_transitions_replay_logistic():
    from stan_gb300 import Model, sampler
    ds = make_dataset("logistic", small=True, seed=3)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 8
    inits = np.zeros((C, m.D))
    kw = dict(num_chains=C, adapt=False, num_warmup=10, num_samples=60, save_warmup=True,
              stepsize=0.25, inits=inits, max_depth=10, stepsize_jitter=0.3)
    r = sampler.run(m, random_seed=21, **kw)
    o = om.sample(seed=21, **kw)
    _compare(r, o, 70)


def test_adaptive_run_replays_warmup_and_adaptation():
    """hmc_nuts_diag_e_adapt with a short schedule: the step-size searches,
    dual averaging and the variance windows follow the oracle."""
    from stan_gb300 import Model, sampler
    ds = make_dataset("logistic", small=True, seed=4)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 4
    kw = dict(num_chains=C, adapt=True, num_warmup=150, num_samples=50, save_warmup=True,
              init_buffer=30, term_buffer=20, window=20, stepsize=1.0)
    r = sampler.run(m, random_seed=8, init_radius=2.0, **kw)
    o = om.sample(seed=8, init_radius=2.0, **kw)
    assert np.all(r.status == 0)
    assert np.allclose(r.init, o["init"], rtol=0, atol=0)
    # the first 40 warmup iterations replay exactly; after that the
    # trajectories carry round-off from the differently ordered gradient sums,
    # which the adaptation amplifies: the adapted step size and metric are
    # compared at 1e-4 relative (observed differences ~4e-6).
    _compare(r, o, 40)
    assert np.allclose(r.stepsize, o["stepsize"], rtol=1e-4)
    assert np.allclose(r.inv_metric, o["inv_metric"], rtol=1e-4)
    assert np.all(np.abs(r.n_grad - o["n_grad"]) <= 0.02 * o["n_grad"])


def test_draw_stream_matches_host():
    """Uniforms drawn for random inits on the device equal the host stream."""
    import oracle
    from stan_gb300 import Model, sampler
    ds = make_dataset("logistic", small=True, seed=5)
    m = Model.from_dataset(ds)
    r = sampler.run(m, num_chains=3, adapt=False, num_warmup=0, num_samples=1, stepsize=0.1,
                    random_seed=1234, init_chain_id=7, init_radius=1.5)
    for c in range(3):
        u = oracle.draws(1234, 7 + c, 0, 0, m.D)
        assert np.array_equal(r.init[c], (2.0 * u - 1.0) * 1.5)


@pytest.mark.parametrize("J,team", [(300, 0), (1100, 0), (1100, 4)])
def test_multi_warp_chains_replay(J, team):
    """Large dimensions run one chain per CTA of 2 (D <= 1024) or 8 warps
    (team 0: the built-in rule; team 4 forces four warps); their transitions
    replay the oracle like the warp-per-chain form."""
    from stan_gb300 import Model, _lib, sampler, workloads
    ds = workloads.hier_normal(J=J, K=6, mean_size=4, seed=11)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 3
    inits = np.random.default_rng(2).normal(size=(C, m.D)) * 0.1
    kw = dict(num_chains=C, adapt=False, num_warmup=0, num_samples=4, stepsize=0.05,
              inits=inits, max_depth=6)
    lib = _lib.load()
    _lib.check(lib.gbnuts_set_launch_shape(0, team), "gbnuts_set_launch_shape")
    try:
        r = sampler.run(m, random_seed=9, **kw)
    finally:
        _lib.check(lib.gbnuts_set_launch_shape(0, 0), "gbnuts_set_launch_shape")
    o = om.sample(seed=9, **kw)
    assert np.all(r.status == 0) and np.all(o["return_code"] == 0)
    _compare(r, o, 4)


def test_device_reproduces_the_reference_golden_transition():
    """unit_e_nuts_test.cpp:311-355 on the device: the gauss3D model (written
    as a Poisson GLM whose single row, x = 0 and y = 0, adds the constant -1
    to lp), one non-adaptive transition from q = (1, -1, 1) with step size
    0.1 and the draws recovered from the reference's expected values
    (tests/golden/gauss3d_transition.json).  The device's row must carry the
    reference's depth, leapfrog count, draw, log_prob and accept_stat to
    EXPECT_FLOAT_EQ precision (4 float ulps)."""
    import ctypes
    import json
    import os

    from stan_gb300 import Model, _lib, sampler
    with open(os.path.join(os.path.dirname(__file__), "golden", "gauss3d_transition.json")) as f:
        fx = json.load(f)
    g = fx["golden"]
    m = Model(2, np.zeros((1, 3)), np.zeros(1), hp=[1.0], intercept=False)
    cfg, out, res = sampler.prepare(3, 1, adapt=False, num_warmup=0, num_samples=1,
                                    stepsize=fx["stepsize"], stepsize_jitter=0.0, max_depth=10,
                                    inits=np.array(fx["q0"]), inv_metrics=np.ones(3),
                                    precision="fp64")
    n = max(len(fx["uniforms"]), 3) + 8
    u = np.full(n, np.nan)
    u[:len(fx["uniforms"])] = fx["uniforms"]
    z = np.full(n, np.nan)
    z[:3] = fx["normals"]
    lib = _lib.load()
    f = lib.gbnuts_sample_run_scripted
    f.restype = ctypes.c_int
    dp = ctypes.POINTER(ctypes.c_double)
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(_lib.RunConfig), ctypes.POINTER(_lib.RunOutput),
                  dp, dp, ctypes.c_int]
    rc = f(m.handle, ctypes.byref(cfg), ctypes.byref(out), u.ctypes.data_as(dp),
           z.ctypes.data_as(dp), n)
    assert rc == 0, _lib.last_error()
    sampler.finish(out, res)
    row = res.draws[0, 0]
    ulp4 = lambda v: 4 * float(np.spacing(np.float32(abs(v))))  # noqa: E731
    assert int(row[3]) == g["depth"] and int(row[4]) == g["n_leapfrog"] and row[5] == 0
    for i in range(3):
        assert abs(row[7 + i] - g["q"][i]) <= ulp4(g["q"][i]), (i, row[7 + i])
    assert abs(row[0] + 1.0 - g["log_prob"]) <= ulp4(g["log_prob"]), row[0]
    assert abs(row[1] - g["accept_stat"]) <= ulp4(g["accept_stat"]), row[1]
