"""Device ESS (gbnuts_ess) against the NumPy restatement of the reference's
analysis code (itself pinned to the reference's bern1-4 vectors in
tests/test_analyze.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _draws(C, rows, n_cols, seed, phi=0.6):
    rng = np.random.default_rng(seed)
    d = np.zeros((C, rows, n_cols))
    for q in range(n_cols):
        for c in range(C):
            x = rng.normal()
            for r in range(rows):
                x = phi * x + rng.normal() * np.sqrt(1 - phi * phi)
                d[c, r, q] = x + 0.1 * c
    return d


@pytest.mark.parametrize("C,rows", [(4, 500), (4, 501), (8, 300), (2, 16)])
def test_device_ess_matches_numpy(C, rows):
    from stan_gb300 import _lib, analyze
    d = _draws(C, rows, 3, seed=C * 1000 + rows)
    d[:, :, 2] = np.round(d[:, :, 2], 1)  # many ties
    out = np.zeros(6)
    rc = _lib.load().gbnuts_ess(np.ascontiguousarray(d).ctypes.data_as(_lib._dp), C, rows, 3,
                                0, rows, 0, 3, out.ctypes.data_as(_lib._dp))
    assert rc == 0, _lib.last_error()
    for q in range(3):
        b, t = analyze.split_rank_normalized_ess(d[:, :, q].T)
        assert abs(out[2 * q] - b) <= 1e-8 * b, (q, out[2 * q], b)
        assert abs(out[2 * q + 1] - t) <= 1e-8 * t, (q, out[2 * q + 1], t)


def test_device_ess_nan_cases():
    from stan_gb300 import _lib
    C, rows = 4, 100
    d = _draws(C, rows, 3, seed=5)
    d[:, :, 0] = 1.5           # constant
    d[1, 7, 1] = np.inf        # not finite
    out = np.zeros(6)
    rc = _lib.load().gbnuts_ess(np.ascontiguousarray(d).ctypes.data_as(_lib._dp), C, rows, 3,
                                0, rows, 0, 3, out.ctypes.data_as(_lib._dp))
    assert rc == 0
    assert np.isnan(out[0]) and np.isnan(out[1]) and np.isnan(out[2]) and np.isnan(out[3])
    assert np.isfinite(out[4]) and np.isfinite(out[5])


def test_fit_report_matches_host():
    from stan_gb300 import Model, analyze, diagnostics, sampler
    from tests.datasets import make_dataset
    ds = make_dataset("hier_logistic", small=True, seed=3)
    r = sampler.run(Model.from_dataset(ds), num_chains=4, num_warmup=200, num_samples=300,
                    random_seed=4)
    bulk, tail = diagnostics.split_rank_ess(r)
    d = r.sampling_draws()
    q = np.concatenate([d[:, :, 0:1], d[:, :, 7:]], axis=2)
    for k in range(q.shape[2]):
        b, t = analyze.split_rank_normalized_ess(q[:, :, k])
        assert abs(bulk[k] - b) <= 1e-8 * b and abs(tail[k] - t) <= 1e-8 * t, k


def test_run_reports_ess_alone_and_in_pool():
    """RunResult.ess (computed on the device at the end of the run) equals the
    host restatement, for an alone run and the same fit inside a pool."""
    from stan_gb300 import Model, analyze, sampler
    from stan_gb300.serving import Pool
    from tests.datasets import make_dataset
    ds = make_dataset("hier_normal", small=True, seed=5)
    kw = dict(num_chains=4, num_warmup=150, num_samples=200, random_seed=6, report_ess=True)
    r = sampler.run(Model.from_dataset(ds, x_dtype="f32"), precision="fp32", **kw)
    d = r.sampling_draws()
    q = np.concatenate([d[:, :, 0:1], d[:, :, 7:]], axis=2)
    for k in range(q.shape[2]):
        b, t = analyze.split_rank_normalized_ess(q[:, :, k])
        assert abs(r.ess[k, 0] - b) <= 1e-8 * b and abs(r.ess[k, 1] - t) <= 1e-8 * t, k
    pool = Pool(precision="fp32", x_dtype="f32", reserve_bytes=0)
    fid = pool.submit(ds, **kw)
    pool.run_all()
    rp = pool.pop(fid)
    assert np.array_equal(rp.ess, r.ess)
    pool.close()
