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


def _host_summary(x):
    """The six summary values of one quantity (x: draws x chains) from the
    NumPy restatement."""
    from stan_gb300 import analyze
    b, t = analyze.split_rank_normalized_ess(x)
    rb, rt = analyze.split_rank_normalized_rhat(x)
    return np.array([b, t, rb, rt, analyze.mcse_mean(x), analyze.mcse_sd(x)])


def _close(dev, host, rtol):
    both_nan = np.isnan(dev) & np.isnan(host)
    ok = both_nan | (np.abs(dev - host) <= rtol * np.abs(host))
    return bool(np.all(ok))


@pytest.mark.parametrize("C,rows", [(4, 500), (4, 501), (8, 300), (2, 16), (4, 7), (16, 512)])
def test_device_summary_matches_numpy(C, rows):
    from stan_gb300 import _lib
    d = _draws(C, rows, 3, seed=C * 7 + rows)
    d[:, :, 2] = np.round(d[:, :, 2], 1)  # many ties
    out = np.zeros(18)
    rc = _lib.load().gbnuts_summary(np.ascontiguousarray(d).ctypes.data_as(_lib._dp), C, rows,
                                    3, 0, rows, 0, 3, out.ctypes.data_as(_lib._dp))
    assert rc == 0, _lib.last_error()
    for q in range(3):
        host = _host_summary(d[:, :, q].T)
        assert _close(out[6 * q:6 * q + 6], host, 1e-8), (q, out[6 * q:6 * q + 6], host)


def test_device_summary_bern_golden():
    """The reference's bern1-4 chains (lp__, theta) on the device against the
    reference's own expected values (R posterior)."""
    import os
    from stan_gb300 import _lib
    f = np.load(os.path.join(os.path.dirname(__file__), "golden", "bern_draws.npz"))
    d = np.ascontiguousarray(np.stack([f["lp"].T, f["theta"].T], axis=2))  # (4, 1000, 2)
    out = np.zeros(12)
    rc = _lib.load().gbnuts_summary(d.ctypes.data_as(_lib._dp), 4, 1000, 2, 0, 1000, 0, 2,
                                    out.ctypes.data_as(_lib._dp))
    assert rc == 0, _lib.last_error()
    lp, th = out[:6], out[6:]
    # split_rank_normalized_ess_test.cpp:37-53, split_rank_normalized_rhat_test.cpp:40-52,
    # mcse_test.cpp:39-49
    assert lp[0] == pytest.approx(1512.7684, abs=1e-4) and lp[1] == pytest.approx(1591.9707, abs=1e-4)
    assert th[0] == pytest.approx(1407.5124, abs=1e-4) and th[1] == pytest.approx(1291.7131, abs=1e-4)
    assert max(lp[2], lp[3]) == pytest.approx(1.00073, abs=1e-5)
    assert max(th[2], th[3]) == pytest.approx(1.006789, abs=1e-5)
    assert lp[4] == pytest.approx(0.02016, abs=1e-4) and th[4] == pytest.approx(0.00323, abs=1e-4)
    assert lp[5] == pytest.approx(0.03553, abs=1e-4) and th[5] == pytest.approx(0.00216, abs=1e-4)


def test_device_summary_nan_cases():
    from stan_gb300 import _lib
    C, rows = 4, 100
    d = _draws(C, rows, 3, seed=9)
    d[:, :, 0] = 1.5           # constant: every value NaN
    d[1, 7, 1] = np.inf        # not finite: every value NaN
    out = np.zeros(18)
    rc = _lib.load().gbnuts_summary(np.ascontiguousarray(d).ctypes.data_as(_lib._dp), C, rows,
                                    3, 0, rows, 0, 3, out.ctypes.data_as(_lib._dp))
    assert rc == 0
    assert np.all(np.isnan(out[:12])) and np.all(np.isfinite(out[12:]))
    # more than 8192 draws per quantity is refused
    big = np.zeros((16, 600, 1))
    rc = _lib.load().gbnuts_summary(big.ctypes.data_as(_lib._dp), 16, 600, 1, 0, 600, 0, 1,
                                    out.ctypes.data_as(_lib._dp))
    assert rc == _lib.USAGE


def test_run_reports_summary_alone_and_in_pool():
    """RunResult.summary (on the device at the end of the run) equals the host
    restatement, and the same fit in a pool reports the same values."""
    from stan_gb300 import Model, diagnostics, sampler
    from stan_gb300.serving import Pool
    from tests.datasets import make_dataset
    ds = make_dataset("hier_logistic", small=True, seed=8)
    kw = dict(num_chains=4, num_warmup=150, num_samples=200, random_seed=2, report_summary=True,
              report_ess=True)
    r = sampler.run(Model.from_dataset(ds, x_dtype="f32"), precision="fp32", **kw)
    d = r.sampling_draws()
    q = np.concatenate([d[:, :, 0:1], d[:, :, 7:]], axis=2)
    for k in range(q.shape[2]):
        assert _close(r.summary[k], _host_summary(q[:, :, k]), 1e-8), k
    assert np.array_equal(r.ess, r.summary[:, :2])
    assert np.array_equal(diagnostics.summary(r), r.summary)
    assert diagnostics.max_rhat(r) < 1.1
    pool = Pool(precision="fp32", x_dtype="f32", reserve_bytes=0)
    fid = pool.submit(ds, **kw)
    pool.run_all()
    rp = pool.pop(fid)
    assert np.array_equal(rp.summary, r.summary)
    pool.close()
