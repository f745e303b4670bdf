"""Batched log density and gradient on the GPU against the FP64 oracle.

Tolerances: FP64 form <= 1e-12 relative (lp; gradient in the max norm);
FP32 form: gradient <= 1e-4 relative in the 2-norm, lp <= 1e-5 relative.
"""
import numpy as np
import pytest

from tests.datasets import make_dataset

pytestmark = pytest.mark.gpu

KINDS = ["logistic", "logistic_100k", "poisson", "hier_normal", "hier_logistic"]


@pytest.fixture(scope="module")
def models():
    from stan_gb300 import Model
    out = {}
    for kind in KINDS:
        ds = make_dataset(kind, small=True, seed=7)
        out[kind] = (ds, Model.from_dataset(ds), ds.oracle_model())
    return out


def _points(D, C, seed, scale=0.3):
    return np.random.default_rng(seed).normal(size=(C, D)) * scale


@pytest.mark.parametrize("kind", KINDS)
def test_fp64_single_point_matches_oracle(models, kind):
    ds, m, om = models[kind]
    for th in _points(m.D, 4, 1):
        for propto in (True, False):
            for jac in (True, False):
                lp, g = m.log_prob_grad(th, propto=propto, jacobian=jac)
                lpo, go = om.log_prob_grad(th, propto=propto, jacobian=jac)
                assert abs(lp - lpo) <= 1e-12 * max(1.0, abs(lpo))
                assert np.max(np.abs(g - go)) <= 1e-12 * max(1.0, np.max(np.abs(go)))
                assert m.log_prob(th, propto=propto, jacobian=jac) == pytest.approx(lp, rel=1e-15, abs=1e-15)


@pytest.mark.parametrize("kind", KINDS)
def test_fp64_batch_matches_oracle(models, kind):
    ds, m, om = models[kind]
    C = 37
    th = _points(m.D, C, 2)
    lp, g = m.log_prob_grad_batch(th, "fp64")
    for c in range(C):
        lpo, go = om.log_prob_grad(th[c])
        assert abs(lp[c] - lpo) <= 1e-12 * max(1.0, abs(lpo))
        assert np.max(np.abs(g[c] - go)) <= 1e-12 * max(1.0, np.max(np.abs(go)))


@pytest.mark.parametrize("kind", KINDS)
def test_fp32_batch_within_stated_tolerance(models, kind):
    ds, m, om = models[kind]
    C = 19
    th = _points(m.D, C, 3)
    lp, g = m.log_prob_grad_batch(th, "fp32")
    for c in range(C):
        lpo, go = om.log_prob_grad(th[c])
        assert abs(lp[c] - lpo) <= 1e-5 * abs(lpo)
        assert np.linalg.norm(g[c] - go) <= 1e-4 * np.linalg.norm(go)


def test_full_size_logistic_batch():
    """N = 100000, K = 100 (X stored FP32): FP64 batch vs oracle at 8 points."""
    from stan_gb300 import Model
    ds = make_dataset("logistic_100k", small=False, seed=1)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    th = _points(m.D, 8, 4, scale=0.05)
    lp, g = m.log_prob_grad_batch(th, "fp64")
    lp32, g32 = m.log_prob_grad_batch(th, "fp32")
    for c in range(8):
        lpo, go = om.log_prob_grad(th[c])
        assert abs(lp[c] - lpo) <= 1e-12 * abs(lpo)
        assert np.max(np.abs(g[c] - go)) <= 1e-12 * np.max(np.abs(go))
        assert np.linalg.norm(g32[c] - go) <= 1e-4 * np.linalg.norm(go)


@pytest.mark.parametrize("K", [3, 16, 17])
@pytest.mark.parametrize("C", [3, 5, 20])
def test_group_sums_with_single_row_groups_and_large_groups(K, C):
    """Segmented group reduction across tile, run and chunk boundaries: groups
    of one row, an empty group, groups longer than a tile; chain blocks of 4,
    8 and 16 chains; up to 16 features the per-thread row runs, above that
    the general form."""
    from stan_gb300 import Model
    from stan_gb300.workloads import Dataset, HIER_NORMAL
    rng = np.random.default_rng(5 + K + C)
    sizes = np.array([1, 1, 300, 2, 31, 32, 33, 0, 64, 65, 1, 500, 7, 16, 15, 17, 1, 1, 260])
    J = sizes.size
    g = np.repeat(np.arange(J, dtype=np.int32), sizes)
    N = g.size
    X = rng.normal(size=(N, K))
    y = rng.normal(size=N)
    ds = Dataset("groups", HIER_NORMAL, X, y, "f64", group=g, J=J, hp=(5.0, 1.0, 1.0, 1.0))
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    th = _points(m.D, C, 6)
    lp, gr = m.log_prob_grad_batch(th, "fp64")
    lp32, gr32 = m.log_prob_grad_batch(th, "fp32")
    for c in range(C):
        lpo, go = om.log_prob_grad(th[c])
        assert abs(lp[c] - lpo) <= 1e-12 * abs(lpo)
        assert np.max(np.abs(gr[c] - go)) <= 1e-12 * np.max(np.abs(go))
        assert abs(lp32[c] - lpo) <= 1e-5 * abs(lpo)
        assert np.linalg.norm(gr32[c] - go) <= 1e-4 * np.linalg.norm(go)
    lp2, gr2 = m.log_prob_grad_batch(th, "fp32")
    assert np.array_equal(lp2, lp32) and np.array_equal(gr2, gr32)  # deterministic


def test_non_finite_density_is_reported_not_raised(models):
    ds, m, om = models["poisson"]
    th = np.full(m.D, 400.0)
    lp, g = m.log_prob_grad(th)
    assert not np.isfinite(lp)


def test_full_size_hier_normal_config_c():
    """J = 2000 groups (~42k rows), D = 2013: FP64 to 1e-12, FP32 within its
    stated tolerance, against the oracle."""
    from stan_gb300 import Model
    ds = make_dataset("hier_normal", small=False, seed=1)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 32
    th = np.random.default_rng(8).normal(size=(C, m.D)) * 0.2
    lp64, g64 = m.log_prob_grad_batch(th, "fp64")
    lp32, g32 = m.log_prob_grad_batch(th, "fp32")
    for c in (0, 7, 31):
        lpo, go = om.log_prob_grad(th[c])
        assert abs(lp64[c] - lpo) <= 1e-12 * abs(lpo)
        assert np.linalg.norm(g64[c] - go) <= 1e-12 * np.linalg.norm(go)
        assert abs(lp32[c] - lpo) <= 1e-5 * abs(lpo)
        assert np.linalg.norm(g32[c] - go) <= 1e-4 * np.linalg.norm(go)


def test_full_size_poisson_config_d():
    """N = 262144, K = 512, X stored bf16: FP64 to 1e-12 against the oracle;
    the bf16 tensor-core forms within their stated tolerances."""
    from stan_gb300 import Model
    ds = make_dataset("poisson", small=False, seed=1)
    m = Model.from_dataset(ds)
    om = ds.oracle_model()
    C = 16
    th = np.random.default_rng(9).normal(size=(C, m.D)) * 0.05
    lp64, g64 = m.log_prob_grad_batch(th, "fp64")
    lp3, g3 = m.log_prob_grad_batch(th, "bf16x3")
    lp1, g1 = m.log_prob_grad_batch(th, "bf16")
    for c in (0, 15):
        lpo, go = om.log_prob_grad(th[c])
        assert abs(lp64[c] - lpo) <= 1e-12 * abs(lpo)
        assert np.linalg.norm(g64[c] - go) <= 1e-12 * np.linalg.norm(go)
        assert abs(lp3[c] - lpo) <= 1e-5 * abs(lpo)
        assert np.linalg.norm(g3[c] - go) <= 1e-4 * np.linalg.norm(go)
        assert abs(lp1[c] - lpo) <= 1e-3 * abs(lpo)
        assert np.linalg.norm(g1[c] - go) <= 1e-2 * np.linalg.norm(go)


def _fixture():
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "logdensity_exact.npz")
    return np.load(path)


@pytest.mark.parametrize("name", ["logistic_1k", "logistic_f32", "poisson", "poisson_bf16",
                                  "hier_normal", "hier_logistic"])
def test_fp64_matches_exact_restatement(name):
    """The device's FP64 form against the extended-precision restatement of
    the densities from their definitions (tests/logdensity_exact.py; values
    in tests/golden/logdensity_exact.npz): every propto / jacobian setting on
    the single-point entry points, and the batched entry point, within 1e-12
    relative (lp; gradient in the 2-norm)."""
    from stan_gb300 import Model
    f = _fixture()
    group = f[name + "__group"] if name + "__group" in f.files else None
    m = Model(int(f[name + "__kind"]), f[name + "__X"], f[name + "__y"], group=group,
              J=int(f[name + "__J"]), hp=list(f[name + "__hp"]),
              intercept=bool(f[name + "__intercept"]), x_dtype=str(f[name + "__xdtype"]))
    th = f[name + "__theta"]
    lps, grads = f[name + "__lp"], f[name + "__grad"]
    for v, (propto, jac) in enumerate([(True, True), (True, False), (False, True), (False, False)]):
        for i in range(th.shape[0]):
            lp, g = m.log_prob_grad(th[i], propto=propto, jacobian=jac)
            assert abs(lp - lps[v, i]) <= 1e-12 * abs(lps[v, i]), (v, i)
            assert np.linalg.norm(g - grads[v, i]) <= 1e-12 * np.linalg.norm(grads[v, i]), (v, i)
    lp, g = m.log_prob_grad_batch(th, "fp64")
    assert np.all(np.abs(lp - lps[0]) <= 1e-12 * np.abs(lps[0]))
    assert np.all(np.linalg.norm(g - grads[0], axis=1) <= 1e-12 * np.linalg.norm(grads[0], axis=1))
    m.close()
