"""The reference's golden NUTS transition replayed by the oracle.

src/test/unit/mcmc/hmc/nuts/unit_e_nuts_test.cpp:311-355 pins one transition
of the gauss3D model (x ~ normal(0, 1), 3 dimensions, unit metric) from
q = (1, -1, 1) with step size 0.1: depth 3, 15 leapfrog steps, draw
(0.70149082, -0.69831347, 0.54392564), log_prob -0.63779306, accept_stat
0.99912512, all with the reference's mixmax stream.  That stream is not
restated here: tests/golden/gauss3d_transition.json holds a momentum draw
and uniforms recovered from those expected values
(tests/golden/make_gauss3d_transition.py).  Replayed through the oracle's
base_nuts restatement, they must reproduce every expected value at the
precision the reference's test checks (EXPECT_FLOAT_EQ: 4 float ulps), and
consume exactly the recovered draws.

gauss3D is written as a Poisson GLM with no rows of data contributing:
one row with x = 0 and y = 0 adds the constant -1 to lp, and the normal(0, 1)
prior on the three coefficients is the model's density.
"""
import json
import os

import numpy as np

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture():
    with open(os.path.join(HERE, "golden", "gauss3d_transition.json")) as f:
        return json.load(f)


def float_eq(a, b):
    """EXPECT_FLOAT_EQ: within 4 units in the last place of a float."""
    return abs(a - b) <= 4 * np.spacing(np.float32(abs(b))).astype(np.float64) + 1e-300


def gauss3d_oracle():
    return oracle.OracleModel(2, np.zeros((1, 3)), np.zeros(1), hp=[1.0], intercept=False)


def test_oracle_reproduces_the_golden_transition():
    f = fixture()
    g = f["golden"]
    m = gauss3d_oracle()
    r = m.transition_scripted(f["q0"], f["uniforms"], f["normals"], f["stepsize"], max_depth=10)
    assert r["depth"] == g["depth"]
    assert r["n_leapfrog"] == g["n_leapfrog"]
    assert r["divergent"] == g["divergent"]
    for i in range(3):
        assert float_eq(r["q"][i], g["q"][i]), (i, r["q"][i], g["q"][i])
    assert float_eq(r["lp"] + 1.0, g["log_prob"]), r["lp"]
    assert float_eq(r["accept_stat"], g["accept_stat"]), r["accept_stat"]
    assert r["normals_used"] == 3
    assert r["uniforms_used"] == len(f["uniforms"])


def test_fixture_script_recovers_the_fixture():
    """The recovery is deterministic: rerunning it gives the committed draws."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_gauss3d", os.path.join(HERE, "golden", "make_gauss3d_transition.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    f = fixture()
    p0 = mod.momentum_for(f["position"])
    assert np.allclose(p0, f["normals"], rtol=0, atol=1e-15)
