"""Pins the CPU oracle to the reference's own unit-test vectors.

Each test names the reference test it restates (paths relative to the
stan-dev/stan tree).  The oracle is the checker for every GPU parity test, so
these run first and on the CPU only.
"""
import math

import numpy as np
import pytest

import oracle


# --- draw stream ------------------------------------------------------------
def test_philox_known_answers():
    # Published Philox4x32-10 known-answer vectors (Random123 kat_vectors).
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _philox_np(c0, c1, c2, c3, k0, k1):
    """Independent NumPy restatement of Philox4x32-10 for cross-checking."""
    M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
    c = [np.uint64(v) for v in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(k0), np.uint64(k1)
    mask = np.uint64(0xFFFFFFFF)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(W0)) & mask
            k1 = (k1 + np.uint64(W1)) & mask
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        c = [((p1 >> np.uint64(32)) ^ c[1] ^ k0) & mask, p1 & mask,
             ((p0 >> np.uint64(32)) ^ c[3] ^ k1) & mask, p0 & mask]
    return [int(v) for v in c]


def test_uniform_stream_matches_numpy_restatement():
    seed, chain = 1234, 7
    u = oracle.draws(seed, chain, 0, 0, 64)
    for n in range(64):
        w = _philox_np(n >> 1, 0, 0, 0, seed, chain)
        a, b = (w[2], w[3]) if n & 1 else (w[0], w[1])
        m = (a << 21) | (b >> 11)
        assert u[n] == m * 2.0 ** -53


def test_normal_pairs_equal_single_normals():
    # the GPU sampler draws momenta a Box-Muller pair at a time
    # (gbds_normal_pair_at); every value must equal gbds_normal_at's, bit for bit
    for seed, chain, start in [(99, 3, 0), (1, 0, 7), (2 ** 31 + 5, 1023, 10 ** 9 + 1)]:
        a = oracle.draws(seed, chain, 1, start, 257)
        b = oracle.draws(seed, chain, 2, start, 257)
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_normal_stream_moments_and_box_muller():
    z = oracle.draws(99, 3, 1, 0, 400000)
    assert abs(z.mean()) < 5 / math.sqrt(z.size)
    assert abs(z.var() - 1) < 5 * math.sqrt(2 / z.size)
    # Box-Muller pairs from one Philox block agree with libm to a few ulp.
    for n in range(0, 20, 2):
        w = _philox_np(n >> 1, 0, 1, 0, 99, 3)
        u = ((w[0] << 21) | (w[1] >> 11)) * 2.0 ** -53
        v = ((w[2] << 21) | (w[3] >> 11)) * 2.0 ** -53
        r = math.sqrt(-2 * math.log(1 - u))
        assert z[n] == pytest.approx(r * math.cos(2 * math.pi * v), rel=1e-14, abs=1e-14)
        assert z[n + 1] == pytest.approx(r * math.sin(2 * math.pi * v), rel=1e-14, abs=1e-14)


# --- base_nuts mock tests: src/test/unit/mcmc/hmc/nuts/base_nuts_test.cpp ---
def test_build_tree_mock():
    # base_nuts_test.cpp:139-198
    out = oracle.mock_scenario(1, [0.5] * 64)
    valid, rho, p_begin, ps_begin, p_end, ps_end, q, p, nlf, lsw, smp = out
    assert valid == 1
    assert rho == 1.5 * (nlf + 1)
    assert (p_begin, ps_begin, p_end, ps_end) == (1.5, 1.5, 1.5, 12)
    assert q == 8 * 1.5 and p == 1.5 and nlf == 8
    assert lsw == pytest.approx(-0.1 + math.log(8), rel=1e-6)
    assert smp == pytest.approx(math.exp(-0.1) * 8, rel=1e-6)


def test_rho_aggregation_mock():
    # base_nuts_test.cpp:200-266
    r = oracle.mock_scenario(2, [0.5] * 64) / 1.5
    assert len(r) == 21
    assert list(r[0::3]) == [2, 2, 4, 2, 2, 4, 8]
    assert list(r[1::3]) == [2, 2, 3, 2, 2, 3, 5]
    assert list(r[2::3]) == [2, 2, 3, 2, 2, 3, 5]


def test_divergence_mock():
    # base_nuts_test.cpp:268-333
    assert list(oracle.mock_scenario(3)) == [1, 0, 1, 0, 0, 1]


def test_transition_mock_reaches_max_depth():
    # base_nuts_test.cpp:335-373: depth == max_depth (5), n_leapfrog == 31,
    # lp 0, accept 1; the reference's draw 23 * 1.5 depends on its mixmax
    # stream (seed 0, chain 0).  Replaying a stream that takes every subtree
    # forward and picks local leaf 7 of the last 16-leaf subtree reproduces it.
    u = [0.9] * 36
    for i in (24, 25, 26):  # inner merges along the path to local leaf 7
        u[i] = 0.1
    depth, nlf, div, q, lp, acc, used = oracle.mock_scenario(4, u)[:7]
    assert (depth, nlf, div) == (5, 31, 0)
    assert q == 23 * 1.5
    assert lp == 0 and acc == 1 and used == 36


def test_transition_edge_momenta_mock():
    # base_nuts_test.cpp:375-438 (max_depth 2, both doublings forward)
    out = oracle.mock_scenario(5, [0.9] * 16)
    depth, nlf, div = out[:3]
    assert (depth, nlf, div) == (2, 3, 0)
    pairs = out[7:].reshape(-1, 2)
    expect = np.array([[0, 1], [0, 1], [0, 1], [2, 3], [2, 3], [2, 3], [0, 3], [0, 2], [1, 3]]) * 1.5
    assert pairs.shape == (9, 2)
    assert np.array_equal(pairs, expect)


# --- adaptation: src/test/unit/mcmc/*adaptation_test.cpp ---------------------
@pytest.mark.parametrize("state,eps,stat,expect_eps,expect_state", [
    # stepsize_adaptation_test.cpp:174-182
    ([273, 0.00513820936953773, 0.886351350781597, 2.488109515349, 0.5, 0.05, 0.75, 10],
     2.2037632781885, 1.0, 3.95863527373545, None),
    # stepsize_adaptation_test.cpp:184-200
    ([79, 0.0209457573689391, 0.821976337071218, 4.13018724667137, 0.5, 0.05, 0.75, 10],
     1.50198560950968, 0.728285153733299, 2.40769920051673,
     (80, 0.0181765250233587, 0.824095816988227)),
    # stepsize_adaptation_test.cpp:202-218 (epsilon tolerance 5e-14 there)
    ([79, 0.0206811620891896, 0.825842987938587, 4.13018305456267, 0.5, 0.05, 0.75, 10],
     1.574313439903, 0.684248188546772, 2.31161210908631,
     (80, 0.0184041693043455, 0.826295412288499)),
])
def test_dual_averaging_vectors(state, eps, stat, expect_eps, expect_state):
    st, e = oracle.learn_stepsize(state, eps, stat)
    assert abs(e - expect_eps) < 5e-14
    if expect_state:
        assert abs(st[0] - expect_state[0]) < 1e-14
        assert abs(st[1] - expect_state[1]) < 1e-14
        assert abs(st[2] - expect_state[2]) < 1e-14


def test_learn_stepsize_hits_target():
    # stepsize_adaptation_test.cpp:55-70: mu = log(1), delta = stat -> eps = 1
    st, e = oracle.learn_stepsize([0, 0, 0, math.log(1), 0.65, 0.05, 0.75, 10], 0.0, 0.65)
    assert e == 1.0


def test_var_adaptation_regularisation():
    # var_adaptation_test.cpp:5-27
    n, n_learn = 10, 10
    rc, var, upd, lines = oracle.var_adaptation(50, 0, 0, n_learn, np.zeros((n_learn, n)), np.zeros(n))
    assert rc == 0 and lines == []
    assert np.all(var == 1e-3 * 5.0 / (n_learn + 5.0))
    assert upd[-1] == 1 and upd[:-1].sum() == 0


def test_window_messages():
    # windowed_adaptation_test.cpp:5-48
    _, _, _, lines = oracle.var_adaptation(10, 1, 1, 1, np.zeros((1, 1)), np.zeros(1))
    assert "info|WARNING: No variance estimation is" in lines
    assert "info|         performed for num_warmup < 20" in lines
    _, _, _, lines = oracle.var_adaptation(100, 75, 50, 25, np.zeros((1, 1)), np.zeros(1))
    for want in ["WARNING: There aren't enough warmup iterations to fit the",
                 "         three stages of adaptation as currently configured.",
                 "         Reducing each adaptation stage to 15%/75%/10% of",
                 "         the given number of warmup iterations:",
                 "           init_buffer = 15", "           adapt_window = 75",
                 "           term_buffer = 10"]:
        assert "info|" + want in lines
    _, _, _, lines = oracle.var_adaptation(1000, 75, 50, 25, np.zeros((1, 1)), np.zeros(1))
    assert lines == []


def test_window_schedule_default():
    # 1000 warmup, 75/50/25: windows end at 99, 149, 249, 449, 949
    rng = np.random.default_rng(0)
    _, _, upd, _ = oracle.var_adaptation(1000, 75, 50, 25, rng.normal(size=(1000, 2)), np.ones(2))
    assert list(np.nonzero(upd)[0]) == [99, 149, 249, 449, 949]


def test_window_schedule_short_warmup_never_updates():
    # The 15%/75%/10% fallback (windowed_adaptation.hpp:339-371) returns without
    # restart(), so the end-of-window index keeps its unsigned wrap-around value
    # and the metric is never updated; restated as the reference behaves.
    rng = np.random.default_rng(0)
    _, _, upd, _ = oracle.var_adaptation(100, 75, 50, 25, rng.normal(size=(100, 2)), np.ones(2))
    assert upd.sum() == 0
