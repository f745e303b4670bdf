"""Recovers the draws of the reference's golden NUTS transition and writes
tests/golden/gauss3d_transition.json.

The reference pins one base_nuts transition with its own RNG
(src/test/unit/mcmc/hmc/nuts/unit_e_nuts_test.cpp:311-355): the gauss3D model
(x ~ normal(0, 1), 3 dimensions, unit metric), start q = (1, -1, 1), step
size 0.1 without jitter, draws from create_rng(4839294, 0) (boost mixmax with
Boost's normal_distribution).  Expected: tree depth 3, 15 leapfrog steps, not
divergent, draw q = (0.70149082, -0.69831347, 0.54392564), log_prob
-0.63779306, accept_stat 0.99912512.

That RNG is not restated here, so the transition's draws are recovered from
those expected values instead.  The momentum draw p0 (3 normals) and the
direction uniforms of the first three subtrees fix the trajectory; on a
standard normal target the leapfrog map is linear, so for a candidate
position k of the returned draw on the trajectory, p0 follows from
q_k(p0) = q.  Every direction pattern and position is tried; for each, a
restatement of base_nuts::transition / build_tree below (base_nuts.hpp:78-352)
searches the acceptance decisions that return that state, and the candidate
is kept when it also gives depth 3, 15 leapfrog steps and the expected
accept_stat.  Two mirror-image candidates remain (the trajectory read
forwards or backwards); the first is written.  Acceptance uniforms are set
to the middle of the interval that gives the decision, direction uniforms to
0.25 / 0.75.

The fixture then lets the oracle and the GPU sampler replay the transition
(tests/test_oracle_gauss3d_transition.py, tests/test_gpu_nuts_parity.py): a
pin of the transition's arithmetic (trajectory, energies, multinomial
sampling, U-turn criterion, accept_stat) against the reference's numbers,
with the reference's draws recovered rather than regenerated.

    python tests/golden/make_gauss3d_transition.py
"""
import itertools
import json
import math
import os

import numpy as np

EPS = 0.1
Q0 = np.array([1.0, -1.0, 1.0])
GOLDEN = {"depth": 3, "n_leapfrog": 15, "divergent": False,
          "q": [0.70149082, -0.69831347, 0.54392564], "log_prob": -0.63779306,
          "accept_stat": 0.99912512}


def leapfrog(q, p, h):
    """expl_leapfrog on V = |q|^2 / 2 with a unit metric."""
    p = p - h / 2 * q
    q = q + h * p
    p = p - h / 2 * q
    return q, p


def hamiltonian(q, p):
    return 0.5 * q @ q + 0.5 * p @ p


def log_sum_exp(a, b):
    if a == -math.inf:
        return b
    if b == -math.inf:
        return a
    return max(a, b) + math.log1p(math.exp(-abs(a - b)))


def criterion(p_sharp_minus, p_sharp_plus, rho):
    return p_sharp_plus @ rho > 0 and p_sharp_minus @ rho > 0


def transition(p0, forward, decide, max_depth=10):
    """base_nuts::transition with the given momentum, subtree directions and
    acceptance decisions.  Returns (q of the draw, accept_stat, depth,
    n_leapfrog, uniforms consumed)."""
    uniforms = []
    z = [Q0.copy(), p0.copy()]
    H0 = hamiltonian(*z)
    z_fwd, z_bck = [Q0.copy(), p0.copy()], [Q0.copy(), p0.copy()]
    z_sample, z_propose = [Q0.copy(), p0.copy()], [Q0.copy(), p0.copy()]
    p_ff = ps_ff = p_fb = ps_fb = p_bf = ps_bf = p_bb = ps_bb = p0.copy()
    rho = p0.copy()
    lsw = 0.0
    count = {"nlf": 0, "metro": 0.0}

    def accept(prob):
        yes = decide(prob)
        uniforms.append(prob / 2 if yes else (1 + prob) / 2)
        return yes

    def build(depth, prop, sign, st):
        if depth == 0:
            z[0], z[1] = leapfrog(z[0], z[1], sign * EPS)
            count["nlf"] += 1
            h = hamiltonian(*z)
            st["lsw"] = log_sum_exp(st["lsw"], H0 - h)
            count["metro"] += 1 if H0 - h > 0 else math.exp(H0 - h)
            prop[0], prop[1] = z[0].copy(), z[1].copy()
            st.update(ps_beg=z[1].copy(), ps_end=z[1].copy(), rho=st["rho"] + z[1],
                      p_beg=z[1].copy(), p_end=z[1].copy())
            return True
        init = dict(rho=np.zeros(3), lsw=-math.inf)
        if not build(depth - 1, prop, sign, init):
            st.update(ps_beg=init["ps_beg"], p_beg=init["p_beg"])
            return False
        prop_final = [z[0].copy(), z[1].copy()]
        final = dict(rho=np.zeros(3), lsw=-math.inf)
        if not build(depth - 1, prop_final, sign, final):
            st.update(ps_beg=init["ps_beg"], p_beg=init["p_beg"])
            return False
        lsw_sub = log_sum_exp(init["lsw"], final["lsw"])
        st["lsw"] = log_sum_exp(st["lsw"], lsw_sub)
        if final["lsw"] > lsw_sub or accept(math.exp(final["lsw"] - lsw_sub)):
            prop[0], prop[1] = prop_final
        rho_sub = init["rho"] + final["rho"]
        st.update(rho=st["rho"] + rho_sub, ps_beg=init["ps_beg"], ps_end=final["ps_end"],
                  p_beg=init["p_beg"], p_end=final["p_end"])
        ok = criterion(init["ps_beg"], final["ps_end"], rho_sub)
        ok &= criterion(init["ps_beg"], final["ps_beg"], init["rho"] + final["p_beg"])
        ok &= criterion(init["ps_end"], final["ps_end"], final["rho"] + init["p_end"])
        return ok

    depth = 0
    while depth < max_depth:
        fwd = forward[depth] if depth < len(forward) else True
        uniforms.append(0.75 if fwd else 0.25)
        if fwd:
            z[0], z[1] = z_fwd[0].copy(), z_fwd[1].copy()
            rho_b, p_bf, ps_bf = rho.copy(), p_ff.copy(), ps_ff.copy()
            st = dict(rho=np.zeros(3), lsw=-math.inf)
            valid = build(depth, z_propose, 1, st)
            ps_fb, ps_ff, rho_f = st["ps_beg"], st.get("ps_end", st["ps_beg"]), st["rho"]
            p_fb, p_ff = st["p_beg"], st.get("p_end", st["p_beg"])
            z_fwd = [z[0].copy(), z[1].copy()]
        else:
            z[0], z[1] = z_bck[0].copy(), z_bck[1].copy()
            rho_f, p_fb, ps_fb = rho.copy(), p_bb.copy(), ps_bb.copy()
            st = dict(rho=np.zeros(3), lsw=-math.inf)
            valid = build(depth, z_propose, -1, st)
            ps_bf, ps_bb, rho_b = st["ps_beg"], st.get("ps_end", st["ps_beg"]), st["rho"]
            p_bf, p_bb = st["p_beg"], st.get("p_end", st["p_beg"])
            z_bck = [z[0].copy(), z[1].copy()]
        if not valid:
            break
        depth += 1
        if st["lsw"] > lsw or accept(math.exp(st["lsw"] - lsw)):
            z_sample = [z_propose[0].copy(), z_propose[1].copy()]
        lsw = log_sum_exp(lsw, st["lsw"])
        rho = rho_b + rho_f
        if not (criterion(ps_bb, ps_ff, rho) and criterion(ps_bb, ps_fb, rho_b + p_fb)
                and criterion(ps_bf, ps_ff, rho_f + p_bf)):
            break
    return z_sample[0], count["metro"] / count["nlf"], depth, count["nlf"], uniforms


def momentum_for(k):
    """p0 such that the k-th leapfrog state (backwards for k < 0) is at the
    golden q (the map from p0 to q_k is affine)."""
    h = EPS if k > 0 else -EPS

    def q_at(p0):
        q, p = Q0.copy(), p0.copy()
        for _ in range(abs(k)):
            q, p = leapfrog(q, p, h)
        return q

    base = q_at(np.zeros(3))
    slope = q_at(np.ones(3)) - base
    return (np.array(GOLDEN["q"]) - base) / slope


def main():
    target = np.array(GOLDEN["q"])
    found = []
    for pattern in itertools.product([True, False], repeat=4):
        positions, fwd_len, bck_len = [], 0, 0
        for j in range(3):
            n = 2 ** j
            if pattern[j]:
                positions += [fwd_len + i + 1 for i in range(n)]
                fwd_len += n
            else:
                positions += [-(bck_len + i + 1) for i in range(n)]
                bck_len += n
        for k in positions:
            p0 = momentum_for(k)
            # depth, leapfrog count and accept_stat do not depend on the
            # acceptance decisions; only the returned state does
            _, acc, depth, nlf, _ = transition(p0, list(pattern), lambda prob: True)
            if (depth != GOLDEN["depth"] or nlf != GOLDEN["n_leapfrog"]
                    or abs(acc - GOLDEN["accept_stat"]) >= 1e-7):
                continue
            for bits in range(1 << 16):
                choice = iter((bits >> i) & 1 for i in range(16))
                q, acc, depth, nlf, uniforms = transition(
                    p0, list(pattern), lambda prob: next(choice, 1) == 1)
                if (depth == GOLDEN["depth"] and nlf == GOLDEN["n_leapfrog"]
                        and np.max(np.abs(q - target)) < 1e-8
                        and abs(acc - GOLDEN["accept_stat"]) < 1e-7):
                    found.append({"p0": p0.tolist(), "uniforms": uniforms,
                                  "directions": list(pattern), "position": k,
                                  "accept_stat_recovered": acc})
                    break
    if not found:
        raise SystemExit("no draw sequence reproduces the golden transition")
    out = {"source": "src/test/unit/mcmc/hmc/nuts/unit_e_nuts_test.cpp:311-355",
           "q0": Q0.tolist(), "stepsize": EPS, "golden": GOLDEN,
           "normals": found[0]["p0"], "uniforms": found[0]["uniforms"],
           "candidates": len(found), "position": found[0]["position"]}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gauss3d_transition.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst, "candidates:", len(found))


if __name__ == "__main__":
    main()
