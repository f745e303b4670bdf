"""The four log densities restated from their definitions in extended
precision: an independent check of the oracle's (and the device's) values.

Stan Math is not present, so its semantics are written out here from the
distributions' definitions, as the sampler calls them
(src/stan/model/log_prob_grad.hpp:40-44,79-83, log_prob<propto, jacobian>):

  bernoulli_logit(y | eta)   = y eta - log(1 + e^eta)
  poisson_log(y | eta)       = y eta - e^eta - log(y!)          [log(y!) dropped under propto]
  normal(y | m, s)           = -(y - m)^2 / (2 s^2) - log s - log(2 pi) / 2
                               [with s a constant, -log s - log(2 pi)/2 drops under propto;
                                with s a parameter only -log(2 pi)/2 drops]
  tau = e^u, sigma = e^v     Jacobian terms u, v added when jacobian is true
  half-normal priors         normal_lpdf on the positive parameter (no truncation term)

Arithmetic: every product x * theta is split exactly into two doubles
(Dekker's product), eta_n and every gradient sum add those pieces in
double-double (pairwise error-free additions), and each row's link term is
evaluated in mpmath at 30 digits, so the returned lp and gradient are correct
to far below 1e-14 relative.  Parameter layouts and default prior scales are the library's:
  logistic / poisson : [alpha], beta[K]        prior normal(0, hp0) on every coordinate
  hier_normal        : mu, log tau, log sigma, z[J], beta[K]
                       mu ~ N(0, hp0), tau ~ N+(0, hp1), sigma ~ N+(0, hp2),
                       z ~ N(0, 1), beta ~ N(0, hp3)
  hier_logistic      : alpha, log tau, z[J], beta[K]
                       alpha ~ N(0, hp0), tau ~ N+(0, hp1), z ~ N(0, 1), beta ~ N(0, hp2)
"""
import math

import mpmath as mp
import numpy as np

LOGISTIC, POISSON, HIER_NORMAL, HIER_LOGISTIC = 1, 2, 3, 4
_SPLIT = 134217729.0  # 2^27 + 1


def _two_prod(a, b):
    """a * b = p + e exactly (Dekker), elementwise for float64 arrays."""
    p = a * b
    c = _SPLIT * a
    ah = c - (c - a)
    al = a - ah
    c = _SPLIT * b
    bh = c - (c - b)
    bl = b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def _two_sum_tree(a):
    """Sum of a along axis 0 as a double-double (hi, lo): pairwise error-free
    additions (Knuth's two-sum), the rounding errors of every level summed
    apart; accurate to about 2^-100 of the sum of magnitudes."""
    err = np.zeros(a.shape[1:])
    while a.shape[0] > 1:
        if a.shape[0] % 2:
            a = np.concatenate([a, np.zeros((1,) + a.shape[1:])])
        x, y = a[0::2], a[1::2]
        s = x + y
        bp = s - x
        err = err + ((x - (s - bp)) + (y - bp)).sum(axis=0)
        a = s
    hi = a[0] + err
    return hi, err - (hi - a[0])


def _row_dots(X, beta, block=8192):
    """x_n . beta for every row as a double-double (hi, lo)."""
    hi = np.empty(X.shape[0])
    lo = np.empty(X.shape[0])
    for b in range(0, X.shape[0], block):
        p, e = _two_prod(X[b:b + block], beta[None, :])
        h, l = _two_sum_tree(np.concatenate([p, e], axis=1).T)
        hi[b:b + block], lo[b:b + block] = h, l
    return hi, lo


def _col_sums(X, r_hi, r_lo, block=8192):
    """sum_n x_nk r_n for every column, r given as (hi, lo) doubles."""
    parts = []
    for b in range(0, X.shape[0], block):
        xb = X[b:b + block]
        p, e = _two_prod(xb, r_hi[b:b + block, None])
        h, l = _two_sum_tree(np.concatenate([p, e, xb * r_lo[b:b + block, None]], axis=0))
        parts += [h, l]
    h, l = _two_sum_tree(np.stack(parts))
    return h + l


def _dd(v):
    hi = float(v)
    return hi, float(v - hi)


def lp_grad(kind, X, y, theta, group=None, J=0, hp=(), intercept=True, propto=True,
            jacobian=True):
    """(lp, grad) of one point, exact to double precision."""
    mp.mp.dps = 30
    X = np.ascontiguousarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    th = np.asarray(theta, dtype=np.float64)
    N, K = X.shape
    hpv = lambda i, d: hp[i] if i < len(hp) else d  # noqa: E731
    half_log_2pi = mp.log(2 * mp.pi) / 2
    lp = mp.mpf(0)
    grad = np.zeros(th.size)

    def normal_prior(v, s):
        # normal(0, s) on a coordinate with a constant scale
        out = -(mp.mpf(v) / s) ** 2 / 2
        if not propto:
            out += -mp.log(s) - half_log_2pi
        return out

    if kind in (LOGISTIC, POISSON):
        off = 1 if intercept else 0
        alpha = th[0] if intercept else 0.0
        beta = th[off:]
        hi, lo = _row_dots(X, beta)
        r_hi = np.empty(N)
        r_lo = np.empty(N)
        terms = []
        for n in range(N):
            eta = mp.mpf(hi[n]) + mp.mpf(lo[n]) + mp.mpf(alpha)
            if kind == LOGISTIC:
                terms.append(y[n] * eta - mp.log1p(mp.exp(eta)))
                r = y[n] - 1 / (1 + mp.exp(-eta))
            else:
                mu = mp.exp(eta)
                t = y[n] * eta - mu
                if not propto:
                    t -= mp.loggamma(y[n] + 1)
                terms.append(t)
                r = y[n] - mu
            r_hi[n], r_lo[n] = _dd(r)
        lp = mp.fsum(terms)
        s = hpv(0, 2.5 if kind == LOGISTIC else 1.0)
        lp += mp.fsum(normal_prior(v, s) for v in th)
        g = _col_sums(X, r_hi, r_lo)
        grad[off:] = g
        if intercept:
            grad[0] = math.fsum(np.concatenate([r_hi, r_lo]))
        grad -= th / (s * s)
        return float(lp), grad

    group = np.asarray(group)
    if kind == HIER_NORMAL:
        mu_, ut, us = th[0], th[1], th[2]
        z = th[3:3 + J]
        beta = th[3 + J:]
        s_mu, s_tau, s_sig, s_beta = hpv(0, 5.0), hpv(1, 1.0), hpv(2, 1.0), hpv(3, 1.0)
        base = mu_
    else:
        alpha, ut = th[0], th[1]
        us = None
        z = th[2:2 + J]
        beta = th[2 + J:]
        s_a, s_tau, s_beta = hpv(0, 2.5), hpv(1, 1.0), hpv(2, 2.5)
        base = alpha
    tau = mp.exp(ut)
    hi, lo = _row_dots(X, beta)
    r_hi = np.empty(N)
    r_lo = np.empty(N)
    terms, sq = [], []
    if kind == HIER_NORMAL:
        sigma = mp.exp(us)
        inv_s2 = 1 / (sigma * sigma)
    for n in range(N):
        eta = mp.mpf(hi[n]) + mp.mpf(lo[n]) + mp.mpf(base) + tau * mp.mpf(z[group[n]])
        if kind == HIER_NORMAL:
            e = y[n] - eta
            terms.append(-e * e * inv_s2 / 2)
            sq.append(e * e)
            r = e * inv_s2
        else:
            terms.append(y[n] * eta - mp.log1p(mp.exp(eta)))
            r = y[n] - 1 / (1 + mp.exp(-eta))
        r_hi[n], r_lo[n] = _dd(r)
    lp = mp.fsum(terms)
    # group sums of r, then d/dz_j = tau gz_j - z_j, d/dtau = sum_j z_j gz_j
    gz = [mp.mpf(0)] * J
    order = np.argsort(group, kind="stable")
    bounds = np.searchsorted(group[order], np.arange(J + 1))
    for j in range(J):
        idx = order[bounds[j]:bounds[j + 1]]
        gz[j] = mp.mpf(math.fsum(np.concatenate([r_hi[idx], r_lo[idx]])))
    g_base = mp.mpf(math.fsum(np.concatenate([r_hi, r_lo])))
    g_tau = mp.fsum(mp.mpf(z[j]) * gz[j] for j in range(J))
    g_beta = _col_sums(X, r_hi, r_lo)
    zoff = 3 if kind == HIER_NORMAL else 2
    if kind == HIER_NORMAL:
        lp += -N * mp.mpf(us)
        if not propto:
            lp += -N * half_log_2pi
        lp += normal_prior(mu_, s_mu)
        # tau and sigma: normal(0, s) on the positive value
        lp += -(tau / s_tau) ** 2 / 2 - (sigma / s_sig) ** 2 / 2
        if not propto:
            lp += -mp.log(s_tau) - mp.log(s_sig) - 2 * half_log_2pi
        if jacobian:
            lp += mp.mpf(ut) + mp.mpf(us)
        grad[0] = float(g_base - mp.mpf(mu_) / s_mu ** 2)
        grad[1] = float(tau * (g_tau - tau / s_tau ** 2) + (1 if jacobian else 0))
        gsq = mp.fsum(sq)
        grad[2] = float(sigma * (-N / sigma + gsq / sigma ** 3 - sigma / s_sig ** 2) +
                        (1 if jacobian else 0))
    else:
        lp += normal_prior(alpha, s_a)
        lp += -(tau / s_tau) ** 2 / 2
        if not propto:
            lp += -mp.log(s_tau) - half_log_2pi
        if jacobian:
            lp += mp.mpf(ut)
        grad[0] = float(g_base - mp.mpf(alpha) / s_a ** 2)
        grad[1] = float(tau * (g_tau - tau / s_tau ** 2) + (1 if jacobian else 0))
    lp += mp.fsum(normal_prior(v, 1.0) for v in z)
    lp += mp.fsum(normal_prior(v, s_beta) for v in beta)
    for j in range(J):
        grad[zoff + j] = float(tau * gz[j] - mp.mpf(z[j]))
    grad[zoff + J:] = g_beta - beta / (s_beta * s_beta)
    return float(lp), grad


def for_dataset(ds, theta, propto=True, jacobian=True):
    """lp_grad for a stan_gb300.workloads.Dataset."""
    return lp_grad(ds.kind, ds.X, ds.y, theta, group=ds.group, J=ds.J, hp=tuple(ds.hp),
                   intercept=ds.intercept, propto=propto, jacobian=jacobian)
