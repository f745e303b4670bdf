"""Post-hoc convergence diagnostics used for the min-bulk-ESS metric.

NumPy restatement of the reference's analysis code (paths relative to the
stan-dev/stan tree):
  src/stan/analyze/mcmc/autocovariance.hpp:38-99        biased FFT autocovariance
  src/stan/analyze/mcmc/ess.hpp:28-103                  Geyer initial monotone ESS
  src/stan/analyze/mcmc/split_chains.hpp:47-66          split chains in halves
  src/stan/analyze/mcmc/rank_normalization.hpp:23-56    average ranks -> normal scores
  src/stan/analyze/mcmc/check_chains.hpp                is_finite_and_varies
  src/stan/analyze/mcmc/split_rank_normalized_ess.hpp:28-55   (bulk, tail)
  src/stan/analyze/mcmc/mcse.hpp:22-61                  mcse_mean, mcse_sd
  src/stan/analyze/mcmc/rhat.hpp:20-45                  rhat from W and B
  src/stan/analyze/mcmc/split_rank_normalized_rhat.hpp:28-45  (bulk, tail) R-hat
The normal quantile is scipy.special.ndtri (the reference uses Boost's
quantile(normal)); the sample quantile is the linear-interpolation (R type 7)
estimator of Stan Math's quantile().  Chains are the columns of a
draws_per_chain x num_chains matrix, as in the reference.
"""
import math

import numpy as np
from scipy import special, stats


def _autocovariance_cols(x):
    """Biased autocovariance of every column: acov[t] = (1/N) sum c_i c_{i+t}."""
    n = x.shape[0]
    c = x - x.mean(axis=0, keepdims=True)
    nfft = 1 << int(math.ceil(math.log2(max(2 * n, 2))))
    f = np.fft.rfft(c, n=nfft, axis=0)
    ac = np.fft.irfft(f * np.conj(f), n=nfft, axis=0)[:n].real
    ac0 = ac[0:1].copy()
    with np.errstate(invalid="ignore", divide="ignore"):
        ac = ac / ac0
    var_pop = (c * c).mean(axis=0, keepdims=True)
    return ac * var_pop


def ess(chains):
    """ess.hpp:28-103 for one quantity; chains: (draws_per_chain, num_chains)."""
    chains = np.asarray(chains, dtype=np.float64)
    n, m = chains.shape
    acov = _autocovariance_cols(chains)
    chain_mean = chains.mean(axis=0)
    chain_var = acov[0] * n / (n - 1)
    w = chain_var.mean()
    var_plus = w * (n - 1) / n
    if m > 1:
        var_plus += chain_mean.var(ddof=1)
    rho_hat_t = np.zeros(n)
    rho_hat_even = 1.0
    rho_hat_t[0] = rho_hat_even
    rho_hat_odd = 1 - (w - acov[1].mean()) / var_plus
    rho_hat_t[1] = rho_hat_odd
    t = 1
    acov_mean = acov.mean(axis=1)
    while (t < n - 4 and (rho_hat_even + rho_hat_odd > 0)
           and not math.isnan(rho_hat_even + rho_hat_odd)):
        rho_hat_even = 1 - (w - acov_mean[t + 1]) / var_plus
        rho_hat_odd = 1 - (w - acov_mean[t + 2]) / var_plus
        if rho_hat_even + rho_hat_odd >= 0:
            rho_hat_t[t + 1] = rho_hat_even
            rho_hat_t[t + 2] = rho_hat_odd
        if rho_hat_t[t + 1] + rho_hat_t[t + 2] > rho_hat_t[t - 1] + rho_hat_t[t]:
            rho_hat_t[t + 1] = (rho_hat_t[t - 1] + rho_hat_t[t]) / 2
            rho_hat_t[t + 2] = rho_hat_t[t + 1]
        t += 2
    max_t = t
    if rho_hat_even > 0:
        rho_hat_t[max_t + 1] = rho_hat_even
    draws_total = m * n
    tau_hat = -1 + 2 * rho_hat_t[:max_t].sum() + rho_hat_t[max_t + 1]
    tau_hat = max(tau_hat, 1 / math.log10(draws_total))
    return draws_total / tau_hat


def split_chains(chains):
    chains = np.asarray(chains, dtype=np.float64)
    n, m = chains.shape
    half = n // 2
    tail = (n + 1) // 2
    out = np.empty((half, 2 * m))
    out[:, 0::2] = chains[:half]
    out[:, 1::2] = chains[tail:tail + half]
    return out


def _approx_constant(v, c, prec=1e-12):
    return bool(np.all(np.abs(v - c) <= prec * np.minimum(np.abs(v), abs(c))))


def is_finite_and_varies(chains):
    chains = np.asarray(chains, dtype=np.float64)
    if not np.all(np.isfinite(chains)):
        return False
    first = chains[0]
    for i in range(chains.shape[1]):
        if _approx_constant(chains[:, i], first[i]):
            return False
    if chains.shape[1] > 1 and _approx_constant(first, first[0]):
        return False
    return True


def rank_transform(chains):
    chains = np.asarray(chains, dtype=np.float64)
    s = chains.size
    r = stats.rankdata(chains.reshape(-1, order="F"), method="average")
    z = special.ndtri((r - 0.375) / (s + 0.25))
    return z.reshape(chains.shape, order="F")


def quantile(x, p):
    x = np.sort(np.asarray(x, dtype=np.float64).reshape(-1))
    idx = (x.size - 1) * p
    lo, hi = int(math.floor(idx)), int(math.ceil(idx))
    h = idx - lo
    return (1 - h) * x[lo] + h * x[hi]


def split_rank_normalized_ess(chains):
    """(bulk ESS, tail ESS) of one quantity."""
    sp = split_chains(chains)
    if not is_finite_and_varies(sp) or sp.shape[0] < 4:
        return float("nan"), float("nan")
    bulk = ess(rank_transform(sp))
    flat = sp.reshape(-1, order="F")
    q05 = (sp <= quantile(flat, 0.05)).astype(np.float64)
    q95 = (sp >= quantile(flat, 0.95)).astype(np.float64)
    e05, e95 = ess(q05), ess(q95)
    if math.isnan(e05):
        tail = e95
    elif math.isnan(e95):
        tail = e05
    else:
        tail = min(e05, e95)
    return bulk, tail


def rhat(chains):
    """sqrt(((n - 1)/n W + B/n) / W) with B, W the between- and within-chain variances."""
    chains = np.asarray(chains, dtype=np.float64)
    n, m = chains.shape
    means = chains.mean(axis=0)
    b = n * ((means - means.mean()) ** 2).sum() / (m - 1)
    w = (((chains - means) ** 2).sum(axis=0) / (n - 1.0)).sum() / m
    return math.sqrt((b / w + n - 1) / n)


def split_rank_normalized_rhat(chains):
    """(bulk R-hat, tail R-hat) of one quantity: R-hat of the normal scores of the
    split draws and of their distances from the median."""
    sp = split_chains(chains)
    if not is_finite_and_varies(sp):
        return float("nan"), float("nan")
    bulk = rhat(rank_transform(sp))
    med = quantile(sp.reshape(-1, order="F"), 0.5)
    tail = rhat(rank_transform(np.abs(sp - med)))
    return bulk, tail


def mcse_mean(chains):
    chains = np.asarray(chains, dtype=np.float64)
    if chains.shape[0] < 4 or not is_finite_and_varies(chains):
        return float("nan")
    sample_var = ((chains - chains.mean()) ** 2).sum() / (chains.size - 1)
    return math.sqrt(sample_var / ess(chains))


def mcse_sd(chains):
    chains = np.asarray(chains, dtype=np.float64)
    if chains.shape[0] < 4 or not is_finite_and_varies(chains):
        return float("nan")
    ctr = np.abs(chains - chains.mean())
    ess_mean = ess(split_chains(ctr))
    evar = (ctr ** 2).mean()
    fourth = (ctr ** 4).mean()
    varvar = (fourth - evar ** 2) / ess_mean
    varsd = varvar / evar / 4.0
    return math.sqrt(varsd)


def min_bulk_ess(draws, names=None):
    """Minimum bulk ESS over the last axis of draws (iterations, chains, quantities)."""
    draws = np.asarray(draws, dtype=np.float64)
    best, arg = float("inf"), None
    for j in range(draws.shape[2]):
        b, _ = split_rank_normalized_ess(draws[:, :, j])
        if not math.isnan(b) and b < best:
            best, arg = b, j
    return best, (names[arg] if names is not None and arg is not None else arg)
