"""Convergence diagnostics on the device (gbnuts_ess, gbnuts_summary): split
rank-normalised bulk and tail ESS, bulk and tail R-hat and the Monte Carlo
standard errors of every quantity of a fit, for the serving loop's reports.

Restates src/stan/analyze/mcmc/split_rank_normalized_ess.hpp:28-55,
split_rank_normalized_rhat.hpp:28-45 and mcse.hpp:22-61 like the NumPy module
`analyze` (which the tests use to check this one); fits of up to 8192 split
draws per quantity (ESS) or 8192 draws per quantity (full summary).
"""
import numpy as np

from . import _lib


def _columns(result, quantities, fn, width):
    """Runs gbnuts_ess / gbnuts_summary over the quantities' columns of a
    RunResult's post-warmup draws (the same rows for every chain)."""
    draws = np.ascontiguousarray(result.draws, dtype=np.float64)
    C, max_rows, n_cols = draws.shape
    w = int(result.n_warmup_rows.max()) if result.n_warmup_rows.size else 0
    n = int(result.n_rows.min()) - w
    cols = [0] + list(range(7, n_cols)) if quantities == "all" else list(quantities)
    out = np.full((len(cols), width), np.nan)
    f = getattr(_lib.load(), fn)
    # contiguous runs of columns go to the device in one call
    i = 0
    while i < len(cols):
        j = i
        while j + 1 < len(cols) and cols[j + 1] == cols[j] + 1:
            j += 1
        buf = np.zeros(width * (j - i + 1))
        rc = f(draws.ctypes.data_as(_lib._dp), C, max_rows, n_cols, w, max(n, 0), cols[i],
               j - i + 1, buf.ctypes.data_as(_lib._dp))
        _lib.check(rc, fn)
        out[i:j + 1] = buf.reshape(-1, width)
        i = j + 1
    return out


def split_rank_ess(result, quantities="all"):
    """(bulk, tail) ESS arrays over lp__ and the parameters of a RunResult's
    post-warmup draws (the same rows for every chain)."""
    out = _columns(result, quantities, "gbnuts_ess", 2)
    return out[:, 0], out[:, 1]


def summary(result, quantities="all"):
    """(quantities, 6) array: bulk ESS, tail ESS, bulk R-hat, tail R-hat,
    mcse_mean, mcse_sd of lp__ and each parameter (sampler.SUMMARY_COLUMNS)."""
    return _columns(result, quantities, "gbnuts_summary", 6)


def max_rhat(result):
    """Largest of the bulk and tail R-hats over lp__ and the parameters."""
    s = summary(result)
    r = s[:, 2:4]
    return float(np.nanmax(r)) if np.any(np.isfinite(r)) else float("nan")


def min_bulk_ess(result):
    bulk, _ = split_rank_ess(result)
    return float(np.nanmin(bulk)) if np.any(np.isfinite(bulk)) else float("nan")
