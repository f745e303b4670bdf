"""Convergence diagnostics on the device (gbnuts_ess): split rank-normalised
bulk and tail ESS of every quantity of a fit, for the serving loop's reports.

Restates src/stan/analyze/mcmc/split_rank_normalized_ess.hpp:28-55 like the
NumPy module `analyze` (which the tests use to check this one); fits of up to
8192 split draws per quantity.
"""
import numpy as np

from . import _lib


def split_rank_ess(result, quantities="all"):
    """(bulk, tail) ESS arrays over lp__ and the parameters of a RunResult's
    post-warmup draws (the same rows for every chain)."""
    draws = np.ascontiguousarray(result.draws, dtype=np.float64)
    C, max_rows, n_cols = draws.shape
    w = int(result.n_warmup_rows.max()) if result.n_warmup_rows.size else 0
    n = int(result.n_rows.min()) - w
    cols = [0] + list(range(7, n_cols)) if quantities == "all" else list(quantities)
    out = np.full((len(cols), 2), np.nan)
    lib = _lib.load()
    # contiguous runs of columns go to the device in one call
    i = 0
    while i < len(cols):
        j = i
        while j + 1 < len(cols) and cols[j + 1] == cols[j] + 1:
            j += 1
        buf = np.zeros(2 * (j - i + 1))
        rc = lib.gbnuts_ess(draws.ctypes.data_as(_lib._dp), C, max_rows, n_cols, w, max(n, 0),
                            cols[i], j - i + 1, buf.ctypes.data_as(_lib._dp))
        _lib.check(rc, "gbnuts_ess")
        out[i:j + 1] = buf.reshape(-1, 2)
        i = j + 1
    return out[:, 0], out[:, 1]


def min_bulk_ess(result):
    bulk, _ = split_rank_ess(result)
    return float(np.nanmin(bulk)) if np.any(np.isfinite(bulk)) else float("nan")
