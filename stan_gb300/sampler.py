"""Array interface to the device run (gbnuts_sample_run): draws as NumPy arrays."""
import ctypes
import dataclasses

import numpy as np

from . import _lib

SAMPLER_COLUMNS = ["lp__", "accept_stat__", "stepsize__", "treedepth__", "n_leapfrog__",
                   "divergent__", "energy__"]
SUMMARY_COLUMNS = ["ess_bulk", "ess_tail", "rhat_bulk", "rhat_tail", "mcse_mean", "mcse_sd"]
_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


@dataclasses.dataclass
class RunResult:
    draws: np.ndarray        # (chains, rows, 7 + D); rows beyond n_rows are zero
    n_rows: np.ndarray
    n_warmup_rows: np.ndarray
    status: np.ndarray
    stepsize: np.ndarray
    inv_metric: np.ndarray
    init: np.ndarray
    n_grad: np.ndarray
    seconds: np.ndarray
    total_ms: float
    grad_ms: float           # mean duration of one batched-gradient partial kernel
    steps: int
    kernel_launches: int
    diagnostics: np.ndarray = None
    ess: np.ndarray = None   # (1 + D, 2): bulk, tail ESS of lp__ and each parameter
    # (1 + D, 6): bulk ESS, tail ESS, bulk R-hat, tail R-hat, mcse_mean, mcse_sd
    summary: np.ndarray = None

    def sampling_draws(self):
        """(iterations, chains, 7 + D) post-warmup draws (the chainset layout)."""
        w = int(self.n_warmup_rows.max()) if self.n_warmup_rows.size else 0
        n = int(self.n_rows.min())
        return np.transpose(self.draws[:, w:n], (1, 0, 2))


def prepare(D, num_chains=4, adapt=True, num_warmup=1000, num_samples=1000, num_thin=1,
            save_warmup=False, stepsize=1.0, stepsize_jitter=0.0, max_depth=10, delta=0.8,
            gamma=0.05, kappa=0.75, t0=10.0, init_buffer=75, term_buffer=50, window=25,
            init_radius=2.0, random_seed=0, init_chain_id=1, precision="fp64",
            inits=None, inv_metrics=None, save_diagnostics=False, report_ess=False,
            report_summary=False, metric="diag"):
    """Run configuration and caller-owned output buffers for a fit of dimension D.

    report_ess: also compute the split rank-normalised bulk / tail ESS of every
    quantity on the device when the fit ends (RunResult.ess).
    metric: "diag" (diag_e) or "dense" (dense_e; inv_metrics and
    RunResult.inv_metric are then (chains, D, D)).
    report_summary: also the full convergence summary (ESS, R-hat, MCSE) of every
    quantity, on the device (RunResult.summary; SUMMARY_COLUMNS).

    Returns (config, output, result): the ctypes structures point into the
    arrays of `result`, which must stay alive until the run has written them.
    """
    C = num_chains
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    ini = None if inits is None else np.ascontiguousarray(inits, dtype=np.float64).reshape(C, D)
    dense = metric == "dense"
    mshape = (C, D, D) if dense else (C, D)
    imi = None if inv_metrics is None else np.ascontiguousarray(
        inv_metrics, dtype=np.float64).reshape(mshape)
    cfg = _lib.RunConfig(C, int(adapt), num_warmup, num_samples, num_thin, int(save_warmup),
                         stepsize, stepsize_jitter, max_depth, delta, gamma, kappa, t0,
                         init_buffer, term_buffer, window, init_radius, random_seed,
                         init_chain_id, prec, int(save_diagnostics),
                         None if ini is None else _ptr(ini), None if imi is None else _ptr(imi),
                         _lib.METRIC_DENSE if dense else _lib.METRIC_DIAG)
    rows = ((num_warmup + num_thin - 1) // num_thin if save_warmup else 0) + \
        (num_samples + num_thin - 1) // num_thin
    rows = max(rows, 1)
    ncol = 7 + D
    res = RunResult(np.zeros((C, rows, ncol)), np.zeros(C, dtype=np.int32),
                    np.zeros(C, dtype=np.int32), np.zeros(C, dtype=np.int32), np.zeros(C),
                    np.zeros(mshape), np.zeros((C, D)), np.zeros(C, dtype=np.int64),
                    np.zeros((C, 2)), 0.0, 0.0, 0, 0,
                    np.zeros((C, rows, 3 * D)) if save_diagnostics else None)
    if report_ess:
        res.ess = np.full((1 + D, 2), np.nan)
    if report_summary:
        res.summary = np.full((1 + D, 6), np.nan)
    res._keep = (ini, imi)
    ip = ctypes.POINTER(ctypes.c_int)
    out = _lib.RunOutput(rows, ncol, _ptr(res.draws),
                         None if res.diagnostics is None else _ptr(res.diagnostics),
                         res.n_rows.ctypes.data_as(ip), res.n_warmup_rows.ctypes.data_as(ip),
                         res.status.ctypes.data_as(ip), _ptr(res.stepsize), _ptr(res.inv_metric),
                         _ptr(res.init), res.n_grad.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                         _ptr(res.seconds), 0.0, 0.0, 0, 0,
                         None if res.ess is None else _ptr(res.ess),
                         None if res.summary is None else _ptr(res.summary))
    res._run = (cfg, out)
    return cfg, out, res


def finish(out, res):
    """Copies the run totals of `out` into `res`."""
    res.total_ms, res.grad_ms = out.total_ms, out.grad_ms
    res.steps, res.kernel_launches = out.steps, out.kernel_launches
    return res


def write_csv(model, result, csv):
    """Writes a finished run (a RunResult of run(), or of a pool) as Stan CSV
    through a callbacks.CsvFiles, in the service functions' protocol
    (gbnuts_write_run; chains formatted concurrently)."""
    cfg, out = result._run
    cb = csv.open(cfg.num_chains, cfg.init_chain_id)
    try:
        rc = _lib.load().gbnuts_write_run(model.handle, ctypes.byref(cfg), ctypes.byref(out),
                                          ctypes.byref(cb))
    finally:
        csv.close()
    _lib.check(rc, "gbnuts_write_run")


def run(model, num_chains=4, **kwargs):
    """One fit through gbnuts_sample_run (the keyword arguments of prepare())."""
    lib = _lib.load()
    cfg, out, res = prepare(model.D, num_chains, **kwargs)
    rc = lib.gbnuts_sample_run(model.handle, ctypes.byref(cfg), ctypes.byref(out), None)
    _lib.check(rc, "gbnuts_sample_run")
    return finish(out, res)
