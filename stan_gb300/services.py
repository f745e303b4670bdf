"""stan::services::sample::{hmc_nuts_diag_e_adapt, hmc_nuts_diag_e} with the
reference's argument order and callback protocol
(src/stan/services/sample/hmc_nuts_diag_e_adapt.hpp:331-343, :57-68;
src/stan/services/sample/hmc_nuts_diag_e.hpp:48-60), running every chain on
the GPU through the C ABI.  Returns the reference's error codes."""
import ctypes

import numpy as np

from . import _lib
from .callbacks import Interrupt, Logger, StructuredWriter, Writer

_dp = ctypes.POINTER(ctypes.c_double)


def _as_list(w, n, factory):
    if w is None:
        return [factory() for _ in range(n)]
    if isinstance(w, (list, tuple)):
        if len(w) != n:
            raise ValueError("need one writer per chain")
        return list(w)
    return [w] * n


def _context_matrix(values, num_chains, D, key, dense=False):
    """init / init_inv_metric contexts: None, one vector (one D x D matrix when
    dense) for all chains, a per-chain array, or a list of dicts holding `key`."""
    if values is None:
        return None
    if isinstance(values, (list, tuple)) and len(values) and isinstance(values[0], dict):
        if any(key not in v for v in values):
            return None
        values = [v[key] for v in values]
    a = np.asarray(values, dtype=np.float64)
    if dense:
        if a.ndim == 2:
            a = np.tile(a, (num_chains, 1, 1))
        return np.ascontiguousarray(a.reshape(num_chains, D, D))
    if a.ndim == 1:
        a = np.tile(a, (num_chains, 1))
    return np.ascontiguousarray(a.reshape(num_chains, D))


class _Bridge:
    """Routes the C callbacks to the per-chain Python writer objects."""

    def __init__(self, num_chains, logger, interrupt, init_w, sample_w, diag_w, metric_w):
        self.logger = logger or Logger()
        self.interrupt = interrupt or Interrupt()
        self.writers = {_lib.INIT_WRITER: init_w, _lib.SAMPLE_WRITER: sample_w,
                        _lib.DIAGNOSTIC_WRITER: diag_w}
        self.metric = metric_w
        self.error = None
        cb = _lib.Callbacks()
        cb.ctx = None
        cb.write_names = _lib.WRITE_NAMES(self._names)
        cb.write_values = _lib.WRITE_VALUES(self._values)
        cb.write_message = _lib.WRITE_MESSAGE(self._message)
        cb.write_blank = _lib.WRITE_BLANK(self._blank)
        cb.log = _lib.LOG(self._log)
        cb.interrupt = _lib.INTERRUPT(self._interrupt)
        cb.write_metric = _lib.WRITE_METRIC(self._metric)
        cb.want_diagnostics = int(any(type(w) is not Writer for w in diag_w))
        self.cb = cb

    def _guard(self, f):
        try:
            f()
        except Exception as e:  # never let an exception unwind through C
            if self.error is None:
                self.error = e

    def _names(self, ctx, chain, w, names, n):
        self._guard(lambda: self.writers[w][chain]([names[i].decode() for i in range(n)]))

    def _values(self, ctx, chain, w, vals, n):
        self._guard(lambda: self.writers[w][chain]([vals[i] for i in range(n)]))

    def _message(self, ctx, chain, w, msg):
        self._guard(lambda: self.writers[w][chain](msg.decode()))

    def _blank(self, ctx, chain, w):
        self._guard(lambda: self.writers[w][chain]())

    def _log(self, ctx, level, msg):
        m = msg.decode()
        f = [self.logger.debug, self.logger.info, self.logger.warn, self.logger.error,
             self.logger.fatal][level]
        self._guard(lambda: f(m))

    def _interrupt(self, ctx):
        try:
            return 1 if self.interrupt() else 0
        except Exception:
            return 1

    def _metric(self, ctx, chain, stepsize, metric_type, inv, n):
        w = self.metric[chain]

        def f():
            w.begin_record()
            w.write("stepsize", stepsize)
            w.write("metric_type", metric_type.decode())
            vals = [inv[i] for i in range(n)]
            if metric_type == b"dense_e":  # n = D * D, row-major
                d = int(round(n ** 0.5))
                vals = [vals[i * d:(i + 1) * d] for i in range(d)]
            w.write("inv_metric", vals)
            w.end_record()
        self._guard(f)


def _callbacks(bridge, csv, num_chains, chain_id0):
    """The bridge's callbacks, or the native CSV writer's with the bridge's
    logger and interrupt."""
    if csv is None:
        return bridge.cb
    cb = csv.open(num_chains, chain_id0)
    cb.log = bridge.cb.log
    cb.interrupt = bridge.cb.interrupt
    return cb


def _finish(bridge, csv):
    if csv is not None:
        csv.close()
    if bridge.error is not None:
        raise bridge.error


def hmc_nuts_diag_e_adapt(model, num_chains, init, init_inv_metric, random_seed, init_chain_id,
                          init_radius, num_warmup, num_samples, num_thin, save_warmup, refresh,
                          stepsize, stepsize_jitter, max_depth, delta, gamma, kappa, t0,
                          init_buffer, term_buffer, window, interrupt=None, logger=None,
                          init_writer=None, sample_writer=None, diagnostic_writer=None,
                          metric_writer=None, precision="fp64", csv=None,
                          _metric=0):
    """Adaptive diag_e NUTS for num_chains chains; writers are lists (one per chain),
    or csv: a callbacks.CsvFiles that writes Stan CSV files natively."""
    D = model.D
    bridge = _Bridge(num_chains, logger, interrupt,
                     _as_list(init_writer, num_chains, Writer),
                     _as_list(sample_writer, num_chains, Writer),
                     _as_list(diagnostic_writer, num_chains, Writer),
                     _as_list(metric_writer, num_chains, StructuredWriter))
    ini = _context_matrix(init, num_chains, D, "theta")
    imi = _context_matrix(init_inv_metric, num_chains, D, "inv_metric",
                          dense=_metric == _lib.METRIC_DENSE)
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    cb = _callbacks(bridge, csv, num_chains, init_chain_id)
    fn = "gbnuts_hmc_nuts_dense_e_adapt" if _metric else "gbnuts_hmc_nuts_diag_e_adapt"
    rc = getattr(_lib.load(), fn)(
        model.handle, num_chains, None if ini is None else ini.ctypes.data_as(_dp),
        None if imi is None else imi.ctypes.data_as(_dp), random_seed, init_chain_id,
        init_radius, num_warmup, num_samples, num_thin, int(save_warmup), refresh, stepsize,
        stepsize_jitter, max_depth, delta, gamma, kappa, t0, init_buffer, term_buffer, window,
        prec, ctypes.byref(cb))
    _finish(bridge, csv)
    return rc


def hmc_nuts_diag_e(model, num_chains, init, init_inv_metric, random_seed, init_chain_id,
                    init_radius, num_warmup, num_samples, num_thin, save_warmup, refresh,
                    stepsize, stepsize_jitter, max_depth, interrupt=None, logger=None,
                    init_writer=None, sample_writer=None, diagnostic_writer=None,
                    precision="fp64", csv=None, _metric=0):
    """Non-adaptive diag_e NUTS (the resume path) for num_chains chains (csv as
    for hmc_nuts_diag_e_adapt)."""
    D = model.D
    bridge = _Bridge(num_chains, logger, interrupt,
                     _as_list(init_writer, num_chains, Writer),
                     _as_list(sample_writer, num_chains, Writer),
                     _as_list(diagnostic_writer, num_chains, Writer),
                     [StructuredWriter() for _ in range(num_chains)])
    ini = _context_matrix(init, num_chains, D, "theta")
    imi = _context_matrix(init_inv_metric, num_chains, D, "inv_metric",
                          dense=_metric == _lib.METRIC_DENSE)
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    cb = _callbacks(bridge, csv, num_chains, init_chain_id)
    fn = "gbnuts_hmc_nuts_dense_e" if _metric else "gbnuts_hmc_nuts_diag_e"
    rc = getattr(_lib.load(), fn)(
        model.handle, num_chains, None if ini is None else ini.ctypes.data_as(_dp),
        None if imi is None else imi.ctypes.data_as(_dp), random_seed, init_chain_id,
        init_radius, num_warmup, num_samples, num_thin, int(save_warmup), refresh, stepsize,
        stepsize_jitter, max_depth, prec, ctypes.byref(cb))
    _finish(bridge, csv)
    return rc


def _dense(fn, name):
    """The dense_e form of a diag_e service wrapper: same arguments, with
    init_inv_metric as D x D matrices (one for all chains or one per chain)."""
    import functools

    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        return fn(*args, _metric=_lib.METRIC_DENSE, **kwargs)
    wrapper.__name__ = name
    wrapper.__doc__ = fn.__doc__.replace("diag_e", "dense_e") + (
        "  Dense form: init_inv_metric D x D.")
    return wrapper


hmc_nuts_dense_e_adapt = _dense(hmc_nuts_diag_e_adapt, "hmc_nuts_dense_e_adapt")
hmc_nuts_dense_e = _dense(hmc_nuts_diag_e, "hmc_nuts_dense_e")
