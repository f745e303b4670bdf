"""Python counterparts of the reference's callback interfaces
(src/stan/callbacks/writer.hpp:16-61, stream_writer.hpp:16-103, logger.hpp:24-97,
stream_logger.hpp:17, interrupt.hpp:14-28, structured_writer.hpp:16-150).

A writer is called with a list of names, a list of values, a message string, or
nothing (a blank line), exactly as the reference's writer::operator() overloads.
"""
import io


class Writer:
    """No-op writer (the reference's base class)."""

    def names(self, names):
        pass

    def values(self, values):
        pass

    def message(self, message):
        pass

    def blank(self):
        pass

    def __call__(self, *args):
        if not args:
            return self.blank()
        a = args[0]
        if isinstance(a, str):
            return self.message(a)
        if len(a) and isinstance(a[0], str):
            return self.names(list(a))
        if len(a) == 0:
            return self.names([])
        return self.values(list(a))


class StreamWriter(Writer):
    """stream_writer: comma-separated rows; messages prefixed (default "# ")."""

    def __init__(self, stream=None, prefix="# "):
        self.stream = stream if stream is not None else io.StringIO()
        self.prefix = prefix

    def names(self, names):
        self.stream.write(",".join(names) + "\n")

    def values(self, values):
        self.stream.write(",".join(f"{v:g}" for v in values) + "\n")

    def message(self, message):
        self.stream.write(self.prefix + message + "\n")

    def blank(self):
        self.stream.write(self.prefix + "\n")


class Logger:
    def debug(self, msg):
        pass

    def info(self, msg):
        pass

    def warn(self, msg):
        pass

    def error(self, msg):
        pass

    def fatal(self, msg):
        pass


class StreamLogger(Logger):
    def __init__(self, info=None, err=None):
        self.out = info if info is not None else io.StringIO()
        self.err = err if err is not None else self.out

    def debug(self, msg):
        self.out.write(msg + "\n")

    def info(self, msg):
        self.out.write(msg + "\n")

    def warn(self, msg):
        self.err.write(msg + "\n")

    def error(self, msg):
        self.err.write(msg + "\n")

    def fatal(self, msg):
        self.err.write(msg + "\n")


class Interrupt:
    """Called once per iteration in the reference; raising (here: returning
    True) stops sampling."""

    def __call__(self):
        return False


class StructuredWriter:
    """Receives the adapted {stepsize, metric_type, inv_metric} record."""

    def __init__(self):
        self.records = []

    def begin_record(self):
        self.records.append({})

    def write(self, key, value):
        self.records[-1][key] = value

    def end_record(self):
        pass


class CsvFiles:
    """Native Stan CSV output (gbnuts_csv_open): per chain <sample_prefix>_<id>.csv,
    optionally <diagnostic_prefix>_<id>.csv and the metric record
    <metric_prefix>_<id>.json, ids from the service's init_chain_id.  The
    service formats rows in native code, chains in parallel; pass it as
    `csv=` to the service functions (their Python writer arguments are then
    unused; logger and interrupt still apply)."""

    def __init__(self, sample_prefix, diagnostic_prefix=None, metric_prefix=None, sig_figs=6):
        self.sample_prefix = sample_prefix
        self.diagnostic_prefix = diagnostic_prefix
        self.metric_prefix = metric_prefix
        self.sig_figs = sig_figs
        self._h = None

    def open(self, num_chains, chain_id0):
        import ctypes

        from . import _lib
        cb = _lib.Callbacks()
        h = ctypes.c_void_p()
        enc = (lambda s: None if s is None else str(s).encode())
        rc = _lib.load().gbnuts_csv_open(enc(self.sample_prefix), enc(self.diagnostic_prefix),
                                         enc(self.metric_prefix), num_chains, chain_id0,
                                         self.sig_figs, ctypes.byref(cb), ctypes.byref(h))
        _lib.check(rc, "gbnuts_csv_open")
        self._h = h
        return cb

    def close(self):
        from . import _lib
        if self._h is not None:
            h, self._h = self._h, None
            _lib.check(_lib.load().gbnuts_csv_close(h), "gbnuts_csv_close")
