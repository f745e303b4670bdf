"""Loads libgbnuts.so (the in-tree CUDA build) and declares its C ABI.

There is no CPU fallback: if the library is missing or cannot be loaded, every
entry point raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgbnuts.so")

OK, USAGE, DATAERR, NOINPUT, SOFTWARE, CONFIG = 0, 64, 65, 66, 70, 78
LOGISTIC, POISSON, HIER_NORMAL, HIER_LOGISTIC = 1, 2, 3, 4
F64, F32, BF16 = 0, 1, 2
PREC_FP64, PREC_FP32, PREC_BF16X3, PREC_BF16, PREC_F16X3 = 0, 1, 2, 3, 4
METRIC_DIAG, METRIC_DENSE = 0, 1
PRECISIONS = {"fp64": PREC_FP64, "fp32": PREC_FP32, "bf16x3": PREC_BF16X3, "bf16": PREC_BF16,
              "f16x3": PREC_F16X3}
INIT_WRITER, SAMPLE_WRITER, DIAGNOSTIC_WRITER = 0, 1, 2
CHAIN_STATUS = {0: "ok", 1: "init_failed", 2: "stepsize_init_failed", 3: "stepsize_failed",
                4: "metric_overflow", 5: "interrupted", 6: "bad_metric"}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_llp = ctypes.POINTER(ctypes.c_longlong)

WRITE_NAMES = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_char_p), ctypes.c_int)
WRITE_VALUES = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int)
WRITE_MESSAGE = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p)
WRITE_BLANK = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int)
LOG = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p)
INTERRUPT = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p)
WRITE_METRIC = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                ctypes.c_char_p, _dp, ctypes.c_int)


class Callbacks(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("write_names", WRITE_NAMES),
                ("write_values", WRITE_VALUES), ("write_message", WRITE_MESSAGE),
                ("write_blank", WRITE_BLANK), ("log", LOG), ("interrupt", INTERRUPT),
                ("write_metric", WRITE_METRIC), ("want_diagnostics", ctypes.c_int),
                ("chains_concurrent", ctypes.c_int)]


class RunConfig(ctypes.Structure):
    _fields_ = [("num_chains", ctypes.c_int), ("adapt", ctypes.c_int),
                ("num_warmup", ctypes.c_int), ("num_samples", ctypes.c_int),
                ("num_thin", ctypes.c_int), ("save_warmup", ctypes.c_int),
                ("stepsize", ctypes.c_double), ("stepsize_jitter", ctypes.c_double),
                ("max_depth", ctypes.c_int), ("delta", ctypes.c_double),
                ("gamma", ctypes.c_double), ("kappa", ctypes.c_double), ("t0", ctypes.c_double),
                ("init_buffer", ctypes.c_uint), ("term_buffer", ctypes.c_uint),
                ("window", ctypes.c_uint), ("init_radius", ctypes.c_double),
                ("random_seed", ctypes.c_uint), ("init_chain_id", ctypes.c_uint),
                ("precision", ctypes.c_int), ("save_diagnostics", ctypes.c_int),
                ("inits", _dp), ("inv_metrics", _dp), ("metric", ctypes.c_int)]


class RunOutput(ctypes.Structure):
    _fields_ = [("max_rows", ctypes.c_int), ("n_cols", ctypes.c_int), ("draws", _dp),
                ("diagnostics", _dp), ("n_rows", _ip), ("n_warmup_rows", _ip), ("status", _ip),
                ("stepsize", _dp), ("inv_metric", _dp), ("init", _dp), ("n_grad", _llp),
                ("seconds", _dp), ("total_ms", ctypes.c_double), ("grad_ms", ctypes.c_double),
                ("steps", ctypes.c_longlong), ("kernel_launches", ctypes.c_longlong),
                ("ess", _dp), ("summary", _dp)]


# Every exported symbol and its signature (restype, argtypes).
SIGNATURES = {
    "gbnuts_model_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _dp, _ip,
                                           ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, _dp, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "gbnuts_model_destroy": (None, [ctypes.c_void_p]),
    "gbnuts_num_params_r": (ctypes.c_int, [ctypes.c_void_p]),
    "gbnuts_param_name": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_char_p, ctypes.c_int]),
    "gbnuts_log_prob": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int, _dp]),
    "gbnuts_log_prob_grad": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int,
                                            _dp, _dp]),
    "gbnuts_log_prob_grad_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp,
                                                  ctypes.c_int]),
    "gbnuts_log_prob_grad_batch_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int,
                                                         ctypes.c_void_p, ctypes.c_void_p,
                                                         ctypes.c_void_p, ctypes.c_int,
                                                         ctypes.c_void_p]),
    "gbnuts_log_prob_grad_batch_device_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int,
                                                                 ctypes.c_void_p, ctypes.c_void_p,
                                                                 ctypes.c_void_p, ctypes.c_int,
                                                                 ctypes.c_void_p]),
    "gbnuts_write_array": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "gbnuts_unconstrain_array": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "gbnuts_hmc_nuts_diag_e_adapt": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_uint, ctypes.c_uint, ctypes.c_double,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
        ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
        ctypes.POINTER(Callbacks)]),
    "gbnuts_hmc_nuts_dense_e_adapt": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_uint, ctypes.c_uint, ctypes.c_double,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
        ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
        ctypes.POINTER(Callbacks)]),
    "gbnuts_hmc_nuts_diag_e": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_uint, ctypes.c_uint, ctypes.c_double,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
        ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Callbacks)]),
    "gbnuts_hmc_nuts_dense_e": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_uint, ctypes.c_uint, ctypes.c_double,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
        ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Callbacks)]),
    "gbnuts_sample_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RunConfig),
                                         ctypes.POINTER(RunOutput), ctypes.POINTER(Callbacks)]),
    "gbnuts_pool_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_longlong, ctypes.c_longlong,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "gbnuts_pool_destroy": (None, [ctypes.c_void_p]),
    "gbnuts_pool_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_int, _dp, _ip, ctypes.c_longlong,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp,
                                          ctypes.c_int, ctypes.POINTER(RunConfig),
                                          ctypes.POINTER(RunOutput), _llp]),
    "gbnuts_pool_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _ip, _ip]),
    "gbnuts_pool_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, _ip, _ip]),
    "gbnuts_pool_stats": (ctypes.c_int, [ctypes.c_void_p, _llp, _llp]),
    "gbnuts_ess_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "gbnuts_ess": (ctypes.c_int, [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]),
    "gbnuts_summary_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p]),
    "gbnuts_summary": (ctypes.c_int, [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      _dp]),
    "gbnuts_write_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RunConfig),
                                        ctypes.POINTER(RunOutput), ctypes.POINTER(Callbacks)]),
    "gbnuts_csv_open": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(Callbacks),
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "gbnuts_csv_close": (ctypes.c_int, [ctypes.c_void_p]),
    "gbnuts_set_launch_shape": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int]),
    "gbnuts_device_info": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    "gbnuts_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
}

_lib = None


def load(build_if_missing=True):
    """Returns the loaded library; builds it first when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"gbnuts CUDA library not built: {LIB_PATH} is missing")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    load().gbnuts_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


class GbnutsError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"{where} returned {code}: {last_error()}")
        self.code = code


def check(code, where):
    if code != OK:
        raise GbnutsError(code, where)
    return code


def device_info():
    buf = ctypes.create_string_buffer(512)
    load().gbnuts_device_info(buf, 512)
    return buf.value.decode()
