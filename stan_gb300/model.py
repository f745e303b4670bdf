"""Model handle: the stand-in for stan::model::model_base as the sampler uses it
(src/stan/model/model_base.hpp:36-707; log_prob_grad.hpp:27-88)."""
import ctypes

import numpy as np

from . import _lib
from .workloads import Dataset

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _x_buffer(X, x_dtype):
    X = np.asarray(X)
    if x_dtype == "f64":
        return np.ascontiguousarray(X, dtype=np.float64), _lib.F64
    if x_dtype == "f32":
        return np.ascontiguousarray(X, dtype=np.float32), _lib.F32
    if x_dtype == "bf16":
        f = np.ascontiguousarray(X, dtype=np.float32)
        u = f.view(np.uint32).astype(np.uint64)
        lsb = (u >> np.uint64(16)) & np.uint64(1)
        b = ((u + np.uint64(0x7FFF) + lsb) >> np.uint64(16)).astype(np.uint16)
        return np.ascontiguousarray(b), _lib.BF16
    raise ValueError(f"unknown x_dtype {x_dtype}")


class Model:
    """A log density with its data resident on the GPU."""

    def __init__(self, kind, X, y, group=None, J=0, hp=None, intercept=True, x_dtype="f64"):
        lib = _lib.load()
        kind = kind if isinstance(kind, int) else {"logistic": 1, "poisson": 2,
                                                   "hier_normal": 3, "hier_logistic": 4}[kind]
        Xb, dt = _x_buffer(X, x_dtype)
        N, K = Xb.shape
        yb = np.ascontiguousarray(y, dtype=np.float64)
        gb = None if group is None else np.ascontiguousarray(group, dtype=np.int32)
        hpb = None if hp is None or len(hp) == 0 else np.ascontiguousarray(hp, dtype=np.float64)
        h = ctypes.c_void_p()
        rc = lib.gbnuts_model_create(
            kind, Xb.ctypes.data_as(ctypes.c_void_p), dt, _ptr(yb),
            None if gb is None else gb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            N, K, J, 1 if intercept else 0, None if hpb is None else _ptr(hpb),
            0 if hpb is None else len(hpb), ctypes.byref(h))
        _lib.check(rc, "gbnuts_model_create")
        self._h = h
        self.kind, self.N, self.K, self.J = kind, N, K, J
        self.D = lib.gbnuts_num_params_r(h)

    @classmethod
    def from_dataset(cls, ds: Dataset, x_dtype=None):
        return cls(ds.kind, ds.X, ds.y, group=ds.group, J=ds.J, hp=list(ds.hp),
                   intercept=ds.intercept, x_dtype=x_dtype or ds.x_dtype)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().gbnuts_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_params_r(self):
        return self.D

    def param_names(self, constrained=True):
        buf = ctypes.create_string_buffer(256)
        out = []
        for i in range(self.D):
            _lib.load().gbnuts_param_name(self._h, i, int(constrained), buf, 256)
            out.append(buf.value.decode())
        return out

    def log_prob(self, theta, propto=True, jacobian=True):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        lp = ctypes.c_double()
        _lib.check(_lib.load().gbnuts_log_prob(self._h, _ptr(th), int(propto), int(jacobian),
                                               ctypes.byref(lp)), "gbnuts_log_prob")
        return lp.value

    def log_prob_grad(self, theta, propto=True, jacobian=True):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        g = np.zeros(self.D)
        lp = ctypes.c_double()
        _lib.check(_lib.load().gbnuts_log_prob_grad(self._h, _ptr(th), int(propto), int(jacobian),
                                                    ctypes.byref(lp), _ptr(g)),
                   "gbnuts_log_prob_grad")
        return lp.value, g

    def log_prob_grad_batch(self, thetas, precision="fp64"):
        th = np.ascontiguousarray(thetas, dtype=np.float64)
        C = th.shape[0]
        lp = np.zeros(C)
        g = np.zeros((C, self.D))
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
        _lib.check(_lib.load().gbnuts_log_prob_grad_batch(self._h, C, _ptr(th), _ptr(lp), _ptr(g),
                                                          prec), "gbnuts_log_prob_grad_batch")
        return lp, g

    def write_array(self, theta):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        out = np.zeros(self.D)
        _lib.check(_lib.load().gbnuts_write_array(self._h, _ptr(th), _ptr(out)), "gbnuts_write_array")
        return out

    def unconstrain_array(self, theta):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        out = np.zeros(self.D)
        _lib.check(_lib.load().gbnuts_unconstrain_array(self._h, _ptr(th), _ptr(out)),
                   "gbnuts_unconstrain_array")
        return out
