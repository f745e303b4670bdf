"""TEST INFRASTRUCTURE: ctypes wrapper around the CPU oracle (oracle/oracle.cpp).

The oracle is a C++ FP64 restatement of the reference's NUTS path (see the
header of oracle.cpp for the file:line map).  Only tests/, the smoke check and
bench.py's CPU-baseline leg use it, and only as the checker or the timed CPU
baseline, never as part of the product path.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

LOGISTIC, POISSON, HIER_NORMAL, HIER_LOGISTIC = 1, 2, 3, 4
N_SAMPLER_COLS = 7  # lp__, accept_stat__, stepsize__, treedepth__, n_leapfrog__, divergent__, energy__


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


class _ModelSpec(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("N", ctypes.c_int), ("K", ctypes.c_int),
        ("J", ctypes.c_int), ("intercept", ctypes.c_int),
        ("X", ctypes.POINTER(ctypes.c_double)), ("y", ctypes.POINTER(ctypes.c_double)),
        ("group", ctypes.POINTER(ctypes.c_int)), ("hp", ctypes.POINTER(ctypes.c_double)),
        ("n_hp", ctypes.c_int), ("compensated", ctypes.c_int),
    ]


class _SamplerConfig(ctypes.Structure):
    _fields_ = [
        ("num_warmup", ctypes.c_int), ("num_samples", ctypes.c_int),
        ("num_thin", ctypes.c_int), ("save_warmup", ctypes.c_int), ("refresh", ctypes.c_int),
        ("stepsize", ctypes.c_double), ("stepsize_jitter", ctypes.c_double),
        ("max_depth", ctypes.c_int), ("delta", ctypes.c_double), ("gamma", ctypes.c_double),
        ("kappa", ctypes.c_double), ("t0", ctypes.c_double),
        ("init_buffer", ctypes.c_uint), ("term_buffer", ctypes.c_uint), ("window", ctypes.c_uint),
        ("init_radius", ctypes.c_double), ("seed", ctypes.c_uint), ("init_chain_id", ctypes.c_uint),
        ("adapt", ctypes.c_int), ("dense", ctypes.c_int),
    ]


class _ChainOut(ctypes.Structure):
    _fields_ = [
        ("rows", ctypes.POINTER(ctypes.c_double)), ("unc", ctypes.POINTER(ctypes.c_double)),
        ("init", ctypes.POINTER(ctypes.c_double)), ("inv_metric", ctypes.POINTER(ctypes.c_double)),
        ("stepsize", ctypes.POINTER(ctypes.c_double)), ("n_grad", ctypes.POINTER(ctypes.c_longlong)),
        ("n_saved", ctypes.POINTER(ctypes.c_int)), ("return_code", ctypes.POINTER(ctypes.c_int)),
        ("seconds", ctypes.POINTER(ctypes.c_double)),
        ("draws_used", ctypes.POINTER(ctypes.c_ulonglong)),
        ("n_grad_total", ctypes.POINTER(ctypes.c_longlong)),
    ]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.oracle_model_create.restype = ctypes.c_void_p
        L.oracle_model_create.argtypes = [ctypes.POINTER(_ModelSpec)]
        L.oracle_model_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_model_dim.argtypes = [ctypes.c_void_p]
        L.oracle_log_prob.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_int, dp]
        L.oracle_log_prob_grad.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_int, dp, dp]
        L.oracle_write_array.argtypes = [ctypes.c_void_p, dp, dp]
        L.oracle_draws.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
                                   ctypes.c_ulonglong, ctypes.c_int, dp]
        L.oracle_philox.argtypes = [ctypes.POINTER(ctypes.c_uint)] * 3
        L.oracle_sample.argtypes = [ctypes.c_void_p, ctypes.POINTER(_SamplerConfig), ctypes.c_int,
                                    dp, dp, ctypes.c_int, ctypes.POINTER(_ChainOut)]
        L.oracle_learn_stepsize.argtypes = [dp, dp, ctypes.c_double]
        L.oracle_var_adaptation.argtypes = [ctypes.c_uint] * 4 + [
            ctypes.c_int, ctypes.c_int, dp, dp, ctypes.POINTER(ctypes.c_int),
            ctypes.c_char_p, ctypes.c_int]
        L.oracle_mock_scenario.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, ctypes.c_int]
        L.oracle_transition_scripted.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_double,
                                                 ctypes.c_int, dp, ctypes.c_int, dp,
                                                 ctypes.c_int, dp]
        L.oracle_covar_adaptation.argtypes = [ctypes.c_uint] * 4 + [
            ctypes.c_int, ctypes.c_int, dp, dp, ctypes.POINTER(ctypes.c_int)]
        L.oracle_dense_metric.argtypes = [ctypes.c_int, dp, dp, dp, dp, ctypes.c_uint,
                                          ctypes.c_uint, ctypes.c_int, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleModel:
    """One log density (logistic / Poisson GLM, hierarchical normal / logistic)."""

    def __init__(self, kind, X, y, group=None, J=0, hp=None, intercept=True, compensated=True):
        X = np.ascontiguousarray(X, dtype=np.float64)
        self.N, self.K = X.shape
        self._X = X
        self._y = np.ascontiguousarray(y, dtype=np.float64)
        self._g = None if group is None else np.ascontiguousarray(group, dtype=np.int32)
        self._hp = None if hp is None else np.ascontiguousarray(hp, dtype=np.float64)
        spec = _ModelSpec(kind, self.N, self.K, J, 1 if intercept else 0, _dp(self._X), _dp(self._y),
                          None if self._g is None else self._g.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                          None if self._hp is None else _dp(self._hp),
                          0 if self._hp is None else len(self._hp), int(compensated))
        self._h = lib().oracle_model_create(ctypes.byref(spec))
        if not self._h:
            raise ValueError("oracle model creation failed")
        self.D = lib().oracle_model_dim(self._h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.oracle_model_destroy(self._h)
            self._h = None

    def log_prob(self, theta, propto=True, jacobian=True):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        lp = ctypes.c_double()
        lib().oracle_log_prob(self._h, _dp(th), int(propto), int(jacobian), ctypes.byref(lp))
        return lp.value

    def log_prob_grad(self, theta, propto=True, jacobian=True):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        g = np.zeros(self.D)
        lp = ctypes.c_double()
        lib().oracle_log_prob_grad(self._h, _dp(th), int(propto), int(jacobian), ctypes.byref(lp), _dp(g))
        return lp.value, g

    def transition_scripted(self, q0, uniforms, normals, stepsize, max_depth=10,
                            inv_metric=None):
        """One base_nuts transition from q0 with the given draws (diag_e).
        Returns dict(q, lp, accept_stat, depth, n_leapfrog, divergent, energy,
        uniforms_used, normals_used)."""
        D = self.D
        q0 = np.ascontiguousarray(q0, dtype=np.float64)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        z = np.ascontiguousarray(normals, dtype=np.float64)
        im = None if inv_metric is None else np.ascontiguousarray(inv_metric, dtype=np.float64)
        out = np.zeros(D + 8)
        rc = lib().oracle_transition_scripted(self._h, _dp(q0), None if im is None else _dp(im),
                                              stepsize, max_depth, _dp(u), u.size, _dp(z),
                                              z.size, _dp(out))
        if rc != 0:
            raise RuntimeError("scripted draws exhausted")
        return {"q": out[:D].copy(), "lp": out[D], "accept_stat": out[D + 1],
                "depth": int(out[D + 2]), "n_leapfrog": int(out[D + 3]),
                "divergent": bool(out[D + 4]), "energy": out[D + 5],
                "uniforms_used": int(out[D + 6]), "normals_used": int(out[D + 7])}

    def write_array(self, theta):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        out = np.zeros(self.D)
        lib().oracle_write_array(self._h, _dp(th), _dp(out))
        return out

    def sample(self, num_chains=4, num_warmup=1000, num_samples=1000, num_thin=1,
               save_warmup=False, stepsize=1.0, stepsize_jitter=0.0, max_depth=10,
               delta=0.8, gamma=0.05, kappa=0.75, t0=10.0, init_buffer=75, term_buffer=50,
               window=25, init_radius=2.0, seed=0, init_chain_id=1, adapt=True,
               inits=None, inv_metrics=None, num_threads=None, dense=False):
        """Runs hmc_nuts_diag_e_adapt (adapt=True) or hmc_nuts_diag_e on the CPU;
        dense=True: the dense_e services (inverse metrics D x D per chain)."""
        D = self.D
        cfg = _SamplerConfig(num_warmup, num_samples, num_thin, int(save_warmup), 0,
                             stepsize, stepsize_jitter, max_depth, delta, gamma, kappa, t0,
                             init_buffer, term_buffer, window, init_radius, seed,
                             init_chain_id, int(adapt), int(dense))
        n_rows = (num_warmup if save_warmup else 0) + num_samples
        n_rows = (n_rows + num_thin - 1) // num_thin + 2
        C = num_chains
        rows = np.zeros((C, n_rows, N_SAMPLER_COLS + D))
        unc = np.zeros((C, n_rows, D))
        init = np.zeros((C, D))
        im = np.zeros((C, D, D) if dense else (C, D))
        eps = np.zeros(C)
        ng = np.zeros(C, dtype=np.int64)
        ns = np.zeros(C, dtype=np.int32)
        rc = np.zeros(C, dtype=np.int32)
        secs = np.zeros((C, 2))
        used = np.zeros((C, 2), dtype=np.uint64)
        ngt = np.zeros(C, dtype=np.int64)
        outs = (_ChainOut * C)()
        for i in range(C):
            outs[i] = _ChainOut(
                _dp(rows[i]), _dp(unc[i]), _dp(init[i]), _dp(im[i]),
                _dp(eps[i:i + 1]),
                ng[i:i + 1].ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                ns[i:i + 1].ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                rc[i:i + 1].ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                _dp(secs[i]),
                used[i].ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)),
                ngt[i:i + 1].ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        ini = None if inits is None else np.ascontiguousarray(inits, dtype=np.float64).reshape(C, D)
        imi = None if inv_metrics is None else np.ascontiguousarray(
            inv_metrics, dtype=np.float64).reshape((C, D, D) if dense else (C, D))
        nt = num_threads or os.cpu_count() or 1
        lib().oracle_sample(self._h, ctypes.byref(cfg), C, None if ini is None else _dp(ini),
                            None if imi is None else _dp(imi), nt, outs)
        m = int(ns.max()) if C else 0
        return {
            "rows": rows[:, :m], "unc": unc[:, :m], "init": init, "inv_metric": im,
            "stepsize": eps, "n_grad": ng, "n_saved": ns, "return_code": rc,
            "seconds": secs, "draws_used": used, "n_grad_total": ngt,
        }


def draws(seed, chain, stream, start, n):
    out = np.zeros(n)
    lib().oracle_draws(seed, chain, stream, start, n, _dp(out))
    return out


def philox(ctr, key):
    c = (ctypes.c_uint * 4)(*ctr)
    k = (ctypes.c_uint * 2)(*key)
    o = (ctypes.c_uint * 4)()
    lib().oracle_philox(c, k, o)
    return list(o)


def learn_stepsize(state, epsilon, adapt_stat):
    st = np.ascontiguousarray(state, dtype=np.float64).copy()
    e = np.array([epsilon], dtype=np.float64)
    lib().oracle_learn_stepsize(_dp(st), _dp(e), adapt_stat)
    return st, float(e[0])


def var_adaptation(num_warmup, init_buffer, term_buffer, window, q, var0):
    q = np.ascontiguousarray(q, dtype=np.float64)
    n, d = q.shape
    var = np.ascontiguousarray(var0, dtype=np.float64).copy()
    upd = np.zeros(n, dtype=np.int32)
    buf = ctypes.create_string_buffer(8192)
    rc = lib().oracle_var_adaptation(num_warmup, init_buffer, term_buffer, window, d, n,
                                     _dp(q), _dp(var), upd.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                     buf, 8192)
    lines = [l for l in buf.value.decode().split("\n") if l]
    return rc, var, upd, lines


def covar_adaptation(num_warmup, init_buffer, term_buffer, window, q, covar0):
    """covar_adaptation.learn_covariance over the rows of q; returns (rc, covar, updates)."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    n, d = q.shape
    covar = np.ascontiguousarray(covar0, dtype=np.float64).reshape(d, d).copy()
    upd = np.zeros(n, dtype=np.int32)
    rc = lib().oracle_covar_adaptation(num_warmup, init_buffer, term_buffer, window, d, n,
                                       _dp(q), _dp(covar),
                                       upd.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return rc, covar, upd


def dense_metric(inv_metric, p=None, seed=0, chain=1, n=0):
    """dense_e_metric at inverse metric a: (T(p), dtau_dp(p), n momenta from
    sample_p); None when a fails the services' validation."""
    a = np.ascontiguousarray(inv_metric, dtype=np.float64)
    d = a.shape[0]
    T = np.zeros(1)
    dt = np.zeros(d)
    pv = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros((max(n, 1), d))
    rc = lib().oracle_dense_metric(d, _dp(a), None if pv is None else _dp(pv), _dp(T), _dp(dt),
                                   seed, chain, n, _dp(out))
    if rc != 0:
        return None
    return float(T[0]), dt, out[:n]


def mock_scenario(scenario, uniforms=()):
    u = np.ascontiguousarray(np.asarray(uniforms, dtype=np.float64))
    if u.size == 0:
        u = np.zeros(1)
        nu = 0
    else:
        nu = u.size
    out = np.zeros(512)
    n = lib().oracle_mock_scenario(scenario, _dp(u), nu, _dp(out), 512)
    if n < 0:
        raise RuntimeError(f"mock scenario {scenario} failed ({n})")
    return out[:n]
