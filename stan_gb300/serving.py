"""Serving many posterior fits on one GPU: a fit pool with continuous batching.

`Pool` wraps the gbnuts_pool_* entry points: fits are submitted with their
data and run configuration, admitted while slots, the chain budget and device
memory allow, stepped together (every chain of every admitted fit advances in
the same two launches per step) and retired with their draws as soon as all of
their chains have finished, while later fits keep arriving.

`serve()` drives a pool with fits that arrive as a Poisson process and records
each fit's latency (arrival to results on the host).  The reference has no
counterpart: its service runs one fit per call
(src/stan/services/sample/hmc_nuts_diag_e_adapt.hpp:331-407).
"""
import ctypes
import dataclasses
import time

import numpy as np

from . import _lib, sampler
from .model import _x_buffer

QUEUED, RUNNING, DONE, UNKNOWN = 0, 1, 2, 3


class Pool:
    def __init__(self, precision="fp32", x_dtype="f32", max_fits=64, max_chains=1 << 16,
                 reserve_bytes=4 << 30):
        lib = _lib.load()
        self.precision = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
        self.x_dtype = x_dtype
        h = ctypes.c_void_p()
        _, dt = _x_buffer(np.zeros((1, 1)), x_dtype)
        rc = lib.gbnuts_pool_create(self.precision, dt, max_fits, max_chains, reserve_bytes,
                                    ctypes.byref(h))
        _lib.check(rc, "gbnuts_pool_create")
        self._h = h
        self._fits = {}  # id -> (result, output struct, host arrays kept alive)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().gbnuts_pool_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, ds, num_chains=4, **run_kwargs):
        """Queues a fit of dataset `ds` (workloads.Dataset); returns its id."""
        lib = _lib.load()
        Xb, dt = _x_buffer(ds.X, self.x_dtype)
        N, K = Xb.shape
        yb = np.ascontiguousarray(ds.y, dtype=np.float64)
        gb = None if ds.group is None else np.ascontiguousarray(ds.group, dtype=np.int32)
        hpb = np.ascontiguousarray(ds.hp, dtype=np.float64) if len(ds.hp) else None
        run_kwargs.setdefault("precision", self.precision)
        cfg, out, res = sampler.prepare(ds.D, num_chains, **run_kwargs)
        fid = ctypes.c_longlong()
        rc = lib.gbnuts_pool_submit(
            self._h, ds.kind, Xb.ctypes.data_as(ctypes.c_void_p), dt,
            yb.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            None if gb is None else gb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            N, K, ds.J, 1 if ds.intercept else 0,
            None if hpb is None else hpb.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            0 if hpb is None else len(hpb), ctypes.byref(cfg), ctypes.byref(out),
            ctypes.byref(fid))
        _lib.check(rc, "gbnuts_pool_submit")
        self._fits[fid.value] = (res, out)
        return fid.value

    def step(self, n_steps=32):
        """Admits, runs n_steps steps, retires; returns (fits running, fits queued)."""
        run, q = ctypes.c_int(), ctypes.c_int()
        rc = _lib.load().gbnuts_pool_step(self._h, n_steps, ctypes.byref(run), ctypes.byref(q))
        _lib.check(rc, "gbnuts_pool_step")
        return run.value, q.value

    def status(self, fit_id):
        st, rc = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.load().gbnuts_pool_status(self._h, fit_id, ctypes.byref(st),
                                                  ctypes.byref(rc)), "gbnuts_pool_status")
        return st.value, rc.value

    def stats(self):
        steps, chains = ctypes.c_longlong(), ctypes.c_longlong()
        _lib.check(_lib.load().gbnuts_pool_stats(self._h, ctypes.byref(steps), ctypes.byref(chains)),
                   "gbnuts_pool_stats")
        return steps.value, chains.value

    def result(self, fit_id):
        """The finished fit's RunResult (raises if it failed or is not done)."""
        st, rc = self.status(fit_id)
        if st != DONE:
            raise RuntimeError(f"fit {fit_id} is not done (state {st})")
        _lib.check(rc, f"pool fit {fit_id}")
        res, out = self._fits[fit_id]
        return sampler.finish(out, res)

    def pop(self, fit_id):
        """result() and forget the fit's buffers."""
        r = self.result(fit_id)
        del self._fits[fit_id]
        return r

    def run_all(self, n_steps=64):
        """Steps until every submitted fit is done."""
        while True:
            running, queued = self.step(n_steps)
            if running == 0 and queued == 0:
                return


def poisson_arrivals(rate, n, seed=0):
    """Arrival times (seconds from 0) of n events of a Poisson process of `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def latency_stats(latencies):
    a = np.asarray(latencies, dtype=np.float64)
    if a.size == 0:
        return {"n": 0, "p50": None, "p99": None, "mean": None, "max": None}
    return {"n": int(a.size), "p50": float(np.percentile(a, 50)),
            "p99": float(np.percentile(a, 99)), "mean": float(a.mean()), "max": float(a.max())}


@dataclasses.dataclass
class ServeReport:
    latencies: np.ndarray    # per fit, seconds from arrival to results on the host
    wall_s: float            # first arrival to last completion
    fits_per_s: float
    steps: int
    max_running: int

    def summary(self):
        d = latency_stats(self.latencies)
        d.update(wall_s=self.wall_s, fits_per_s=self.fits_per_s, steps=self.steps,
                 max_running=self.max_running)
        return d


def serve(pool, datasets, arrivals, steps_per_call=32, run_kwargs=None, on_done=None,
          clock=time.perf_counter):
    """Submits datasets[i] at arrivals[i] seconds after the start and steps the
    pool until every fit is done.  on_done(i, result) is called per fit."""
    run_kwargs = run_kwargs or {}
    n = len(datasets)
    order = np.argsort(arrivals, kind="stable")
    lat = np.zeros(n)
    ids = {}
    nxt = 0
    done = 0
    max_running = 0
    t0 = clock()
    while done < n:
        now = clock() - t0
        if not ids and nxt < n and arrivals[order[nxt]] > now:
            time.sleep(min(arrivals[order[nxt]] - now, 0.05))
            now = clock() - t0
        while nxt < n and arrivals[order[nxt]] <= now:
            i = int(order[nxt])
            ids[pool.submit(datasets[i], **run_kwargs)] = i
            nxt += 1
        running, _ = pool.step(steps_per_call)
        max_running = max(max_running, running)
        t_done = clock() - t0
        for fid, i in list(ids.items()):
            st, _ = pool.status(fid)
            if st == DONE:
                r = pool.pop(fid)
                lat[i] = t_done - arrivals[i]
                done += 1
                del ids[fid]
                if on_done is not None:
                    on_done(i, r)
    wall = clock() - t0 - float(np.min(arrivals))
    steps, _ = pool.stats()
    return ServeReport(lat, wall, n / wall if wall > 0 else float("inf"), steps, max_running)
