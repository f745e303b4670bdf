"""The batched gradient entry point that allocates no device memory.

Some callers cannot call cudaMalloc when they need a gradient (their device
memory is pre-reserved by their own pool, or they run under another
framework's allocator lock).  gbnuts_log_prob_grad_batch_device_noalloc
serves them from a fixed device array inside the library.  This file checks,
through the C ABI, that it returns what the regular batched entry point
returns, bit for bit, on two calls in a row (the array keeps the previous
call's contents), for a GLM and for a hierarchical model (whose group sums
must be cleared on every call), on a stream the caller created with two
models calling in turn, and that an oversized request is refused.  It is
named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from tests.datasets import make_dataset

pytestmark = pytest.mark.gpu


class _Dev:
    """Device buffers for the test's inputs and outputs (the test allocates
    them; the entry point under test does not)."""

    def __init__(self):
        self.rt = ctypes.CDLL("libcudart.so")
        self.rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        self.rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        self.rt.cudaFree.argtypes = [ctypes.c_void_p]
        self.rt.cudaMemset.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t]
        self.ptrs = []

    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), nbytes) == 0
        self.ptrs.append(p)
        return p

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        p = self.alloc(arr.nbytes)
        assert self.rt.cudaMemcpy(p, arr.ctypes.data, arr.nbytes, 1) == 0
        return p

    def get(self, p, shape):
        out = np.zeros(shape)
        assert self.rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, 2) == 0
        return out

    def sync(self):
        assert self.rt.cudaDeviceSynchronize() == 0

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)


def _both(model, theta, precision, stream=None):
    from stan_gb300 import _lib
    lib = _lib.load()
    dev = _Dev()
    C, D = theta.shape
    d_th = dev.put(theta)
    outs = []
    for fn in (lib.gbnuts_log_prob_grad_batch_device, lib.gbnuts_log_prob_grad_batch_device_noalloc):
        d_lp, d_g = dev.alloc(C * 8), dev.alloc(C * D * 8)
        rc = fn(model.handle, C, d_th, d_lp, d_g, _lib.PRECISIONS[precision], stream)
        assert rc == 0, _lib.last_error()
        dev.sync()
        outs.append((dev.get(d_lp, (C,)), dev.get(d_g, (C, D))))
    dev.free()
    return outs


@pytest.mark.parametrize("kind,precision", [("logistic_100k", "fp64"), ("hier_normal", "fp64"),
                                            ("logistic", "fp32")])
def test_no_alloc_matches_regular_entry_point_twice(kind, precision):
    """Both entry points run the same kernels with the same row splits, so
    their results are equal bit for bit, in either precision."""
    from stan_gb300 import Model
    ds = make_dataset(kind, small=True, seed=12)
    m = Model.from_dataset(ds)
    rng = np.random.default_rng(3)
    for call in range(2):  # the second call sees the first call's leftovers
        th = rng.normal(size=(48, m.D)) * 0.3
        (lp_a, g_a), (lp_b, g_b) = _both(m, th, precision)
        assert np.array_equal(lp_b, lp_a), call
        assert np.array_equal(g_b, g_a), call


def test_no_alloc_on_a_caller_stream_with_two_models_in_turn():
    """A stream the caller created, and two models of different families
    calling in turn on it: each call clears and rewrites what it reads from
    the shared array (split bounds, group sums), so the hierarchical model
    after the GLM, and the GLM after it, still equal the regular entry point."""
    from stan_gb300 import Model
    rt = _Dev().rt
    rt.cudaStreamCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
    rt.cudaStreamDestroy.argtypes = [ctypes.c_void_p]
    st = ctypes.c_void_p()
    assert rt.cudaStreamCreate(ctypes.byref(st)) == 0
    try:
        glm = Model.from_dataset(make_dataset("logistic_100k", small=True, seed=5))
        hier = Model.from_dataset(make_dataset("hier_normal", small=True, seed=6))
        rng = np.random.default_rng(9)
        for m in (glm, hier, glm, hier):
            th = rng.normal(size=(16, m.D)) * 0.3
            (lp_a, g_a), (lp_b, g_b) = _both(m, th, "fp64", st)
            assert np.array_equal(lp_b, lp_a)
            assert np.array_equal(g_b, g_a)
    finally:
        rt.cudaStreamSynchronize(st)
        rt.cudaStreamDestroy(st)


def test_no_alloc_refuses_oversized_requests():
    """40000 chains x (4 + 100) partial sums x 8 bytes = 33 MB of scratch, twice
    the fixed array: refused on the host.  The buffers are real and sized for
    the request, so the call would be valid even if it were not refused."""
    from stan_gb300 import Model, _lib
    ds = make_dataset("logistic_100k", small=False, seed=1)
    m = Model.from_dataset(ds)
    C = 40000
    dev = _Dev()
    d_th = dev.alloc(C * m.D * 8)
    d_lp = dev.alloc(C * 8)
    d_g = dev.alloc(C * m.D * 8)
    assert dev.rt.cudaMemset(d_th, 0, C * m.D * 8) == 0
    rc = _lib.load().gbnuts_log_prob_grad_batch_device_noalloc(m.handle, C, d_th, d_lp, d_g,
                                                               _lib.PREC_FP64, None)
    dev.sync()
    dev.free()
    assert rc == _lib.USAGE
    assert "bytes of scratch" in _lib.last_error()
