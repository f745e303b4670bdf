"""Failure detection without a GPU fault: every device wait in the library
is bounded and reports through an error code instead of hanging.  A wait on
an mbarrier that nothing arrives on, with a short limit, must give up, record
its code and leave the device usable (a regular gradient call after it
succeeds)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_that_nothing_satisfies_gives_up_and_reports():
    from stan_gb300 import Model, _lib
    from tests.datasets import make_dataset
    lib = _lib.load()
    f = lib.gbnuts_wait_probe
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_longlong, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    code, done = ctypes.c_int(-1), ctypes.c_int(-1)
    assert f(2_000_000, ctypes.byref(code), ctypes.byref(done)) == 0, _lib.last_error()
    assert done.value == 0 and code.value == 77
    ds = make_dataset("logistic", small=True, seed=2)
    m = Model.from_dataset(ds)
    lp, g = m.log_prob_grad(np.zeros(m.D))
    assert np.isfinite(lp) and np.all(np.isfinite(g))
