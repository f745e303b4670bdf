"""The native Stan CSV / JSON metric writer (gbnuts_csv_open) on the CPU: its
callbacks are called directly, as the service calls them, and the files are
compared byte for byte with the reference's writer formats:
  src/stan/callbacks/stream_writer.hpp:16-103 (stream_writer_test.cpp:20-60:
  "0,1,2,3,4\\n", a blank is the prefix and a newline, a message is the prefix,
  the message and a newline; values as operator<< prints them, printf %.*g)
  src/stan/callbacks/json_writer.hpp (json_writer_test.cpp: record layout with
  two-space indentation, " : " after keys, NaN / Inf / -Inf)
"""
import ctypes
import os
import threading

import numpy as np
import pytest

from stan_gb300 import _lib

_dp = ctypes.POINTER(ctypes.c_double)


def _open(tmp_path, chains=2, diag=True, metric=True, sig_figs=6, chain_id0=1):
    lib = _lib.load()
    cb = _lib.Callbacks()
    h = ctypes.c_void_p()
    rc = lib.gbnuts_csv_open(str(tmp_path / "out").encode(),
                             str(tmp_path / "diag").encode() if diag else None,
                             str(tmp_path / "metric").encode() if metric else None,
                             chains, chain_id0, sig_figs, ctypes.byref(cb), ctypes.byref(h))
    assert rc == 0, _lib.last_error()
    return lib, cb, h


def _values(cb, chain, writer, vals):
    a = np.ascontiguousarray(vals, dtype=np.float64)
    cb.write_values(cb.ctx, chain, writer, a.ctypes.data_as(_dp), a.size)


def _names(cb, chain, writer, names):
    arr = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
    cb.write_names(cb.ctx, chain, writer, arr, len(names))


def _g(v, p=6):
    # operator<< of a double with precision p: C's %.*g
    return "%.*g" % (p, v)


def test_rows_messages_and_blank_match_stream_writer(tmp_path):
    lib, cb, h = _open(tmp_path)
    assert cb.want_diagnostics == 1 and cb.chains_concurrent == 1
    _names(cb, 0, 1, ["lp__", "accept_stat__", "beta.1"])
    _values(cb, 0, 1, [0, 1, 2])
    _values(cb, 0, 1, [-7.123456789, 0.000012345678, 1234567.0])
    cb.write_message(cb.ctx, 0, 1, b"Adaptation terminated")
    cb.write_blank(cb.ctx, 0, 1)
    _values(cb, 0, 1, [np.inf, -np.inf, np.nan])
    _values(cb, 1, 1, [3.5])
    _values(cb, 1, 2, [1e-300, 1e300])
    _values(cb, 0, 0, [1.0])  # the init writer has no file
    assert lib.gbnuts_csv_close(h) == 0, _lib.last_error()
    got = (tmp_path / "out_1.csv").read_text()
    want = ("lp__,accept_stat__,beta.1\n"
            "0,1,2\n"
            + ",".join(_g(v) for v in [-7.123456789, 0.000012345678, 1234567.0]) + "\n"
            "# Adaptation terminated\n"
            "# \n"
            "inf,-inf,nan\n")
    assert got == want
    assert (tmp_path / "out_2.csv").read_text() == "3.5\n"
    assert (tmp_path / "diag_2.csv").read_text() == "1e-300,1e+300\n"
    assert (tmp_path / "diag_1.csv").read_text() == ""


@pytest.mark.parametrize("p", [1, 3, 6, 9, 17])
def test_values_at_every_precision_equal_printf(tmp_path, p):
    rng = np.random.default_rng(p)
    v = np.concatenate([rng.normal(size=200) * 10.0 ** rng.integers(-12, 12, size=200),
                        [0.0, -0.0, 1.0, 0.1, 123456789.0, 5e-324, 1.7976931348623157e308,
                         0.5, 2.5, 1e-5, 1e-4, 99999.95, 999999.5]])
    lib, cb, h = _open(tmp_path, chains=1, diag=False, metric=False, sig_figs=p)
    _values(cb, 0, 1, v)
    assert lib.gbnuts_csv_close(h) == 0
    got = (tmp_path / "out_1.csv").read_text().rstrip("\n").split(",")
    assert got == [_g(x, p) for x in v]


def test_metric_record_matches_json_writer(tmp_path):
    lib, cb, h = _open(tmp_path, chains=2, chain_id0=5)
    inv = np.array([1.0, 0.25, np.nan, np.inf, -np.inf, 1.23456789])
    cb.write_metric(cb.ctx, 1, 0.123456789, b"diag_e", inv.ctypes.data_as(_dp), inv.size)
    assert lib.gbnuts_csv_close(h) == 0
    got = (tmp_path / "metric_6.json").read_text()
    want = ('\n{\n  "stepsize" : 0.123457,\n  "metric_type" : "diag_e",\n'
            '  "inv_metric" : [ 1, 0.25, NaN, Inf, -Inf, 1.23457 ]\n}\n')
    assert got == want
    assert not os.path.exists(tmp_path / "metric_5.json")


def test_chains_written_concurrently(tmp_path):
    """Each chain's writers are used by one thread at a time while other
    chains' writers run on other threads (the service's concurrent emission)."""
    C, rows, n = 16, 3000, 12
    lib, cb, h = _open(tmp_path, chains=C, diag=False, metric=False)
    data = [np.random.default_rng(c).normal(size=(rows, n)) for c in range(C)]

    def chain(c):
        _names(cb, c, 1, [f"x{i}" for i in range(n)])
        for r in range(rows):
            _values(cb, c, 1, data[c][r])
        cb.write_message(cb.ctx, c, 1, b"done")

    ts = [threading.Thread(target=chain, args=(c,)) for c in range(C)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert lib.gbnuts_csv_close(h) == 0
    for c in range(C):
        lines = (tmp_path / f"out_{c + 1}.csv").read_text().split("\n")
        assert lines[0] == ",".join(f"x{i}" for i in range(n))
        assert lines[rows + 1] == "# done" and lines[rows + 2] == ""
        back = np.array([[float(x) for x in ln.split(",")] for ln in lines[1:rows + 1]])
        assert np.allclose(back, data[c], rtol=1e-5, atol=0)


def test_open_errors(tmp_path):
    lib = _lib.load()
    cb = _lib.Callbacks()
    h = ctypes.c_void_p()
    missing = str(tmp_path / "no_such_dir" / "out").encode()
    assert lib.gbnuts_csv_open(missing, None, None, 2, 1, 6, ctypes.byref(cb),
                               ctypes.byref(h)) == _lib.NOINPUT
    assert lib.gbnuts_csv_open(str(tmp_path / "x").encode(), None, None, 0, 1, 6,
                               ctypes.byref(cb), ctypes.byref(h)) == _lib.USAGE
    assert lib.gbnuts_csv_open(str(tmp_path / "x").encode(), None, None, 1, 1, 0,
                               ctypes.byref(cb), ctypes.byref(h)) == _lib.USAGE


def test_dense_metric_record_matches_json_writer(tmp_path):
    # json_writer's Eigen matrix: "[ " rows as "[ a, b ]" joined by ", " " ]"
    lib, cb, h = _open(tmp_path, chains=1)
    inv = np.array([1.0, 0.5, 0.5, 2.0])
    cb.write_metric(cb.ctx, 0, 0.5, b"dense_e", inv.ctypes.data_as(_dp), inv.size)
    assert lib.gbnuts_csv_close(h) == 0
    got = (tmp_path / "metric_1.json").read_text()
    assert got == ('\n{\n  "stepsize" : 0.5,\n  "metric_type" : "dense_e",\n'
                   '  "inv_metric" : [ [ 1, 0.5 ], [ 0.5, 2 ] ]\n}\n')
