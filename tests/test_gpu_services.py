"""The service functions' writer protocol (hmc_nuts_diag_e_adapt_test.cpp:19-196,
mcmc_writer.hpp:63-259): names, warmup rows, the adaptation block, sampling
rows and the timing block per chain; and the native CSV writer's files equal to
the Python stream writers' text for the same run (the native writer formats
the chains concurrently)."""
import io

import numpy as np
import pytest

from tests.datasets import make_dataset

pytestmark = pytest.mark.gpu

KW = dict(init=None, init_inv_metric=None, random_seed=11, init_chain_id=1, init_radius=2.0,
          num_warmup=120, num_samples=80, num_thin=1, save_warmup=False, refresh=0,
          stepsize=1.0, stepsize_jitter=0.0, max_depth=10, delta=0.8, gamma=0.05, kappa=0.75,
          t0=10.0, init_buffer=30, term_buffer=20, window=20)


def _strip_timing(text):
    """The text without the values of the elapsed-time lines (they differ run to run)."""
    out = []
    for ln in text.split("\n"):
        if "seconds (" in ln:
            ln = ln.split("seconds (")[1]
        out.append(ln)
    return "\n".join(out)


def _python_run(m, C):
    from stan_gb300 import services
    from stan_gb300.callbacks import StreamWriter, StructuredWriter
    sample = [StreamWriter(io.StringIO()) for _ in range(C)]
    diag = [StreamWriter(io.StringIO()) for _ in range(C)]
    metric = [StructuredWriter() for _ in range(C)]
    rc = services.hmc_nuts_diag_e_adapt(m, C, sample_writer=sample, diagnostic_writer=diag,
                                        metric_writer=metric, **KW)
    return rc, [w.stream.getvalue() for w in sample], [w.stream.getvalue() for w in diag]


def test_service_protocol():
    from stan_gb300 import Model
    ds = make_dataset("logistic", small=True, seed=3)
    m = Model.from_dataset(ds)
    C = 3
    rc, sample, diag = _python_run(m, C)
    assert rc == 0
    D = m.D
    for c in range(C):
        lines = sample[c].split("\n")
        names = lines[0].split(",")
        assert names[:7] == ["lp__", "accept_stat__", "stepsize__", "treedepth__",
                             "n_leapfrog__", "divergent__", "energy__"]
        assert len(names) == 7 + D
        assert lines[1] == "# Adaptation terminated"
        assert lines[2].startswith("# Step size = ")
        assert lines[3] == "# Diagonal elements of inverse mass matrix:"
        assert len(lines[4][2:].split(", ")) == D
        rows = lines[5:5 + KW["num_samples"]]
        assert all(len(r.split(",")) == 7 + D for r in rows)
        assert lines[5 + KW["num_samples"]] == "# "
        assert "Elapsed Time" in lines[6 + KW["num_samples"]]
        dl = diag[c].split("\n")
        assert len(dl[0].split(",")) == 7 + 3 * D
        assert dl[0].split(",")[7 + D].startswith("p_")


def test_native_csv_equals_stream_writers(tmp_path):
    from stan_gb300 import Model, services
    from stan_gb300.callbacks import CsvFiles
    ds = make_dataset("hier_logistic", small=True, seed=4)
    m = Model.from_dataset(ds)
    C = 6
    rc, sample, diag = _python_run(m, C)
    assert rc == 0
    csv = CsvFiles(tmp_path / "out", tmp_path / "diag", tmp_path / "metric")
    rc2 = services.hmc_nuts_diag_e_adapt(m, C, csv=csv, **KW)
    assert rc2 == 0
    for c in range(C):
        got = (tmp_path / f"out_{c + 1}.csv").read_text()
        assert _strip_timing(got) == _strip_timing(sample[c]), c
        got = (tmp_path / f"diag_{c + 1}.csv").read_text()
        assert _strip_timing(got) == _strip_timing(diag[c]), c
        js = (tmp_path / f"metric_{c + 1}.json").read_text()
        assert js.startswith('\n{\n  "stepsize" : ') and '"metric_type" : "diag_e"' in js
        inv = js.split("[ ")[1].split(" ]")[0].split(", ")
        assert len(inv) == m.D


def test_write_run_after_array_run(tmp_path):
    """gbnuts_write_run on a finished array-API run writes the same files as the
    service with the same arguments."""
    from stan_gb300 import Model, sampler, services
    from stan_gb300.callbacks import CsvFiles
    ds = make_dataset("logistic", small=True, seed=6)
    m = Model.from_dataset(ds)
    C = 4
    rc = services.hmc_nuts_diag_e_adapt(m, C, csv=CsvFiles(tmp_path / "svc"), **KW)
    assert rc == 0
    kw = {k: v for k, v in KW.items()
          if k not in ("init", "init_inv_metric", "refresh")}
    r = sampler.run(m, num_chains=C, **kw)
    sampler.write_csv(m, r, CsvFiles(tmp_path / "arr"))
    for c in range(C):
        a = (tmp_path / f"svc_{c + 1}.csv").read_text()
        b = (tmp_path / f"arr_{c + 1}.csv").read_text()
        assert _strip_timing(a) == _strip_timing(b), c


def test_resume_service_given_stepsize_and_metric():
    """hmc_nuts_diag_e (hmc_nuts_diag_e.hpp:48-315, run_sampler.hpp): no
    adaptation, the given step size and inverse metric in every row and in
    the adaptation block run_sampler still writes, and the same draws as the
    array API's non-adaptive run with the same seed."""
    from stan_gb300 import Model, sampler, services
    from stan_gb300.callbacks import StreamWriter
    ds = make_dataset("logistic", small=True, seed=4)
    m = Model.from_dataset(ds)
    C, D = 2, m.D
    inv = np.linspace(0.5, 1.5, D)
    sample = [StreamWriter(io.StringIO()) for _ in range(C)]
    rc = services.hmc_nuts_diag_e(m, C, None, inv, 17, 1, 2.0, 50, 60, 1, False, 0, 0.25, 0.0,
                                  10, sample_writer=sample)
    assert rc == 0
    ref = sampler.run(m, num_chains=C, adapt=False, num_warmup=50, num_samples=60,
                      stepsize=0.25, random_seed=17, init_radius=2.0,
                      inv_metrics=np.tile(inv, (C, 1)))
    for c in range(C):
        lines = sample[c].stream.getvalue().split("\n")
        assert lines[1] == "# Adaptation terminated"
        assert lines[2] == "# Step size = 0.25"
        assert lines[3] == "# Diagonal elements of inverse mass matrix:"
        got = np.array([float(v) for v in lines[4][2:].split(", ")])
        assert np.allclose(got, inv, rtol=1e-6)
        rows = np.array([[float(v) for v in ln.split(",")] for ln in lines[5:5 + 60]])
        assert np.all(rows[:, 2] == 0.25)
        assert np.allclose(rows, ref.draws[c, :60], rtol=1e-5, atol=1e-6)


def test_interrupt_callback_stops_the_run():
    """The interrupt callback is polled between steps; a true answer stops
    every chain (generate_transitions.hpp:52, where the interface's interrupt
    throws): the service returns SOFTWARE, logs "Sampling interrupted." and
    the chains have written fewer rows than requested."""
    from stan_gb300 import Model, _lib, services
    from stan_gb300.callbacks import Logger, StreamWriter
    ds = make_dataset("logistic_100k", small=True, seed=5)
    m = Model.from_dataset(ds)
    C = 2
    polls = []

    class Stop:
        def __call__(self):
            polls.append(1)
            return len(polls) >= 3

    class Record(Logger):
        def __init__(self):
            self.lines = []

        def error(self, msg):
            self.lines.append(msg)

    log = Record()
    sample = [StreamWriter(io.StringIO()) for _ in range(C)]
    kw = dict(KW, num_warmup=2000, num_samples=2000)
    rc = services.hmc_nuts_diag_e_adapt(m, C, sample_writer=sample, interrupt=Stop(),
                                        logger=log, **kw)
    assert rc == _lib.SOFTWARE
    assert len(polls) >= 3
    assert "Sampling interrupted." in log.lines
    for w in sample:
        rows = [ln for ln in w.stream.getvalue().split("\n") if ln and not ln.startswith(("#", "lp__"))]
        assert len(rows) < 2000


def test_rows_reach_the_writers_during_the_run():
    """The host drain: rows go to the writer callbacks while the device run
    is still going (the interrupt callback, polled between step chunks on the
    calling thread, sees rows arrive), and the output equals the post-run
    protocol's (every row once, in order, the adaptation block between the
    warmup and sampling rows)."""
    from stan_gb300 import Model, _lib, sampler, services
    from stan_gb300.callbacks import StreamWriter
    ds = make_dataset("logistic_100k", small=True, seed=7)
    m = Model.from_dataset(ds)
    C = 2
    sample = [StreamWriter(io.StringIO()) for _ in range(C)]

    def n_rows():
        return sum(w.stream.getvalue().count("\n") for w in sample)

    seen = []

    class Watch:
        def __call__(self):
            seen.append(n_rows())
            return False

    kw = dict(KW, num_warmup=400, num_samples=400, save_warmup=1)
    rc = services.hmc_nuts_diag_e_adapt(m, C, sample_writer=sample, interrupt=Watch(), **kw)
    assert rc == _lib.OK
    assert len(seen) > 3
    assert any(0 < n < n_rows() for n in seen[:-1]), seen[:20]
    ref = sampler.run(m, num_chains=C, **{k: v for k, v in kw.items()
                                          if k not in ("init", "init_inv_metric", "refresh")})
    for c in range(C):
        lines = sample[c].stream.getvalue().split("\n")
        rows = [ln for ln in lines if ln and not ln.startswith(("#", "lp__"))]
        assert len(rows) == 800
        i_adapt = next(i for i, ln in enumerate(lines) if ln == "# Adaptation terminated")
        assert sum(1 for ln in lines[:i_adapt] if ln and not ln.startswith(("#", "lp__"))) == 400
        got = np.array([[float(v) for v in ln.split(",")] for ln in rows])
        assert np.allclose(got, ref.draws[c, :800], rtol=1e-5, atol=1e-6)
