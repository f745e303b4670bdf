"""Host logic of the serving loop (no GPU): arrivals, latency statistics and
the submit / step / retire bookkeeping of serve() against a fake pool."""
import numpy as np

from stan_gb300 import serving


def test_poisson_arrivals_rate_and_order():
    t = serving.poisson_arrivals(rate=50.0, n=20000, seed=1)
    assert np.all(np.diff(t) > 0)
    assert abs(len(t) / t[-1] - 50.0) < 1.5
    assert np.array_equal(t, serving.poisson_arrivals(rate=50.0, n=20000, seed=1))


def test_latency_stats():
    s = serving.latency_stats(np.arange(1, 101, dtype=float))
    assert s["n"] == 100 and s["p50"] == 50.5 and abs(s["p99"] - 99.01) < 1e-9
    assert s["mean"] == 50.5 and s["max"] == 100
    assert serving.latency_stats([])["p50"] is None


class FakePool:
    """Each fit needs `work` steps once admitted; at most `slots` run at once."""

    def __init__(self, work, slots):
        self.work, self.slots = work, slots
        self.queue, self.running, self.left, self.done = [], [], {}, set()
        self.steps = 0
        self.next_id = 1
        self.submitted = []

    def submit(self, ds, **kw):
        fid = self.next_id
        self.next_id += 1
        self.queue.append(fid)
        self.submitted.append((ds, kw))
        return fid

    def step(self, n):
        while self.queue and len(self.running) < self.slots:
            fid = self.queue.pop(0)
            self.running.append(fid)
            self.left[fid] = self.work
        self.steps += n
        for fid in list(self.running):
            self.left[fid] -= n
            if self.left[fid] <= 0:
                self.running.remove(fid)
                self.done.add(fid)
        return len(self.running), len(self.queue)

    def status(self, fid):
        return (serving.DONE, 0) if fid in self.done else (serving.RUNNING, 0)

    def pop(self, fid):
        self.done.discard(fid)
        return ("result", fid)

    def stats(self):
        return self.steps, 0


class FakeClock:
    def __init__(self, pool, step_s):
        self.t, self.pool, self.step_s, self.last = 0.0, pool, step_s, 0

    def __call__(self):
        # time advances with the steps the pool has run
        self.t += (self.pool.steps - self.last) * self.step_s
        self.last = self.pool.steps
        return self.t


def test_serve_bookkeeping(monkeypatch):
    pool = FakePool(work=10, slots=2)
    clock = FakeClock(pool, step_s=0.01)
    slept = []

    def fake_sleep(s):
        slept.append(s)
        clock.t += s

    monkeypatch.setattr(serving.time, "sleep", fake_sleep)
    arrivals = np.array([0.0, 0.0, 0.0, 1.0])
    got = []
    rep = serving.serve(pool, ["a", "b", "c", "d"], arrivals, steps_per_call=5,
                        run_kwargs={"num_chains": 2}, on_done=lambda i, r: got.append(i),
                        clock=clock)
    assert sorted(got) == [0, 1, 2, 3]
    # two slots: a, b finish after 10 steps (0.1 s); c is admitted then and
    # finishes at 0.2 s; d arrives at 1.0 s (the loop sleeps) and takes 0.1 s
    assert np.allclose(rep.latencies, [0.1, 0.1, 0.2, 0.1])
    assert rep.max_running == 2
    assert slept and all(s <= 0.05 + 1e-12 for s in slept)
    assert [d for d, _ in pool.submitted] == ["a", "b", "c", "d"]
    assert all(kw == {"num_chains": 2} for _, kw in pool.submitted)
