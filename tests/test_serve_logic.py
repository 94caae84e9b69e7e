"""Host logic of the continuous-batching server, with a fake engine (CPU).

The fake engine finishes a system after a number of steps proportional to
its size, refuses admission above a memory budget, and reports results; the
server must admit requests as they arrive, keep refused ones queued until
memory frees, overlap running systems, retire finished ones and record
their latency.
"""
import numpy as np
import pytest

from mpla_gb300.serve import Request, Server, latency_stats, poisson_arrivals


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-6)


class NoMemory(Exception):
    status = 3


class BadInput(Exception):
    status = 2


class FakeEngine:
    def __init__(self, clock, budget):
        self.clock = clock
        self.budget = budget
        self.used = 0
        self.left = {}
        self.sizes = {}
        self.next = 0
        self.max_concurrent = 0

    def add(self, points, nugget, b, precision, eps, iter_max, reserve_bytes):
        n = b.shape[0]
        if n == 0:
            raise BadInput()
        if self.used + n > self.budget:
            raise NoMemory()
        h = self.next
        self.next += 1
        self.used += n
        self.sizes[h] = n
        self.left[h] = n // 100
        self.max_concurrent = max(self.max_concurrent, len(self.left))
        return h

    def run(self, max_steps):
        self.clock.t += 0.01
        for h in list(self.left):
            self.left[h] -= 1
        return sum(1 for v in self.left.values() if v > 0)

    def run_async(self, max_steps):
        self.pending = max_steps

    def wait(self):
        self.waits = getattr(self, "waits", 0) + 1
        return self.run(self.pending)

    def ready(self):
        return True

    def finished(self):
        return [h for h, v in self.left.items() if v <= 0]

    def result(self, h, n, r, release):
        del self.left[h]
        self.used -= self.sizes.pop(h)
        return np.zeros((n, r)), [None] * r


def test_server_admits_overlaps_and_retires():
    clock = FakeClock()
    eng = FakeEngine(clock, budget=5000)
    srv = Server(eng, clock=clock, sleep=clock.sleep)
    rng = np.random.default_rng(0)
    arrivals = poisson_arrivals(20.0, 2.0, rng)
    for k, t in enumerate(arrivals):
        n = int(rng.integers(200, 3000))
        srv.submit(Request(arrival=t, rid=k, points=np.zeros((2, n)), b=np.zeros((n, 1))))
    srv.serve(until=2.0, drain_until=100.0)
    assert len(srv.done) == len(arrivals)
    assert eng.max_concurrent > 1             # work of several requests overlapped
    assert srv.refusals > 0                   # the memory budget forced waiting
    assert eng.used == 0                      # every slot released
    for c in srv.done:
        assert c.finished >= c.admitted >= c.arrival
    st = latency_stats(srv.done)
    assert st["completed"] == len(arrivals) and st["p99_s"] >= st["p50_s"] > 0


def test_server_waits_for_late_arrivals():
    clock = FakeClock()
    eng = FakeEngine(clock, budget=10**9)
    srv = Server(eng, clock=clock, sleep=clock.sleep)
    srv.submit(Request(arrival=5.0, rid=0, points=np.zeros((2, 500)), b=np.zeros((500, 1))))
    srv.serve(until=6.0, drain_until=50.0)
    assert len(srv.done) == 1 and srv.done[0].admitted >= 5.0


def test_other_admission_errors_propagate():
    clock = FakeClock()
    srv = Server(FakeEngine(clock, budget=10), clock=clock, sleep=clock.sleep)
    srv.submit(Request(arrival=0.0, rid=0, points=np.zeros((2, 0)), b=np.zeros((0, 1))))
    with pytest.raises(BadInput):
        srv.serve(until=1.0, drain_until=2.0)


def test_poisson_arrivals_rate():
    rng = np.random.default_rng(1)
    a = poisson_arrivals(50.0, 100.0, rng)
    assert abs(len(a) / 100.0 - 50.0) < 3.0
    assert all(x < y for x, y in zip(a, a[1:]))


def test_server_keeps_precisions_in_their_own_engines():
    """FP64 and mixed requests go to separate engines, both of which advance
    in every round (their device work overlaps); each engine's handles are
    its own."""
    clock = FakeClock()
    engines = {0: FakeEngine(clock, budget=10**9), 1: FakeEngine(clock, budget=10**9)}
    srv = Server(engines, clock=clock, sleep=clock.sleep)
    for k in range(6):
        n = 300 + 100 * k
        srv.submit(Request(arrival=0.01 * k, rid=k, points=np.zeros((2, n)), b=np.zeros((n, 1)), precision=k % 2))
    srv.serve(until=0.1, drain_until=100.0)
    assert sorted(c.rid for c in srv.done) == list(range(6))
    assert all(e.used == 0 and e.next == 3 for e in engines.values())
    assert all(c.precision == c.rid % 2 for c in srv.done)
    assert engines[0].waits > 1 and engines[1].waits > 1


class SlowEngine(FakeEngine):
    """Finishes a slice only every `period`-th time it is asked."""

    def __init__(self, clock, budget, period):
        super().__init__(clock, budget)
        self.period = period
        self.asked = 0

    def ready(self):
        self.asked += 1
        return self.asked % self.period == 0


def test_fast_engine_does_not_wait_for_slow_engine():
    clock = FakeClock()
    engines = {0: SlowEngine(clock, 10**9, period=50), 1: FakeEngine(clock, 10**9)}
    srv = Server(engines, clock=clock, sleep=clock.sleep)
    srv.submit(Request(arrival=0.0, rid=0, points=np.zeros((2, 5000)), b=np.zeros((5000, 1)), precision=0))
    srv.submit(Request(arrival=0.0, rid=1, points=np.zeros((2, 300)), b=np.zeros((300, 1)), precision=1))
    srv.serve(until=0.0, drain_until=1000.0)
    fin = {c.rid: c.finished for c in srv.done}
    assert fin[1] < fin[0]
    # the small request needed 3 slices of its engine and finished while the
    # slow engine had completed only a few of its 50
    assert engines[1].waits == 3
