"""Continuous-batching solve server on top of the batched CG engine.

Requests (a Gaussian system with 1..8 right-hand sides and a precision)
arrive over time.  The loop:
  1. admits every arrived request whose buffers fit in free device memory
     (the engine refuses otherwise; the request waits in the queue) into the
     engine of its precision,
  2. advances all admitted systems by a slice of CG iterations: each engine
     enqueues its graph replays on its own stream, then the loop waits for
     all of them, so FP64 and mixed work overlap on the device (FP64 on the
     FP64 pipe, mixed on the FP32 and SFU pipes) and a mixed request's
     steps never wait for the much slower FP64 steps,
  3. retires the systems whose right-hand sides have all finished, records
     their latency (arrival to result on the host), and frees their slots.
So requests arriving while others are on the GPU join at the next slice, and
slots and memory are reused as soon as systems finish.  The engine keeps
each system's arithmetic independent of the others, so a result is the same
alone and in the mix.
"""
from __future__ import annotations

import heapq
import math
import time
from dataclasses import dataclass, field

import numpy as np

NOMEM = 3  # MGB_ERR_NOMEM: admission refused, retry when memory frees


@dataclass(order=True)
class Request:
    arrival: float
    rid: int = field(compare=False)
    points: np.ndarray = field(compare=False, repr=False)   # dim x n, scaled
    b: np.ndarray = field(compare=False, repr=False)        # n x r
    nugget: float = field(compare=False, default=1e-4)
    precision: int = field(compare=False, default=1)
    eps: float = field(compare=False, default=1e-10)


@dataclass
class Completion:
    rid: int
    n: int
    nrhs: int
    precision: int
    arrival: float
    admitted: float
    finished: float
    x: np.ndarray = field(repr=False)
    infos: list = field(repr=False)

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class Server:
    """Drives engines with the Batch interface (add / run_async / wait /
    finished / result): one engine for every precision, or one engine for
    all (``engine`` may be a single engine or a dict precision -> engine)."""

    def __init__(self, engine, slice_steps: int = 64, reserve_bytes: int = 2 << 30, iter_max: int = 200000,
                 clock=time.perf_counter, sleep=time.sleep):
        self.engines = engine if isinstance(engine, dict) else None
        self.engine = None if self.engines else engine
        self.slice_steps = slice_steps
        self.reserve_bytes = reserve_bytes
        self.iter_max = iter_max
        self.clock = clock
        self.sleep = sleep
        self.queue: list[Request] = []       # submitted, not yet admitted (ordered by arrival)
        self.running: dict[tuple, tuple] = {}  # (engine key, handle) -> (request, admitted time)
        self.done: list[Completion] = []
        self.refusals = 0
        self.inflight: set = set()           # engines with a slice enqueued

    def _engine_of(self, precision: int):
        if self.engines is None:
            return 0, self.engine
        return precision, self.engines[precision]

    def _all_engines(self):
        return [(0, self.engine)] if self.engines is None else list(self.engines.items())

    def submit(self, req: Request) -> None:
        heapq.heappush(self.queue, req)

    def _admit(self, now: float) -> None:
        waiting = []
        while self.queue and self.queue[0].arrival <= now:
            req = heapq.heappop(self.queue)
            key, eng = self._engine_of(req.precision)
            try:
                h = eng.add(req.points, req.nugget, req.b, precision=req.precision, eps=req.eps,
                            iter_max=self.iter_max, reserve_bytes=self.reserve_bytes)
            except Exception as e:  # noqa: BLE001 - only a memory/slot refusal is retried
                if getattr(e, "status", None) == NOMEM:
                    self.refusals += 1
                    waiting.append(req)
                    continue
                raise
            self.running[(key, h)] = (req, self.clock())
        for r in waiting:
            heapq.heappush(self.queue, r)

    def _retire(self, key, eng) -> None:
        for h in eng.finished():
            if (key, h) not in self.running:
                continue
            req, admitted = self.running.pop((key, h))
            n, r = req.b.shape[0], req.b.shape[1]
            x, infos = eng.result(h, n, r, release=True)
            self.done.append(Completion(req.rid, n, r, req.precision, req.arrival, admitted, self.clock(), x, infos))

    def step(self) -> int:
        """One scheduling round; returns the number of running systems.
        Every engine with running systems works on its own slice: an engine
        whose last slice has finished is retired and given the next one at
        once, while the others keep running (so a fast engine never waits
        for a slow one)."""
        self._admit(self.clock())
        started = False
        for key, eng in self._all_engines():
            busy = any(k == key for k, _ in self.running)
            if key in self.inflight:
                if not eng.ready():
                    continue
                self.inflight.discard(key)
                eng.wait()
                self._retire(key, eng)
                busy = any(k == key for k, _ in self.running)
            if busy:
                eng.run_async(self.slice_steps)
                self.inflight.add(key)
                started = True
        if not started and self.inflight:
            self.sleep(0.0002)
        return len(self.running)

    def drain(self) -> None:
        """Wait for every slice in flight (their systems stay admitted)."""
        for key, eng in self._all_engines():
            if key in self.inflight:
                eng.wait()
                self._retire(key, eng)
        self.inflight.clear()

    def serve(self, until: float, drain_until: float | None = None) -> None:
        """Run rounds until every submitted request has finished, or the clock
        passes `drain_until` (requests still running then stay unfinished).
        `until` is the end of the arrival window: the loop never stops before
        it while requests may still arrive."""
        drain_until = drain_until if drain_until is not None else math.inf
        while True:
            now = self.clock()
            if now > drain_until:
                self.drain()
                break
            if not self.running and not self.queue:
                if now >= until:
                    break
                self.sleep(min(0.005, until - now))
                continue
            if not self.running and self.queue and self.queue[0].arrival > now:
                self.sleep(min(0.005, self.queue[0].arrival - now))
                continue
            self.step()


def poisson_arrivals(rate: float, duration: float, rng: np.random.Generator) -> list[float]:
    """Arrival times of a Poisson process of `rate` per second over [0, duration)."""
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            return out
        out.append(t)


def latency_stats(done: list[Completion]) -> dict:
    if not done:
        return {"completed": 0}
    lat = np.array([c.latency for c in done])
    span = max(c.finished for c in done) - min(c.arrival for c in done)
    return {"completed": len(done), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "solves_per_s": len(done) / span if span > 0 else None}
