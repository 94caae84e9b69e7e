"""Continuous batching on the GPU: requests arriving over time (Poisson),
half FP64 and half mixed, are admitted while others run, all finish at the
FP64 tolerance, and a request's result is bitwise the same when it is solved
alone as when it was served in the mix.

Residual checks use the oracle's double-double residual with the bounds of
the batch tests: 1.2e-10 for mixed requests (which certify 1e-10 on their
own double-double true residual), 1e-8 for FP64 requests (which stop on the
recursive residual like the reference's CG)."""
import time

import numpy as np
import pytest

from mpla_gb300 import synth
from mpla_gb300.serve import Request, Server, latency_stats, poisson_arrivals

pytestmark = pytest.mark.gpu


def make_request(k, arrival, rng, n=None):
    n = n or int(np.exp(rng.uniform(np.log(300), np.log(1500))))
    dim = 2 + int(rng.random() < 0.5)
    ell = float(rng.uniform(0.03, 0.2))
    r = int(rng.integers(1, 5))
    pts = synth.gauss_points(n, dim, 700 + k) / (np.sqrt(2.0) * ell)
    b = np.stack([synth.normal(700 + k, 900 + j, n) for j in range(r)], axis=1)
    return Request(arrival=arrival, rid=k, points=pts, b=b, nugget=1e-4, precision=k % 2)


def test_served_results_are_correct_and_match_solo_solves(gpu, orc):
    rng = np.random.default_rng(3)
    arrivals = poisson_arrivals(12.0, 1.0, rng)
    t0 = time.perf_counter()
    reqs = [make_request(k, t0 + a, rng) for k, a in enumerate(arrivals)]
    # one mixed and one FP64 request of the serving configuration's larger
    # sizes, arriving while the others run
    reqs += [make_request(len(reqs) + j, t0 + 0.5, rng, n=8192 + 96 * j) for j in range(2)]
    engines = {gpu.PREC_FP64: gpu.Batch(64), gpu.PREC_MIXED: gpu.Batch(64)}
    srv = Server(engines, slice_steps=32)
    for r in reqs:
        srv.submit(r)
    srv.serve(until=t0 + 1.0, drain_until=t0 + 300.0)
    assert len(srv.done) == len(reqs)
    stats = latency_stats(srv.done)
    assert stats["p99_s"] >= stats["p50_s"] > 0
    by_id = {c.rid: c for c in srv.done}
    for req in reqs:
        c = by_id[req.rid]
        op = orc.GaussOp(req.points, req.nugget)
        for j in range(req.b.shape[1]):
            assert c.infos[j].status == 0, (req.rid, req.precision, c.infos[j].as_dict())
            assert c.infos[j].final_res < 1e-10
            tol = 1.2e-10 if req.precision == 1 else 1e-8
            assert orc.true_relres_accurate(op, req.b[:, j], c.x[:, j]) < tol
    for req in reqs[:2]:
        solo = gpu.Batch(2)
        h = solo.add(req.points, req.nugget, req.b, precision=req.precision, iter_max=200000)
        solo.run()
        x, _ = solo.result(h, req.b.shape[0], req.b.shape[1])
        solo.close()
        assert np.array_equal(x, by_id[req.rid].x)
    for e in engines.values():
        e.close()
