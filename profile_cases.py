"""Small, self-contained kernel workloads for Nsight Compute captures.

Each case launches one hot kernel a few times on inputs sized for a capture
that ends by itself (a few hundred MB on the device at most):

  python profile_cases.py dgemv       # dense dgemv, n = 4096 (134 MB matrix)
  python profile_cases.py gauss_f64   # FP64 Gaussian matvec, n = 16384, d = 2
  python profile_cases.py gauss_mixed # FP32/SFU Gaussian matvec, n = 65536, d = 2
  python profile_cases.py mixed_cg    # 300 mixed-CG iterations, n = 16384, d = 2
  python profile_cases.py batch       # 100 steps of a 24-system batch (n <= 4096)
  python profile_cases.py batch128    # 16 timed steps of 128 batch systems (n <= 16384)
  python profile_cases.py batch128_solve  # the same 128 systems solved to 1e-10
  python profile_cases.py mixed_c3    # full mixed solve, n = 131072, d = 3, l = 0.08
  python profile_cases.py batch_trace # all 512 batch systems to 1e-10, per-replay times
  python profile_cases.py batch512    # 16 timed steps of all 512 batch systems
  python profile_cases.py serving_sweep  # the serving configuration, 3 rates x ~32 requests
  python profile_cases.py serving_sweep 0.2,0.4 32  # chosen rates and requests per rate
  python profile_cases.py all

Prints the CUDA-event time per launch of each case.  The cases that write a
record (batch_trace, serving_sweep) put it in the folder named by the
environment variable PROFILE_OUT (default: profile_out).
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

import mpla_gb300 as mg
from mpla_gb300 import synth


def case_dgemv(reps=3):
    n = 4096
    rng = np.random.default_rng(0)
    A = mg.DeviceArray.from_numpy(rng.uniform(-1, 1, n * n))
    x = mg.DeviceArray.from_numpy(rng.uniform(-1, 1, n))
    y = mg.DeviceArray(n)
    ms = mg.time_dgemv(n, A.ptr, x.ptr, y.ptr, reps=reps)
    print(f"dgemv n={n}: {ms:.4f} ms/launch, {(8.0 * n * n + 16 * n) / ms / 1e6:.1f} GB/s")


def _gauss(n, dim, ell, precision, reps):
    prob = synth.gauss_problem(n, dim, ell, 1e-4, seed=0)
    dp = mg.GaussPoints(prob.scaled())
    x = mg.DeviceArray.from_numpy(np.random.default_rng(1).standard_normal(n))
    y = mg.DeviceArray(n)
    ms = mg.time_gauss_matvec(dp, 1e-4, precision, x.ptr, y.ptr, reps=reps)
    name = "fp64" if precision == mg.PREC_FP64 else "mixed"
    print(f"gauss_{name} n={n} d={dim}: {ms:.4f} ms/launch, {float(n) * n / ms / 1e6:.2f} Gentries/s")


def case_gauss_f64(reps=2):
    _gauss(16384, 2, 0.05, mg.PREC_FP64, reps)


def case_gauss_mixed(reps=20):
    _gauss(65536, 2, 0.05, mg.PREC_MIXED, reps)


def case_mixed_cg(iters=300):
    """The headline solve's kernel mix (FP32 matvec, fused vector kernels,
    FP64 true residuals) on the n = 16384 member of its family, capped at
    `iters` iterations so that a launch list stays short."""
    n = 16384
    prob = synth.gauss_problem(n, 2, 0.05, 1e-4, seed=0)
    dp = mg.GaussPoints(prob.scaled())
    b = mg.DeviceArray.from_numpy(prob.b)
    x = mg.DeviceArray(n)
    x.zero()
    info = mg.cg_gauss(dp, 1e-4, b.ptr, x.ptr, iter_max=iters, eps=1e-10, precision=mg.PREC_MIXED)
    print(f"mixed_cg n={n}: {info.iterations} iterations, relres {info.true_relres:.3e}")


def case_batch(steps=100):
    """The batched engine's kernel mix: 24 systems of the batch workload with
    n <= 4096, advanced by `steps` iterations."""
    spec = synth.batch_spec(24, n_hi=4096)
    batch = mg.Batch(24)
    for k in range(24):
        g = synth.batch_system(spec, k)
        batch.add(g.scaled(), g.nugget, g.b, precision=mg.PREC_MIXED)
    active = batch.run(max_steps=steps)
    print(f"batch: {active} of 24 systems still running after {steps} steps")
    batch.close()


def case_batch128(steps=16):
    """The batch workload's step at its busiest: the first 128 of the 512
    systems (n log-uniform in [256, 16384]) admitted together, one warm-up
    replay, then `steps` timed iterations (host wall time around whole graph
    replays, which end with a device synchronisation)."""
    import time

    spec = synth.batch_spec(512)
    batch = mg.Batch(128)
    for k in range(128):
        g = synth.batch_system(spec, k)
        batch.add(g.scaled(), g.nugget, g.b, precision=mg.PREC_MIXED)
    batch.run(max_steps=8)
    t0 = time.perf_counter()
    active = batch.run(max_steps=steps)
    ms = (time.perf_counter() - t0) * 1e3 / steps
    rpt, tune = batch.tuning()
    print(f"batch128: {ms:.3f} ms per step, {active} of 128 systems running, rows per thread {rpt}, "
          f"FP32 matvec ms per class (2 / 4 rows per thread) {[[round(t, 4) for t in c[1:]] for c in tune]}")
    batch.close()


def case_batch512(steps=16):
    """All 512 batch systems admitted together: one warm-up replay, then
    `steps` iterations (the busiest step of the batch workload, for launch
    lists)."""
    import time

    spec = synth.batch_spec(512)
    batch = mg.Batch(512)
    for k in range(512):
        g = synth.batch_system(spec, k)
        batch.add(g.scaled(), g.nugget, g.b, precision=mg.PREC_MIXED, iter_max=300000)
    batch.run(max_steps=8)
    t0 = time.perf_counter()
    active = batch.run(max_steps=steps)
    ms = (time.perf_counter() - t0) * 1e3 / steps
    print(f"batch512: {ms:.3f} ms per step, {active} of 512 systems running")
    batch.close()


def case_batch128_solve():
    """The same 128 systems run to relres 1e-10: wall time, and per system
    (slowest ten) the iterations and FP64 true residuals of its slowest
    right-hand side."""
    import time

    spec = synth.batch_spec(512)
    batch = mg.Batch(128)
    handles = []
    for k in range(128):
        g = synth.batch_system(spec, k)
        handles.append((k, batch.add(g.scaled(), g.nugget, g.b, precision=mg.PREC_MIXED)))
    t0 = time.perf_counter()
    active = batch.run()
    sec = time.perf_counter() - t0
    rows = []
    for k, h in handles:
        n, r = int(spec.n[k]), int(spec.nrhs[k])
        _, infos = batch.result(h, n, r)
        rows.append((max(i.iterations for i in infos), max(i.fp64_matvecs for i in infos),
                      sum(i.fp64_matvecs for i in infos), n, int(spec.dim[k]), float(spec.ell[k]), r))
    rows.sort(reverse=True)
    print(f"batch128_solve: {sec:.2f} s, {active} unfinished, {sum(x[2] for x in rows)} FP64 true residuals "
          f"over all right-hand sides")
    for it, rep, _, n, d, ell, r in rows[:10]:
        print(f"  n={n} d={d} l={ell:.3f} nrhs={r}: {it} iterations, {rep} FP64 true residuals")
    batch.close()


OUT_DIR = Path(os.environ.get("PROFILE_OUT", "profile_out"))


def case_batch_trace(count=512, out=None):
    """All `count` systems of the batch workload admitted together and run to
    relres 1e-10 one graph replay (8 steps) at a time: per replay the host
    wall time and the systems still running (a CSV), then the total, the
    replay-time distribution and the slowest systems."""
    import time

    spec = synth.batch_spec(512)
    batch = mg.Batch(count)
    handles = []
    for k in range(count):
        g = synth.batch_system(spec, k)
        handles.append((k, batch.add(g.scaled(), g.nugget, g.b, precision=mg.PREC_MIXED, iter_max=300000)))
    batch.run(max_steps=0)
    rows = []
    t0 = time.perf_counter()
    active = count
    while active > 0:
        t = time.perf_counter()
        active = batch.run(max_steps=8)
        rows.append((len(rows), time.perf_counter() - t, active))
    sec = time.perf_counter() - t0
    out = Path(out) if out is not None else OUT_DIR / "batch_trace.csv"
    out.parent.mkdir(parents=True, exist_ok=True)
    with open(out, "w") as f:
        f.write("replay,seconds,active\n")
        for r in rows:
            f.write(f"{r[0]},{r[1]:.6f},{r[2]}\n")
    dts = np.array([r[1] for r in rows])
    res = []
    for k, h in handles:
        n, r = int(spec.n[k]), int(spec.nrhs[k])
        _, infos = batch.result(h, n, r)
        res.append((max(i.iterations for i in infos), sum(i.fp64_matvecs for i in infos), n, int(spec.dim[k]),
                    float(spec.ell[k]), r))
    res.sort(reverse=True)
    print(f"batch_trace {count}: {sec:.2f} s over {len(rows)} replays; replay ms p50 {np.median(dts) * 1e3:.2f}, "
          f"p90 {np.percentile(dts, 90) * 1e3:.2f}, max {dts.max() * 1e3:.2f}; the slowest 10 % of replays take "
          f"{np.sort(dts)[-max(1, len(dts) // 10):].sum():.2f} s; FP64 true residuals {sum(x[1] for x in res)}")
    for it, rep, n, d, ell, r in res[:10]:
        print(f"  n={n} d={d} l={ell:.3f} nrhs={r}: {it} iterations, {rep} FP64 true residuals (all lanes)")
    batch.close()


def case_serving_sweep(rates=(0.1, 0.2, 0.4), per_rate=32, out=None):
    """The serving configuration as specified: per arrival rate, Poisson
    arrivals of about `per_rate` requests, n log-uniform in [1024, 32768],
    d in {2,3}, l ~ U[0.03, 0.2], 1-4 N(0,1) right-hand sides, half FP64,
    relres 1e-10, drained until every request has finished; p50/p99 latency
    and solves/s per rate and per precision (JSON)."""
    import json
    import time

    from mpla_gb300.serve import Request, Server, latency_stats

    res = []
    for q, rate in enumerate(rates):
        window = per_rate / rate
        reqs = synth.serving_requests(rate, window, seed=100 + q)
        engines = {mg.PREC_FP64: mg.Batch(128), mg.PREC_MIXED: mg.Batch(128)}
        srv = Server(engines, slice_steps=64)
        t0 = time.perf_counter()
        for a, k, pts, b, prec in reqs:
            srv.submit(Request(arrival=t0 + a, rid=k, points=pts, b=b, precision=prec))
        srv.serve(until=t0 + window)
        st = latency_stats(srv.done)
        for p, name in ((0, "fp64"), (1, "mixed")):
            lat = [c.latency for c in srv.done if c.precision == p]
            if lat:
                st[name] = {"completed": len(lat), "p50_s": float(np.percentile(lat, 50)),
                            "p99_s": float(np.percentile(lat, 99)), "n_max": max(c.n for c in srv.done if c.precision == p)}
        st.update({"rate_per_s": rate, "window_s": window, "submitted": len(reqs),
                   "unfinished": len(reqs) - len(srv.done),
                   "all_converged": all(int(i.status) == 0 for c in srv.done for i in c.infos),
                   "wall_s": time.perf_counter() - t0})
        for e in engines.values():
            e.close()
        print(json.dumps(st), flush=True)
        res.append(st)
    out = Path(out) if out is not None else OUT_DIR / "serving_sweep.json"
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text(json.dumps(res, indent=1))


def case_mixed_c3():
    """The mixed-precision configuration: n = 131072 points U[0,1]^3, l = 0.08,
    nugget 1e-4, b = sin(2 pi x1) cos(2 pi x2), solved to relres 1e-10."""
    import time

    n = 131072
    prob = synth.config_gauss_mixed(0)
    dp = mg.GaussPoints(prob.scaled())
    b = mg.DeviceArray.from_numpy(prob.b)
    x = mg.DeviceArray(n)
    x.zero()
    mv_ms = mg.time_gauss_matvec(dp, 1e-4, mg.PREC_MIXED, b.ptr, x.ptr, reps=5)
    evaluated = mg.gauss_mixed_work(dp)
    x.zero()
    t0 = time.perf_counter()
    info = mg.cg_gauss(dp, 1e-4, b.ptr, x.ptr, iter_max=200000, eps=1e-10, precision=mg.PREC_MIXED)
    sec = time.perf_counter() - t0
    print(f"mixed_c3 n={n} d=3: matvec {mv_ms:.3f} ms ({evaluated} evaluated entries), {info.iterations} iterations, "
          f"{info.fp64_matvecs} FP64 true residuals, {sec:.2f} s, true relres {info.true_relres:.3e}, "
          f"status {info.status}")


CASES = {"dgemv": case_dgemv, "gauss_f64": case_gauss_f64, "gauss_mixed": case_gauss_mixed,
         "mixed_cg": case_mixed_cg, "batch": case_batch, "batch128": case_batch128,
         "batch128_solve": case_batch128_solve, "mixed_c3": case_mixed_c3, "batch_trace": case_batch_trace,
         "batch512": case_batch512, "serving_sweep": case_serving_sweep}


def main(argv):
    mg.init(0)
    long_cases = ("mixed_c3", "batch128", "batch128_solve", "batch_trace", "batch512", "serving_sweep")
    if argv and argv[0] == "serving_sweep" and len(argv) > 1:
        # serving_sweep RATES [PER_RATE]: e.g. serving_sweep 0.2,0.4 24
        rates = tuple(float(r) for r in argv[1].split(","))
        per_rate = int(argv[2]) if len(argv) > 2 else 32
        case_serving_sweep(rates=rates, per_rate=per_rate,
                           out=OUT_DIR / f"serving_sweep_{argv[1].replace(',', '_')}.json")
        mg.synchronize()
        return
    names = [k for k in CASES if k not in long_cases] if (not argv or argv[0] == "all") else argv
    for name in names:
        CASES[name]()
    mg.synchronize()


if __name__ == "__main__":
    main(sys.argv[1:])
