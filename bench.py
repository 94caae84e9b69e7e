#!/usr/bin/env python3
"""Benchmark of the GB300 MPLA hot path: kernel-CG solves/s at relres 1e-10.

Workload (one "step" = one full solve): the Gaussian kernel system of the
matrix-free FP64 configuration -- n = 65536 points uniform in [0,1]^2,
K_ij = exp(-|x_i - x_j|^2 / (2 * 0.05^2)) + 1e-4 delta_ij,
b_i = sin(2 pi x_i1) cos(2 pi x_i2), x0 = 0 -- solved to a relative
residual of 1e-10 with the mixed-precision CG (FP32/SFU matvec, FP64
vectors, dots, scalars and FP64 true-residual replacement).  The plain FP64
CG on the same system is timed on a bounded sample of iterations (a full
FP64 solve takes tens of minutes on GB300's FP64 pipe) and reported beside it.

  value     solves/s with points, b and x resident in HBM (device-timed)
  e2e       the same solve through mgb_cg_gauss_host from pinned host buffers
            (host->device copies of points, b, x0 and the copy of x back
            inside the timed region)
  dense     the dense configuration: FP64 CG solves/s and the dgemv, n = 4096
  mixed_c3  the mixed configuration's matvec (n = 131072, d = 3) against the
            SFU peak
  batched   all 512 systems of the batch configuration to relres 1e-10, with
            plain FP64 extrapolated from per-step times and an iteration ratio
  serving   continuous batching at three arrival rates (requests up to
            n = 8192; profile_cases.py serving_sweep runs the full sizes)

``--impl reference`` times the reference MPLA (compiled from its sources into
oracle/_ref by oracle/build_ref.py) on the same system through its own API:
FP64 CG with the Gaussian system_assembler plugin, on a bounded sample of
iterations, and the dense configuration (mpla_dgemv, its cublasDgemv call,
the dense CG).  Under torchrun every rank runs its own replica (the path does
not shard); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "kernel-CG solves/s & p99 latency at relres 1e-10: mixed vs plain FP64, 1 GB300"
N_FULL, DIM, ELL, NUGGET, EPS = 65536, 2, 0.05, 1e-4, 1e-10
L2_FLUSH_BYTES = 512 << 20
# FP64 CG iterations of the full n = 65536 solve, measured once on GB300 with
# mgb_cg_gauss (plain FP64, 1163.6 s); used to turn sampled FP64 and
# reference iterations into solves/s.  Other sizes fall back to the mixed
# count (a lower bound on the FP64 count for this family).
FP64_ITERATIONS_N65536 = 18958
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the FP32 group kernel at n = 65536, d = 2, from one ncu capture of that
# launch (points, slots and x stay in L2).  Not measured per run: ncu is not
# run inside the benchmark.
GROUP_KERNEL_DRAM_BYTES_N65536 = 1.441024e6 + 0.295936e6
SFU_EX2_PER_CLK_SM = 32.0
SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi sampling during the timed region (every 200 ms)."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={SMI_FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def aggregate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput: units processed by all ranks / max time."""
    return units_per_rank * world / seconds_max


# -------------------------------------------------------------- CPU baseline
_T0 = time.perf_counter()


def progress(msg: str) -> None:
    print(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)


def measured_peak(key: str):
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())[key])
    except (OSError, KeyError, ValueError, TypeError):
        return None


def fp64_iterations(args, fallback: int) -> int:
    if args.fp64_iterations:
        return args.fp64_iterations
    return FP64_ITERATIONS_N65536 if args.n == N_FULL else fallback


def cpu_baseline(points_scaled: np.ndarray, nugget: float, iterations: int, budget_s: float = 10.0) -> dict:
    """FP64 oracle matvec rows on the host cores for about budget_s seconds;
    solves/s = entries/s / (n^2 * iterations)."""
    import oracle

    op = oracle.GaussOp(points_scaled, nugget)
    n = op.n
    x = np.ones(n)
    rows = 256
    done_entries = 0
    t0 = time.perf_counter()
    r0 = 0
    while time.perf_counter() - t0 < budget_s:
        nr = min(rows, n - r0)
        op.matvec(x, rows=nr, cols=n, roff=r0, coff=0)
        done_entries += nr * n
        r0 = (r0 + nr) % n
    dt = time.perf_counter() - t0
    eps = done_entries / dt
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": eps / (float(n) * n * iterations), "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"{done_entries / 1e9:.2f}e9 FP64 kernel entries of the C oracle matvec ({dt:.1f} s, "
                      f"OpenMP over rows), scaled by n^2 x {iterations} CG iterations per solve",
            "entries_per_s": eps}


# ------------------------------------------------------- secondary sections
def bench_mixed_c3(mg, stream, sms: int, sm_mhz: float) -> dict:
    """The mixed-precision configuration's operator (n = 131072 points
    U[0,1]^3, l = 0.08, nugget 1e-4): time of one mixed matvec (20 launches,
    CUDA events) and its rate against the SFU peak.  A full solve of this
    system takes about a minute; its record is a profile case
    (profile_cases.py mixed_c3), not a bench step."""
    from mpla_gb300 import synth

    prob = synth.config_gauss_mixed(0)
    n = prob.n
    dp = mg.GaussPoints(prob.scaled())
    dxr = mg.DeviceArray.from_numpy(np.random.default_rng(0).standard_normal(n))
    dy = mg.DeviceArray(n)
    ms = mg.time_gauss_matvec(dp, NUGGET, mg.PREC_MIXED, dxr.ptr, dy.ptr, reps=20, stream=stream.cuda_stream)
    evaluated = float(mg.gauss_mixed_work(dp))
    rate = evaluated / (ms * 1e-3)
    peak = SFU_EX2_PER_CLK_SM * sms * sm_mhz * 1e6
    return {"workload": "mixed matvec, n=131072, points U[0,1]^3, l=0.08, nugget 1e-4",
            "matvec_ms": ms, "evaluated_per_launch": evaluated, "ex2_per_s": rate, "sfu_frac": rate / peak,
            "algorithmic_entries_per_s": float(n) * n / (ms * 1e-3)}


def bench_dense(mg, torch, stream, hbm_peak_gbs: float | None) -> dict:
    """Dense FP64 CG (n = 4096, A = M^T M / n + I, b = 1, relres 1e-10) and
    the dgemv on the same A."""
    from mpla_gb300 import synth

    n = 4096
    A, b, _ = synth.config_dense(0)
    dA = mg.DeviceArray.from_numpy(np.asfortranarray(A).ravel(order="F"))
    db = mg.DeviceArray.from_numpy(b)
    dy = mg.DeviceArray(n)
    x_t = torch.zeros(n, dtype=torch.float64, device="cuda")  # zeroed in order on the bench stream
    torch.cuda.synchronize()
    sp = stream.cuda_stream
    reps = 20

    def solve():
        with torch.cuda.stream(stream):
            x_t.zero_()
            return mg.cg_dense(n, dA.ptr, db.ptr, x_t.data_ptr(), iter_max=1000, eps=EPS, stream=sp)

    for _ in range(3):
        info = solve()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        info = solve()
    e1.record(stream)
    torch.cuda.synchronize()
    solve_ms = e0.elapsed_time(e1) / reps
    gemv_ms = mg.time_dgemv(n, dA.ptr, db.ptr, dy.ptr, reps=50, stream=sp)
    gemv_bytes = 8.0 * n * n + 16.0 * n
    gbs = gemv_bytes / (gemv_ms * 1e-3) / 1e9
    return {"workload": "dense FP64 CG, n=4096, A = M^T M/n + I (M ~ U[-1,1], seed 0), b = 1, relres 1e-10",
            "solves_per_s": 1e3 / solve_ms, "ms_per_solve": solve_ms, "iterations": int(info.iterations),
            "converged": int(info.status) == 0,
            "dgemv": {"ms": gemv_ms, "achieved_gbs": gbs, "peak_gbs": hbm_peak_gbs,
                      "frac": gbs / hbm_peak_gbs if hbm_peak_gbs else None,
                      "bytes": gemv_bytes, "note": "A is 128 MiB: back-to-back launches partly hit L2"}}


def bench_batched(mg, count: int) -> dict:
    """Batched mixed-precision solves: `count` Gaussian systems of the batch
    workload (n log-uniform in [256, 16384], d in {2,3}, l ~ U[0.03, 0.2],
    nugget 1e-4, 1-8 N(0,1) right-hand sides; 512 is the whole workload),
    admitted together from host buffers and run to relres 1e-10.

    Plain FP64 on the same systems is not run to the end (it would take tens
    of minutes on GB300's FP64 pipe).  Its batch time is extrapolated from
    three measurements: the mixed batch's wall time, the FP64 / mixed time
    per step with every system running (16 steps each), and the FP64 / mixed
    iteration ratio of the slowest right-hand side, measured by solving a
    sample of the batch's systems (every system with n <= 2048, up to 24) to
    the end in both precisions."""
    from mpla_gb300 import synth

    spec = synth.batch_spec(512)
    systems = [synth.batch_system(spec, k) for k in range(count)]
    batch = mg.Batch(count)
    t_add0 = time.perf_counter()
    handles = []
    for g in systems:
        handles.append(batch.add(g.scaled(), g.nugget, g.b, precision=mg.PREC_MIXED, eps=EPS, iter_max=300000))
    mg.synchronize()
    t_add = time.perf_counter() - t_add0
    launches0 = mg.kernel_launches()
    t0 = time.perf_counter()
    left = batch.run()
    mg.synchronize()
    sec = time.perf_counter() - t0
    launches = mg.kernel_launches() - launches0
    t_res0 = time.perf_counter()
    iters, statuses, worst = [], [], 0.0
    rhs_total = 0
    for h, g in zip(handles, systems):
        x, infos = batch.result(h, g.n, g.b.shape[1])
        rhs_total += g.b.shape[1]
        iters += [i.iterations for i in infos]
        statuses += [int(i.status) for i in infos]
        # each mixed lane's FP64 double-double true residual at convergence
        worst = max([worst] + [i.true_relres for i in infos])
    t_res = time.perf_counter() - t_res0
    rpt, _ = batch.tuning()
    batch.close()

    def ms_per_step(precision: int, subset, steps: int = 16) -> float:
        bt = mg.Batch(len(subset))
        for g in subset:
            bt.add(g.scaled(), g.nugget, g.b, precision=precision, eps=EPS, iter_max=300000)
        bt.run(max_steps=8)
        mg.synchronize()
        t = time.perf_counter()
        bt.run(max_steps=steps)
        mg.synchronize()
        dt = (time.perf_counter() - t) / steps
        bt.close()
        return dt * 1e3

    def solve_iterations(precision: int, subset) -> list[int]:
        bt = mg.Batch(len(subset))
        hs = [bt.add(g.scaled(), g.nugget, g.b, precision=precision, eps=EPS, iter_max=300000) for g in subset]
        bt.run()
        out = [max(i.iterations for i in bt.result(h, g.n, g.b.shape[1])[1]) for h, g in zip(hs, subset)]
        bt.close()
        return out

    fp64_step, mixed_step = ms_per_step(mg.PREC_FP64, systems), ms_per_step(mg.PREC_MIXED, systems)
    sample = [g for g in systems if g.n <= 2048][:24]
    k64, k32 = solve_iterations(mg.PREC_FP64, sample), solve_iterations(mg.PREC_MIXED, sample)
    ratio_iters = float(sum(k64)) / float(sum(k32))
    fp64_seconds_est = sec * (fp64_step / mixed_step) * ratio_iters
    return {"workload": f"{count} of the 512 Gaussian systems, n log-uniform [256,16384], d in {{2,3}}, "
                        "l ~ U[0.03,0.2], nugget 1e-4, 1-8 N(0,1) right-hand sides, mixed precision, relres 1e-10",
            "systems_per_s": count / sec, "rhs_solves_per_s": rhs_total / sec, "seconds": sec,
            "e2e_systems_per_s": count / (sec + t_add + t_res), "admission_seconds": t_add,
            "result_readback_seconds": t_res,
            "unfinished": left, "all_converged": all(s == 0 for s in statuses),
            "rhs_total": rhs_total, "iterations_median": float(np.median(iters)), "iterations_max": int(max(iters)),
            "worst_true_relres": worst, "gpu_launches": int(launches),
            "fp64_ms_per_step": fp64_step, "mixed_ms_per_step": mixed_step,
            "fp64_over_mixed_per_step": fp64_step / mixed_step,
            "fp64_over_mixed_iterations": ratio_iters,
            "iteration_sample": f"{len(sample)} systems with n <= 2048 solved to the end in both precisions "
                                f"(slowest right-hand side): FP64 {sum(k64)}, mixed {sum(k32)} iterations",
            "fp64_systems_per_s_extrapolated": count / fp64_seconds_est,
            "fp64_seconds_extrapolated": fp64_seconds_est,
            "mixed_over_fp64_solves": fp64_seconds_est / sec,
            "extrapolation": "FP64 batch time = mixed batch time x FP64/mixed time per step (all systems running) "
                             "x FP64/mixed iterations (sample)",
            "autotuner_rows_per_thread": rpt}


def bench_serving(mg, rates, per_rate: int, n_hi: int, drain: float, seed: int = 0) -> list:
    """Continuous batching at several arrival rates: per rate, Poisson
    arrivals over a window of per_rate / rate seconds (about `per_rate`
    requests), n log-uniform in [1024, n_hi], d in {2,3}, l ~ U[0.03, 0.2],
    1-4 N(0,1) right-hand sides, half FP64 and half mixed, relres 1e-10,
    drained until every request has finished (or `drain` seconds)."""
    from mpla_gb300 import synth
    from mpla_gb300.serve import Request, Server, latency_stats

    out = []
    for q, rate in enumerate(rates):
        window = per_rate / rate
        reqs = synth.serving_requests(rate, window, seed=seed + q, n_hi=n_hi)
        engines = {mg.PREC_FP64: mg.Batch(128), mg.PREC_MIXED: mg.Batch(128)}
        srv = Server(engines, slice_steps=64)
        t0 = time.perf_counter()
        for a, k, pts, b, prec in reqs:
            srv.submit(Request(arrival=t0 + a, rid=k, points=pts, b=b, precision=prec))
        srv.serve(until=t0 + window, drain_until=t0 + window + drain)
        st = latency_stats(srv.done)
        conv = all(int(i.status) == 0 for c in srv.done for i in c.infos)
        by_prec = {}
        for p, name in ((0, "fp64"), (1, "mixed")):
            lat = [c.latency for c in srv.done if c.precision == p]
            if lat:
                by_prec[name] = {"completed": len(lat), "p50_s": float(np.percentile(lat, 50)),
                                 "p99_s": float(np.percentile(lat, 99)),
                                 "n_max": int(max(c.n for c in srv.done if c.precision == p))}
        for e in engines.values():
            e.close()
        st.update({"rate_per_s": rate, "window_s": window,
                   "workload": f"Poisson arrivals {rate}/s for {window:g} s, n log-uniform [1024,{n_hi}], "
                               "d in {2,3}, l ~ U[0.03,0.2], 1-4 N(0,1) right-hand sides, half FP64 / half mixed, "
                               "relres 1e-10",
                   "submitted": len(reqs), "unfinished": len(reqs) - len(srv.done), "all_converged": conv,
                   "admission_refusals": srv.refusals, "by_precision": by_prec})
        out.append(st)
    return out


# ---------------------------------------------------------------- our arm
def run_ours(args, world, rank, local):
    import torch

    import mpla_gb300 as mg
    from mpla_gb300 import synth

    if not mg.LIB_PATH.exists():
        from mpla_gb300 import _build

        _build.build()
    torch.cuda.set_device(local)
    mg.init(local)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    n = args.n
    prob = synth.gauss_problem(n, DIM, ELL, NUGGET, seed=0)
    pts_scaled = prob.scaled()
    b = prob.b
    dp = mg.GaussPoints(pts_scaled)
    db = mg.DeviceArray.from_numpy(b)
    # x and the L2-flush buffer are torch tensors so that zeroing them is
    # ordered on the benchmark stream together with the solve.
    x_t = torch.zeros(n, dtype=torch.float64, device="cuda")
    flush_t = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    class _Ptr:
        def __init__(self, t):
            self.ptr = t.data_ptr()

    dx = _Ptr(x_t)

    def step():
        with torch.cuda.stream(stream):
            flush_t.zero_()  # L2 flush
            x_t.zero_()
            return mg.cg_gauss(dp, NUGGET, db.ptr, dx.ptr, iter_max=args.iter_max, eps=EPS,
                               precision=mg.PREC_MIXED, stream=sp)

    for _ in range(args.warmup):
        info = step()
    torch.cuda.synchronize()
    barrier(world)
    launches0 = mg.kernel_launches()
    infos = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            infos.append(step())
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    launches = mg.kernel_launches() - launches0
    sec = e0.elapsed_time(e1) / 1e3
    sec_max = max_over_ranks(sec, world)
    value = aggregate(args.steps, sec_max, world)
    info = infos[-1]
    # the solver's own FP64 true residual ||b - K x|| / ||b|| of the returned
    # x (parity of that residual with the FP64 oracle is a test, not a bench
    # step)
    true_rel = float(info.true_relres)

    # ---- e2e through the host-buffer entry point
    pin_pts = pts_scaled.copy()
    e2e_times = []
    # (the device path above has warmed the library; every e2e call is timed)
    for k in range(args.e2e_steps):
        barrier(world)
        t0 = time.perf_counter()
        x_host, einfo = mg.cg_gauss_host(pin_pts, NUGGET, b, iter_max=args.iter_max, eps=EPS, precision=mg.PREC_MIXED)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    e2e_sec = max_over_ranks(sum(e2e_times), world)
    e2e_value = aggregate(args.e2e_steps, e2e_sec, world) if args.e2e_steps > 0 else None

    # ---- plain FP64 CG: bounded sample of iterations
    fp_iters = args.fp64_sample_iters
    with torch.cuda.stream(stream):
        x_t.zero_()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        finfo = mg.cg_gauss(dp, NUGGET, db.ptr, dx.ptr, iter_max=fp_iters + 1, eps=EPS, precision=mg.PREC_FP64,
                            stream=sp)
        t1.record(stream)
    torch.cuda.synchronize()
    fp_ms_per_iter = t0.elapsed_time(t1) / max(1, finfo.iterations + 1)

    # ---- dominant kernel: the mixed matvec, per-launch device time
    dy = mg.DeviceArray(n)
    dxr = mg.DeviceArray.from_numpy(np.random.default_rng(0).standard_normal(n))
    mixed_ms = mg.time_gauss_matvec(dp, NUGGET, mg.PREC_MIXED, dxr.ptr, dy.ptr, reps=20, stream=sp)
    f64_ms = mg.time_gauss_matvec(dp, NUGGET, mg.PREC_FP64, dxr.ptr, dy.ptr, reps=3, stream=sp)
    clocks = clk.summary()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = clocks.get("sm_mhz") or 1900.0
    entries = float(n) * n
    evaluated = float(mg.gauss_mixed_work(dp))   # exponentials one mixed matvec evaluates
    mixed_rate = evaluated / (mixed_ms * 1e-3)
    sfu_peak = SFU_EX2_PER_CLK_SM * sms * sm_mhz * 1e6
    fp64_rate = entries / (f64_ms * 1e-3)
    fp64_evaluated = float(mg.gauss_fp64_work(dp))   # entries one FP64 matvec evaluates

    iters_mixed = int(info.iterations)
    iters_fp64 = fp64_iterations(args, iters_mixed)
    fp64_solves_est = 1.0 / (fp_ms_per_iter * 1e-3 * iters_fp64)

    if rank != 0:
        return
    extra = {}
    progress(f"headline done: {iters_mixed} mixed iterations, {sec_max / args.steps:.2f} s per solve")
    if not args.no_dense:
        extra["dense"] = bench_dense(mg, torch, stream, measured_peak("hbm_gbs"))
        progress("dense done")
        extra["mixed_c3"] = bench_mixed_c3(mg, stream, sms, sm_mhz)
        progress("mixed C3 matvec done")
    if not args.no_batched:
        extra["batched"] = bench_batched(mg, args.batch_systems)
        progress("batched done")
    if not args.no_serving:
        extra["serving"] = bench_serving(mg, [float(r) for r in args.serve_rates.split(",")], args.serve_per_rate,
                                         args.serve_n_max, args.serve_drain)
        progress("serving done")
    cpu = cpu_baseline(pts_scaled, NUGGET, iters_fp64, budget_s=args.cpu_seconds) if not args.no_cpu else None
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": sec_max * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 matvec (SFU exp2) + f64 vectors/dots/scalars/true residual",
        "data": "synthetic: seeded splitmix64, points U[0,1]^2, b = sin(2 pi x1) cos(2 pi x2)",
        "config": {"workload": f"Gaussian kernel CG, n={n}, d={DIM}, l={ELL}, nugget={NUGGET}, relres {EPS}, x0=0",
                   "solver": "mixed CG with FP64 reliable residual replacement",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer zeroed before every step"},
        "iterations": iters_mixed,
        "converged": all(int(i.status) == 0 for i in infos),
        "fp64_true_residual_replacements": int(info.fp64_matvecs),
        "true_relres": true_rel,
        "p50_ms": statistics.median([sec_max * 1e3 / args.steps]),
        "e2e": {"value": e2e_value, "unit": "solves/s",
                "h2d_bytes_per_step": int(pts_scaled.nbytes + b.nbytes + 8 * n),
                "d2h_bytes_per_step": int(8 * n)},
        "fp64": {"ms_per_iteration": fp_ms_per_iter, "sample_iterations": int(finfo.iterations + 1),
                 "matvec_ms": f64_ms, "entries_per_s": fp64_rate,
                 "evaluated_per_launch": fp64_evaluated, "evaluated_per_s": fp64_evaluated / (f64_ms * 1e-3),
                 "iterations_assumed": iters_fp64,
                 "solves_per_s_est": fp64_solves_est,
                 "mixed_over_fp64": value / fp64_solves_est},
        "roofline": {"bound": "sfu", "kernel": "sym_f32_group_kernel (+ gather, reduce)",
                     "achieved": mixed_rate / 1e12, "peak": sfu_peak / 1e12, "unit": "Tex2/s",
                     "frac": mixed_rate / sfu_peak,
                     "traffic": GROUP_KERNEL_DRAM_BYTES_N65536 if (n == N_FULL and DIM == 2) else None,
                     "traffic_unit": "DRAM bytes per launch",
                     "traffic_source": "one ncu capture of this kernel at n=65536, d=2 (not measured in this run)",
                     "per_unit": "1 evaluated kernel entry = 1 ex2 (+ 6 FP32 lane operations in 3 packed FMA-pipe "
                                 "instructions, d = 2); each unordered pair of points evaluated once, tile pairs "
                                 "below 2^-40 skipped",
                     "evaluated_per_launch": evaluated, "algorithmic_entries_per_launch": entries,
                     "algorithmic_entries_per_s": entries / (mixed_ms * 1e-3), "matvec_ms": mixed_ms,
                     "peak_source": f"{SFU_EX2_PER_CLK_SM:.0f} ex2/clk/SM (the XU pipe peak ncu reports on GB300) "
                                    f"x {sms} SMs x {sm_mhz:.0f} MHz median SM clock"},
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    line.update(extra)
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------- reference arm
def reference_dense(ref, n: int = 4096, reps: int = 10) -> dict:
    """C1 on the reference: mpla_dgemv (cuBLAS Dgemv inside, mpla.cpp:716-751)
    and the dense CG of mpla_generic_conjugate_gradient_with_checkpoint_restart
    with the cuBLAS user core of the reference's test_cg.cpp:38-43."""
    from mpla_gb300 import synth

    A, b, x0 = synth.config_dense(0)
    _, gemv_ms = ref.dgemv(A, np.linspace(-1.0, 1.0, n), reps=50)
    cublas_ms = ref.cublas_dgemv_ms(A, reps=50)
    for _ in range(2):
        ref.solve_dense(A, b, x0, 1000, EPS, ref.SOLVER_CG_REL)
    times, mvs = [], []
    for _ in range(reps):
        _, mv, ms = ref.solve_dense(A, b, x0, 1000, EPS, ref.SOLVER_CG_REL)
        times.append(ms)
        mvs.append(mv)
    solve_ms = float(np.median(times))
    gemv_bytes = 8.0 * n * n + 16.0 * n
    return {"workload": "dense FP64 CG, n=4096, A = M^T M/n + I (M ~ U[-1,1], seed 0), b = 1, relres 1e-10",
            "solves_per_s": 1e3 / solve_ms, "ms_per_solve": solve_ms,
            "iterations": ref.iterations(ref.SOLVER_CG_REL, mvs[-1]),
            "dgemv": {"ms": gemv_ms, "achieved_gbs": gemv_bytes / (gemv_ms * 1e-3) / 1e9, "bytes": gemv_bytes,
                      "what": "mpla_dgemv (cuBLAS Dgemv plus the reference's per-call allocations and copies)"},
            "cublas_dgemv": {"ms": cublas_ms, "achieved_gbs": gemv_bytes / (cublas_ms * 1e-3) / 1e9,
                             "what": "the cublasDgemv call inside mpla_dgemv alone, on resident operands"}}


def run_reference(args, world, rank, local):
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    refdir = ROOT / "oracle" / "_ref"
    lib = refdir / "libmplaref.so"
    if not lib.exists():
        try:
            import build_ref

            build_ref.build()
        except Exception as e:  # noqa: BLE001
            print(json.dumps({"impl": "reference", "unavailable": f"reference MPLA not built: {e}"}))
            return
    from oracle import reference as ref
    from mpla_gb300 import synth

    try:
        ref.lib(local)
    except RuntimeError as e:
        print(json.dumps({"impl": "reference", "unavailable": str(e)}))
        return
    L = ref.lib(local)
    import ctypes as C

    n = args.n
    prob = synth.gauss_problem(n, DIM, ELL, NUGGET, seed=0)
    pts = np.ascontiguousarray(prob.scaled())
    b = np.ascontiguousarray(prob.b)
    sample_iters = args.ref_sample_iters
    ms = C.c_double()
    mv = C.c_int()
    for _ in range(args.warmup):
        L.ref_cg_gauss_sample(n, DIM, pts.ctypes.data, NUGGET, b.ctypes.data, sample_iters, EPS, C.byref(ms),
                              C.byref(mv))
    total_ms, total_mv = 0.0, 0
    for _ in range(args.steps):
        st = L.ref_cg_gauss_sample(n, DIM, pts.ctypes.data, NUGGET, b.ctypes.data, sample_iters, EPS, C.byref(ms),
                                   C.byref(mv))
        if st != 0:
            print(json.dumps({"impl": "reference", "unavailable": f"reference CG sample failed (status {st})"}))
            return
        total_ms += ms.value
        total_mv += mv.value
    # every matvec of the sample is inside the timed call: the r0 matvec and
    # one per iteration, so the time per iteration is the time per matvec
    ms_per_iter = total_ms / max(1, total_mv)
    iters_fp64 = fp64_iterations(args, 0)
    value = (1.0 / (ms_per_iter * 1e-3 * iters_fp64)) if iters_fp64 else None
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded splitmix64, points U[0,1]^2, b = sin(2 pi x1) cos(2 pi x2)",
        "config": {"workload": f"Gaussian kernel CG, n={n}, d={DIM}, l={ELL}, nugget={NUGGET}, relres {EPS}, x0=0",
                   "solver": "reference MPLA FP64 CG (mpla_generic_conjugate_gradient_with_checkpoint_restart, "
                             "gaussian system_assembler, streamed cuBLAS core)"},
        "ms_per_iteration": ms_per_iter,
        "sample_matvecs": total_mv,
        "iterations_assumed": iters_fp64,
        "extrapolation": f"each step runs {sample_iters} CG iterations ({sample_iters + 1} matvecs, all timed) of the "
                         f"reference MPLA built from its sources (GPU, 1 rank); solves/s = 1 / (ms per matvec x "
                         f"{iters_fp64} iterations, this library's FP64 CG count on the same system)",
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_dense:
        line["dense"] = reference_dense(ref)
    print(json.dumps(line), flush=True)


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=N_FULL)
    p.add_argument("--iter-max", type=int, default=100000)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--fp64-sample-iters", type=int, default=20)
    p.add_argument("--fp64-iterations", type=int, default=0,
                   help="FP64 CG iteration count of the full solve, when known (used to scale sampled iterations)")
    p.add_argument("--ref-sample-iters", type=int, default=3)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-dense", action="store_true")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--batch-systems", type=int, default=512,
                   help="systems of the 512-system batch workload to run (a prefix; 512 is all of it)")
    p.add_argument("--serve-rates", default="0.5,1,2", help="arrival rates per second, comma-separated")
    p.add_argument("--serve-per-rate", type=int, default=8, help="expected requests per rate")
    p.add_argument("--serve-n-max", type=int, default=8192,
                   help="largest request size (the serving configuration's 32768 makes single FP64 requests run "
                        "for minutes on GB300's FP64 pipe; the full sweep is profile_cases.py serving_sweep)")
    p.add_argument("--serve-drain", type=float, default=300.0)
    args = p.parse_args(argv)
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    world, rank, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    try:
        if args.impl == "reference":
            run_reference(args, world, rank, local)
        else:
            run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
