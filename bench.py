#!/usr/bin/env python3
"""Benchmark of the particle-history hot path on GB300.

Workload (the metric's configuration, "config 1" of the reference's
headline): slab [0, 1] in 10,000 cells decomposed into 64 contiguous
sub-domains (decompose_domain, per-layer dx), sigma_a(x) = 0.5 + 0.4 sin(6 pi x),
sigma_s(x) = 2.0 + 1.5 cos(4 pi x) at cell centres (fp32), particles born at
x = 0, mu = 1, weight 1.0, seeds from the reference's rnd_seed chain started
at 5127801, minimum weight 1e-12 (implicit capture, as Layer::simulate).
The full problem is 1e8 histories; one bench step runs one batch of
--batch consecutive histories of that source (default: all 1e8 in one
launch, so the launch's tail, where the SMs wait on the longest histories,
is paid once per 1e8).  Synthetic data: the reference has no dataset.

batched / adjoint : the metric's other two forms (batched slabs of
        configuration 2 at full size, autotuned, against one launch per slab;
        forward+adjoint of configuration 3), each timed with CUDA events on
        its own launch.
worker : the workers with on-device hand-over queues (asynchronous rings,
        and the synchronous cycle) on the first 1e7 histories, against the
        fused tracker (identical tallies).
fit   : configuration 4, the batched inverse fit (200 Adam steps of batched
        forward+adjoint launches replayed from a CUDA graph).
value : histories/s of the strict tracker with the batch's particles
        already resident in HBM (mcg_simulate_device), CUDA-event time of
        the kernel, L2 flushed (256 MB memset) between steps.
e2e   : histories/s through the C ABI with host buffers (mcg_simulate on
        pinned host particles and results, which the tracker reads and
        writes in place over the host link, + the tally read), wall time per
        step.
--impl reference : the reference's CPU implementation of the path (the
        oracle port of src/layer.cpp on all host cores), same metric.
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "histories/s on 1 GB300 (plain vs batched vs fwd+adjoint) at matched tally std err"
NB_CELLS, N_LAYERS, N_TOTAL = 10000, 64, 100_000_000
BASE_SEED = 5127801
MIN_W = 1e-12
# DRAM bytes (read + write) per history of the strict tracker, from an ncu
# capture of 3e6 histories of this workload
DRAM_BYTES_PER_HISTORY = 112.44e6 / 3e6
WORKLOAD = ("slab 10000 cells / 64 sub-domains (decompose_domain), sigma_a=0.5+0.4sin(6pi x), "
            "sigma_s=2+1.5cos(4pi x), 1e8 histories from x=0 mu=1 w=1, rnd_seed chain 5127801, "
            "min weight 1e-12")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), "measured"
    except OSError:
        return 6800.0, "fallback"


def conversion_roofline(steps, scatters, seconds, mode, rates):
    """64-bit int<->float conversions per second against the rate of that
    pipe measured in this run (mcg_measure_conversion_rates).  The strict
    tracker converts a state to a float only where the value itself is
    needed: the flight sample and the new direction of a scatter (2 per
    scatter; the certain-crossing test compares the state's top bits as an
    integer, and deposits below 2^31 fixed-point units take the 32-bit
    conversion).  The near-ties that also need the flight sample (about 2e-5
    of the crossings) and the rare deposits of 2^31 units and more are not
    counted.  The fast tracker uses no 64-bit conversion per step."""
    per = 2 * scatters if mode == "strict" else 0
    peak = min(rates["u64_f32"], rates["f32_s64"])
    achieved = per / seconds
    return {"bound": "64-bit int/float conversion rate (not binding)", "achieved": achieved,
            "peak": peak, "unit": "conversions/s", "frac": achieved / peak,
            "peak_source": "measured in this run (mcg_measure_conversion_rates)",
            "measured_rates": rates}


def physics(nb=NB_CELLS):
    xc = (np.arange(nb, dtype=np.float64) + 0.5) / nb
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    rates = (sa / sigs).astype(np.float32)
    return sigs, rates


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ------------------------------------------------------------------ CPU leg
def cpu_rate(n_hist, threads, first=0):
    """Oracle port of Layer::simulate over the decomposed slab on host cores:
    histories/s on histories first .. first+n_hist-1 of the source."""
    import oracle as O
    sigs, rates = physics()
    layers = list(O.decompose(0.0, 1.0, NB_CELLS, N_LAYERS))
    p = np.zeros(n_hist, O.PARTICLE_DTYPE)
    s = O.lcg_skip(BASE_SEED, first, True)
    p["seed"] = O.rnd_seed_chain(s, n_hist)
    p["x"], p["mu"], p["wmc"], p["index"] = 0.0, 1.0, 1.0, 0
    t0 = time.perf_counter()
    r = O.simulate_histories(layers, sigs, rates, MIN_W, p, 2.0 ** 35, nthreads=threads)
    dt = time.perf_counter() - t0
    steps = int(r["traces"]["steps"].sum())
    return n_hist / dt, steps, dt


def cpu_calibrate(threads):
    """Histories/s of the port on a sample large enough to keep every thread
    busy (512 histories per thread), used to size the timed samples."""
    rate, _, _ = cpu_rate(threads * 512, threads, first=1_000_000)
    return rate


def cpu_baseline(budget_s=10.0, threads=None):
    threads = threads or os.cpu_count()
    rate = cpu_calibrate(threads)
    n = int(max(threads * 8, min(4_000_000, rate * budget_s)))
    rate, steps, dt = cpu_rate(n, threads, first=7_000_000)
    return {"value": rate, "unit": "histories/s", "cores": threads, "kind": "port",
            "sample": f"{n} histories of the 1e8-history source (indices 7e6..), {steps} steps, "
                      f"{dt:.1f} s on {threads} threads",
            "steps_per_s": steps / dt}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count()
    rate = cpu_calibrate(threads)
    per_step = int(max(threads * 8, min(2_000_000, rate * 4.0)))
    times = []
    for k in range(args.warmup + args.steps):
        rate, steps, dt = cpu_rate(per_step, threads, first=3_000_000 + k * per_step)
        if k >= args.warmup:
            times.append(dt)
    value = per_step * len(times) / sum(times)
    line = {
        "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD,
                   "batch": per_step, "l2": "n/a (host)"},
        "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} histories per step of the same 1e8-history "
                                   "source (consecutive indices from 3e6), sized to about four "
                                   "seconds of host work per step; the GPU arm runs all 1e8 "
                                   "per step",
                         "note": "the oracle's restatement of Layer::simulate (bit-exact with "
                                 "the reference's compiled Layer; its speed measured at 0.98x "
                                 "of it single-threaded), OpenMP over all host cores: the "
                                 "reference's own intra-rank parallelism, mpirun being "
                                 "unavailable on this box"},
        "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU leg
def run_gpu(args):
    import torch
    import importlib.util
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    spec = importlib.util.spec_from_file_location(
        "mc_mpi_gb300", os.path.join(ROOT, "mc-mpi_gb300", "__init__.py"),
        submodule_search_locations=[os.path.join(ROOT, "mc-mpi_gb300")])
    mcg = importlib.util.module_from_spec(spec)
    sys.modules["mc_mpi_gb300"] = mcg
    spec.loader.exec_module(mcg)

    B = args.batch
    sigs, rates = physics()
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, NB_CELLS, N_LAYERS)
    ctx = mcg.Context(mode=args.mode, device=local)
    ctx.set_layers(st, m, dx, sigs, rates, MIN_W)
    ctx.set_tally_scale(35)
    ctx.set_algorithm(args.algorithm, args.event_steps)

    # device-resident particles of the batch: built on the device by the
    # source kernel before the timed region (histories k*B .. of this rank)
    part = torch.empty(B * 24, dtype=torch.uint8, device="cuda")
    res = torch.empty(B, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    host_p = torch.empty(B * 24, dtype=torch.uint8).pin_memory()
    host_r = torch.empty(B, dtype=torch.int32).pin_memory()

    def batch_first(k):
        return (rank * (args.warmup + args.steps) + k) * B % N_TOTAL

    built = [None]

    def make_batch(k):
        """Born particles of step k in the pinned host buffer (rebuilt only
        when the step's histories differ from the buffer's)."""
        if built[0] == batch_first(k):
            return
        arr = np.frombuffer(host_p.numpy(), dtype=mcg.PARTICLE_DTYPE)
        src = mcg.Source(0, 0, BASE_SEED, 0.0, 1.0, 1.0, 0)
        mcg._check(mcg.load_library().mcg_create_particles(
            ctx.h, C.byref(src), batch_first(k), B, arr.ctypes.data_as(C.c_void_p)))
        built[0] = batch_first(k)

    def device_step(k):
        make_batch(k)
        part.copy_(host_p, non_blocking=False)
        flush.zero_()
        torch.cuda.synchronize()
        ctx.simulate_device_ptr(part.data_ptr(), B, res.data_ptr())
        return ctx.last_kernel_ms()

    for k in range(args.warmup):
        device_step(k)
    ctx.tally_reset()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    kernel_ms = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            kernel_ms.append(device_step(args.warmup + k))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    counters = ctx.counters()
    dev_s = sum(kernel_ms) / 1e3
    if dist:
        t = torch.tensor([dev_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s = float(t.item())
    value = ws * B * args.steps / dev_s

    # e2e through the C ABI with pinned host buffers
    lib = mcg.load_library()
    e2e_times = []
    for k in range(0 if args.no_e2e else max(1, min(args.steps, 3)) + 1):
        make_batch(args.warmup + k)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        mcg._check(lib.mcg_simulate(ctx.h, C.c_void_p(host_p.data_ptr()), B,
                                    C.c_void_p(host_r.data_ptr()), None, None))
        tq = ctx.tally_q()
        e2e_times.append(time.perf_counter() - t1)
        built[0] = None  # the call wrote the final particle states back
    e2e_val = B / statistics.median(e2e_times[1:]) if e2e_times else None

    # roofline of the tracker kernel: algorithmic bytes per launch
    hbm_peak, peak_kind = peaks()
    bytes_per_hist = 24 + 24 + 4  # particle in, particle out, result
    # DRAM bytes (read + write) per history from one ncu capture of this
    # kernel on 3e6 histories of the same workload (a constant of this file,
    # not measured by this run), scaled to the launch: below the algorithmic
    # 52 B because part of the particle write-back is still in L2 when the
    # kernel ends
    dram_per_hist = DRAM_BYTES_PER_HISTORY
    mean_ms = sum(kernel_ms) / len(kernel_ms)
    achieved = bytes_per_hist * B / (mean_ms / 1e3) / 1e9
    steps_per_s = counters["steps"] / dev_s if not dist else None
    clocks = clk.summary()
    f_sm = (clocks["sm_mhz"] or 1470.0) * 1e6
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    n_alg = 20.0 + 6.0 * counters["scatters"] / max(counters["steps"], 1)
    issue_frac = (counters["steps"] / dev_s) * n_alg / (sms * 128 * f_sm) if steps_per_s else None

    line = {
        "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "batch": B, "mode": args.mode, "algorithm": args.algorithm,
                   "parallelism": f"histories sharded x{ws}",
                   "l2": "flushed between steps (256 MB memset)"},
        "steps_per_s": counters["steps"] / dev_s * ws,
        "collisions_per_s": counters["scatters"] / dev_s * ws,
        "wall_s": wall,
        "gpu_launches": args.steps,
        "e2e": None if e2e_val is None else {
            "value": e2e_val * ws, "unit": "histories/s",
            "h2d_bytes_per_step": 24 * B, "d2h_bytes_per_step": 28 * B + 8 * NB_CELLS,
            "path": "mcg_simulate on pinned host buffers: the tracker reads and writes "
                    "them in place over the host link during the launch"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak,
                     "traffic": dram_per_hist * B if args.mode == "strict" else None,
                     "traffic_unit": "bytes per launch",
                     "traffic_source": "constant from an ncu capture of 3e6 histories of this "
                                       "workload (dram__bytes_read.sum + dram__bytes_write.sum), "
                                       "scaled by histories; not measured by this run",
                     "peak_source": peak_kind,
                     "note": "not HBM-bound: instruction issue bounds the tracker; see "
                             "issue_roofline"},
        "conversion_roofline": conversion_roofline(counters["steps"] * ws,
                                                   counters["scatters"] * ws, dev_s, args.mode,
                                                   ctx.conversion_rates()),
        "issue_roofline": {"bound": "issue", "n_alg_ops_per_step": n_alg,
                           "achieved_gops": (counters["steps"] / dev_s) * n_alg / 1e9,
                           "peak_gops": sms * 128 * f_sm / 1e9, "frac": issue_frac,
                           # the step's two algorithmic transcendentals (log, exp) against
                           # 16 special-function results per SM per clock
                           "mufu_alg_per_step": 2,
                           "mufu_frac": (counters["steps"] / dev_s) * 2 / (sms * 16 * f_sm)
                           if steps_per_s else None},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_extra:
        line["fom"] = figure_of_merit(ctx, value / ws)
    if rank == 0 and not args.no_extra and args.algorithm == "history":
        line["event"] = bench_event(mcg, args.mode, local, st, m, dx, sigs, rates)
    if rank == 0 and not args.no_extra and args.mode == "strict":
        # the same steps with fast arithmetic (hardware log2/exp2, a series
        # for the flight's log near h = 1; tallies statistically equivalent,
        # not bit-identical)
        fctx = mcg.Context(mode="fast", device=local)
        fctx.set_layers(st, m, dx, sigs, rates, MIN_W)
        fctx.set_tally_scale(35)
        fms = []
        for k in range(3):
            make_batch(args.warmup)
            part.copy_(host_p, non_blocking=False)
            flush.zero_()
            torch.cuda.synchronize()
            fctx.simulate_device_ptr(part.data_ptr(), B, res.data_ptr())
            fms.append(fctx.last_kernel_ms())
        fc = fctx.counters()
        line["fast"] = {"value": B / (statistics.median(fms[1:]) / 1e3), "unit": "histories/s",
                        "warmup": 1, "steps": 2,
                        "steps_per_s": fc["steps"] / (sum(fms) / 1e3)}
        fctx.close()
    if rank == 0 and not args.no_extra:
        line["batched"] = bench_batched(mcg, args.mode, local)
        line["adjoint"] = bench_adjoint(mcg, args.mode, local)
        line["worker"] = bench_worker(mcg, args.mode, local, st, m, dx, sigs, rates)
        line["fit"] = bench_fit(mcg, local)
    if dist:
        # exact multi-rank reduction: every rank runs its share of 1e5
        # histories, the int64 tallies are summed over ranks, and rank 0
        # compares with one rank running all of them
        from mc_mpi_gb300 import dist as mdist
        n_check = 100_000

        def run_shard(first, count):
            ctx.tally_reset()
            ctx.simulate_source(N_TOTAL + first, count)
            return torch.from_numpy(ctx.tally_q())

        red = mdist.sharded_tally(run_shard, n_check, ws, rank, device="cuda")
        if rank == 0:
            ctx.tally_reset()
            ctx.simulate_source(N_TOTAL, n_check)
            line["multi_rank_check"] = {
                "histories": n_check, "ranks": ws,
                "identical_tallies": bool(np.array_equal(red.cpu().numpy(), ctx.tally_q()))}
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def bench_batched(mcg, mode, device, scale=1.0, reps=2):
    """Configuration 2 (4096 slabs, cells U{16..4096}, L ~ U[0.5, 5], per-cell
    sigma_a ~ U[0.1, 5], sigma_s ~ U[0, 10], histories log-uniform in
    [1e3, 1e6] scaled by `scale`), launch shape and algorithm picked by the
    autotuner: one persistent CUDA-graph launch against one ordinary launch
    per slab, same histories, same tallies."""
    from mc_mpi_gb300 import workloads
    slabs, sigs, rates = workloads.config2(scale_histories=scale)
    n = sum(d["n_histories"] for d in slabs)
    with mcg.Context(mode=mode, device=device) as ctx:
        ctx.set_tally_scale(30)
        ctx.batch_set(slabs, sigs, rates, MIN_W)
        tune = ctx.batch_autotune(0.05)
        ctx.batch_run()  # warm-up, builds the graph
        ms = []
        for _ in range(reps):
            ctx.batch_tally_reset()
            ctx.batch_run()
            ms.append(ctx.last_kernel_ms())
        q_batch = ctx.batch_tally_q()
        steps = ctx.counters()["steps"]
        ctx.batch_tally_reset()
        ctx.batch_run_per_slab()
        ms_plain = ctx.last_kernel_ms()
        same = bool(np.array_equal(ctx.batch_tally_q(), q_batch))
    fast_ms = None
    if mode == "strict":
        # the same histories with the fast arithmetic, in the strict run's
        # launch shape (statistically equivalent tallies)
        with mcg.Context(mode="fast", device=device) as fctx:
            fctx.set_tally_scale(30)
            fctx.batch_set(slabs, sigs, rates, MIN_W)
            fctx.batch_set_launch(tune["block"], tune["item_histories"], tune["tally_mode"])
            fctx.batch_set_deferral(tune["defer"])
            if tune["algorithm"] == 1:
                fctx.batch_set_algorithm("event", tune["steps_per_pass"])
            fctx.batch_run()
            fctx.batch_tally_reset()
            fctx.batch_run()
            fast_ms = fctx.last_kernel_ms()
    t = min(ms) / 1e3
    return {"value": n / t, "unit": "histories/s", "per_slab_value": n / (ms_plain / 1e3),
            "speedup_vs_per_slab": (ms_plain / 1e3) / t, "identical_tallies": same,
            "fast_value": None if fast_ms is None else n / (fast_ms / 1e3),
            "steps_per_s": steps / t, "histories": n, "launches": 1, "autotuned": tune,
            "workload": f"4096 slabs, cells U{{16..4096}}, L~U[0.5,5], sigma_a~U[0.1,5], "
                        f"sigma_s~U[0,10], histories log-uniform [1e3,1e6] x {scale}",
            "note": None if scale >= 1.0 else
                    "reduced histories: each per-slab launch is then mostly its fixed cost "
                    "(set-up and the tail of its longest histories), which inflates the "
                    "speed-up"}


def bench_worker(mcg, mode, device, st, m, dx, sigs, rates, n=10_000_000):
    """The workers with on-device hand-over queues, the forms that replace
    WorkerSync/Async/Rma's MPI exchange, on the first n histories of the
    workload, against the fused tracker on the same histories (identical
    tallies expected): `value` is the asynchronous form (mcg_worker_run_async,
    one persistent launch with bounded rings), `sync_value` the cycle form
    (mcg_worker_run)."""
    with mcg.Context(mode=mode, device=device) as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, MIN_W)
        ctx.set_tally_scale(35)
        ctx.simulate_source(0, n // 10)  # warm-up
        ctx.tally_reset()
        ctx.simulate_source(0, n)
        t_fused = ctx.last_kernel_ms() / 1e3
        q_fused = ctx.tally_q()
        ctx.tally_reset()
        ctx.worker_run_async(n // 10)  # warm-up, sizes the rings
        ctx.tally_reset()
        hand = ctx.worker_run_async(n)
        t_a = ctx.last_kernel_ms() / 1e3
        same_a = bool(np.array_equal(ctx.tally_q(), q_fused))
        ctx.tally_reset()
        ctx.worker_run(n // 10)  # warm-up
        ctx.tally_reset()
        cycles, hand_s = ctx.worker_run(n)
        t_s = ctx.last_kernel_ms() / 1e3
        same_s = bool(np.array_equal(ctx.tally_q(), q_fused))
    return {"value": n / t_a, "unit": "histories/s", "fused_value": n / t_fused,
            "ratio_vs_fused": t_fused / t_a, "identical_tallies": same_a and same_s,
            "handoffs_per_history": hand / n, "sync_value": n / t_s,
            "sync_ratio_vs_fused": t_fused / t_s, "sync_cycles": cycles, "histories": n,
            "workload": "the plain workload's first 1e7 histories, 64 sub-domains with "
                        "on-device hand-over queues"}


def bench_fit(mcg, device, scale=1.0, n_steps=200):
    """Configuration 4: 64 slabs with cells U{64..1024}, hidden
    sigma_a = 1 + 0.8 sin(2 pi k x + phi), sigma_s = 1.5; targets from 1e7
    histories per slab; 200 Adam steps (lr 1e-2) from sigma_a = 1, each a
    batched forward+adjoint launch of 1e6 histories per slab (fast
    arithmetic), all replayed from one CUDA graph.  Reports histories/s of
    the fit and the final relative L2 error of sigma_a."""
    from mc_mpi_gb300 import workloads
    slabs, hidden, sig_s = workloads.config4(histories=int(1e6 * scale))
    tslabs = [dict(d, n_histories=int(1e7 * scale), base_seed=d["base_seed"] + 1)
              for d in slabs]
    sigs = (hidden + sig_s).astype(np.float32)
    rates = (hidden / sigs).astype(np.float32)
    with mcg.Context(mode="fast", device=device) as ctx:
        ctx.batch_set(tslabs, sigs, rates, MIN_W)
        ctx.batch_run()
        npc = np.concatenate([np.full(d["n_cells"], d["n_histories"]) for d in tslabs])
        target = ctx.batch_tally() / npc
        ctx.fit_set(slabs, np.ones_like(hidden), sig_s, target, max_steps=n_steps)
        ctx.fit_run(n_steps, lr=1e-2)
        ms = ctx.last_kernel_ms()
        sig, loss = ctx.fit_read()
    hist = n_steps * sum(d["n_histories"] for d in slabs)
    err0 = float(np.linalg.norm(1.0 - hidden) / np.linalg.norm(hidden))
    err = float(np.linalg.norm(sig - hidden) / np.linalg.norm(hidden))
    return {"value": hist / (ms / 1e3), "unit": "histories/s", "adam_steps": n_steps,
            "histories": hist, "ms_per_adam_step": ms / n_steps, "gpu_launches": 3 * n_steps,
            "rel_l2_error": err, "rel_l2_error_start": err0, "loss_first": float(loss[0]),
            "loss_last": float(loss[-1]), "mode": "fast",
            "workload": f"configuration 4: 64 slabs, cells U{{64..1024}}, hidden "
                        f"sigma_a=1+0.8sin(2pi k x+phi), sigma_s=1.5, {n_steps} Adam steps lr "
                        f"1e-2, {int(1e6 * scale)} histories per slab and step, targets from "
                        f"{int(1e7 * scale)} per slab"}


def figure_of_merit(ctx, hist_per_s, n_batches=20, size=100_000):
    """FOM = 1 / (SE^2 T) of the per-cell tally at this throughput: the
    per-history variance of each cell's absorbed weight comes from
    n_batches independent batches (disjoint histories of the same source)
    run on the GPU; SE^2 = var / N and T = N / (histories/s), so
    FOM = (histories/s) / var.  Reported averaged over the visited cells,
    and as the relative-error form (mean^2 / var, MCNP's figure of merit)
    as a median over them.  The reference's estimator is the same, so the
    two arms' FOM ratio equals their throughput ratio."""
    means = []
    for b in range(n_batches):
        ctx.tally_reset()
        ctx.simulate_source(N_TOTAL + b * size, size)
        means.append(ctx.tally() / size)
    ctx.tally_reset()
    M = np.array(means)
    var = M.var(axis=0, ddof=1) * size
    mu = M.mean(axis=0)
    seen = var > 0
    return {"value": float(np.mean(hist_per_s / var[seen])), "unit": "1/s (1/(SE^2 T), mean over cells)",
            "relative_median": float(np.median(hist_per_s * mu[seen] ** 2 / var[seen])),
            "cells": int(seen.sum()), "variance_from": f"{n_batches} batches of {size} histories"}


def bench_event(mcg, mode, device, st, m, dx, sigs, rates, n=10_000_000, k=16):
    """The event-based tracker (SoA particle bank, K events per pass, per
    event type compaction) on the first n histories of the workload, against
    the history-based tracker on the same histories (identical tallies)."""
    with mcg.Context(mode=mode, device=device) as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, MIN_W)
        ctx.set_tally_scale(35)
        ctx.simulate_source(0, n // 10)  # warm-up
        ctx.tally_reset()
        ctx.simulate_source(0, n)
        t_hist = ctx.last_kernel_ms() / 1e3
        q_hist = ctx.tally_q()
        steps = ctx.counters()["steps"]
        ctx.set_algorithm("event", k)
        ctx.simulate_source(0, n // 10)  # sizes the bank
        ctx.tally_reset()
        ctx.simulate_source(0, n)
        t_ev = ctx.last_kernel_ms() / 1e3
        same = bool(np.array_equal(ctx.tally_q(), q_hist))
    return {"value": n / t_ev, "unit": "histories/s", "steps_per_s": steps / t_ev,
            "events_per_pass": k, "histories": n, "history_value": n / t_hist,
            "identical_tallies": same,
            "bank_bytes_per_event": 72 / k, "bank_gbs": 72 / k * steps / t_ev / 1e9}


def bench_adjoint(mcg, mode, device, n=10_000_000):
    """Configuration 3 (1000 cells on [0, 2], sigma_a ~ U[0.2, 2], sigma_s ~
    U[0.5, 5], loss weights ~ N(0, 1)): forward + adjoint of all 2,000 cross
    sections against the forward pass alone, 1e7 histories."""
    rng = np.random.default_rng(3)
    M, L = 1000, np.float32(2.0)
    sig_a = (rng.uniform(0.2, 2.0, M).astype(np.float32) * L).astype(np.float32)
    sig_s = (rng.uniform(0.5, 5.0, M).astype(np.float32) * L).astype(np.float32)
    w = rng.standard_normal(M).astype(np.float32)
    with mcg.Context(mode=mode, device=device) as ctx:
        ctx.set_layers_xs([0], [M], [np.float32(1.0 / M)], sig_a, sig_s, MIN_W)
        ctx.adjoint_set_weights(w)
        ctx.simulate_source(0, n // 10)  # warm-up
        ctx.tally_reset()
        ctx.simulate_source(0, n)
        t_plain = ctx.last_kernel_ms() / 1e3
        ctx.adjoint_reset()
        ctx.adjoint_run(0, n, with_gradient=True)
        t_adj = ctx.last_kernel_ms() / 1e3
        ctx.adjoint_reset()
        ctx.adjoint_run(0, n, with_gradient=False)
        t_fwd = ctx.last_kernel_ms() / 1e3
    return {"value": n / t_adj, "unit": "histories/s", "forward_value": n / t_plain,
            "cost_vs_forward": t_adj / t_plain, "cost_vs_forward_with_loss": t_adj / t_fwd,
            "parameters": 2 * M,
            "workload": "1000 cells on [0,2], sigma_a~U[0.2,2], sigma_s~U[0.5,5], "
                        "loss weights~N(0,1), 1e7 histories from x=0 mu=1"}


def run_workload(args):
    """Full-size runs of the metric's other forms, one JSON line each:
    batch   configuration 2 (4096 slabs, ~5.9e8 histories): batched launch vs
            one launch per slab, autotuned;
    adjoint configuration 3 (1e7 histories, 2,000 parameters): forward +
            adjoint vs forward;
    fit     configuration 4 (64 slabs, 1e6 histories per slab and step, 200
            Adam steps): final relative L2 error of sigma_a, histories/s."""
    import importlib.util
    import torch
    torch.cuda.set_device(0)
    spec = importlib.util.spec_from_file_location(
        "mc_mpi_gb300", os.path.join(ROOT, "mc-mpi_gb300", "__init__.py"),
        submodule_search_locations=[os.path.join(ROOT, "mc-mpi_gb300")])
    mcg = importlib.util.module_from_spec(spec)
    sys.modules["mc_mpi_gb300"] = mcg
    spec.loader.exec_module(mcg)
    from mc_mpi_gb300 import workloads
    base = {"metric": METRIC, "unit": "histories/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic"}
    if args.workload == "batch":
        slabs, sigs, rates = workloads.config2(scale_histories=args.scale)
        n = sum(d["n_histories"] for d in slabs)
        with mcg.Context(mode=args.mode) as ctx, ClockSampler(0) as clk:
            ctx.set_tally_scale(30)
            ctx.batch_set(slabs, sigs, rates, MIN_W)
            tune = ctx.batch_autotune(0.05)
            if args.defer >= 0:
                ctx.batch_set_deferral(args.defer)
                tune["defer"] = args.defer
            ctx.batch_run()
            ms = []
            for _ in range(args.steps):
                ctx.batch_tally_reset()
                ctx.batch_run()
                ms.append(ctx.last_kernel_ms())
            c = ctx.counters()
            q = ctx.batch_tally_q()
            ctx.batch_tally_reset()
            ctx.batch_run_per_slab()
            ms_plain = ctx.last_kernel_ms()
            same = bool(np.array_equal(q, ctx.batch_tally_q()))
        t = statistics.median(ms) / 1e3
        base.update(value=n / t, ms_per_step=t * 1e3, gpu_launches=1,
                    config={"workload": "configuration 2: 4096 slabs, cells U{16..4096}, "
                                        "L~U[0.5,5], sigma_a~U[0.1,5], sigma_s~U[0,10], histories "
                                        f"log-uniform [1e3,1e6] x {args.scale}", "histories": n,
                            "mode": args.mode, "autotuned": tune, "l2": "inputs born on device"},
                    per_slab_value=n / (ms_plain / 1e3), speedup_vs_per_slab=ms_plain / 1e3 / t,
                    identical_tallies=same, steps_per_s=c["steps"] / t,
                    clocks=clk.summary())
    elif args.workload == "adjoint":
        base.update(bench_adjoint(mcg, args.mode, 0))
        base["config"] = {"workload": base.pop("workload"), "mode": args.mode}
    elif args.workload == "fit":
        with ClockSampler(0) as clk:
            r = bench_fit(mcg, 0, scale=args.scale)
        base.update(value=r["value"], ms_per_step=r["ms_per_adam_step"],
                    gpu_launches=r["gpu_launches"],
                    config={"workload": r["workload"], "mode": "fast"},
                    rel_l2_error=r["rel_l2_error"], rel_l2_error_start=r["rel_l2_error_start"],
                    loss_first=r["loss_first"], loss_last=r["loss_last"], clocks=clk.summary())
    elif args.workload == "worker":
        sigs, rates = physics()
        st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, NB_CELLS, N_LAYERS)
        with ClockSampler(0) as clk:
            r = bench_worker(mcg, args.mode, 0, st, m, dx, sigs, rates,
                             n=int(1e7 * args.scale))
        base.update(value=r["value"], gpu_launches=1, clocks=clk.summary(),
                    config={"workload": r["workload"], "mode": args.mode},
                    **{k: r[k] for k in ("fused_value", "ratio_vs_fused", "identical_tallies",
                                         "handoffs_per_history", "sync_value",
                                         "sync_ratio_vs_fused", "sync_cycles")})
    print(json.dumps(base))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="strict", choices=["strict", "fast"])
    ap.add_argument("--batch", type=int, default=N_TOTAL)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the e2e measurement (profiling runs)")
    ap.add_argument("--algorithm", default="history", choices=["history", "event"],
                    help="single-chain tracker: history-based (default) or event-based")
    ap.add_argument("--event-steps", type=int, default=4, help="event mode: events per pass")
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "batch", "adjoint", "fit", "worker"])
    ap.add_argument("--scale", type=float, default=1.0,
                    help="fraction of the configuration's histories (batch, fit)")
    ap.add_argument("--defer", type=int, default=-1,
                    help="batch: waiting lanes of the deferred full step after the autotuner "
                         "(0 off; default: the autotuner's choice)")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the fast, event, batched, adjoint, worker and fit measurements")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "plain":
        return run_workload(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
