#!/usr/bin/env python3
"""Benchmark of the phase-space hot path on the N=5 D0 workload (2^24 events).

Workload (one "step"): mother M = 1.86484 GeV at rest -> K (0.493677) + 4 pi (0.13957),
Philox2x64-7, seed 0x3039, 2^24 events:
  * store path: Generate into Decays columns (5 x Vector4R) + generation-time weight +
    Decays::Unweight hit-or-miss flags  (32*5 + 8 + 1 = 169 bytes written per event);
  * storage-free AverageOn of |BW(m(K pi1))|^2, mass 0.8955 GeV, width 0.0473 GeV.
value = events of the step / step time (events/s).  Outputs written per step (2.84 GB)
exceed the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--precision fp64]

--impl reference times the reference itself on the host cores: Hydra's own Generate + AverageOn
(OMP backend, all threads), built from its headers by oracle/build_ref.sh, on a bounded sample of
the same workload (the oracle port where that build is absent).

After the contract's timed loop, `parts` adds the other workloads the metric names, each timed
once on the same GPU (skip with --no-parts):
  * the same N=5 workload at FP64 (the reference's arithmetic): Generate and AverageOn ms;
  * 256 channels of N in 2..10 (seeded mix, ~37 M events) as one batched graph launch: events/s,
    fraction of the HBM copy peak, max relative error against the FP64 form of the same events;
  * a seeded Poisson serving trace (2000 requests/s, 50% store / 50% AverageOn |BW|^2): p50/p99
    latency and served events/s of the continuous-batching server, the same trace through the
    plain FP64 one-launch-per-request form, and their throughput ratio;
  * a capacity sweep: the arrival rate raised until the server no longer keeps up, with the
    saturated events/s and its p99.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

N_DAUGHTERS = 5
MOTHER = 1.86484
MASSES = [0.493677, 0.13957, 0.13957, 0.13957, 0.13957]
SEED = 0x3039
BW = (0, 1, 0.8955, 0.0473)
UNWEIGHT_SEED = 0x180EC6D33CFD0ABA
BYTES_PER_EVENT = 32 * N_DAUGHTERS + 8 + 1
METRIC = "events/s (N=5 phase-space Generate+weights+unweight flags, then AverageOn |BW|^2)"


def workload_config(n, precision):
    return {"workload": "D0 -> K pi pi pi pi phase space: Generate (5 Vector4R + weight + unweight flag) "
                        "+ AverageOn |BW(m_K_pi1)|^2",
            "n_events": n, "n_daughters": N_DAUGHTERS, "mother_mass": MOTHER, "engine": "philox2x64-7",
            "seed": SEED, "precision": precision, "bytes_per_event_stored": BYTES_PER_EVENT,
            "l2": "outputs per step (%.2f GB) exceed L2; no flush" % (n * BYTES_PER_EVENT / 1e9)}


def measured_peak_hbm():
    p = REPO / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


DEFAULT_N = 1 << 24          # events per step of the D0 -> K pi pi pi pi bench workload


def profiled_traffic(precision):
    """DRAM bytes per launch of the store kernel from the committed ncu summary, if any."""
    p = REPO / "profiles" / "traffic.json"
    try:
        d = json.loads(p.read_text())
        return d.get(f"generate_n5_{precision}")
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0, period_ms=50):
        self.proc = None
        self.lines = []            # (host time, csv line)
        self.device_index = device_index
        self.period_ms = period_ms
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0:     # sampler running before timing
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def mark(self, t_start, t_end):
        """Timed-region bounds (host clock); samples within one period of it count."""
        self.window = (t_start - self.period_ms / 1e3, t_end + self.period_ms / 1e3)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.window is not None:
            inside = [ln for ln in lines if self.window[0] <= ln[0] <= self.window[1]]
            if not inside and lines:       # region shorter than a period: nearest sample
                mid = 0.5 * (self.window[0] + self.window[1])
                inside = [min(lines, key=lambda ln: abs(ln[0] - mid))]
            lines = inside
        for _, line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gpu" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------------------ CPU baseline

def cpu_sample(seconds=3.0, n_sample=1 << 21, nthreads=0):
    """Oracle port of the reference (FP64, -O3, OpenMP over all host threads): store step +
    AverageOn on chunks of the workload until `seconds` of wall time have elapsed.  All host
    cores are used even when a launcher (torchrun) has set OMP_NUM_THREADS=1 for its ranks."""
    import numpy as np
    from oracle import oracle as O
    if nthreads <= 0:
        nthreads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    O.build()
    ch = O.make_channel(MASSES, MOTHER, SEED, O.ENGINE_PHILOX)
    fn = O.make_functor(2, *BW)
    four = np.empty((N_DAUGHTERS, n_sample, 4))
    w = np.empty(n_sample)
    fl = np.empty(n_sample, dtype=np.uint8)
    O.store_step(ch, 0, 4096, UNWEIGHT_SEED, four[:, :4096].copy(), w[:4096].copy(), fl[:4096].copy(), nthreads)
    t0 = time.perf_counter()
    done, first = 0, 0
    while True:
        O.store_step(ch, first, n_sample, UNWEIGHT_SEED, four, w, fl, nthreads)
        O.average_on(ch, fn, first, n_sample, nthreads=nthreads if nthreads else 0)
        done += n_sample
        first += n_sample
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    cores = nthreads if nthreads > 0 else O.max_threads()
    return done / dt, cores, f"{done} events ({done // n_sample} chunks of {n_sample}), {dt:.2f} s wall"


REF_HARNESS = REPO / "oracle" / "_ref" / "ref_harness_omp"
REF_HARNESS_CPP = REPO / "oracle" / "_ref" / "ref_harness_cpp"


def host_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def reference_cpu(n_sample, reps):
    """The reference itself on the host cores: Hydra's PhaseSpace<5>::Generate into a Decays and
    AverageOn(|BW|^2) through its public API, OMP backend with every host thread, built from the
    unmodified Hydra headers by oracle/build_ref.sh (oracle/ref_harness.cpp, mode `time`).  Returns
    (events/s of each repetition, threads), or None where the harness was not built.  The
    reference's Generate drops the weight and stores no unweight flag, so it does less per event
    than the GPU step it is compared with."""
    return _time_harness(REF_HARNESS, n_sample, reps, host_threads())


def reference_cpu_single_core(n_sample=1 << 20, reps=2):
    """The same through the reference's CPP backend (one host thread), the single-core figure of
    the reference's CPU path; the median events/s after one warm-up, or None where not built."""
    r = _time_harness(REF_HARNESS_CPP, n_sample, reps, 1)
    return None if r is None else statistics.median(r[0][1:])


def _time_harness(harness, n_sample, reps, threads):
    if not harness.exists():
        return None
    cmd = [str(harness), "time", str(N_DAUGHTERS), "0", str(SEED), str(n_sample), repr(MOTHER),
           *map(repr, MASSES), "2", str(BW[0]), str(BW[1]), repr(BW[2]), repr(BW[3]), str(reps)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, check=True,
                       env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
    d = json.loads(r.stdout.strip().splitlines()[-1])
    rates = [n_sample / (g + a) for g, a in zip(d["generate_all"], d["average_all"])]
    return rates, int(d["threads"])


def run_reference(args):
    world, rank = dist_setup(args)
    if rank != 0:
        return 0
    n_sample = 1 << 22
    ref = reference_cpu(n_sample, args.warmup + args.steps)
    port_rate, port_cores, port_sample = cpu_sample(seconds=2.0)
    if ref is not None:
        rates, cores = ref
        value = statistics.median(rates[args.warmup:])
        kind = "reference"
        sample = (f"per step: {n_sample} events of the workload through the reference's own Generate + "
                  f"AverageOn (Hydra OMP backend, {cores} threads; oracle/ref_harness.cpp built by "
                  f"oracle/build_ref.sh); median of {args.steps} steps after {args.warmup} warm-up")
    else:
        value, cores, kind = port_rate, port_cores, "port"
        sample = f"{port_sample}; oracle port of Hydra's omp path (reference harness not built here)"
    n = args.n
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * n / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded counter-based RNG)",
        "config": workload_config(n, "fp64"), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": cores, "kind": kind, "sample": sample,
                         "port_value": port_rate, "port_sample": port_sample,
                         "single_core_value": reference_cpu_single_core(),
                         "single_core_sample": "2^20 events through the reference's CPP backend, one thread"},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------ GPU arm

def run_gpu(args):
    import torch
    world, rank = dist_setup(args)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from hydra_gb300 import api
    import hydra_gb300
    hydra_gb300.lib()          # raises if the CUDA library is missing: no fallback

    n = args.n
    first = rank * n           # weak scaling: each rank owns its own event range
    ch = api.make_channel(MASSES, MOTHER, SEED, "philox")
    fn = api.functor_bw2(*BW)
    dev = torch.device("cuda", local)
    four = torch.empty((N_DAUGHTERS, n, 4), dtype=torch.float64, device=dev)
    w = torch.empty(n, dtype=torch.float64, device=dev)
    fl = torch.empty(n, dtype=torch.uint8, device=dev)
    stats = torch.zeros(3, dtype=torch.float64, device=dev)
    ws = torch.empty(api.average_on_workspace_size(n) // 8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        api.generate(ch, first, four, w, fl, UNWEIGHT_SEED, args.precision, stream)
        if ev is not None:
            ev[1].record(stream)
        api.average_on(ch, first, n, fn, stats, ws, args.precision, stream)
        if ev is not None:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        barrier(world)
        torch.cuda.synchronize()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        h0 = time.time()
        t_start.record(stream)
        for k in range(args.steps):
            step(evs[k])
        t_end.record(stream)
        torch.cuda.synchronize()
        clocks.mark(h0, time.time())
        barrier(world)
    total_ms = t_start.elapsed_time(t_end)
    # the same two outputs from one pass (hps_generate_average), timed after the contract's loop
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    api.generate_average(ch, first, four, w, fl, fn, stats, ws, UNWEIGHT_SEED, args.precision, stream)
    f0.record(stream)
    for _ in range(args.steps):
        api.generate_average(ch, first, four, w, fl, fn, stats, ws, UNWEIGHT_SEED, args.precision, stream)
    f1.record(stream)
    torch.cuda.synchronize()
    fused_ms = f0.elapsed_time(f1) / args.steps
    gen_ms = [e[0].elapsed_time(e[1]) for e in evs]
    avg_ms = [e[1].elapsed_time(e[2]) for e in evs]
    total_ms = max_over_ranks(total_ms, world)
    ms_per_step = total_ms / args.steps
    value = world * n / (ms_per_step / 1e3)

    # end to end through the host-output entry point: Decays land in pinned host memory,
    # the AverageOn result is read back; copies are inside the timed region.
    e2e = None
    if not args.no_e2e:
        hfour = torch.empty((N_DAUGHTERS, n, 4), dtype=torch.float64).pin_memory()
        hw = torch.empty(n, dtype=torch.float64).pin_memory()
        hfl = torch.empty(n, dtype=torch.uint8).pin_memory()
        hstats = torch.zeros(3, dtype=torch.float64).pin_memory()

        def e2e_step():
            # Generate into pinned host Decays and AverageOn of the same events: one kernel writes
            # the events across the link and reduces meanwhile (hps_generate_average_host)
            api.generate_average_host(ch, first, hfour, hw, hfl, fn, stats, UNWEIGHT_SEED, args.precision, stream)
            hstats.copy_(stats, non_blocking=True)
            stream.synchronize()

        for _ in range(max(1, min(args.warmup, 2))):
            e2e_step()
        e2e_steps = max(2, min(args.steps, 5))
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        barrier(world)
        dt = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": world * n * e2e_steps / dt, "unit": "events/s", "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": n * BYTES_PER_EVENT + 24, "steps": e2e_steps,
               "note": "hps_generate_average_host: Decays into pinned host memory + AverageOn, result read back"}

    peak, peak_kind = measured_peak_hbm()
    gen_avg_s = statistics.mean(gen_ms) / 1e3
    achieved = n * BYTES_PER_EVENT / gen_avg_s / 1e9
    traffic = profiled_traffic(args.precision) if n == DEFAULT_N else None   # captured for the default size
    roofline = {"bound": "hbm", "kernel": "k_generate (store path)", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic, "algorithmic_bytes_per_launch": n * BYTES_PER_EVENT,
                "kernel_ms": statistics.mean(gen_ms)}

    precision_report = None
    if rank == 0 and not args.no_check:
        precision_report = check_against_oracle(api, torch, ch, fn, first, four, w, fl, stats, args)
        if not args.no_parts:
            precision_report["full_size_fp32_fix_vs_fp64"] = precision_part(api, torch)

    extra = {}
    if rank == 0 and not args.no_parts:
        peak_gbs = measured_peak_hbm()[0]
        extra["fp64_same_workload"] = fp64_part(api, torch, ch, fn, four, w, fl, stats, ws, first, n, stream)
        del four, w, fl, ws
        torch.cuda.empty_cache()
        extra["batched_256_channels"] = batch_part(api, torch, peak_gbs)
        extra["serving"] = serving_part(api, torch)
        extra["serving_capacity"] = capacity_part(api, torch)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, cores, sample = cpu_sample(seconds=2.0)
        cpu = {"value": rate, "unit": "events/s", "cores": cores, "kind": "port", "sample": sample}
        ref = reference_cpu(1 << 22, 4)
        if ref is not None:
            rates, rcores = ref
            cpu = {"value": statistics.median(rates[1:]), "unit": "events/s", "cores": rcores, "kind": "reference",
                   "sample": f"{1 << 22} events of the workload, Generate + AverageOn through the reference's own "
                             f"API (Hydra OMP backend), median of 3 after 1 warm-up",
                   "port_value": rate, "port_sample": sample,
                   "single_core_value": reference_cpu_single_core(),
                   "single_core_sample": "2^20 events through the reference's CPP backend, one thread"}

    csum = clocks.summary()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64fix",
            "data": "synthetic (seeded counter-based RNG; no dataset)",
            "config": workload_config(n, args.precision) | {"parallelism": f"replicas{world}"},
            "parts": {"generate_ms": statistics.mean(gen_ms), "average_on_ms": statistics.mean(avg_ms),
                      "generate_events_per_s": n / gen_avg_s,
                      "average_on_events_per_s": n / (statistics.mean(avg_ms) / 1e3),
                      "fused_generate_average_ms": fused_ms,
                      "fused_events_per_s": world * n / (fused_ms / 1e3),
                      "fused_note": "hps_generate_average: the same Decays, weights, flags and AverageOn "
                                    "result in one pass (bit-identical), not part of value", **extra},
            "max_rel_err": precision_report,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": (4 if args.precision == "fp32_fix" else 3) * args.steps, "clocks": csum,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def timed_ms(torch, fn, reps, stream=None):
    """Median of `reps` CUDA-event timings of fn() after one untimed call."""
    fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return statistics.median(out)


def fp64_part(api, torch, ch, fn, four, w, fl, stats, ws, first, n, stream):
    """The bench workload at FP64 (the reference's arithmetic), Generate and AverageOn timed alone."""
    g = timed_ms(torch, lambda: api.generate(ch, first, four, w, fl, UNWEIGHT_SEED, "fp64", stream), 3, stream)
    a = timed_ms(torch, lambda: api.average_on(ch, first, n, fn, stats, ws, "fp64", stream), 3, stream)
    return {"generate_ms": g, "average_on_ms": a, "generate_events_per_s": n / (g / 1e3),
            "average_on_events_per_s": n / (a / 1e3), "pipeline_events_per_s": n / ((g + a) / 1e3)}


def precision_part(api, torch, total=1 << 26, chunk=1 << 22):
    """The precision workloads at full size: every one of 2^26 events of ten pions from M = 5.0 GeV
    and of B0 -> J/psi K pi, FP32_FIX against the FP64 form of the same events (which follows the
    reference's arithmetic operation for operation)."""
    out = {}
    for name, M, masses in (("ten_pions_M5_2e26", 5.0, [0.13957] * 10),
                            ("b0_jpsi_k_pi_2e26", 5.27934, [3.0969, 0.493677, 0.13957])):
        N = len(masses)
        ch = api.make_channel(masses, M, SEED, "philox")
        a = torch.empty((N, chunk, 4), dtype=torch.float64, device="cuda")
        b = torch.empty_like(a)
        wa = torch.empty(chunk, dtype=torch.float64, device="cuda")
        wb = torch.empty_like(wa)
        e4 = ew = 0.0
        for first in range(0, total, chunk):
            api.generate(ch, first, a, wa, None, precision="fp32_fix")
            api.generate(ch, first, b, wb, None, precision="fp64")
            e4 = max(e4, float(((a - b).abs().amax(dim=2) / b[:, :, 0]).max()))
            ew = max(ew, float(((wa - wb).abs() / wb).max()))
        out[name] = {"four_vectors": e4, "weights": ew, "events_checked": total}
        del a, b, wa, wb
        torch.cuda.empty_cache()
    return out


def batch_part(api, torch, peak, n_channels=256, check_channels=256):
    """256 seeded channels (N uniform in 2..10, masses from the menu, events log-uniform 1e3..1e6),
    store path, one graph launch of the batched FP32_FIX kernels after the project's autotuner."""
    from hydra_gb300 import batch_bench as BB
    chans = BB.make_channels(n_channels)
    total = sum(c[3] for c in chans)
    nbytes = sum(c[3] * (32 * c[0] + 8) for c in chans)
    outs, items, hch = [], [], []
    for N, m, M, n, seed in chans:
        ch = api.make_channel(m, M, seed, "philox")
        four = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        outs.append((four, w))
        hch.append(ch)
        items.append(api.store_item(ch, 0, four, w))
    plan = api.BatchPlan(len(items), 1)
    plan.set_items(items)
    t0 = time.perf_counter()
    tuning = plan.autotune(None)
    tune_s = time.perf_counter() - t0
    ms = timed_ms(torch, plan.launch, 5)
    plan.launch()
    torch.cuda.synchronize()
    # every event of the first `check_channels` channels against the FP64 form of the same events
    e4 = ew = 0.0
    for ch, (four, w) in list(zip(hch, outs))[:check_channels]:
        f64, w64 = torch.empty_like(four), torch.empty_like(w)
        api.generate(ch, 0, f64, w64, None, precision="fp64")
        e4 = max(e4, float(((four - f64).abs().amax(dim=2) / f64[:, :, 0]).max()))
        ew = max(ew, float(((w - w64).abs() / w64).max()))
    checked = sum(c[3] for c in chans[:check_channels])
    plan.close()
    del outs, items
    torch.cuda.empty_cache()
    gbs = nbytes / (ms / 1e3) / 1e9
    return {"workload": f"{n_channels} channels, N in 2..10, {total} events, store path (32N+8 B/event)",
            "events": total, "ms": ms, "events_per_s": total / (ms / 1e3), "gbs": gbs, "hbm_frac": gbs / peak,
            "tuning": {"ctas_per_sm": tuning[0], "store_tile_events": tuning[1],
                       "kernel_form": ["per_N", "one_kernel"][tuning[2]], "threads_per_event": max(1, tuning[3]),
                       "autotune_s": tune_s},
            "max_rel_err": {"four_vectors": e4, "weights": ew, "events_checked": checked,
                            "against": "FP64 form of the same events"}}


def serving_part(api, torch, rate=2000.0, duration=3.0, budget_gb=80.0, drain_plain=4.0):
    """A seeded Poisson trace through the continuous-batching server, then the same trace through
    the plain FP64 one-launch-per-request form (its unfinished requests are reported as backlog)."""
    from hydra_gb300 import serve_bench as SB
    trace = SB.make_trace(rate, duration, 12345)
    offered = sum(x[4] for x in trace)
    served = SB.run_batched(api, trace, int(budget_gb * (1 << 30)), 30.0)
    torch.cuda.empty_cache()
    plain = SB.run_plain(api, torch, trace, "fp64", drain_plain)
    torch.cuda.empty_cache()
    ratio = served["events_per_s"] / plain["events_per_s"] if plain["events_per_s"] else None
    return {"workload": f"Poisson {rate:g} req/s for {duration:g} s, seed 12345 ({len(trace)} requests, "
                        f"{offered} events), 50% store / 50% AverageOn |BW|^2, {budget_gb:g} GB budget",
            "offered_events_per_s": offered / duration,
            "served_fp32fix_batched": served, "plain_fp64_per_request": plain,
            "throughput_ratio_vs_plain_fp64": ratio}


def capacity_part(api, torch, rates=(2000.0, 8000.0, 32000.0), duration=1.0, budget_gb=80.0):
    """Arrival rate raised until the served throughput falls behind the offered load: the
    saturated events/s of the server and the p99 latency at that load."""
    from hydra_gb300 import serve_bench as SB
    points = []
    for i, rate in enumerate(rates):
        trace = SB.make_trace(rate, duration, 777 + i)
        offered = sum(x[4] for x in trace) / duration
        r = SB.run_batched(api, trace, int(budget_gb * (1 << 30)), 60.0)
        torch.cuda.empty_cache()
        points.append({"rate_req_per_s": rate, "requests": len(trace), "offered_events_per_s": offered,
                       "served_events_per_s": r["events_per_s"], "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"],
                       "completed": r["completed"]})
        if r["events_per_s"] < 0.8 * offered:
            break
    sat = max(points, key=lambda p: p["served_events_per_s"])
    return {"points": points, "saturated_events_per_s": sat["served_events_per_s"], "p99_ms_at_saturation":
            sat["p99_ms"], "saturated": points[-1]["served_events_per_s"] < 0.8 * points[-1]["offered_events_per_s"]}


def check_against_oracle(api, torch, ch, fn, first, four, w, fl, stats, args, sample=1 << 18):
    """Maximum relative error of this run's outputs against the FP64 oracle on the first `sample`
    events of the step (four-vectors energy-normalised, weights relative, flags counted) and of
    the AverageOn mean on the first 2^22 events."""
    import numpy as np
    from oracle import oracle as O
    och = O.make_channel(MASSES, MOTHER, SEED, O.ENGINE_PHILOX)
    m = min(sample, args.n)
    rfour, rw = O.generate(och, first, m)
    g4 = four[:, :m].cpu().numpy()
    gw = w[:m].cpu().numpy()
    e4 = float((np.abs(g4 - rfour).max(axis=2) / rfour[:, :, 0]).max())
    ok = rw > 0
    ew = float((np.abs(gw[ok] - rw[ok]) / rw[ok]).max()) if ok.any() else 0.0
    u = O.unweight_uniforms(UNWEIGHT_SEED, first, m)
    rfl = (rw / och.max_weight > u).astype(np.uint8)
    nfl = int((fl[:m].cpu().numpy() != rfl).sum())
    na = min(1 << 22, args.n)
    out = torch.zeros(3, dtype=torch.float64, device=four.device)
    api.average_on(ch, first, na, fn, out, None, args.precision)
    mean = float(out[0].item())
    rmean, rm2, rW = O.average_on(och, O.make_functor(2, *BW), first, na, nthreads=0)
    return {"four_vectors": e4, "weights": ew, "flags_differing": nfl, "sample_events": m,
            "average_on_mean": abs(mean - rmean) / abs(rmean), "average_on_sigma_rel": (rm2 ** 0.5 / rW) / abs(rmean),
            "average_on_events": na,
            "measure": "four-vectors max_k |dp_k|/E; weights |dw|/w; AverageOn |dmean|/mean vs the oracle "
                       "(FP64, the reference's arithmetic)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--precision", choices=["fp64", "fp32_fix"], default="fp32_fix")
    ap.add_argument("--n", type=int, default=DEFAULT_N)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-parts", action="store_true", help="skip the FP64, batch and serving parts")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
