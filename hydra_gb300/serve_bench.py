"""Serving benchmark: Poisson request arrivals against the continuous-batching server.

Trace (seeded): arrivals at `rate` requests/s for `duration` s; each request is one channel with
N uniform in 2..10, daughter masses from {0.13957, 0.493677, 0.938272, 1.86484} GeV, mother mass
uniform in [1.2 sum(m), sum(m) + 6] GeV at rest, events log-uniform in [1e4, 1e7]; half are
Generate-into-Decays (columns + weights), half AverageOn of |BW(m_01)|^2 (0.8955, 0.0473 GeV).

  batched    hps_server: admission under an HBM budget, continuous batching into the persistent
             FP32_FIX kernel; outputs released as soon as each request finishes
  plain      one launch per request in arrival order (hps_generate / hps_average_on), FP64 by
             default; requests still queued when the drain limit is reached are reported as backlog

Latency = finish - arrival; throughput = completed events / (last finish - first arrival).
python -m hydra_gb300.serve_bench [--rate 2000] [--duration 10] [--budget-gb 80] [--plain fp64]
"""
from __future__ import annotations

import argparse
import json
import queue
import sys
import threading
import time

import numpy as np

MASS_MENU = [0.13957, 0.493677, 0.938272, 1.86484]


def make_trace(rate: float, duration: float, seed: int):
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        N = int(rng.integers(2, 11))
        m = [float(x) for x in rng.choice(MASS_MENU, size=N)]
        M = float(rng.uniform(1.2 * sum(m), sum(m) + 6.0))
        n = int(np.exp(rng.uniform(np.log(1e4), np.log(1e7))))
        mode = 0 if rng.random() < 0.5 else 1
        out.append((t, N, m, M, n, mode, len(out)))
    return out


def percentiles(lat):
    if not lat:
        return {"p50_ms": None, "p99_ms": None, "mean_ms": None}
    a = np.asarray(lat) * 1e3
    return {"p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)), "mean_ms": float(a.mean())}


def run_batched(api, trace, budget_bytes, drain_s, slice_events=1 << 22):
    server = api.Server(budget_bytes=budget_bytes, slice_events=slice_events, max_batch_items=1024,
                        max_inflight=8192)
    reqs = []
    for (t, N, m, M, n, mode, c) in trace:
        ch = api.make_channel(m, M, 0x3039 + c, "philox")
        reqs.append(api.store_request(ch, 0, n) if mode == 0 else
                    api.average_request(ch, 0, n, api.functor_bw2(0, 1, 0.8955, 0.0473)))
    t0 = time.monotonic()
    submit_err = []

    def submitter():
        try:
            for (t, *_), r in zip(trace, reqs):
                d = t0 + t - time.monotonic()
                if d > 0:
                    time.sleep(d)
                server.submit(r)
        except Exception as e:           # reported, not raised from the thread
            submit_err.append(repr(e))

    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    lat, events, first_sub, last_done, done = [], 0, None, None, 0
    deadline = t0 + trace[-1][0] + drain_s if trace else t0
    while done < len(trace) and time.monotonic() < deadline:
        got = server.next_done(0.5)
        if got is None:
            continue
        ticket, res = got
        if res.status == 0:
            lat.append(res.t_done - res.t_submit)
            events += res.n_events
            first_sub = res.t_submit if first_sub is None else min(first_sub, res.t_submit)
            last_done = res.t_done if last_done is None else max(last_done, res.t_done)
        done += 1
        server.release(ticket)
    th.join(timeout=5)
    st = server.stats()
    server.close()
    span = (last_done - first_sub) if last_done else float("nan")
    return {"completed": done, "events": events, "span_s": span, "events_per_s": events / span if done else 0.0,
            **percentiles(lat), "launches": st["launches"], "peak_bytes": st["bytes_peak"],
            "submit_errors": submit_err[:3]}


def run_plain(api, torch, trace, precision, drain_s):
    q = queue.Queue()
    t0 = time.monotonic()
    stop = threading.Event()

    def submitter():
        for item in trace:
            d = t0 + item[0] - time.monotonic()
            if d > 0:
                time.sleep(d)
            q.put((time.monotonic(), item))
            if stop.is_set():
                return

    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    lat, events, done = [], 0, 0
    first_sub, last_done = None, None
    deadline = t0 + (trace[-1][0] if trace else 0) + drain_s
    fn = api.functor_bw2(0, 1, 0.8955, 0.0473)
    stats = torch.zeros(3, dtype=torch.float64, device="cuda")
    while done < len(trace) and time.monotonic() < deadline:
        try:
            t_sub, (t, N, m, M, n, mode, c) = q.get(timeout=0.5)
        except queue.Empty:
            continue
        ch = api.make_channel(m, M, 0x3039 + c, "philox")
        if mode == 0:
            four = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
            w = torch.empty(n, dtype=torch.float64, device="cuda")
            api.generate(ch, 0, four, w, None, precision=precision)
        else:
            api.average_on(ch, 0, n, fn, stats, None, precision=precision)
        torch.cuda.synchronize()
        t_done = time.monotonic()
        if mode == 0:
            del four, w
        lat.append(t_done - t_sub)
        events += n
        first_sub = t_sub if first_sub is None else min(first_sub, t_sub)
        last_done = t_done
        done += 1
    stop.set()
    span = (last_done - first_sub) if last_done else float("nan")
    return {"completed": done, "backlog": len(trace) - done, "events": events, "span_s": span,
            "events_per_s": events / span if done else 0.0, **percentiles(lat),
            "note": "latencies of completed requests only"}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--duration", type=float, default=10.0)
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--budget-gb", type=float, default=80.0)
    ap.add_argument("--plain", choices=["fp64", "fp32_fix", "none"], default="fp64")
    ap.add_argument("--drain", type=float, default=20.0, help="seconds after the last arrival to keep serving")
    ap.add_argument("--slice-events", type=int, default=1 << 22, help="largest store slice per launch")
    args = ap.parse_args(argv)
    import torch
    from hydra_gb300 import api
    trace = make_trace(args.rate, args.duration, args.seed)
    total_events = sum(x[4] for x in trace)
    batched = run_batched(api, trace, int(args.budget_gb * (1 << 30)), args.drain, args.slice_events)
    line = {"workload": f"Poisson {args.rate:g} req/s for {args.duration:g} s ({len(trace)} requests, "
                        f"{total_events} events offered), 50% store / 50% AverageOn |BW|^2",
            "offered_events_per_s": total_events / args.duration, "slice_events": args.slice_events,
            "batched_fp32fix": batched}
    if args.plain != "none":
        torch.cuda.empty_cache()
        plain = run_plain(api, torch, trace, args.plain, args.drain)
        line[f"plain_{args.plain}_per_request"] = plain
        if plain["events_per_s"]:
            line["throughput_ratio"] = batched["events_per_s"] / plain["events_per_s"]
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
