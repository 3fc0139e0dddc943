"""Batched-channels benchmark: 256 decay channels of uneven N and event counts.

Workload (seeded): for channel c, N uniform in 2..10, each daughter mass drawn from
{0.13957, 0.493677, 0.938272, 1.86484} GeV, mother mass uniform in [1.2 sum(m), sum(m) + 6] GeV at
rest, events log-uniform in [1e3, 1e6] (about 37M in total), Philox seed 0x3039 + c; store path
(Decays columns + generation-time weight, 32N + 8 bytes per event).

Compared on the same GPU:
  batched   one graph launch of the persistent FP32_FIX kernels, one per N (hps_batch_*), autotuned shape
  plain64   one hps_generate launch per channel, FP64 arithmetic (the reference's)
  plain32   one hps_generate launch per channel, FP32_FIX arithmetic
Prints one JSON line.  python -m hydra_gb300.batch_bench [--channels 256] [--reps 5] [--tuning C,T[,FORM]]
"""
from __future__ import annotations

import argparse
import json
import statistics
import sys
import time
from pathlib import Path

import numpy as np

MASS_MENU = [0.13957, 0.493677, 0.938272, 1.86484]


def make_channels(n_channels: int, seed: int = 0x3039):
    rng = np.random.default_rng(seed)
    chans = []
    for c in range(n_channels):
        N = int(rng.integers(2, 11))
        m = [float(x) for x in rng.choice(MASS_MENU, size=N)]
        sm = sum(m)
        M = float(rng.uniform(1.2 * sm, sm + 6.0))
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(1e6))))
        chans.append((N, m, M, n, seed + c))
    return chans


def timed(fn, torch, reps):
    fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return statistics.median(out)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--channels", type=int, default=256)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--tune-cache", default=None)
    ap.add_argument("--tuning", default=None,
                    help="CTAS_PER_SM,STORE_TILE[,FORM[,THREADS_PER_EVENT]] instead of autotuning")
    args = ap.parse_args(argv)
    import torch
    from hydra_gb300 import api

    chans = make_channels(args.channels)
    total = sum(c[3] for c in chans)
    nbytes = sum(c[3] * (32 * c[0] + 8) for c in chans)
    outs = []
    items = []
    hch = []
    for N, m, M, n, seed in chans:
        ch = api.make_channel(m, M, seed, "philox")
        four = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        outs.append((four, w))
        hch.append(ch)
        items.append(api.store_item(ch, 0, four, w))

    plan = api.BatchPlan(len(items), 1)
    plan.set_items(items)
    if args.tuning:
        plan.set_tuning(*(int(x) for x in args.tuning.split(",")))
        tuning = plan.tuning()
    else:
        tuning = plan.autotune(args.tune_cache)
    t_batch = timed(plan.launch, torch, args.reps)

    def plain(prec):
        def run():
            for ch, (four, w) in zip(hch, outs):
                api.generate(ch, 0, four, w, None, precision=prec)
        return run

    t_plain32 = timed(plain("fp32_fix"), torch, args.reps)
    t_plain64 = timed(plain("fp64"), torch, max(1, min(args.reps, 3)))

    # the batch wrote the same bytes the per-channel FP32_FIX launches write
    ref = []
    for ch, (four, w) in zip(hch[:8], outs[:8]):
        f2, w2 = torch.empty_like(four), torch.empty_like(w)
        api.generate(ch, 0, f2, w2, None, precision="fp32_fix")
        ref.append((f2, w2))
    plan.launch()
    torch.cuda.synchronize()
    same = all(torch.equal(a, c) and torch.equal(b, d) for (a, b), (c, d) in zip(outs[:8], ref))

    peak = None
    try:
        peak = json.loads((Path(__file__).resolve().parent.parent / "MEASURED_PEAKS.json").read_text())["hbm_gbs"]
    except Exception:
        pass
    gbs = nbytes / (t_batch / 1e3) / 1e9
    line = {
        "workload": f"{args.channels} channels, N in 2..10, {total} events, store path (32N+8 B/event)",
        "events": total, "bytes": nbytes,
        "batched": {"ms": t_batch, "events_per_s": total / (t_batch / 1e3), "gbs": gbs,
                    "hbm_frac": (gbs / peak) if peak else None, "tuning": {"ctas_per_sm": tuning[0],
                                                                           "store_tile_events": tuning[1],
                                                                           "kernel_form": ["per_N", "one_kernel"][tuning[2]],
                                                                           "threads_per_event": max(1, tuning[3])}},
        "plain_fp64_per_channel": {"ms": t_plain64, "events_per_s": total / (t_plain64 / 1e3)},
        "plain_fp32fix_per_channel": {"ms": t_plain32, "events_per_s": total / (t_plain32 / 1e3)},
        "speedup_vs_plain_fp64": t_plain64 / t_batch,
        "batch_equals_alone": same,
    }
    print(json.dumps(line), flush=True)
    plan.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
