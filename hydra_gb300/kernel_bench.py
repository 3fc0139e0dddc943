"""One entry point on one channel, timed alone: Generate, AverageOn or Evaluate.

Channels (Philox, seed 0x3039, mother at rest):
  2    D0 -> K pi             M = 1.86484, m = (0.493677, 0.13957)
  3    B0 -> J/psi K pi       M = 5.27934, m = (3.0969, 0.493677, 0.13957)
  4, 5 D0 -> K + 3 or 4 pi    M = 1.86484, m = (0.493677, 0.13957 x (N-1))
  6-9  six to nine pions     M = 3.0,     m = 0.13957 x N
(--mother / --masses replace them, e.g. to time a channel that takes the float-float boosts)
  10   ten pions             M = 5.0,     m = 0.13957 x 10
The functor of AverageOn and Evaluate is |BW(m_01)|^2 (m0 = 0.8955, G0 = 0.0473); Evaluate
stores the generation-time weight and the functor value (16 bytes per event), Generate the
Decays columns, the weight and the unweight flag (32N + 9 bytes per event); dalitz bins
m^2(d0 d1) against m^2(d1 d2) on a 64 x 48 grid as the events are made (N >= 3).

Prints one JSON line: ms per call (CUDA events, mean of --steps calls after --warmup), events/s
and, for the storing forms, the GB/s of algorithmic bytes written.

    python -m hydra_gb300.kernel_bench --op evaluate --n-daughters 5 --events 16777216 --precision fp32_fix
"""
from __future__ import annotations

import argparse
import json

CHANNELS = {
    2: (1.86484, [0.493677, 0.13957]),
    3: (5.27934, [3.0969, 0.493677, 0.13957]),
    4: (1.86484, [0.493677] + [0.13957] * 3),
    5: (1.86484, [0.493677] + [0.13957] * 4),
    6: (3.0, [0.13957] * 6),
    7: (3.0, [0.13957] * 7),
    8: (3.0, [0.13957] * 8),
    9: (3.0, [0.13957] * 9),
    10: (5.0, [0.13957] * 10),
}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", choices=["generate", "average", "evaluate", "dalitz"], default="evaluate")
    ap.add_argument("--n-daughters", default="5", help="N, or a comma-separated list of N (one line each)")
    ap.add_argument("--events", type=int, default=1 << 24)
    ap.add_argument("--precision", choices=["fp64", "fp32_fix"], default="fp32_fix")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--mother", type=float, default=None, help="mother mass in place of the channel's")
    ap.add_argument("--bare", action="store_true", help="generate the Decays columns only (no weights, no flags)")
    ap.add_argument("--masses", default=None, help="comma-separated daughter masses in place of the channel's")
    args = ap.parse_args(argv)
    ns = [int(x) for x in args.n_daughters.split(",")]
    if any(N not in CHANNELS for N in ns):
        ap.error(f"--n-daughters takes values in {sorted(CHANNELS)}")
    for N in ns:
        run(ap, args, N)
    return 0


def run(ap, args, N):
    import torch
    from hydra_gb300 import api

    n = args.events
    M, masses = CHANNELS[N]
    if args.masses:
        masses = [float(x) for x in args.masses.split(",")]
        if len(masses) != N:
            ap.error("--masses needs one mass per daughter")
    if args.mother is not None:
        M = args.mother
    ch = api.make_channel(masses, M, 0x3039, "philox")
    fn = api.functor_bw2(0, 1, 0.8955, 0.0473)
    dev = "cuda"
    stored = 0
    if args.op == "generate":
        four = torch.empty((N, n, 4), dtype=torch.float64, device=dev)
        w = torch.empty(n, dtype=torch.float64, device=dev)
        fl = torch.empty(n, dtype=torch.uint8, device=dev)
        stored = n * (32 * N + (0 if args.bare else 9))

        def step():
            if args.bare:
                api.generate(ch, 0, four, None, None, precision=args.precision)
            else:
                api.generate(ch, 0, four, w, fl, precision=args.precision)
    elif args.op == "dalitz":
        # Generate + Dalitz histogram fused: m^2(d0 d1) against m^2(d1 d2) on a 64 x 48 grid over
        # their kinematic ranges, weighted by the generation-time weight; nothing stored
        lo = ((masses[0] + masses[1]) ** 2, (masses[1] + masses[2]) ** 2)
        hi = ((M - sum(masses[2:])) ** 2, (M - masses[0] - sum(masses[3:])) ** 2)
        hist = api.hist2d((0, 1), (1, 2), (64, 48), lo, hi)
        bins = torch.empty(64 * 48 + 2, dtype=torch.float64, device=dev)

        def step():
            api.generate_dalitz(ch, 0, n, hist, bins, "phsp", args.precision)
    elif args.op == "average":
        out = torch.empty(3, dtype=torch.float64, device=dev)
        ws = torch.empty(api.average_on_workspace_size(n), dtype=torch.uint8, device=dev)

        def step():
            api.average_on(ch, 0, n, fn, out, ws, precision=args.precision)
    else:
        w = torch.empty(n, dtype=torch.float64, device=dev)
        f = torch.empty(n, dtype=torch.float64, device=dev)
        stored = n * 16

        def step():
            api.evaluate(ch, 0, n, [fn], w, [f], precision=args.precision)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps):
        step()
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.steps
    line = {"op": args.op, "n_daughters": N, "mother_mass": M, "events": n, "precision": args.precision, "ms": ms,
            "events_per_s": n / ms * 1e3}
    if stored:
        line["stored_gbs"] = stored / ms / 1e6
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    raise SystemExit(main())
