"""Store-path measurements of the single-channel workloads other than the bench line.

  b0_1e6        B0 -> J/psi K pi: N=3, M=5.27934 at rest, m=(3.0969, 0.493677, 0.13957), 10^6
                events, Philox seed 0x3039: Decays + weight (104 B/event), FP64 and FP32_FIX
  b0_2e26       the same channel at 2^26 events
  pions10_2e26  ten pions from M=5.0 (10 x 0.13957) at 2^26 events (328 B/event)
For each, FP64 and FP32_FIX; at 2^26 events the maximum error of every FP32_FIX output against
the FP64 form of the same events is taken over ALL events (the FP64 kernels follow the
reference's arithmetic operation for operation).

Each line: kernel time (median of --reps CUDA-event timings after a warm-up), events/s, achieved
GB/s of algorithmic bytes against the measured HBM copy peak, and for FP32_FIX the max errors.
python -m hydra_gb300.config_bench [--reps 5] [--workloads b0_1e6,b0_2e26,pions10_2e26]
"""
from __future__ import annotations

import argparse
import json
import statistics
import sys
from pathlib import Path

K, PI = 0.493677, 0.13957


def hbm_peak():
    p = Path(__file__).resolve().parent.parent / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


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


def max_errors(torch, four, w, ref_four, ref_w, chunk=1 << 22):
    """max_k |dp_k|/E over events and max |dw|/w, chunked to bound temporary memory."""
    n = four.shape[1]
    e4 = ew = 0.0
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        d = (four[:, lo:hi] - ref_four[:, lo:hi]).abs().amax(dim=2) / ref_four[:, lo:hi, 0].abs()
        e4 = max(e4, float(d.max()))
        ew = max(ew, float(((w[lo:hi] - ref_w[lo:hi]).abs() / ref_w[lo:hi].abs()).max()))
    return e4, ew


def run_case(api, torch, name, masses, M, n, precisions, reps, peak, check):
    N = len(masses)
    ch = api.make_channel(masses, M, 0x3039, "philox")
    fn = api.functor_bw2(0, 1, 0.8955, 0.0473) if N > 2 else api.functor_mass2(0, 1)
    out = {}
    store = {}
    for prec in precisions:
        four = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        ms = timed(lambda: api.generate(ch, 0, four, w, None, precision=prec), torch, reps)
        stats = torch.zeros(3, dtype=torch.float64, device="cuda")
        ws = torch.empty(api.average_on_workspace_size(n), dtype=torch.uint8, device="cuda")
        ams = timed(lambda: api.average_on(ch, 0, n, fn, stats, ws, prec), torch, reps)
        b = n * (32 * N + 8)
        out[prec] = {"generate_ms": ms, "events_per_s": n / (ms / 1e3), "gbs": b / (ms / 1e3) / 1e9,
                     "hbm_frac": b / (ms / 1e3) / 1e9 / peak, "average_on_ms": ams,
                     "average_on_events_per_s": n / (ams / 1e3), "average_on": stats.tolist()}
        store[prec] = (four, w)
    if check and "fp64" in store and "fp32_fix" in store:
        e4, ew = max_errors(torch, store["fp32_fix"][0], store["fp32_fix"][1], store["fp64"][0], store["fp64"][1])
        m64, m32 = out["fp64"]["average_on"][0], out["fp32_fix"]["average_on"][0]
        out["max_rel_err_fp32_fix"] = {"four_vectors": e4, "weights": ew, "events_checked": n,
                                       "average_on_mean": abs(m32 - m64) / abs(m64)}
    return {"workload": name, "n_daughters": N, "mother_mass": M, "n_events": n, "bytes_per_event": 32 * N + 8,
            "peak_gbs": peak, **out}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--workloads", default="b0_1e6,b0_2e26,pions10_2e26")
    args = ap.parse_args(argv)
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import torch
    from hydra_gb300 import api
    peak, _ = hbm_peak()
    known = {
        "b0_1e6": ("B0 -> J/psi K pi, 10^6 events", [3.0969, K, PI], 5.27934, 10**6),
        "b0_2e26": ("B0 -> J/psi K pi, 2^26 events", [3.0969, K, PI], 5.27934, 1 << 26),
        "pions10_2e26": ("10 pions from M=5.0, 2^26 events", [PI] * 10, 5.0, 1 << 26),
    }
    cases = []
    for w in args.workloads.split(","):
        if w not in known:
            ap.error(f"unknown workload {w}; known: {', '.join(known)}")
        cases.append((*known[w], ("fp64", "fp32_fix"), True))
    for name, m, M, n, precs, check in cases:
        print(json.dumps(run_case(api, torch, name, m, M, n, precs, args.reps, peak, check)), flush=True)
        torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
