"""The reference's own CUDA functors on the GPU -- TEST INFRASTRUCTURE ONLY.

Loads ``_ref/ref_gpu.cubin`` (``ref_gpu.cu`` compiled for sm_103a from the unmodified
Hydra headers by ``build_ref.sh``) with the CUDA driver API, in the CUDA context torch
uses, and launches its kernels on torch's current stream:

* ``generate``   -- hydra::detail::DecayMother::operator()(evt) per event, the N
  Vector4R it returns stored as N columns (the Decays layout), as Generate does;
* ``average_bw`` -- hydra::detail::AverageMother::operator()(evt) with the
  Breit-Wigner |BW(m_ij)|^2 functor, folded with AddStatsPHSP, as AverageOn does;
* ``evaluate`` -- hydra::detail::EvalMother (Evaluate) with |BW|^2 and m^2 functors;
* ``generate_mothers`` / ``average_mothers_bw`` -- DecayMothers / AverageMothers with one
  mother per event.

The tests use it to check the product against the reference's own CUDA arithmetic;
``python oracle/ref_gpu.py`` times it on the GPU at the benchmark workloads and prints
one JSON line per case.  The product never loads it.  The cubin needs the Hydra tree
to build; where it is absent ``available()`` is False.
"""
from __future__ import annotations

import ctypes
import functools
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "ref_gpu.cubin"
THREADS = 256
AVG_BLOCKS = 152 * 8
ENGINES = {0: "philox", 1: "squares3"}


def available() -> bool:
    return CUBIN.exists()


@functools.lru_cache(maxsize=None)
def _mother_args(n: int):
    class MotherArgs(ctypes.Structure):
        _fields_ = [("seed", ctypes.c_uint64), ("ecm", ctypes.c_double), ("maxw", ctypes.c_double),
                    ("beta", ctypes.c_double * 3), ("masses", ctypes.c_double * n)]
    return MotherArgs


class _BW(ctypes.Structure):
    _fields_ = [("i", ctypes.c_int32), ("j", ctypes.c_int32), ("a", ctypes.c_double), ("b", ctypes.c_double)]


@functools.lru_cache(maxsize=None)
def _mothers_args(n: int):
    class MothersArgs(ctypes.Structure):
        _fields_ = [("seed", ctypes.c_uint64), ("ecm", ctypes.c_double), ("maxw", ctypes.c_double),
                    ("masses", ctypes.c_double * n)]
    return MothersArgs


_state = {}


def _driver():
    if "cu" not in _state:
        cu = ctypes.CDLL("libcuda.so.1")
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                ctypes.POINTER(ctypes.c_void_p),
                                                                                ctypes.c_void_p]
        _state["cu"] = cu
    return _state["cu"]


def _check(rc: int, what: str):
    if rc != 0:
        msg = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(msg))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({(msg.value or b'?').decode()})")


def _function(name: str):
    import torch
    if "mod" not in _state:
        if not available():
            raise FileNotFoundError(f"{CUBIN} not built (oracle/build_ref.sh needs the Hydra sources)")
        torch.zeros(1, device="cuda")          # makes torch's (primary) context current on this thread
        mod = ctypes.c_void_p()
        _check(_driver().cuModuleLoad(ctypes.byref(mod), str(CUBIN).encode()), "cuModuleLoad")
        _state["mod"] = mod
        _state["fn"] = {}
    fns = _state["fn"]
    if name not in fns:
        f = ctypes.c_void_p()
        _check(_driver().cuModuleGetFunction(ctypes.byref(f), _state["mod"], name.encode()), name)
        fns[name] = f
    return fns[name]


def _launch(name: str, grid: int, args):
    import torch
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _check(_driver().cuLaunchKernel(_function(name), grid, 1, 1, THREADS, 1, 1, 0, stream, params, None), name)


def _args(ch):
    n = ch.n_daughters
    a = _mother_args(n)()
    a.seed = ch.seed
    a.ecm = ch.ecm
    a.maxw = ch.max_weight
    for k in range(3):
        a.beta[k] = ch.beta[k]
    for k in range(n):
        a.masses[k] = ch.masses[k]
    return a


def generate(ch, first: int, n: int, out=None):
    """The reference's DecayMother over events [first, first+n): float64 (N, n, 4) on cuda.

    ``ch`` is any object with the oracle's Channel fields (n_daughters, engine, seed,
    ecm, max_weight, beta, masses)."""
    import torch
    N = ch.n_daughters
    if out is None:
        out = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
    cols = torch.tensor([out[i].data_ptr() for i in range(N)], dtype=torch.int64, device="cuda")
    if n:
        grid = (n + THREADS - 1) // THREADS
        _launch(f"ref_generate_{N}_{ENGINES[ch.engine]}", grid,
                [_args(ch), ctypes.c_uint64(first), ctypes.c_uint64(n), ctypes.c_void_p(cols.data_ptr())])
    out._ref_cols = cols            # the pointer array must outlive the launch
    return out


def _margs(ch):
    n = ch.n_daughters
    a = _mothers_args(n)()
    a.seed = ch.seed
    a.ecm = ch.ecm
    a.maxw = ch.max_weight
    for k in range(n):
        a.masses[k] = ch.masses[k]
    return a


def _grid(n: int) -> int:
    return max(1, (n + THREADS - 1) // THREADS)


def evaluate(ch, first: int, n: int, bw=(0, 1, 0.8955, 0.0473), m2=(0, 1)):
    """The reference's EvalMother with two functors, |BW(m_ij)|^2 and m^2(p_k + p_l): float64
    cuda tensors (weight, bw, m2) of n events each."""
    import torch
    w, fb, fm = (torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(3))
    if n:
        _launch(f"ref_evaluate_{ch.n_daughters}_{ENGINES[ch.engine]}", _grid(n),
                [_args(ch), _BW(*bw), _BW(m2[0], m2[1], 0.0, 0.0), ctypes.c_uint64(first), ctypes.c_uint64(n),
                 ctypes.c_void_p(w.data_ptr()), ctypes.c_void_p(fb.data_ptr()), ctypes.c_void_p(fm.data_ptr())])
    return w, fb, fm


def generate_mothers(ch, first: int, mothers):
    """The reference's DecayMothers: mothers is a float64 (n, 4) cuda tensor; returns (N, n, 4)."""
    import torch
    N, n = ch.n_daughters, mothers.shape[0]
    out = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
    cols = torch.tensor([out[i].data_ptr() for i in range(N)], dtype=torch.int64, device="cuda")
    if n:
        _launch(f"ref_generate_mothers_{N}_{ENGINES[ch.engine]}", _grid(n),
                [_margs(ch), ctypes.c_uint64(first), ctypes.c_uint64(n), ctypes.c_void_p(mothers.data_ptr()),
                 ctypes.c_void_p(cols.data_ptr())])
    out._ref_cols = cols
    return out


def average_mothers_bw(ch, i: int, j: int, a: float, b: float, first: int, mothers):
    """The reference's AverageMothers with |BW(m_ij)|^2 (indices count the mother as 0);
    returns (mean, sqrt(M2)/W)."""
    import torch
    n = mothers.shape[0]
    grid = max(1, min(_grid(n), AVG_BLOCKS))
    partial = torch.empty((grid, 3), dtype=torch.float64, device="cuda")
    _launch(f"ref_average_mothers_bw_{ch.n_daughters}_{ENGINES[ch.engine]}", grid,
            [_margs(ch), _BW(i, j, a, b), ctypes.c_uint64(first), ctypes.c_uint64(n),
             ctypes.c_void_p(mothers.data_ptr()), ctypes.c_void_p(partial.data_ptr())])
    return fold(partial)


def add_stats(x, y):
    """AddStatsPHSP (hydra/detail/functors/StatsPHSP.h:62-84) on (mean, M2, W) triples."""
    w = x[2] + y[2]
    delta = y[0] - x[0]
    return ((x[0] * x[2] + y[0] * y[2]) / w, x[1] + y[1] + delta * delta * x[2] * y[2] / w, w)


@functools.lru_cache(maxsize=None)
def _avg_args(n: int):
    class AvgArgs(ctypes.Structure):
        _fields_ = [("m", _mother_args(n)), ("f", _BW)]
    return AvgArgs


def average_bw_partials(ch, i: int, j: int, a: float, b: float, first: int, n: int):
    """Launches the reference's AverageMother; returns the (blocks, 3) float64 cuda tensor
    of per-block StatsPHSP {mean, M2, W}."""
    import torch
    N = ch.n_daughters
    grid = max(1, min((n + THREADS - 1) // THREADS, AVG_BLOCKS))
    partial = torch.empty((grid, 3), dtype=torch.float64, device="cuda")

    args = _avg_args(N)()
    args.m = _args(ch)
    args.f = _BW(i, j, a, b)
    _launch(f"ref_average_bw_{N}_{ENGINES[ch.engine]}", grid,
            [args, ctypes.c_uint64(first), ctypes.c_uint64(n), ctypes.c_void_p(partial.data_ptr())])
    return partial


def fold(partial) -> tuple:
    """Folds per-block partials in block order; returns (mean, sqrt(M2)/W) as AverageOn does
    (hydra/detail/PhaseSpace.inl:255-273)."""
    p = np.asarray(partial.cpu() if hasattr(partial, "cpu") else partial, dtype=np.float64)
    acc = None
    for row in p:
        if row[2] == 0.0:
            continue
        acc = tuple(row) if acc is None else add_stats(acc, tuple(row))
    if acc is None:
        return float("nan"), float("nan")
    return acc[0], float(np.sqrt(acc[1]) / acc[2])


def average_bw(ch, i, j, a, b, first, n):
    return fold(average_bw_partials(ch, i, j, a, b, first, n))


def _time(fn, steps: int, warmup: int) -> float:
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(steps):
        fn()
    t1.record()
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / steps


def main(argv=None):
    """Times the reference's CUDA functors at the benchmark workloads (one JSON line each):
    N=5 D0 -> K pi pi pi pi (2^24 events, Generate and AverageOn |BW(m_K pi)|^2), the
    N=3 B0 -> J/psi K pi channel (10^6 and 2^26 events) and ten pions (2^26 events), Generate.
    Every output but the 10^6-event one (96 MB) exceeds the L2; the time of that one includes
    whatever of the previous step's output the L2 still holds."""
    import argparse
    import json
    import sys
    import torch
    sys.path.insert(0, str(HERE.parent))
    from oracle import oracle

    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--scale", type=int, default=0, help="log2 shrink of every event count")
    args = ap.parse_args(argv)
    pi, K = 0.13957, 0.493677
    cases = [
        ("generate", "N5_D0_Kpipipipi", [K, pi, pi, pi, pi], 1.86484, 1 << 24),
        ("average_bw", "N5_D0_Kpipipipi", [K, pi, pi, pi, pi], 1.86484, 1 << 24),
        ("generate", "N3_B0_JpsiKpi", [3.0969, K, pi], 5.27934, 10 ** 6),
        ("generate", "N3_B0_JpsiKpi", [3.0969, K, pi], 5.27934, 1 << 26),
        ("generate", "N10_pions", [pi] * 10, 5.0, 1 << 26),
    ]
    for kind, name, masses, M, n in cases:
        n >>= args.scale
        ch = oracle.make_channel(masses, M, 0x3039, oracle.ENGINE_PHILOX)
        if kind == "generate":
            out = torch.empty((len(masses), n, 4), dtype=torch.float64, device="cuda")
            ms = _time(lambda: generate(ch, 0, n, out), args.steps, args.warmup)
            gbs = n * 32 * len(masses) / ms / 1e6
            del out
        else:
            ms = _time(lambda: average_bw_partials(ch, 0, 1, 0.8955, 0.0473, 0, n), args.steps, args.warmup)
            gbs = 0.0
        print(json.dumps({"impl": "reference_cuda", "kind": kind, "workload": name, "events": n,
                          "ms": round(ms, 4), "events_per_s": n / ms * 1e3, "store_gbs": round(gbs, 1),
                          "dtype": "f64"}), flush=True)
        torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
