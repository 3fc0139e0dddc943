"""CPU oracle for the phase-space hot path -- TEST INFRASTRUCTURE ONLY.

ctypes wrapper over ``genbod_oracle.c`` (a plain-C restatement of Hydra's
GENBOD event generator; each function there cites the Hydra source it
follows).  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` use this module, and only as the checker or as the timed
CPU baseline; the product library never loads it.

``build()`` compiles the shared library next to this file with
``-O3 -ffp-contract=off`` (so every double rounds as the reference built the
same way) and OpenMP.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libhps_oracle.so"
SRC = HERE / "genbod_oracle.c"

MAXN = 10
ENGINE_PHILOX = 0
ENGINE_SQUARES3 = 1
ENGINE_MINSTD = 2          # thrust default_random_engine, phase_space_range only
DEFAULT_FUNCTOR_UNWEIGHT_SEED = 0x39ABDC4529B1661C   # hydra/Decays.h:261
DEFAULT_UNWEIGHT_SEED = 0x180EC6D33CFD0ABA   # hydra/Decays.h:253


class Channel(ctypes.Structure):
    _fields_ = [
        ("n_daughters", ctypes.c_int32),
        ("engine", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("ecm", ctypes.c_double),
        ("max_weight", ctypes.c_double),
        ("beta", ctypes.c_double * 3),
        ("masses", ctypes.c_double * MAXN),
    ]


class Functor(ctypes.Structure):
    _fields_ = [
        ("sel", ctypes.c_int32),
        ("i", ctypes.c_int32),
        ("j", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("a", ctypes.c_double),
        ("b", ctypes.c_double),
    ]


def build(force: bool = False) -> Path:
    """Compile genbod_oracle.c into _build/libhps_oracle.so (host compiler)."""
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB_PATH
    LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-Wall", str(SRC), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.POINTER
        u64, i32, dbl = ctypes.c_uint64, ctypes.c_int, ctypes.c_double
        vp = ctypes.c_void_p
        L.hpso_channel_init.argtypes = [P(Channel), i32, i32, u64, dbl, vp, vp]
        L.hpso_channel_init.restype = i32
        L.hpso_rng_words.argtypes = [i32, i32, u64, u64, u64, vp]
        L.hpso_generate.argtypes = [P(Channel), u64, u64, vp, vp, i32]
        L.hpso_recompute_weights.argtypes = [i32, vp, dbl, u64, vp, vp, i32]
        L.hpso_flags.argtypes = [vp, dbl, u64, u64, u64, vp]
        L.hpso_evaluate.argtypes = [P(Channel), P(Functor), u64, u64, vp, vp, i32]
        L.hpso_average_on.argtypes = [P(Channel), P(Functor), u64, u64, vp, i32]
        L.hpso_store_step.argtypes = [P(Channel), u64, u64, vp, vp, u64, vp, i32]
        L.hpso_unweight_uniforms.argtypes = [u64, u64, u64, vp]
        L.hpso_generate_mothers.argtypes = [P(Channel), u64, u64, vp, vp, vp, i32]
        L.hpso_average_mothers.argtypes = [P(Channel), P(Functor), u64, u64, vp, vp]
        L.hpso_evaluate_mothers.argtypes = [P(Channel), P(Functor), u64, u64, vp, vp, vp, vp, i32]
        L.hpso_reweight.argtypes = [i32, vp, dbl, P(Functor), u64, vp, vp, i32]
        L.hpso_dalitz_histogram.argtypes = [i32, u64, vp, vp, vp, vp, vp, vp, vp]
        L.hpso_max_threads.restype = i32
        for f in ("hpso_reweight", "hpso_dalitz_histogram", "hpso_rng_words", "hpso_generate", "hpso_recompute_weights", "hpso_flags",
                  "hpso_evaluate", "hpso_average_on", "hpso_store_step", "hpso_unweight_uniforms",
                  "hpso_generate_mothers", "hpso_average_mothers", "hpso_evaluate_mothers"):
            getattr(L, f).restype = None
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_channel(masses, mother_mass, seed, engine=ENGINE_PHILOX, mother=None) -> Channel:
    """Channel set-up as hydra::PhaseSpace's constructor + DecayMother's ctor.

    Raises ValueError / RuntimeError where the reference throws
    std::invalid_argument / std::runtime_error.
    """
    m = np.ascontiguousarray(masses, dtype=np.float64)
    mom = np.ascontiguousarray(mother if mother is not None else [mother_mass, 0.0, 0.0, 0.0],
                               dtype=np.float64)
    ch = Channel()
    rc = lib().hpso_channel_init(ctypes.byref(ch), len(m), engine, seed & 0xFFFFFFFFFFFFFFFF,
                                 float(mother_mass), _ptr(m), _ptr(mom))
    if rc == -1:
        raise ValueError("mass of mother or daughter particle is negative or zero")
    if rc == -2:
        raise RuntimeError("not enough energy to generate this decay")
    if rc != 0:
        raise ValueError("bad number of daughters")
    return ch


def make_functor(sel=0, i=0, j=1, a=0.0, b=0.0) -> Functor:
    return Functor(sel, i, j, 0, a, b)


def rng_words(n_daughters, engine, seed, first, n) -> np.ndarray:
    nw = 3 * n_daughters - 4
    out = np.zeros((n, nw), dtype=np.uint64)
    lib().hpso_rng_words(n_daughters, engine, seed, first, n, _ptr(out))
    return out


def generate(ch: Channel, first: int, n: int, nthreads: int = 0):
    """Returns (four [N, n, 4] float64, gen-time weights [n])."""
    N = ch.n_daughters
    four = np.zeros((N, n, 4), dtype=np.float64)
    w = np.zeros(n, dtype=np.float64)
    lib().hpso_generate(ctypes.byref(ch), first, n, _ptr(four), _ptr(w), nthreads)
    return four, w


def recompute_weights(ch: Channel, four: np.ndarray, max_weight=None, nthreads: int = 0):
    four = np.ascontiguousarray(four, dtype=np.float64)
    n = four.shape[1]
    out = np.zeros(n, dtype=np.float64)
    m = np.ascontiguousarray(ch.masses, dtype=np.float64)
    mw = ch.max_weight if max_weight is None else max_weight
    lib().hpso_recompute_weights(ch.n_daughters, _ptr(m), mw, n, _ptr(four), _ptr(out), nthreads)
    return out


def flags(weights: np.ndarray, max_weight: float, useed: int, first: int = 0):
    weights = np.ascontiguousarray(weights, dtype=np.float64)
    out = np.zeros(len(weights), dtype=np.uint8)
    lib().hpso_flags(_ptr(weights), max_weight, useed, first, len(weights), _ptr(out))
    return out


def unweight_uniforms(useed: int, first: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float64)
    lib().hpso_unweight_uniforms(useed, first, n, _ptr(out))
    return out


def evaluate(ch: Channel, fn: Functor, first: int, n: int, nthreads: int = 0):
    w = np.zeros(n, dtype=np.float64)
    f = np.zeros(n, dtype=np.float64)
    lib().hpso_evaluate(ctypes.byref(ch), ctypes.byref(fn), first, n, _ptr(w), _ptr(f), nthreads)
    return w, f


def average_on(ch: Channel, fn: Functor, first: int, n: int, nthreads: int = 1):
    """Returns (mean, M2, W); nthreads=1 is the reference cpp-backend fold order."""
    out = np.zeros(3, dtype=np.float64)
    lib().hpso_average_on(ctypes.byref(ch), ctypes.byref(fn), first, n, _ptr(out), nthreads)
    return float(out[0]), float(out[1]), float(out[2])


def store_step(ch: Channel, first: int, n: int, useed: int, four=None, w=None, fl=None,
               nthreads: int = 0):
    N = ch.n_daughters
    four = np.empty((N, n, 4), dtype=np.float64) if four is None else four
    w = np.empty(n, dtype=np.float64) if w is None else w
    fl = np.empty(n, dtype=np.uint8) if fl is None else fl
    lib().hpso_store_step(ctypes.byref(ch), first, n, _ptr(four), _ptr(w), useed, _ptr(fl),
                          nthreads)
    return four, w, fl


def generate_mothers(ch: Channel, first: int, mothers: np.ndarray, nthreads: int = 0):
    """DecayMothers: (four [N, n, 4], weights [n]) for mothers [n, 4]."""
    mothers = np.ascontiguousarray(mothers, dtype=np.float64)
    n = mothers.shape[0]
    four = np.zeros((ch.n_daughters, n, 4), dtype=np.float64)
    w = np.zeros(n, dtype=np.float64)
    lib().hpso_generate_mothers(ctypes.byref(ch), first, n, _ptr(mothers), _ptr(four), _ptr(w), nthreads)
    return four, w


def average_mothers(ch: Channel, fn: Functor, first: int, mothers: np.ndarray):
    """AverageMothers, sequential fold: (mean, M2, W).  Functor indices: 0 = mother."""
    mothers = np.ascontiguousarray(mothers, dtype=np.float64)
    out = np.zeros(3, dtype=np.float64)
    lib().hpso_average_mothers(ctypes.byref(ch), ctypes.byref(fn), first, mothers.shape[0], _ptr(mothers), _ptr(out))
    return float(out[0]), float(out[1]), float(out[2])


def evaluate_mothers(ch: Channel, fn: Functor, first: int, mothers: np.ndarray, nthreads: int = 0):
    """EvalMothers: (weights [n], functor values [n], four [N, n, 4]).  Functor indices: 0 = mother."""
    mothers = np.ascontiguousarray(mothers, dtype=np.float64)
    n = mothers.shape[0]
    w = np.zeros(n)
    f = np.zeros(n)
    four = np.zeros((ch.n_daughters, n, 4))
    lib().hpso_evaluate_mothers(ctypes.byref(ch), ctypes.byref(fn), first, n, _ptr(mothers), _ptr(w), _ptr(f),
                                _ptr(four), nthreads)
    return w, f, four


def reweight(ch: Channel, fn: Functor, four: np.ndarray, max_weight=None, nthreads: int = 0) -> np.ndarray:
    """PhaseSpaceReweight of stored events [N, n, 4]: PhaseSpaceWeight * functor."""
    four = np.ascontiguousarray(four, dtype=np.float64)
    n = four.shape[1]
    out = np.zeros(n, dtype=np.float64)
    m = np.ascontiguousarray(ch.masses, dtype=np.float64)
    mw = ch.max_weight if max_weight is None else max_weight
    lib().hpso_reweight(ch.n_daughters, _ptr(m), mw, ctypes.byref(fn), n, _ptr(four), _ptr(out), nthreads)
    return out


def unweight_functor(ch: Channel, fn: Functor, four: np.ndarray, weight: float = -1.0,
                     seed: int = DEFAULT_FUNCTOR_UNWEIGHT_SEED, first: int = 0):
    """Decays::Unweight(functor, weight, seed): (reweights, max value used, flags, permutation)."""
    rw = reweight(ch, fn, four)
    mv = float(weight) if weight > 0.0 else float(rw.max())
    fl = flags(rw, mv, seed, first)
    perm = np.concatenate([np.flatnonzero(fl), np.flatnonzero(fl == 0)])
    return rw, mv, fl, perm


def dalitz_histogram(four: np.ndarray, weights, pairs, grid, lower, upper) -> np.ndarray:
    """2-D DenseHistogram::Fill of (m2(p_a0+p_a1), m2(p_b0+p_b1)); weights None -> 1."""
    four = np.ascontiguousarray(four, dtype=np.float64)
    n = four.shape[1]
    pr = np.ascontiguousarray(pairs, dtype=np.int32)
    g = np.ascontiguousarray(grid, dtype=np.uint64)
    lo = np.ascontiguousarray(lower, dtype=np.float64)
    hi = np.ascontiguousarray(upper, dtype=np.float64)
    bins = np.zeros(int(g[0] * g[1]) + 2, dtype=np.float64)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    lib().hpso_dalitz_histogram(four.shape[0], n, _ptr(four), None if w is None else _ptr(w), _ptr(pr),
                                _ptr(g), _ptr(lo), _ptr(hi), _ptr(bins))
    return bins


def mother_mass(mother) -> float:
    """Vector4R::mass(): sqrt(E^2 - px^2 - py^2 - pz^2) when positive, else 0."""
    E, px, py, pz = (float(x) for x in mother)
    m2 = E * E - px * px - py * py - pz * pz
    return float(np.sqrt(m2)) if m2 > 0.0 else 0.0


def range_channel(masses, mother, seed) -> Channel:
    """GenerateDecay's constructor (functors/GenerateDecay.h:121-160): ECM and maximum weight
    from mother.mass(), the moving-mother boost vector, the seed cut to 32 bits, minstd_rand."""
    return make_channel(masses, mother_mass(mother), int(seed) & 0xFFFFFFFF, ENGINE_MINSTD, mother)


def max_threads() -> int:
    return int(lib().hpso_max_threads())
