"""Host-side mirror of Hydra's phase-space interface over the C ABI.

Names, argument meaning and error behaviour follow the reference:
  hydra::PhaseSpace<N,GRND>   hydra/PhaseSpace.h:86-346, hydra/detail/PhaseSpace.inl
  hydra::Decays<tuple<P...>>  hydra/Decays.h:67-651, hydra/detail/Decays.inl
  hydra::Vector4R             hydra/Vector4R.h:59-138
Device memory and streams come from PyTorch; every computation is a libhps.so call.

The low-level functions (generate, evaluate, average_on, ...) take torch CUDA tensors
and launch on the current torch stream (or an explicit one) without synchronising.
The class methods synchronise like the reference's blocking Thrust calls.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Iterable, Sequence

import torch

from . import (
    MODE_AVERAGE, MODE_STORE, HpsBatchItem, HpsBatchTuning, HpsRequest, HpsResult, HpsServerConfig,
    HpsServerStats,
    DEFAULT_FUNCTOR_UNWEIGHT_SEED, HIST_COLUMN, HIST_PHSP_WEIGHT, HIST_UNIT, HpsHist2D,
    DEFAULT_UNWEIGHT_SEED, ENGINE_PHILOX, ENGINE_SQUARES3, ERR_BAD_ARG, ERR_NO_ENERGY, ERR_TIMEOUT, FN_BW2, FN_MASS2, FN_ONE,
    HPS_MAX_DAUGHTERS, PREC_FP32_FIX, PREC_FP64, HpsChannel, HpsError, HpsFunctor, check, lib,
)

_ENGINES = {"philox": ENGINE_PHILOX, "squares3": ENGINE_SQUARES3, "default": ENGINE_SQUARES3,
            ENGINE_PHILOX: ENGINE_PHILOX, ENGINE_SQUARES3: ENGINE_SQUARES3}
_PRECISIONS = {"fp64": PREC_FP64, "fp32_fix": PREC_FP32_FIX, PREC_FP64: PREC_FP64, PREC_FP32_FIX: PREC_FP32_FIX}

Channel = HpsChannel


def _stream_handle(stream) -> ctypes.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    if isinstance(stream, torch.cuda.Stream):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


def _dptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    if t is None:
        return ctypes.c_void_p(0)
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def _double_array(values: Sequence[float]):
    arr = (ctypes.c_double * max(1, len(values)))()
    for i, v in enumerate(values):
        arr[i] = float(v)
    return arr


def _ptr_array(tensors: Sequence[torch.Tensor]):
    arr = (ctypes.c_void_p * max(1, len(tensors)))()
    for i, t in enumerate(tensors):
        arr[i] = _dptr(t).value
    return arr


# ----------------------------------------------------------------------------- functors

def functor_one() -> HpsFunctor:
    return HpsFunctor(FN_ONE, 0, 1, 0, 0.0, 0.0)


def functor_mass2(i: int, j: int) -> HpsFunctor:
    """f = mass2(p_i + p_j)."""
    return HpsFunctor(FN_MASS2, i, j, 0, 0.0, 0.0)


def functor_bw2(i: int, j: int, mass: float, width: float) -> HpsFunctor:
    """f = 1 / ((mass^2 - mass2(p_i+p_j))^2 + (mass*width)^2), |relativistic BW|^2."""
    return HpsFunctor(FN_BW2, i, j, 0, float(mass), float(width))


# ----------------------------------------------------------------------------- channel

def make_channel(masses: Sequence[float], mother_mass: float, seed: int, engine="philox",
                 mother: Sequence[float] | None = None) -> HpsChannel:
    """Channel scalars as hydra::PhaseSpace's constructor computes them (PhaseSpace.inl:42-90).

    Raises ValueError (std::invalid_argument) for a mass <= 0 and RuntimeError
    (std::runtime_error) when M - sum(m) <= 0."""
    ch = HpsChannel()
    m = _double_array(masses)
    mom = _double_array(mother if mother is not None else [mother_mass, 0.0, 0.0, 0.0])
    st = lib().hps_channel_init(ctypes.byref(ch), len(masses), _ENGINES[engine], int(seed) & (2**64 - 1),
                                float(mother_mass), ctypes.cast(m, ctypes.c_void_p),
                                ctypes.cast(mom, ctypes.c_void_p))
    if st == ERR_BAD_ARG:
        raise ValueError(lib().hps_last_error().decode())
    if st == ERR_NO_ENERGY:
        raise RuntimeError(lib().hps_last_error().decode())
    check(st)
    return ch


def default_seed(masses: Sequence[float]) -> int:
    m = _double_array(masses)
    return int(lib().hps_default_seed(len(masses), ctypes.cast(m, ctypes.c_void_p)))


# ----------------------------------------------------------------------------- raw launches

def generate(ch: HpsChannel, first: int, four: torch.Tensor | Sequence[torch.Tensor], weights=None, flags=None,
             unweight_seed: int = DEFAULT_UNWEIGHT_SEED, precision="fp64", stream=None) -> None:
    """four: [N, n, 4] float64 CUDA tensor (or N column tensors [n, 4])."""
    cols = list(four) if not isinstance(four, torch.Tensor) else [four[k] for k in range(four.shape[0])]
    if len(cols) != ch.n_daughters:
        raise ValueError("need one column per daughter")
    n = cols[0].shape[0]
    for c in cols:
        if c.dtype != torch.float64 or tuple(c.shape) != (n, 4) or not c.is_contiguous():
            raise ValueError("columns must be contiguous float64 [n, 4]")
    if weights is not None and (weights.dtype != torch.float64 or weights.numel() < n):
        raise ValueError("weights must be float64 [n]")
    if flags is not None and (flags.dtype != torch.uint8 or flags.numel() < n):
        raise ValueError("flags must be uint8 [n]")
    arr = _ptr_array(cols)
    check(lib().hps_generate(ctypes.byref(ch), first, n, ctypes.cast(arr, ctypes.c_void_p), _dptr(weights),
                             _dptr(flags), unweight_seed & (2**64 - 1), _PRECISIONS[precision],
                             _stream_handle(stream)))


def generate_host(ch: HpsChannel, first: int, four: torch.Tensor, weights=None, flags=None,
                  unweight_seed: int = DEFAULT_UNWEIGHT_SEED, precision="fp64", chunk_events: int = 0,
                  stream=None) -> None:
    """Generate into HOST tensors (pinned for full link bandwidth): four [N, n, 4] float64 on CPU."""
    if four.is_cuda or four.dtype != torch.float64 or four.dim() != 3 or four.shape[2] != 4:
        raise ValueError("four must be a CPU float64 [N, n, 4] tensor")
    if not four.is_contiguous():
        raise ValueError("four must be contiguous")
    N, n = four.shape[0], four.shape[1]
    if N != ch.n_daughters:
        raise ValueError("need one column per daughter")
    arr = (ctypes.c_void_p * N)(*[four[k].data_ptr() for k in range(N)])
    wp = ctypes.c_void_p(weights.data_ptr()) if weights is not None else ctypes.c_void_p(0)
    fp = ctypes.c_void_p(flags.data_ptr()) if flags is not None else ctypes.c_void_p(0)
    check(lib().hps_generate_host(ctypes.byref(ch), first, n, ctypes.cast(arr, ctypes.c_void_p), wp, fp,
                                  unweight_seed & (2**64 - 1), _PRECISIONS[precision], chunk_events,
                                  _stream_handle(stream)))


def evaluate(ch: HpsChannel, first: int, n: int, functors: Sequence[HpsFunctor], weights: torch.Tensor | None,
             outs: Sequence[torch.Tensor], precision="fp64", stream=None) -> None:
    fa = (HpsFunctor * max(1, len(functors)))(*functors)
    arr = _ptr_array(outs)
    check(lib().hps_evaluate(ctypes.byref(ch), first, n, ctypes.cast(fa, ctypes.c_void_p), len(functors),
                             _dptr(weights), ctypes.cast(arr, ctypes.c_void_p), _PRECISIONS[precision],
                             _stream_handle(stream)))


def average_on_workspace_size(n: int) -> int:
    return int(lib().hps_average_on_workspace_size(n))


def average_on(ch: HpsChannel, first: int, n: int, functor: HpsFunctor, out: torch.Tensor,
               workspace: torch.Tensor | None = None, precision="fp64", stream=None) -> None:
    """out: float64 CUDA tensor with >= 3 elements receiving {mean, M2, W}."""
    if out.dtype != torch.float64 or out.numel() < 3:
        raise ValueError("out must be float64 with 3 elements")
    wbytes = 0 if workspace is None else workspace.numel() * workspace.element_size()
    check(lib().hps_average_on(ctypes.byref(ch), first, n, ctypes.byref(functor), _dptr(out), _dptr(workspace),
                               wbytes, _PRECISIONS[precision], _stream_handle(stream)))


def generate_average(ch: HpsChannel, first: int, four: torch.Tensor, weights, flags, functor: HpsFunctor,
                     out: torch.Tensor, workspace: torch.Tensor | None = None,
                     unweight_seed: int = DEFAULT_UNWEIGHT_SEED, precision="fp64", stream=None) -> None:
    """Generate (into four [N, n, 4], weights, flags) and AverageOn (into out {mean, M2, W}) of the
    same events in one pass; each result equals its separate call bit for bit."""
    N, n = four.shape[0], four.shape[1]
    arr = _ptr_array([four[k] for k in range(N)])
    wbytes = 0 if workspace is None else workspace.numel() * workspace.element_size()
    check(lib().hps_generate_average(ctypes.byref(ch), first, n, ctypes.cast(arr, ctypes.c_void_p), _dptr(weights),
                                     _dptr(flags), unweight_seed & (2**64 - 1), ctypes.byref(functor), _dptr(out),
                                     _dptr(workspace), wbytes, _PRECISIONS[precision], _stream_handle(stream)))


def generate_average_host(ch: HpsChannel, first: int, four: torch.Tensor, weights, flags, functor: HpsFunctor,
                          out: torch.Tensor, unweight_seed: int = DEFAULT_UNWEIGHT_SEED, precision="fp64",
                          stream=None) -> None:
    """generate_host and average_on of the same events; with pinned host tensors in one pass.
    four/weights/flags: CPU tensors; out: 3-element float64 CUDA tensor.  Synchronous."""
    if four.is_cuda or four.dtype != torch.float64 or four.dim() != 3 or not four.is_contiguous():
        raise ValueError("four must be a contiguous CPU float64 [N, n, 4] tensor")
    N, n = four.shape[0], four.shape[1]
    arr = (ctypes.c_void_p * N)(*[four[k].data_ptr() for k in range(N)])
    wp = ctypes.c_void_p(weights.data_ptr()) if weights is not None else ctypes.c_void_p(0)
    fp = ctypes.c_void_p(flags.data_ptr()) if flags is not None else ctypes.c_void_p(0)
    check(lib().hps_generate_average_host(ctypes.byref(ch), first, n, ctypes.cast(arr, ctypes.c_void_p), wp, fp,
                                          unweight_seed & (2**64 - 1), ctypes.byref(functor), _dptr(out),
                                          _PRECISIONS[precision], _stream_handle(stream)))


def generate_mothers(ch: HpsChannel, first: int, mothers: torch.Tensor, four: torch.Tensor, weights=None,
                     precision="fp64", stream=None) -> None:
    """DecayMothers: mothers [n, 4] (a Vector4R column), four [N, n, 4]."""
    arr = _ptr_array([four[k] for k in range(four.shape[0])])
    check(lib().hps_generate_mothers(ctypes.byref(ch), first, mothers.shape[0], _dptr(mothers),
                                     ctypes.cast(arr, ctypes.c_void_p), _dptr(weights), _PRECISIONS[precision],
                                     _stream_handle(stream)))


def average_on_mothers(ch: HpsChannel, first: int, mothers: torch.Tensor, functor: HpsFunctor, out: torch.Tensor,
                       precision="fp64", stream=None) -> None:
    """AverageMothers; functor indices count the mother as particle 0."""
    check(lib().hps_average_on_mothers(ctypes.byref(ch), first, mothers.shape[0], _dptr(mothers),
                                       ctypes.byref(functor), _dptr(out), None, 0, _PRECISIONS[precision],
                                       _stream_handle(stream)))


def evaluate_mothers(ch: HpsChannel, first: int, mothers: torch.Tensor, functors: Sequence[HpsFunctor],
                     weights: torch.Tensor | None, outs: Sequence[torch.Tensor], precision="fp64", stream=None):
    """EvalMothers; functor indices count the mother as particle 0."""
    fa = (HpsFunctor * max(1, len(functors)))(*functors)
    arr = _ptr_array(outs)
    check(lib().hps_evaluate_mothers(ctypes.byref(ch), first, mothers.shape[0], _dptr(mothers),
                                     ctypes.cast(fa, ctypes.c_void_p), len(functors), _dptr(weights),
                                     ctypes.cast(arr, ctypes.c_void_p), _PRECISIONS[precision],
                                     _stream_handle(stream)))


def event_weights(n_daughters: int, masses: Sequence[float], max_weight: float, four: torch.Tensor,
                  out: torch.Tensor, stream=None) -> None:
    n = four.shape[1]
    arr = _ptr_array([four[k] for k in range(n_daughters)])
    m = _double_array(masses)
    check(lib().hps_event_weights(n_daughters, ctypes.cast(m, ctypes.c_void_p), max_weight, n,
                                  ctypes.cast(arr, ctypes.c_void_p), _dptr(out), _stream_handle(stream)))


def unweight_flags(n_daughters: int, masses: Sequence[float], max_weight: float, four: torch.Tensor,
                   flags: torch.Tensor, unweight_seed: int = DEFAULT_UNWEIGHT_SEED, first: int = 0,
                   stream=None) -> None:
    n = four.shape[1]
    arr = _ptr_array([four[k] for k in range(n_daughters)])
    m = _double_array(masses)
    check(lib().hps_unweight_flags(n_daughters, ctypes.cast(m, ctypes.c_void_p), max_weight, n,
                                   ctypes.cast(arr, ctypes.c_void_p), unweight_seed & (2**64 - 1), first,
                                   _dptr(flags), _stream_handle(stream)))


def unweight_compact(four: torch.Tensor, flags: torch.Tensor, weights: torch.Tensor | None = None,
                     stream=None):
    """Stable partition of stored events by flags (accepted first): returns (four_out,
    weights_out or None, n_accepted as a 1-element int64 CUDA tensor)."""
    N, n = four.shape[0], four.shape[1]
    out = torch.empty_like(four)
    wout = torch.empty_like(weights) if weights is not None else None
    nacc = torch.zeros(1, dtype=torch.int64, device=four.device)
    cin = _ptr_array([four[k] for k in range(N)])
    cout = _ptr_array([out[k] for k in range(N)])
    check(lib().hps_unweight_compact(N, n, ctypes.cast(cin, ctypes.c_void_p), _dptr(weights), _dptr(flags),
                                     ctypes.cast(cout, ctypes.c_void_p), _dptr(wout), _dptr(nacc), None, 0,
                                     _stream_handle(stream)))
    return out, wout, nacc


def reweight(n_daughters: int, masses: Sequence[float], max_weight: float, functor: HpsFunctor,
             four: torch.Tensor, out: torch.Tensor | None, max_out: torch.Tensor | None = None, stream=None) -> None:
    """PhaseSpaceReweight over stored events: out[e] = PhaseSpaceWeight * functor; max_out (a
    1-element float64 CUDA tensor) receives the largest value."""
    n = four.shape[1]
    arr = _ptr_array([four[k] for k in range(n_daughters)])
    m = _double_array(masses)
    check(lib().hps_reweight(n_daughters, ctypes.cast(m, ctypes.c_void_p), max_weight, ctypes.byref(functor), n,
                             ctypes.cast(arr, ctypes.c_void_p), _dptr(out), _dptr(max_out), _stream_handle(stream)))


def weight_flags(weights: torch.Tensor, flags: torch.Tensor, max_weight: float | torch.Tensor,
                 unweight_seed: int = DEFAULT_FUNCTOR_UNWEIGHT_SEED, first: int = 0, stream=None) -> None:
    """flags[e] = weights[e] / W > u(first + e); W a float or a 1-element CUDA tensor."""
    dev = max_weight if isinstance(max_weight, torch.Tensor) else None
    host = 0.0 if dev is not None else float(max_weight)
    check(lib().hps_weight_flags(weights.shape[0], _dptr(weights), host, _dptr(dev), unweight_seed & (2**64 - 1),
                                 first, _dptr(flags), _stream_handle(stream)))


def hist2d(pair_a=(0, 1), pair_b=(1, 2), grid=(100, 100), lower=(0.0, 0.0), upper=(1.0, 1.0)) -> HpsHist2D:
    h = HpsHist2D()
    h.pair_a[0], h.pair_a[1] = pair_a
    h.pair_b[0], h.pair_b[1] = pair_b
    h.grid[0], h.grid[1] = (int(g) for g in grid)
    h.lower[0], h.lower[1] = (float(x) for x in lower)
    h.upper[0], h.upper[1] = (float(x) for x in upper)
    return h


_HIST_WEIGHTS = {"unit": HIST_UNIT, "column": HIST_COLUMN, "phsp": HIST_PHSP_WEIGHT,
                 HIST_UNIT: HIST_UNIT, HIST_COLUMN: HIST_COLUMN, HIST_PHSP_WEIGHT: HIST_PHSP_WEIGHT}


def dalitz_histogram(n_daughters: int, masses: Sequence[float], max_weight: float, four: torch.Tensor,
                     hist: HpsHist2D, bins: torch.Tensor, weights: torch.Tensor | None = None, weight_mode="phsp",
                     stream=None) -> None:
    n = four.shape[1]
    arr = _ptr_array([four[k] for k in range(n_daughters)])
    m = _double_array(masses)
    check(lib().hps_dalitz_histogram(n_daughters, ctypes.cast(m, ctypes.c_void_p), max_weight, n,
                                     ctypes.cast(arr, ctypes.c_void_p), _dptr(weights), _HIST_WEIGHTS[weight_mode],
                                     ctypes.byref(hist), _dptr(bins), _stream_handle(stream)))


def generate_dalitz(ch: HpsChannel, first: int, n: int, hist: HpsHist2D, bins: torch.Tensor, weight_mode="phsp",
                    precision="fp64", stream=None) -> None:
    check(lib().hps_generate_dalitz(ctypes.byref(ch), first, n, _HIST_WEIGHTS[weight_mode], ctypes.byref(hist),
                                    _dptr(bins), _PRECISIONS[precision], _stream_handle(stream)))


def range_channel(masses: Sequence[float], mother: Sequence[float], seed: int) -> HpsChannel:
    ch = HpsChannel()
    m = _double_array(masses)
    mo = _double_array(list(mother))
    check(lib().hps_range_channel(ctypes.byref(ch), len(masses), ctypes.cast(m, ctypes.c_void_p),
                                  ctypes.cast(mo, ctypes.c_void_p), int(seed) & (2**64 - 1)))
    return ch


def generate_range(ch: HpsChannel, first: int, four: torch.Tensor, weights: torch.Tensor | None = None,
                   stream=None) -> None:
    N, n = four.shape[0], four.shape[1]
    arr = _ptr_array([four[k] for k in range(N)])
    check(lib().hps_generate_range(ctypes.byref(ch), first, n, ctypes.cast(arr, ctypes.c_void_p), _dptr(weights),
                                   _stream_handle(stream)))


def rng_words(n_daughters: int, engine, seed: int, first: int, n: int, out: torch.Tensor, stream=None) -> None:
    if out.dtype not in (torch.int64, torch.uint64) or out.numel() < n * (3 * n_daughters - 4):
        raise ValueError("out must be 64-bit with n*(3N-4) elements")
    check(lib().hps_rng_words(n_daughters, _ENGINES[engine], int(seed) & (2**64 - 1), first, n, _dptr(out),
                              _stream_handle(stream)))


# ----------------------------------------------------------------------------- batched channels

def store_item(ch: HpsChannel, first: int, four: torch.Tensor, weights=None, flags=None,
               unweight_seed: int = DEFAULT_UNWEIGHT_SEED) -> HpsBatchItem:
    it = HpsBatchItem()
    it.channel = ch
    it.first_evt = first
    it.n_events = four.shape[1]
    it.mode = MODE_STORE
    for k in range(ch.n_daughters):
        it.cols[k] = four[k].data_ptr()
    it.weights = weights.data_ptr() if weights is not None else None
    it.flags = flags.data_ptr() if flags is not None else None
    it.unweight_seed = unweight_seed & (2**64 - 1)
    return it


def average_item(ch: HpsChannel, first: int, n: int, functor: HpsFunctor, stats: torch.Tensor) -> HpsBatchItem:
    it = HpsBatchItem()
    it.channel = ch
    it.first_evt = first
    it.n_events = n
    it.mode = MODE_AVERAGE
    it.functor = functor
    it.stats = stats.data_ptr()
    return it


class BatchPlan:
    """Many channels in one graph launch of persistent kernels, one per N (hps_batch_*; FP32_FIX)."""

    def __init__(self, max_items: int, max_average_tiles: int, tuning: tuple[int, ...] | None = None):
        """tuning: (ctas_per_sm, store_tile_events[, kernel_form[, threads_per_event]]); kernel_form
        0 = one kernel per N (default), 1 = one kernel over every N; threads_per_event 1 (default)
        or 2 (the store items with N >= 7 computed by two threads per event)."""
        self._p = ctypes.c_void_p()
        if tuning:
            tuning = tuple(tuning) + (0, 1)[len(tuning) - 2:] if len(tuning) < 4 else tuple(tuning)
        t = HpsBatchTuning(*tuning) if tuning else None
        check(lib().hps_batch_create(ctypes.byref(self._p), max_items, max_average_tiles, PREC_FP32_FIX,
                                     ctypes.byref(t) if t else None))
        self._items = None

    def set_items(self, items: Sequence[HpsBatchItem], stream=None):
        arr = (HpsBatchItem * max(1, len(items)))(*items)
        self._items = arr
        check(lib().hps_batch_set_items(self._p, ctypes.cast(arr, ctypes.c_void_p), len(items),
                                        _stream_handle(stream)))

    def launch(self, stream=None):
        check(lib().hps_batch_launch(self._p, _stream_handle(stream)))

    def tuning(self) -> tuple[int, int, int, int]:
        """(ctas_per_sm, store_tile_events, kernel_form, threads_per_event)."""
        t = HpsBatchTuning()
        check(lib().hps_batch_get_tuning(self._p, ctypes.byref(t)))
        return t.ctas_per_sm, t.store_tile_events, t.kernel_form, t.threads_per_event

    def set_tuning(self, ctas_per_sm: int, store_tile_events: int, kernel_form: int = 0, threads_per_event: int = 1):
        t = HpsBatchTuning(ctas_per_sm, store_tile_events, kernel_form, threads_per_event)
        check(lib().hps_batch_set_tuning(self._p, ctypes.byref(t)))

    def autotune(self, cache_path: str | None = None, stream=None) -> tuple[int, int, int, int]:
        t = HpsBatchTuning()
        check(lib().hps_batch_autotune(self._p, _stream_handle(stream),
                                       cache_path.encode() if cache_path else None, ctypes.byref(t)))
        return t.ctas_per_sm, t.store_tile_events, t.kernel_form, t.threads_per_event

    def close(self):
        if self._p:
            lib().hps_batch_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------------- serving loop

def store_request(ch: HpsChannel, first: int, n: int, want_flags: bool = False,
                  unweight_seed: int = DEFAULT_UNWEIGHT_SEED) -> HpsRequest:
    r = HpsRequest()
    r.channel = ch
    r.first_evt = first
    r.n_events = n
    r.mode = MODE_STORE
    r.want_flags = 1 if want_flags else 0
    r.unweight_seed = unweight_seed & (2**64 - 1)
    return r


def average_request(ch: HpsChannel, first: int, n: int, functor: HpsFunctor) -> HpsRequest:
    r = HpsRequest()
    r.channel = ch
    r.first_evt = first
    r.n_events = n
    r.mode = MODE_AVERAGE
    r.functor = functor
    return r


class Server:
    """Continuous-batching request server (hps_server_*)."""

    def __init__(self, budget_bytes: int, slice_events: int = 0, max_batch_items: int = 0, max_inflight: int = 0,
                 max_average_events: int = 0, fail_alloc_after: int = 0):
        cfg = HpsServerConfig(budget_bytes, slice_events, max_batch_items, max_inflight, max_average_events,
                              fail_alloc_after, 0)
        self._s = ctypes.c_void_p()
        check(lib().hps_server_create(ctypes.byref(self._s), ctypes.byref(cfg)))

    def submit(self, request: HpsRequest) -> int:
        t = ctypes.c_uint64()
        check(lib().hps_server_submit(self._s, ctypes.byref(request), ctypes.byref(t)))
        return t.value

    def poll(self, ticket: int):
        res = HpsResult()
        done = ctypes.c_int32()
        check(lib().hps_server_poll(self._s, ticket, ctypes.byref(res), ctypes.byref(done)))
        return res if done.value else None

    def wait(self, ticket: int, timeout_s: float = 60.0) -> HpsResult:
        res = HpsResult()
        check(lib().hps_server_wait(self._s, ticket, ctypes.byref(res), timeout_s))
        return res

    def next_done(self, timeout_s: float = 1.0):
        """(ticket, result) of the next request to finish, or None after timeout_s."""
        t = ctypes.c_uint64()
        res = HpsResult()
        st = lib().hps_server_next_done(self._s, ctypes.byref(t), ctypes.byref(res), timeout_s)
        if st == ERR_TIMEOUT:
            return None
        check(st)
        return t.value, res

    def cancel(self, ticket: int) -> None:
        check(lib().hps_server_cancel(self._s, ticket))

    def release(self, ticket: int) -> None:
        check(lib().hps_server_release(self._s, ticket))

    def stats(self) -> dict:
        st = HpsServerStats()
        check(lib().hps_server_get_stats(self._s, ctypes.byref(st)))
        return {n: getattr(st, n) for n, _ in HpsServerStats._fields_}

    def close(self) -> None:
        if self._s:
            lib().hps_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceArray:
    """Exposes a raw device pointer through __cuda_array_interface__ (zero-copy torch view)."""

    def __init__(self, ptr: int, shape: tuple, typestr: str):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def result_views(res: HpsResult, n_daughters: int):
    """Zero-copy torch views of a finished request's outputs: (four [N, n, 4], weights [n],
    flags [n] or None) for a store request, valid until the request is released."""
    n = int(res.n_events)
    cols = [torch.as_tensor(_DeviceArray(res.cols[k], (n, 4), "<f8"), device="cuda") for k in range(n_daughters)]
    four = torch.stack(cols) if n else torch.empty((n_daughters, 0, 4), dtype=torch.float64, device="cuda")
    w = torch.as_tensor(_DeviceArray(res.weights, (n,), "<f8"), device="cuda") if res.weights else None
    fl = torch.as_tensor(_DeviceArray(res.flags, (n,), "|u1"), device="cuda") if res.flags else None
    return four, w, fl


# ----------------------------------------------------------------------------- reference-shaped API

@dataclass
class Vector4R:
    """(E, px, py, pz), hydra/Vector4R.h:59."""
    e: float
    px: float = 0.0
    py: float = 0.0
    pz: float = 0.0

    def as_list(self):
        return [self.e, self.px, self.py, self.pz]

    def mass(self) -> float:
        m2 = self.e * self.e - self.px * self.px - self.py * self.py - self.pz * self.pz
        return math.sqrt(m2) if m2 > 0 else 0.0


def _pdk(a, b, c):
    x = (a - b - c) * (a + b + c) * (a - b + c) * (a + b - c)
    return math.sqrt(x) / (2 * a)


class Decays:
    """N columns of Vector4R in device memory (hydra/Decays.h:67-651), plus the optional
    generation-time weight column this implementation can store beside them."""

    def __init__(self, mother_mass: float, masses: Sequence[float], nentries: int = 0, device="cuda",
                 with_weights: bool = True):
        self.mother_mass = float(mother_mass)
        self.masses = [float(m) for m in masses]
        ecm = self.mother_mass - sum(self.masses)
        emmax, emmin, wtmax = ecm + self.masses[0], 0.0, 1.0
        for i in range(1, len(self.masses)):          # Decays.h:100-118
            emmin += self.masses[i - 1]
            emmax += self.masses[i]
            wtmax *= _pdk(emmax, emmin, self.masses[i])
        self.max_weight = 1.0 / wtmax
        self.four = torch.empty((len(self.masses), nentries, 4), dtype=torch.float64, device=device)
        self.weights = torch.empty(nentries, dtype=torch.float64, device=device) if with_weights else None

    def __len__(self):
        return self.four.shape[1]

    def size(self):
        return len(self)

    def GetMaxWeight(self):
        return self.max_weight

    def GetMotherMass(self):
        return self.mother_mass

    def GetMasses(self):
        return list(self.masses)

    def GetDaughters(self, k: int) -> torch.Tensor:
        return self.four[k]

    def __getitem__(self, i):
        return tuple(Vector4R(*self.four[k, i].tolist()) for k in range(self.four.shape[0]))

    def GetEventWeights(self, stream=None) -> torch.Tensor:
        """Events | Events.GetEventWeightFunctor() (Decays.h:235-239), evaluated eagerly."""
        out = torch.empty(len(self), dtype=torch.float64, device=self.four.device)
        event_weights(len(self.masses), self.masses, self.max_weight, self.four, out, stream)
        return out

    def UnweightFlags(self, seed: int = DEFAULT_UNWEIGHT_SEED, stream=None) -> torch.Tensor:
        flags = torch.empty(len(self), dtype=torch.uint8, device=self.four.device)
        unweight_flags(len(self.masses), self.masses, self.max_weight, self.four, flags, seed, 0, stream)
        return flags

    def Unweight(self, seed: int = DEFAULT_UNWEIGHT_SEED) -> int:
        """Decays::Unweight (Decays.inl:415-455): stable-partitions the accepted events to the
        front (hps_unweight_compact) and returns their count."""
        flags = self.UnweightFlags(seed)
        self.four, w, nacc = unweight_compact(self.four, flags, self.weights)
        if self.weights is not None:
            self.weights = w
        return int(nacc.item())

    def GetEventReweights(self, functor: HpsFunctor, stream=None) -> torch.Tensor:
        """Events | Events.GetEventWeightFunctor(functor) (Decays.h:243-250), evaluated eagerly."""
        out = torch.empty(len(self), dtype=torch.float64, device=self.four.device)
        reweight(len(self.masses), self.masses, self.max_weight, functor, self.four, out, None, stream)
        return out

    def UnweightFunctor(self, functor: HpsFunctor, weight: float = -1.0,
                        seed: int = DEFAULT_FUNCTOR_UNWEIGHT_SEED) -> int:
        """Decays::Unweight(functor, weight, seed) (Decays.inl:458-511): hit-or-miss on
        PhaseSpaceWeight * functor against weight, or against the largest such value when weight
        <= 0; accepted events stable-partitioned to the front; returns their count."""
        n = len(self)
        rw = torch.empty(n, dtype=torch.float64, device=self.four.device)
        mx = torch.empty(1, dtype=torch.float64, device=self.four.device)
        reweight(len(self.masses), self.masses, self.max_weight, functor, self.four, rw, mx)
        flags = torch.empty(n, dtype=torch.uint8, device=self.four.device)
        weight_flags(rw, flags, mx if weight <= 0.0 else float(weight), seed, 0)
        self.four, w, nacc = unweight_compact(self.four, flags, self.weights)
        if self.weights is not None:
            self.weights = w
        return int(nacc.item())

    def DalitzHistogram(self, grid=(100, 100), lower=(0.0, 0.0), upper=(1.0, 1.0), pair_a=(0, 1), pair_b=(1, 2),
                        weight_mode="phsp") -> torch.Tensor:
        """make_dense_histogram<double,2>(..., Events | dalitz, Events | GetEventWeightFunctor())
        as in the reference's phsp_basic example: grid0*grid1 bins then underflow, overflow."""
        bins = torch.empty(int(grid[0]) * int(grid[1]) + 2, dtype=torch.float64, device=self.four.device)
        dalitz_histogram(len(self.masses), self.masses, self.max_weight, self.four,
                         hist2d(pair_a, pair_b, grid, lower, upper), bins, self.weights, weight_mode)
        torch.cuda.current_stream().synchronize()
        return bins


def phase_space_range(mother, masses: Sequence[float], seed: int, length: int, first: int = 0):
    """phase_space_range(mother, masses, seed, length) (PhaseSpaceRange.inl:46-73), materialised:
    returns (weights [length], four [N, length, 4]) of events first .. first+length-1."""
    mom = mother.as_list() if isinstance(mother, Vector4R) else list(mother)
    ch = range_channel(masses, mom, seed)
    four = torch.empty((len(masses), length, 4), dtype=torch.float64, device="cuda")
    w = torch.empty(length, dtype=torch.float64, device="cuda")
    generate_range(ch, first, four, w)
    torch.cuda.current_stream().synchronize()
    return w, four


class PhaseSpace:
    """hydra::PhaseSpace<N, GRND> (hydra/PhaseSpace.h:86-346)."""

    def __init__(self, mother_mass: float, masses: Sequence[float], engine="default", precision="fp64"):
        self.masses = [float(m) for m in masses]
        self.N = len(self.masses)
        self.engine = _ENGINES[engine]
        self.precision = precision
        self.mother_mass = float(mother_mass)
        # validates and computes ECM / max weight exactly as the C++ constructor
        ch = make_channel(self.masses, mother_mass, 0, self.engine)
        self._ecm = ch.ecm
        self._max_weight = ch.max_weight
        self._seed = default_seed(self.masses)      # PhaseSpace.inl:44,64

    # seeds are GInt_t through this API (PhaseSpace.h:285-291)
    def SetSeed(self, seed: int) -> None:
        s = int(seed) & 0xFFFFFFFF
        s = s - (1 << 32) if s >= (1 << 31) else s
        self._seed = s & (2**64 - 1)

    def GetSeed(self) -> int:
        s = self._seed & 0xFFFFFFFF
        return s - (1 << 32) if s >= (1 << 31) else s

    def GetMaxWeight(self):
        return self._max_weight

    def GetECM(self):
        return self._ecm

    def GetMasses(self):
        return list(self.masses)

    def GetMotherMass(self):
        return self.mother_mass

    def _channel(self, mother: Vector4R | Sequence[float] | None) -> HpsChannel:
        mom = mother.as_list() if isinstance(mother, Vector4R) else (
            list(mother) if mother is not None else [self.mother_mass, 0.0, 0.0, 0.0])
        ch = make_channel(self.masses, self.mother_mass, self._seed, self.engine, mom)
        ch.max_weight = self._max_weight
        ch.ecm = self._ecm
        return ch

    def Generate(self, mother, events: Decays | int, flags: torch.Tensor | None = None,
                 unweight_seed: int = DEFAULT_UNWEIGHT_SEED) -> Decays:
        if isinstance(events, int):
            events = Decays(self.mother_mass, self.masses, events)
        generate(self._channel(mother), 0, events.four, events.weights, flags, unweight_seed, self.precision)
        torch.cuda.current_stream().synchronize()
        return events

    def AverageOn(self, mother, functor: HpsFunctor, n: int):
        out = torch.zeros(3, dtype=torch.float64, device="cuda")
        average_on(self._channel(mother), 0, n, functor, out, None, self.precision)
        mean, m2, w = out.tolist()
        return mean, (math.sqrt(m2) / w if w != 0 else float("nan"))

    def Evaluate(self, mother, n: int, *functors: HpsFunctor) -> torch.Tensor:
        res = torch.empty((len(functors) + 1, n), dtype=torch.float64, device="cuda")
        evaluate(self._channel(mother), 0, n, functors, res[0], [res[k + 1] for k in range(len(functors))],
                 self.precision)
        torch.cuda.current_stream().synchronize()
        return res

    def DalitzHistogram(self, mother, n: int, grid=(100, 100), lower=(0.0, 0.0), upper=(1.0, 1.0), pair_a=(0, 1),
                        pair_b=(1, 2), weight_mode="phsp") -> torch.Tensor:
        """Generate + Dalitz histogram fused: the events are binned where they are made and
        never stored (in this object's precision; weight_mode "phsp" uses the generation-time weight)."""
        bins = torch.empty(int(grid[0]) * int(grid[1]) + 2, dtype=torch.float64, device="cuda")
        generate_dalitz(self._channel(mother), 0, n, hist2d(pair_a, pair_b, grid, lower, upper), bins, weight_mode,
                        self.precision)
        torch.cuda.current_stream().synchronize()
        return bins


class PhaseSpaceIntegrator:
    """hydra::PhaseSpaceIntegrator<N, Backend, GRND> (hydra/PhaseSpaceIntegrator.h:52-160):
    Integrate(functor) is AverageOn(mother at rest, functor, n) of a PhaseSpace with the
    default seed (PhaseSpaceIntegrator.inl:37-42)."""

    def __init__(self, mother_mass: float, masses: Sequence[float], n: int, engine="default", precision="fp64"):
        self.generator = PhaseSpace(mother_mass, masses, engine, precision)
        self.mother = Vector4R(float(mother_mass), 0.0, 0.0, 0.0)
        self.n_samples = int(n)

    def GetGenerator(self) -> PhaseSpace:
        return self.generator

    def GetMother(self) -> Vector4R:
        return self.mother

    def GetNSamples(self) -> int:
        return self.n_samples

    def Integrate(self, functor: HpsFunctor):
        return self.generator.AverageOn(self.mother, functor, self.n_samples)
