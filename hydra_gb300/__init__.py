"""hydra_gb300 -- GB300-native phase-space generator (Hydra's PhaseSpace hot path).

Python binding of the C ABI in ``include/hps.h`` (``libhps.so``, hand-written sm_103a
kernels).  PyTorch provides device memory and streams; every computation runs in
``libhps.so``.  There is no CPU fallback: if the library is missing, loading raises.

Host-side mirror of the reference API for this path (hydra/PhaseSpace.h:86-346):

    ps = PhaseSpace(5.27934, [3.0969, 0.493677, 0.13957], engine="philox")
    ps.SetSeed(0x3039)
    events = ps.Generate(mother, n)          # Decays: N columns of Vector4R (+ weights)
    mean, err = ps.AverageOn(mother, functor, n)
    w, fvals = ps.Evaluate(mother, n, functor, ...)
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

from .build import LIB as _LIB_PATH

HPS_MAX_DAUGHTERS = 10
HPS_AVG_TILE = 4096

OK, ERR_BAD_ARG, ERR_NO_ENERGY, ERR_OOM, ERR_BUDGET, ERR_TIMEOUT, ERR_CUDA, ERR_UNSUPPORTED = range(8)
ENGINE_PHILOX, ENGINE_SQUARES3, ENGINE_MINSTD = 0, 1, 2
PREC_FP64, PREC_FP32_FIX = 0, 1
FN_ONE, FN_MASS2, FN_BW2 = 0, 1, 2
DEFAULT_UNWEIGHT_SEED = 0x180EC6D33CFD0ABA   # hydra/Decays.h:253
DEFAULT_FUNCTOR_UNWEIGHT_SEED = 0x39ABDC4529B1661C   # hydra/Decays.h:261
HIST_UNIT, HIST_COLUMN, HIST_PHSP_WEIGHT = 0, 1, 2


class HpsChannel(ctypes.Structure):
    _fields_ = [
        ("n_daughters", ctypes.c_int32),
        ("engine", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("ecm", ctypes.c_double),
        ("max_weight", ctypes.c_double),
        ("beta", ctypes.c_double * 3),
        ("masses", ctypes.c_double * HPS_MAX_DAUGHTERS),
    ]


class HpsFunctor(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("i", ctypes.c_int32),
        ("j", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("a", ctypes.c_double),
        ("b", ctypes.c_double),
    ]


class HpsHist2D(ctypes.Structure):
    _fields_ = [
        ("pair_a", ctypes.c_int32 * 2),
        ("pair_b", ctypes.c_int32 * 2),
        ("grid", ctypes.c_uint64 * 2),
        ("lower", ctypes.c_double * 2),
        ("upper", ctypes.c_double * 2),
    ]


class HpsStats(ctypes.Structure):
    _fields_ = [("mean", ctypes.c_double), ("m2", ctypes.c_double), ("w", ctypes.c_double)]


class HpsBatchItem(ctypes.Structure):
    _fields_ = [
        ("channel", HpsChannel),
        ("first_evt", ctypes.c_uint64),
        ("n_events", ctypes.c_uint64),
        ("mode", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("functor", HpsFunctor),
        ("cols", ctypes.c_void_p * HPS_MAX_DAUGHTERS),
        ("weights", ctypes.c_void_p),
        ("flags", ctypes.c_void_p),
        ("unweight_seed", ctypes.c_uint64),
        ("stats", ctypes.c_void_p),
    ]


BATCH_PER_N = 0          # hps_batch_form: one persistent kernel per N, parallel graph branches
BATCH_ONE_KERNEL = 1     # one persistent kernel over every N


class HpsBatchTuning(ctypes.Structure):
    _fields_ = [("ctas_per_sm", ctypes.c_int32), ("store_tile_events", ctypes.c_int32),
                ("kernel_form", ctypes.c_int32), ("threads_per_event", ctypes.c_int32)]


MODE_STORE, MODE_AVERAGE = 0, 1


class HpsServerConfig(ctypes.Structure):
    _fields_ = [
        ("budget_bytes", ctypes.c_uint64),
        ("slice_events", ctypes.c_uint64),
        ("max_batch_items", ctypes.c_int32),
        ("max_inflight", ctypes.c_int32),
        ("max_average_events", ctypes.c_uint64),
        ("fail_alloc_after", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class HpsRequest(ctypes.Structure):
    _fields_ = [
        ("channel", HpsChannel),
        ("first_evt", ctypes.c_uint64),
        ("n_events", ctypes.c_uint64),
        ("mode", ctypes.c_int32),
        ("want_flags", ctypes.c_int32),
        ("functor", HpsFunctor),
        ("unweight_seed", ctypes.c_uint64),
    ]


class HpsResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("n_events", ctypes.c_uint64),
        ("cols", ctypes.c_void_p * HPS_MAX_DAUGHTERS),
        ("weights", ctypes.c_void_p),
        ("flags", ctypes.c_void_p),
        ("stats", HpsStats),
        ("t_submit", ctypes.c_double),
        ("t_admit", ctypes.c_double),
        ("t_done", ctypes.c_double),
    ]


class HpsServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "admitted", "completed", "cancelled", "failed",
                                                 "released", "launches", "events_done", "bytes_in_use",
                                                 "bytes_peak")]


class HpsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"hps status {status}: {message}")
        self.status = status


# Exported symbols and their ctypes signatures; tests check this list against include/hps.h.
_vp, _u64, _i32, _dbl, _sz = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_double, ctypes.c_size_t
SIGNATURES = {
    "hps_channel_init": (_i32, [ctypes.POINTER(HpsChannel), _i32, _i32, _u64, _dbl, _vp, _vp]),
    "hps_generate": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _vp, _vp, _u64, _i32, _vp]),
    "hps_generate_host": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _vp, _vp, _u64, _i32, _u64,
                                 _vp]),
    "hps_evaluate": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _i32, _vp, _vp, _i32, _vp]),
    "hps_average_on_workspace_size": (_sz, [_u64]),
    "hps_average_on": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, ctypes.POINTER(HpsFunctor), _vp, _vp,
                              _sz, _i32, _vp]),
    "hps_average_on_noalloc": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, ctypes.POINTER(HpsFunctor), _vp,
                                      _i32, _vp]),
    "hps_generate_mothers": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _vp, _vp, _i32, _vp]),
    "hps_average_on_mothers": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, ctypes.POINTER(HpsFunctor), _vp,
                                      _vp, _sz, _i32, _vp]),
    "hps_evaluate_mothers": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _vp, _i32, _vp, _vp, _i32, _vp]),
    "hps_event_weights": (_i32, [_i32, _vp, _dbl, _u64, _vp, _vp, _vp]),
    "hps_unweight_flags": (_i32, [_i32, _vp, _dbl, _u64, _vp, _u64, _u64, _vp, _vp]),
    "hps_compact_workspace_size": (_sz, [_u64]),
    "hps_unweight_compact": (_i32, [_i32, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "hps_rng_words": (_i32, [_i32, _i32, _u64, _u64, _u64, _vp, _vp]),
    "hps_generate_average_host": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _vp, _vp, _u64,
                                         ctypes.POINTER(HpsFunctor), _vp, _i32, _vp]),
    "hps_generate_average": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _vp, _vp, _u64,
                                    ctypes.POINTER(HpsFunctor), _vp, _vp, _sz, _i32, _vp]),
    "hps_reweight": (_i32, [_i32, _vp, _dbl, ctypes.POINTER(HpsFunctor), _u64, _vp, _vp, _vp, _vp]),
    "hps_weight_flags": (_i32, [_u64, _vp, _dbl, _vp, _u64, _u64, _vp, _vp]),
    "hps_dalitz_histogram": (_i32, [_i32, _vp, _dbl, _u64, _vp, _vp, _i32, ctypes.POINTER(HpsHist2D), _vp, _vp]),
    "hps_generate_dalitz": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _i32, ctypes.POINTER(HpsHist2D), _vp,
                                   _i32, _vp]),
    "hps_range_channel": (_i32, [ctypes.POINTER(HpsChannel), _i32, _vp, _vp, _u64]),
    "hps_generate_range": (_i32, [ctypes.POINTER(HpsChannel), _u64, _u64, _vp, _vp, _vp]),
    "hps_default_seed": (_u64, [_i32, _vp]),
    "hps_batch_create": (_i32, [_vp, _i32, _u64, _i32, _vp]),
    "hps_batch_set_items": (_i32, [_vp, _vp, _i32, _vp]),
    "hps_batch_launch": (_i32, [_vp, _vp]),
    "hps_batch_get_tuning": (_i32, [_vp, _vp]),
    "hps_batch_set_tuning": (_i32, [_vp, _vp]),
    "hps_batch_autotune": (_i32, [_vp, _vp, ctypes.c_char_p, _vp]),
    "hps_batch_destroy": (_i32, [_vp]),
    "hps_server_create": (_i32, [_vp, ctypes.POINTER(HpsServerConfig)]),
    "hps_server_submit": (_i32, [_vp, ctypes.POINTER(HpsRequest), ctypes.POINTER(ctypes.c_uint64)]),
    "hps_server_poll": (_i32, [_vp, _u64, ctypes.POINTER(HpsResult), ctypes.POINTER(ctypes.c_int32)]),
    "hps_server_wait": (_i32, [_vp, _u64, ctypes.POINTER(HpsResult), _dbl]),
    "hps_server_next_done": (_i32, [_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(HpsResult), _dbl]),
    "hps_server_cancel": (_i32, [_vp, _u64]),
    "hps_server_release": (_i32, [_vp, _u64]),
    "hps_server_get_stats": (_i32, [_vp, ctypes.POINTER(HpsServerStats)]),
    "hps_server_destroy": (_i32, [_vp]),
    "hps_last_error": (ctypes.c_char_p, []),
    "hps_abi_version": (_i32, []),
}

_lib = None


def library_path() -> Path:
    return Path(os.environ.get("HPS_LIBRARY", str(_LIB_PATH)))


def lib():
    """Loads libhps.so (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise RuntimeError(f"libhps.so not found at {path}; build it with `python -m hydra_gb300.build`")
        L = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != OK:
        raise HpsError(status, lib().hps_last_error().decode(errors="replace"))


from .api import (  # noqa: E402
    Channel, Decays, PhaseSpace, Vector4R, functor_bw2, functor_mass2, functor_one, make_channel,
)

__all__ = [
    "lib", "check", "HpsError", "HpsChannel", "HpsFunctor", "HpsStats", "Channel", "Decays", "PhaseSpace",
    "Vector4R", "make_channel", "functor_one", "functor_mass2", "functor_bw2",
]
