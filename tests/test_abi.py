"""C ABI checks that need no GPU: the library builds, loads and exports every symbol
include/*.h declares; host-side set-up (hps_channel_init, default seed, workspace size)
matches the reference fixtures; argument errors map to the reference's exceptions."""
from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import GEN_GOLDEN, REPO, load_golden


def declared_symbols():
    syms = set()
    for h in (REPO / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(hps_\w+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("hps_generate", "hps_average_on", "hps_evaluate", "hps_channel_init"):
        assert s in syms


def test_library_exports_every_declared_symbol(hps):
    L = ctypes.CDLL(str(hps.library_path()))
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    # the Python binding covers the same set
    assert set(declared_symbols()) <= set(hps.SIGNATURES)


def test_abi_version(hps):
    assert hps.lib().hps_abi_version() == 4


@pytest.mark.parametrize("name", GEN_GOLDEN)
def test_channel_init_matches_reference(hps, name):
    from hydra_gb300 import api
    g = load_golden(name)
    ch = api.make_channel(list(g["masses"]), float(g["M"]), 1, int(g["engine"]), list(g["mother"]))
    assert ch.max_weight == g["max_weight"]
    assert ch.ecm == g["ecm"]


def test_default_seed_matches_reference(hps):
    from hydra_gb300 import api
    g = load_golden("n3_philox_defaultseed")
    assert api.default_seed(list(g["masses"])) == int(g["default_seed"])
    ps = api.PhaseSpace(float(g["M"]), list(g["masses"]), engine="philox")
    assert ps.GetSeed() == int(g["get_seed"])


def test_seed_is_gint(hps):
    from hydra_gb300 import api
    ps = api.PhaseSpace(5.27934, [3.0969, 0.493677, 0.13957], engine="philox")
    ps.SetSeed(0x3039)
    assert ps.GetSeed() == 12345
    ps.SetSeed(-5)
    assert ps.GetSeed() == -5 and ps._seed == 2**64 - 5      # sign-extended into size_t
    ps.SetSeed(2**32 + 7)
    assert ps.GetSeed() == 7


def test_channel_errors_map_to_reference_exceptions(hps):
    from hydra_gb300 import api
    with pytest.raises(ValueError, match="daughter particle"):
        api.make_channel([0.1, 0.0], 1.0, 1)
    with pytest.raises(ValueError, match="mother particle"):
        api.make_channel([0.1, 0.2], -1.0, 1)
    with pytest.raises(RuntimeError, match="Not enough energy"):
        api.make_channel([0.6, 0.5], 1.0, 1)
    with pytest.raises(ValueError):
        api.make_channel([0.1], 1.0, 1)
    with pytest.raises(ValueError):
        api.make_channel([0.1] * 11, 5.0, 1)


def test_workspace_size(hps):
    from hydra_gb300 import api
    assert api.average_on_workspace_size(0) == 24
    assert api.average_on_workspace_size(1) == 24
    assert api.average_on_workspace_size(4096) == 24
    assert api.average_on_workspace_size(4097) == 48
    assert api.average_on_workspace_size(2**24) == 24 * 4096


def test_bad_arguments_rejected_before_launch(hps):
    """Validation happens on the host: no device is touched for these calls."""
    lib = hps.lib()
    ch = hps.HpsChannel()
    ch.n_daughters = 11
    st = lib.hps_generate(ctypes.byref(ch), 0, 10, None, None, None, 0, 0, None)
    assert st == hps.ERR_BAD_ARG
    assert b"outside 2..10" in lib.hps_last_error()
    from hydra_gb300 import api
    ch = api.make_channel([0.1, 0.2, 0.3], 1.0, 1)
    st = lib.hps_generate(ctypes.byref(ch), 2**64 - 5, 10, None, None, None, 0, 0, None)
    assert st == hps.ERR_BAD_ARG and b"wraps" in lib.hps_last_error()
    st = lib.hps_generate(ctypes.byref(ch), 0, 10, None, None, None, 0, 7, None)
    assert st == hps.ERR_BAD_ARG
    cols = (ctypes.c_void_p * 3)(8, 16, 32)      # misaligned column 0, never dereferenced
    st = lib.hps_generate(ctypes.byref(ch), 0, 10, ctypes.cast(cols, ctypes.c_void_p), None, None, 0, 0, None)
    assert st == hps.ERR_BAD_ARG and b"aligned" in lib.hps_last_error()
    fn = api.functor_mass2(0, 3)
    out = ctypes.c_void_p(64)
    st = lib.hps_average_on(ctypes.byref(ch), 0, 10, ctypes.byref(fn), out, None, 0, 0, None)
    assert st == hps.ERR_BAD_ARG and b"indices" in lib.hps_last_error()
    # n == 0 is a no-op, as an empty Thrust range
    assert lib.hps_generate(ctypes.byref(ch), 0, 0, None, None, None, 0, 0, None) == hps.OK


@pytest.mark.parametrize("name", [n for n in __import__("conftest").EXTRA_GOLDEN])
def test_range_channel_matches_generate_decay(hps, oracle, name):
    """hps_range_channel sets up GenerateDecay's constructor exactly as the oracle does."""
    from hydra_gb300 import api
    g = load_golden(name)
    ch = api.range_channel(list(g["masses"]), list(g["range_mother"]), int(g["rseed"]))
    och = oracle.range_channel(g["masses"], g["range_mother"], int(g["rseed"]))
    assert ch.engine == hps.ENGINE_MINSTD and ch.seed == och.seed == int(g["rseed"]) & 0xFFFFFFFF
    assert ch.ecm == och.ecm and ch.max_weight == och.max_weight
    assert list(ch.beta) == list(och.beta)


def test_consumer_arguments_rejected_before_launch(hps):
    from hydra_gb300 import api
    lib = hps.lib()
    cols = (ctypes.c_void_p * 3)(256, 512, 768)   # aligned, never dereferenced
    m = (ctypes.c_double * 3)(0.1, 0.2, 0.3)
    bins = ctypes.c_void_p(1024)
    cases = [
        (api.hist2d((0, 0), (1, 2), (10, 10), (0, 0), (1, 1)), b"same daughter"),
        (api.hist2d((0, 1), (1, 3), (10, 10), (0, 0), (1, 1)), b"outside"),
        (api.hist2d((0, 1), (1, 2), (0, 10), (0, 0), (1, 1)), b"grid"),
        (api.hist2d((0, 1), (1, 2), (10, 10), (0, 1), (1, 1)), b"upper"),
    ]
    for h, msg in cases:
        st = lib.hps_dalitz_histogram(3, ctypes.cast(m, ctypes.c_void_p), 1.0, 10, ctypes.cast(cols, ctypes.c_void_p),
                                      None, 0, ctypes.byref(h), bins, None)
        assert st == hps.ERR_BAD_ARG and msg in lib.hps_last_error(), msg
    h = api.hist2d((0, 1), (1, 2), (10, 10), (0, 0), (1, 1))
    st = lib.hps_dalitz_histogram(3, ctypes.cast(m, ctypes.c_void_p), 1.0, 10, ctypes.cast(cols, ctypes.c_void_p),
                                  None, 9, ctypes.byref(h), bins, None)
    assert st == hps.ERR_BAD_ARG and b"weight mode" in lib.hps_last_error()
    st = lib.hps_dalitz_histogram(3, ctypes.cast(m, ctypes.c_void_p), 1.0, 10, ctypes.cast(cols, ctypes.c_void_p),
                                  None, hps.HIST_COLUMN, ctypes.byref(h), bins, None)
    assert st == hps.ERR_BAD_ARG and b"weights is NULL" in lib.hps_last_error()
    # a minstd channel is for hps_generate_range only, and hps_generate_range takes nothing else
    rch = api.range_channel([0.1, 0.2, 0.3], [2.0, 0.0, 0.0, 0.0], 5)
    st = lib.hps_generate(ctypes.byref(rch), 0, 10, None, None, None, 0, 0, None)
    assert st == hps.ERR_BAD_ARG and b"hps_generate_range" in lib.hps_last_error()
    ch = api.make_channel([0.1, 0.2, 0.3], 1.0, 1)
    st = lib.hps_generate_range(ctypes.byref(ch), 0, 10, ctypes.cast(cols, ctypes.c_void_p), None, None)
    assert st == hps.ERR_BAD_ARG and b"hps_range_channel" in lib.hps_last_error()
    st = lib.hps_generate_dalitz(ctypes.byref(ch), 0, 10, hps.HIST_COLUMN, ctypes.byref(h), bins, 0, None)
    assert st == hps.ERR_BAD_ARG
    st = lib.hps_generate_dalitz(ctypes.byref(ch), 0, 10, hps.HIST_UNIT, ctypes.byref(h), bins, 7, None)
    assert st == hps.ERR_BAD_ARG and b"precision" in lib.hps_last_error()
    # GenerateDecay has no checks; the range set-up reports what would otherwise be NaNs
    with pytest.raises(hps.HpsError):
        api.range_channel([0.1, 0.2, 0.3], [0.5, 0.0, 0.0, 0.0], 5)
    fn = hps.HpsFunctor(7, 0, 1, 0, 0.0, 0.0)
    st = lib.hps_reweight(3, ctypes.cast(m, ctypes.c_void_p), 1.0, ctypes.byref(fn), 10,
                          ctypes.cast(cols, ctypes.c_void_p), None, None, None)
    assert st == hps.ERR_BAD_ARG and b"kind" in lib.hps_last_error()
    st = lib.hps_weight_flags(10, None, 1.0, None, 0, 0, None, None)
    assert st == hps.ERR_BAD_ARG


def test_fused_and_mothers_arguments_rejected_before_launch(hps):
    """hps_generate_average(_host) and the FP32_FIX mother forms validate on the host."""
    from hydra_gb300 import api
    lib = hps.lib()
    ch = api.make_channel([0.1, 0.2, 0.3], 1.0, 1)
    fn = api.functor_mass2(0, 1)
    out = ctypes.c_void_p(1024)
    cols = (ctypes.c_void_p * 3)(256, 512 + 8, 768)            # column 1 misaligned, never dereferenced
    st = lib.hps_generate_average(ctypes.byref(ch), 0, 10, ctypes.cast(cols, ctypes.c_void_p), None, None, 0,
                                  ctypes.byref(fn), out, None, 0, 1, None)
    assert st == hps.ERR_BAD_ARG and b"aligned" in lib.hps_last_error()
    bad = api.functor_mass2(0, 5)
    st = lib.hps_generate_average(ctypes.byref(ch), 0, 10, None, None, None, 0, ctypes.byref(bad), out, None, 0, 1,
                                  None)
    assert st == hps.ERR_BAD_ARG and b"indices" in lib.hps_last_error()
    st = lib.hps_generate_average(ctypes.byref(ch), 0, 10, None, None, None, 0, ctypes.byref(fn), out, None, 0, 9,
                                  None)
    assert st == hps.ERR_BAD_ARG and b"precision" in lib.hps_last_error()
    st = lib.hps_generate_average_host(ctypes.byref(ch), 0, 10, None, None, None, 0, ctypes.byref(fn), out, 1, None)
    assert st == hps.ERR_BAD_ARG and b"host_cols" in lib.hps_last_error()
    # the mothers' forms check their precision and outputs before any launch
    mo = ctypes.c_void_p(2048)
    w = ctypes.c_void_p(4096)
    st = lib.hps_evaluate_mothers(ctypes.byref(ch), 0, 10, mo, ctypes.byref(fn), 1, w, None, 1, None)
    assert st == hps.ERR_BAD_ARG and b"output column" in lib.hps_last_error()
    st = lib.hps_evaluate_mothers(ctypes.byref(ch), 0, 10, mo, ctypes.byref(fn), 1, w, None, 5, None)
    assert st == hps.ERR_BAD_ARG and b"precision" in lib.hps_last_error()
    st = lib.hps_generate_mothers(ctypes.byref(ch), 0, 10, mo, None, None, 7, None)
    assert st == hps.ERR_BAD_ARG and b"precision" in lib.hps_last_error()


def test_batch_tuning_checked_before_any_device_call(hps):
    """hps_batch_create validates the launch shape first (no GPU needed to see the errors)."""
    lib = hps.lib()
    plan = ctypes.c_void_p()
    for bad, msg in [((0, 4096, 0, 1), b"ctas_per_sm"), ((2, 1000, 0, 1), b"store_tile_events"),
                     ((2, 4096, 2, 1), b"kernel_form"), ((2, 4096, 0, 3), b"threads_per_event"),
                     ((2, 4096, 1, 2), b"needs kernel_form")]:
        t = hps.HpsBatchTuning(*bad)
        st = lib.hps_batch_create(ctypes.byref(plan), 4, 4, hps.PREC_FP32_FIX, ctypes.byref(t))
        assert st == hps.ERR_BAD_ARG
        assert msg in lib.hps_last_error()
    assert ctypes.sizeof(hps.HpsBatchTuning) == 16
