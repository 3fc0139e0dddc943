"""GPU parity: libhps.so (through its C ABI) against the oracle and the reference fixtures.

Bars (FP64 form):
  * random words, generation-time weights, recomputed weights and unweight flags:
    bit-exact (every operation on their path is a correctly rounded IEEE operation
    issued in the reference's order);
  * four-vectors and functor values: max_k |dp_k| / E <= 1e-12 per daughter, the
    energy-normalised error of the precision contract (only cos/sin of the azimuth
    may differ in the last bit between CUDA and the host libm);
  * AverageOn: mean and M2 agree with the oracle's sequential fold to 1e-10 relative
    (same events, different merge order) and the mean agrees with the reference
    fixture within statistics.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import AVG_GOLDEN, GEN_GOLDEN, RNG_GOLDEN, load_golden

pytestmark = pytest.mark.gpu

TOL_FOUR = 1e-12
TOL_AVG = 1e-10

PI, K = 0.13957, 0.493677


def _seed_of(g):
    seed = int(g["seed"])
    return int(g["default_seed"]) if seed == -1 else seed


def _channels(api, O, g):
    mother = list(g["mother"]) if "mother" in g else None
    hch = api.make_channel(list(g["masses"]), float(g["M"]), _seed_of(g), int(g["engine"]), mother)
    och = O.make_channel(g["masses"], float(g["M"]), _seed_of(g), int(g["engine"]), mother=mother)
    return hch, och


def energy_norm_err(a: np.ndarray, b: np.ndarray) -> float:
    """max over daughters/events of max_k |a_k - b_k| / E_b; a, b shaped [N, n, 4]."""
    if a.size == 0:
        return 0.0
    d = np.abs(a - b).max(axis=2) / np.abs(b[:, :, 0])
    return float(d.max())


def gpu_generate(api, torch, ch, first, n, flags=False, useed=None, align16=False, precision="fp64"):
    N = ch.n_daughters
    if align16:
        # columns that are 16- but not 32-byte aligned exercise the 2 x 128-bit store path
        buf = torch.zeros(N * n * 4 + 2, dtype=torch.float64, device="cuda")
        four = buf[2:].view(N, n, 4)
    else:
        four = torch.zeros((N, n, 4), dtype=torch.float64, device="cuda")
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    fl = torch.zeros(n, dtype=torch.uint8, device="cuda") if flags else None
    kw = {} if useed is None else {"unweight_seed": useed}
    api.generate(ch, first, four, w, fl, precision=precision, **kw)
    torch.cuda.synchronize()
    return four.cpu().numpy(), w.cpu().numpy(), (fl.cpu().numpy() if flags else None)


@pytest.fixture(scope="module")
def api(hps, cuda):
    from hydra_gb300 import api as A
    return A


@pytest.fixture(scope="module")
def torch():
    import torch as T
    return T


# --------------------------------------------------------------------------- random streams

@pytest.mark.parametrize("name", RNG_GOLDEN)
def test_rng_words_match_reference(api, torch, name):
    g = load_golden(name)
    N, n = int(g["N"]), int(g["n"])
    out = torch.zeros(n * (3 * N - 4), dtype=torch.int64, device="cuda")
    api.rng_words(N, int(g["engine"]), int(g["seed"]), 0, n, out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint64).reshape(n, -1), g["words"])


@pytest.mark.parametrize("engine", [0, 1])
@pytest.mark.parametrize("N", [2, 3, 6, 10])
@pytest.mark.parametrize("first", [0, 123456789, 2**64 - 4096])
def test_rng_words_match_oracle_at_offsets(api, torch, oracle, engine, N, first):
    """Includes the last events before 2^64, where evt+3N and the Philox counter wrap."""
    n = 4096
    out = torch.zeros(n * (3 * N - 4), dtype=torch.int64, device="cuda")
    api.rng_words(N, engine, 0xDEADBEEFCAFEF00D, first, n, out)
    torch.cuda.synchronize()
    ref = oracle.rng_words(N, engine, 0xDEADBEEFCAFEF00D, first, n)
    assert np.array_equal(out.cpu().numpy().view(np.uint64).reshape(n, -1), ref)


# --------------------------------------------------------------------------- Generate

@pytest.mark.parametrize("name", GEN_GOLDEN)
def test_generate_matches_reference_fixture(api, torch, oracle, name):
    g = load_golden(name)
    hch, _ = _channels(api, oracle, g)
    four, w, fl = gpu_generate(api, torch, hch, 0, int(g["n"]), flags=True, useed=int(g["useed"]))
    assert np.array_equal(w, g["w_gen"]), "generation-time weights must be bit-exact"
    err = energy_norm_err(four, g["four"])
    assert err <= TOL_FOUR, err
    assert np.array_equal(fl, g["flags"])


@pytest.mark.parametrize("N,engine,M,masses,seed", [
    (3, 0, 5.27934, [3.0969, K, PI], 0x3039),
    (5, 0, 1.86484, [K, PI, PI, PI, PI], 0x3039),
    (10, 0, 5.0, [PI] * 10, 0x3039),
    (2, 1, 3.0, [1.0, 0.5], 11),
    (7, 1, 6.0, [PI, K, 0.938272, PI, PI, K, PI], 2**40 + 3),
    (4, 0, 4 * PI + 1e-4, [PI] * 4, 99),            # just above threshold
])
def test_generate_matches_oracle_large(api, torch, oracle, N, engine, M, masses, seed):
    n = 300_001      # not a multiple of the CTA size
    hch = api.make_channel(masses, M, seed, engine)
    och = oracle.make_channel(masses, M, seed, engine)
    four, w, fl = gpu_generate(api, torch, hch, 0, n, flags=True)
    rfour, rw = oracle.generate(och, 0, n)
    assert np.array_equal(w, rw)
    assert energy_norm_err(four, rfour) <= TOL_FOUR
    rwr = oracle.recompute_weights(och, rfour)
    rfl = oracle.flags(rwr, och.max_weight, oracle.DEFAULT_UNWEIGHT_SEED)
    mism = np.nonzero(fl != rfl)[0]
    # a flag may only differ where the recomputed weight sits within 1e-12 of the threshold u
    if mism.size:
        u = oracle.unweight_uniforms(oracle.DEFAULT_UNWEIGHT_SEED, 0, n)[mism]
        assert np.all(np.abs(rwr[mism] / och.max_weight - u) <= 1e-12 * np.maximum(u, 1e-300)), mism


def test_generate_offsets_and_chunking_identical(api, torch, oracle):
    """[0, n) in one call equals two calls [0, a) + [a, n); event e does not depend on the call."""
    hch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, 0)
    n, a = 100_000, 37_119
    four, w, fl = gpu_generate(api, torch, hch, 0, n, flags=True)
    f1, w1, l1 = gpu_generate(api, torch, hch, 0, a, flags=True)
    f2, w2, l2 = gpu_generate(api, torch, hch, a, n - a, flags=True)
    assert np.array_equal(four, np.concatenate([f1, f2], axis=1))
    assert np.array_equal(w, np.concatenate([w1, w2]))
    assert np.array_equal(fl, np.concatenate([l1, l2]))


def test_generate_near_counter_wrap(api, torch, oracle):
    hch = api.make_channel([PI] * 6, 3.0, 5, 0)
    och = oracle.make_channel([PI] * 6, 3.0, 5, 0)
    first = 2**64 - 5000
    four, w, _ = gpu_generate(api, torch, hch, first, 5000)
    rfour, rw = oracle.generate(och, first, 5000)
    assert np.array_equal(w, rw)
    assert energy_norm_err(four, rfour) <= TOL_FOUR


def test_generate_16_byte_aligned_columns(api, torch, oracle):
    hch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, 0)
    a, wa, _ = gpu_generate(api, torch, hch, 0, 10_000, align16=False)
    b, wb, _ = gpu_generate(api, torch, hch, 0, 10_000, align16=True)
    assert np.array_equal(a, b) and np.array_equal(wa, wb)


@pytest.mark.parametrize("n", [0, 1, 31, 257])
def test_generate_small_and_empty(api, torch, oracle, n):
    hch = api.make_channel([3.0969, K, PI], 5.27934, 0x3039, 0)
    och = oracle.make_channel([3.0969, K, PI], 5.27934, 0x3039, 0)
    four, w, _ = gpu_generate(api, torch, hch, 0, n)
    rfour, rw = oracle.generate(och, 0, n)
    assert np.array_equal(w, rw)
    assert energy_norm_err(four, rfour) <= TOL_FOUR


def test_generate_config2_full_size_properties(api, torch, oracle):
    """2^24 events of the N=5 decay: conservation, mass shells, weight bounds, and a
    strided sample of events checked against the oracle."""
    N, n, M = 5, 2**24, 1.86484
    masses = [K, PI, PI, PI, PI]
    hch = api.make_channel(masses, M, 0x3039, 0)
    four = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    fl = torch.empty(n, dtype=torch.uint8, device="cuda")
    api.generate(hch, 0, four, w, fl)
    tot = four.sum(dim=0)
    assert float((tot[:, 0] - M).abs().max()) < 1e-12
    assert float(tot[:, 1:].abs().max()) < 1e-12
    m2 = four[..., 0] ** 2 - (four[..., 1:] ** 2).sum(-1)
    mt = torch.tensor(masses, dtype=torch.float64, device="cuda")[:, None] ** 2
    assert float(((m2 - mt).abs() / four[..., 0] ** 2).max()) < 1e-12
    assert float(w.min()) >= 0.0 and float(w.max()) <= 1.0 + 1e-12
    acc = float(fl.double().mean())
    assert 0.0 < acc < 0.05
    # strided sample against the oracle
    idx = np.arange(0, n, 4099)
    och = oracle.make_channel(masses, M, 0x3039, 0)
    fs = four[:, torch.as_tensor(idx, device="cuda")].cpu().numpy()
    ws = w[torch.as_tensor(idx, device="cuda")].cpu().numpy()
    for j, e in enumerate(idx[:2000]):
        rf, rw = oracle.generate(och, int(e), 1, nthreads=1)
        assert rw[0] == ws[j]
        assert energy_norm_err(fs[:, j:j + 1], rf) <= TOL_FOUR


# --------------------------------------------------------------------------- Evaluate

@pytest.mark.parametrize("name", GEN_GOLDEN)
def test_evaluate_matches_reference_fixture(api, torch, oracle, name):
    g = load_golden(name)
    hch, _ = _channels(api, oracle, g)
    n = int(g["n"])
    f = g["functor"]
    fn = api.HpsFunctor(int(f[0]), int(f[1]), int(f[2]), 0, float(f[3]), float(f[4]))
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    out = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    fns = [fn, api.functor_one(), api.functor_mass2(0, int(g["N"]) - 1)]
    api.evaluate(hch, 0, n, fns, w, out)
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy(), g["w_gen"])
    fv = out[0].cpu().numpy()
    assert np.allclose(fv, g["f_val"], rtol=TOL_FOUR, atol=0)
    assert np.all(out[1].cpu().numpy() == 1.0)


# --------------------------------------------------------------------------- stored-event passes

@pytest.mark.parametrize("name", GEN_GOLDEN)
def test_event_weights_and_unweight_flags_bit_exact(api, torch, name):
    g = load_golden(name)
    four = torch.as_tensor(g["four"], device="cuda")
    N, n = four.shape[0], four.shape[1]
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    api.event_weights(N, list(g["masses"]), float(g["decays_max_weight"]), four, out)
    fl = torch.zeros(n, dtype=torch.uint8, device="cuda")
    api.unweight_flags(N, list(g["masses"]), float(g["decays_max_weight"]), four, fl, int(g["useed"]))
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), g["w_rec"])
    assert np.array_equal(fl.cpu().numpy(), g["flags"])


def test_decays_unweight_stable_partition(api, torch):
    g = load_golden("b0_jpsikpi_n3_philox")
    ps = api.PhaseSpace(float(g["M"]), list(g["masses"]), engine="philox")
    ps.SetSeed(int(g["seed"]))
    ev = ps.Generate(api.Vector4R(float(g["M"])), int(g["n"]))
    before = ev.four.cpu().numpy()
    kept = ev.Unweight(int(g["useed"]))
    assert kept == int(g["n_unweighted"])
    acc = np.nonzero(g["flags"])[0]
    assert energy_norm_err(ev.four.cpu().numpy()[:, :kept], before[:, acc]) == 0.0


# --------------------------------------------------------------------------- AverageOn

def _gpu_average(api, torch, ch, first, n, fn, workspace=False):
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    ws = None
    if workspace:
        ws = torch.zeros(api.average_on_workspace_size(n) // 8, dtype=torch.float64, device="cuda")
    api.average_on(ch, first, n, fn, out, ws)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("name", AVG_GOLDEN)
def test_average_on_matches_reference(api, torch, oracle, name):
    g = load_golden(name)
    f = g["functor"]
    fn = api.HpsFunctor(int(f[0]), int(f[1]), int(f[2]), 0, float(f[3]), float(f[4]))
    ch = api.make_channel(list(g["masses"]), float(g["M"]), int(g["seed"]), int(g["engine"]))
    mean, m2, w = _gpu_average(api, torch, ch, 0, int(g["n"]), fn)
    err = np.sqrt(m2) / w
    assert abs(mean - g["mean"]) <= TOL_AVG * abs(g["mean"])
    assert abs(err - g["err"]) <= 1e-8 * abs(g["err"]) + 1e-300


@pytest.mark.parametrize("N,M,masses,fn_args", [
    (3, 5.27934, [3.0969, K, PI], ("mass2", 0, 1)),
    (5, 1.86484, [K, PI, PI, PI, PI], ("bw2", 0, 1, 0.8955, 0.0473)),
    (10, 5.0, [PI] * 10, ("bw2", 0, 1, 0.8955, 0.0473)),
])
def test_average_on_matches_oracle_fold(api, torch, oracle, N, M, masses, fn_args):
    n = 1_000_003
    if fn_args[0] == "mass2":
        fn = api.functor_mass2(*fn_args[1:])
        ofn = oracle.make_functor(1, *fn_args[1:])
    else:
        fn = api.functor_bw2(*fn_args[1:])
        ofn = oracle.make_functor(2, *fn_args[1:])
    ch = api.make_channel(masses, M, 0x3039, 0)
    och = oracle.make_channel(masses, M, 0x3039, 0)
    mean, m2, w = _gpu_average(api, torch, ch, 0, n, fn)
    rmean, rm2, rw = oracle.average_on(och, ofn, 0, n, nthreads=0)
    assert abs(mean - rmean) <= TOL_AVG * abs(rmean)
    assert abs(m2 - rm2) <= TOL_AVG * abs(rm2)
    assert abs(w - rw) <= TOL_AVG * abs(rw)


def test_average_on_deterministic(api, torch):
    ch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, 0)
    fn = api.functor_bw2(0, 1, 0.8955, 0.0473)
    a = _gpu_average(api, torch, ch, 0, 2_000_000, fn)
    b = _gpu_average(api, torch, ch, 0, 2_000_000, fn, workspace=True)
    c = _gpu_average(api, torch, ch, 0, 2_000_000, fn)
    assert np.array_equal(a, b) and np.array_equal(a, c)


@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097])
def test_average_on_edges(api, torch, oracle, n):
    ch = api.make_channel([3.0969, K, PI], 5.27934, 0x3039, 0)
    och = oracle.make_channel([3.0969, K, PI], 5.27934, 0x3039, 0)
    mean, m2, w = _gpu_average(api, torch, ch, 0, n, api.functor_mass2(1, 2))
    rmean, rm2, rw = oracle.average_on(och, oracle.make_functor(1, 1, 2), 0, n, nthreads=1)
    if n == 0:
        assert (mean, m2, w) == (0.0, 0.0, 0.0)
    else:
        assert abs(mean - rmean) <= 1e-12 * abs(rmean)
        assert abs(w - rw) <= 1e-12 * abs(rw)


def test_phase_space_class_mirrors_reference(api, torch):
    """hydra::PhaseSpace-shaped API: B0 -> J/psi K pi event 0 and AverageOn through the class."""
    g = load_golden("b0_jpsikpi_n3_philox")
    ps = api.PhaseSpace(5.27934, [3.0969, K, PI], engine="philox")
    ps.SetSeed(0x3039)
    assert ps.GetMaxWeight() == g["max_weight"]
    ev = ps.Generate(api.Vector4R(5.27934), 16)
    assert energy_norm_err(ev.four.cpu().numpy(), g["four"][:, :16]) <= TOL_FOUR
    res = ps.Evaluate(api.Vector4R(5.27934), 16, api.functor_mass2(0, 1))
    assert np.array_equal(res[0].cpu().numpy(), g["w_gen"][:16])
    mean, err = ps.AverageOn(api.Vector4R(5.27934), api.functor_mass2(0, 1), 20000)
    ga = load_golden("avg_b0_jpsikpi_m2")
    assert abs(mean - ga["mean"]) <= TOL_AVG * ga["mean"]


@pytest.mark.parametrize("chunk", [0, 1000, 7777])
def test_generate_host_matches_device(api, torch, chunk):
    """Generate into pinned host memory (chunked, copy overlapped) equals the device path."""
    hch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, 0)
    n = 50_001
    f, w, fl = gpu_generate(api, torch, hch, 17, n, flags=True)
    hf = torch.zeros((5, n, 4), dtype=torch.float64).pin_memory()
    hw = torch.zeros(n, dtype=torch.float64).pin_memory()
    hfl = torch.zeros(n, dtype=torch.uint8).pin_memory()
    api.generate_host(hch, 17, hf, hw, hfl, chunk_events=chunk)
    assert np.array_equal(hf.numpy(), f) and np.array_equal(hw.numpy(), w) and np.array_equal(hfl.numpy(), fl)
    # pageable host memory works too (slower)
    pf = torch.zeros((5, n, 4), dtype=torch.float64)
    api.generate_host(hch, 17, pf, None, None, chunk_events=chunk)
    assert np.array_equal(pf.numpy(), f)


@pytest.mark.parametrize("n", [1, 4095, 4096, 100_003])
def test_unweight_compact_is_stable_partition(api, torch, oracle, n):
    hch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, 0)
    four, w, fl = gpu_generate(api, torch, hch, 0, n, flags=True)
    tf = torch.as_tensor(four, device="cuda")
    tw = torch.as_tensor(w, device="cuda")
    tfl = torch.as_tensor(fl, device="cuda")
    out, wout, nacc = api.unweight_compact(tf, tfl, tw)
    torch.cuda.synchronize()
    order = np.concatenate([np.nonzero(fl)[0], np.nonzero(fl == 0)[0]])
    assert int(nacc.item()) == int(fl.sum())
    assert np.array_equal(out.cpu().numpy(), four[:, order])
    assert np.array_equal(wout.cpu().numpy(), w[order])


def test_unweight_compact_empty_writes_zero_count(api, torch):
    """n = 0 moves nothing and still writes the accepted count (0) to the caller's buffer."""
    tf = torch.empty((5, 0, 4), dtype=torch.float64, device="cuda")
    tfl = torch.empty(0, dtype=torch.uint8, device="cuda")
    nacc = torch.full((1,), 12345, dtype=torch.int64, device="cuda")
    cin = api._ptr_array([tf[k] for k in range(5)])
    cout = api._ptr_array([tf[k] for k in range(5)])
    st = api.lib().hps_unweight_compact(5, 0, api.ctypes.cast(cin, api.ctypes.c_void_p), None, api._dptr(tfl),
                                        api.ctypes.cast(cout, api.ctypes.c_void_p), None, api._dptr(nacc), None, 0,
                                        None)
    assert st == 0
    torch.cuda.synchronize()
    assert int(nacc.item()) == 0
