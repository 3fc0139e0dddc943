"""Consumers of a stored sample and the lazy generator on the GPU, against fixtures made by the
reference itself: PhaseSpaceReweight + Decays::Unweight(functor, weight, seed), the Dalitz
DenseHistogram (stored and fused into generation), phase_space_range (minstd_rand) and
PhaseSpaceIntegrator."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import EXTRA_GOLDEN, load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-12          # FP64 four-vectors: only sin/cos differ from the reference
HIST_RTOL = 1e-12    # bin sums: atomic additions in another order than the reference's


@pytest.fixture(scope="module")
def api(hps, cuda):
    from hydra_gb300 import api as A
    return A


@pytest.fixture(scope="module")
def torch():
    import torch as T
    return T


def enorm(a, b):
    return float((np.abs(a - b).max(axis=2) / np.abs(b[:, :, 0])).max())


def functor(api, g):
    f = g["functor"]
    return api.HpsFunctor(int(f[0]), int(f[1]), int(f[2]), 0, float(f[3]), float(f[4]))


@pytest.mark.parametrize("name", EXTRA_GOLDEN)
def test_reweight_and_unweight_functor(api, torch, name):
    g = load_golden(name)
    N, n = int(g["N"]), int(g["n"])
    four = torch.as_tensor(g["four"], device="cuda")
    masses = list(g["masses"])
    ch = api.make_channel(masses, float(g["M"]), int(g["seed"]), int(g["engine"]))
    fn = functor(api, g)
    rw = torch.empty(n, dtype=torch.float64, device="cuda")
    mx = torch.empty(1, dtype=torch.float64, device="cuda")
    api.reweight(N, masses, ch.max_weight, fn, four, rw, mx)
    torch.cuda.synchronize()
    assert np.array_equal(rw.cpu().numpy(), g["reweight"])
    assert mx.item() == g["reweight"].max()
    for key, weight in (("unw_max", -1.0), ("unw_fixed", float(g["fmax"]))):
        ev = api.Decays(float(g["M"]), masses, n)
        ev.four.copy_(four)
        kept = ev.UnweightFunctor(fn, weight, int(g["fseed"]))
        assert kept == int(g[key + "_kept"])
        assert np.array_equal(ev.four.cpu().numpy(), g[key + "_four"])


@pytest.mark.parametrize("name", [n for n in EXTRA_GOLDEN if int(load_golden(n)["N"]) >= 3])
def test_dalitz_histogram_stored(api, torch, oracle, name):
    g = load_golden(name)
    n = int(g["n"])
    ev = api.Decays(float(g["M"]), list(g["masses"]), n, with_weights=False)
    ev.four.copy_(torch.as_tensor(g["four"], device="cuda"))
    bins = ev.DalitzHistogram(tuple(g["grid"]), tuple(g["lower"]), tuple(g["upper"]))
    got = bins.cpu().numpy()
    np.testing.assert_allclose(got, g["hist"], rtol=HIST_RTOL, atol=0)
    counts = ev.DalitzHistogram(tuple(g["grid"]), tuple(g["lower"]), tuple(g["upper"]), weight_mode="unit")
    ref_counts = oracle.dalitz_histogram(g["four"], None, [0, 1, 1, 2], g["grid"], g["lower"], g["upper"])
    assert np.array_equal(counts.cpu().numpy(), ref_counts)


@pytest.mark.parametrize("engine", ["philox", "squares3"])
def test_dalitz_fused_matches_stored(api, torch, oracle, engine):
    """Generate + histogram in one kernel equals Generate, store, then histogram; unit counts
    equal the oracle's exactly on 2^20 events."""
    M, m = 1.86484, [0.493677, 0.13957, 0.13957]
    n = 1 << 20
    ps = api.PhaseSpace(M, m, engine)
    ps.SetSeed(0x3039)
    lo = ((m[0] + m[1]) ** 2, (m[1] + m[2]) ** 2)
    hi = ((M - m[2]) ** 2, (M - m[0]) ** 2)
    fused_w = ps.DalitzHistogram(api.Vector4R(M), n, (64, 48), lo, hi)
    fused_c = ps.DalitzHistogram(api.Vector4R(M), n, (64, 48), lo, hi, weight_mode="unit")
    ev = ps.Generate(api.Vector4R(M), n)
    stored_w = ev.DalitzHistogram((64, 48), lo, hi, weight_mode="column")
    stored_c = ev.DalitzHistogram((64, 48), lo, hi, weight_mode="unit")
    assert np.array_equal(fused_c.cpu().numpy(), stored_c.cpu().numpy())
    np.testing.assert_allclose(fused_w.cpu().numpy(), stored_w.cpu().numpy(), rtol=1e-10, atol=0)
    och = oracle.make_channel(m, M, 0x3039, oracle.ENGINE_PHILOX if engine == "philox" else oracle.ENGINE_SQUARES3)
    four, w = oracle.generate(och, 0, n)
    ref_c = oracle.dalitz_histogram(four, None, [0, 1, 1, 2], (64, 48), lo, hi)
    ref_w = oracle.dalitz_histogram(four, w, [0, 1, 1, 2], (64, 48), lo, hi)
    assert np.array_equal(fused_c.cpu().numpy(), ref_c)
    np.testing.assert_allclose(fused_w.cpu().numpy(), ref_w, rtol=1e-10, atol=0)
    assert ref_c[-2:].sum() == 0 and ref_c.sum() == n


@pytest.mark.parametrize("N,engine,M,masses", [(3, "philox", 1.86484, [0.493677, 0.13957, 0.13957]),
                                               (3, "squares3", 5.27934, [3.0969, 0.493677, 0.13957]),
                                               (5, "philox", 1.86484, [0.493677] + [0.13957] * 4),
                                               (8, "philox", 3.0, [0.13957] * 8)])
def test_dalitz_fused_fp32fix(api, torch, N, engine, M, masses):
    """The FP32_FIX fused histogram against the FP64 one of the same events (which the test above
    pins to the oracle): every event counted; the only differences are events near a bin edge
    moving to the neighbouring bin.  A pair mass squared carries about 1e-7 of the pair's energy
    squared as float rounding, so about that fraction of a bin width around each of the 64 + 48
    edges is in doubt: |dcount| summed over the bins stays below 1e-3 of n.  The weighted totals
    agree within 1e-6."""
    n = 1 << 21
    ch = api.make_channel(masses, M, 0x3039, engine)
    lo = ((masses[0] + masses[1]) ** 2, (masses[1] + masses[2]) ** 2)
    hi = ((M - sum(masses[2:])) ** 2, (M - masses[0] - sum(masses[3:])) ** 2)
    h = api.hist2d((0, 1), (1, 2), (64, 48), lo, hi)
    out = {}
    for prec in ("fp64", "fp32_fix"):
        for mode in ("unit", "phsp"):
            bins = torch.empty(64 * 48 + 2, dtype=torch.float64, device="cuda")
            api.generate_dalitz(ch, 0, n, h, bins, mode, prec)
            out[prec, mode] = bins.cpu().numpy()
    c64, c32 = out["fp64", "unit"], out["fp32_fix", "unit"]
    assert c32.sum() == n and c64.sum() == n
    moved = float(np.abs(c32 - c64).sum())
    w64, w32 = out["fp64", "phsp"], out["fp32_fix", "phsp"]
    print(f"\n[fp32_fix dalitz] N={N} {engine}: {moved:.0f} of {n} counts moved, weighted total "
          f"{abs(w32.sum() - w64.sum()) / w64.sum():.2e}")
    assert moved <= 1e-3 * n
    assert abs(w32.sum() - w64.sum()) <= 1e-6 * w64.sum()


@pytest.mark.parametrize("name", EXTRA_GOLDEN)
def test_phase_space_range(api, torch, name):
    g = load_golden(name)
    w, four = api.phase_space_range(list(g["range_mother"]), list(g["masses"]), int(g["rseed"]), int(g["n"]))
    assert np.array_equal(w.cpu().numpy(), g["range_w"])
    assert enorm(four.cpu().numpy(), g["range_four"]) <= TOL


def test_phase_space_range_window(api, torch, oracle):
    """Element i of the range does not depend on the window it is materialised in."""
    mother, masses, seed = [5.3, 0.0, 0.0, 0.0], [0.13957] * 6, 77
    w_all, f_all = api.phase_space_range(mother, masses, seed, 4096)
    w_win, f_win = api.phase_space_range(mother, masses, seed, 1000, first=3000)
    assert torch.equal(w_all[3000:4000], w_win) and torch.equal(f_all[:, 3000:4000], f_win)
    och = oracle.range_channel(masses, mother, seed)
    rf, rw = oracle.generate(och, 0, 4096)
    assert np.array_equal(w_all.cpu().numpy(), rw)
    assert enorm(f_all.cpu().numpy(), rf) <= TOL


@pytest.mark.parametrize("name", EXTRA_GOLDEN)
def test_phase_space_integrator(api, name):
    g = load_golden(name)
    engine = "philox" if int(g["engine"]) == 0 else "squares3"
    integ = api.PhaseSpaceIntegrator(float(g["M"]), list(g["masses"]), int(g["n"]), engine)
    assert integ.GetGenerator()._seed == int(g["integ_seed"])
    mean, err = integ.Integrate(functor(api, g))
    assert abs(mean - g["integ_mean"]) <= 1e-10 * abs(g["integ_mean"])
    assert abs(err - g["integ_err"]) <= 1e-8 * abs(g["integ_err"]) + 1e-12 * abs(mean)
