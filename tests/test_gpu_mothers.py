"""Per-event mothers (DecayMothers / AverageMothers / EvalMothers) on the GPU, FP64 form,
against the reference fixtures and the oracle; and a decay chain fed by a daughter column."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import MOTHER_GOLDEN, load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-12


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


@pytest.mark.parametrize("name", MOTHER_GOLDEN)
def test_mothers_match_reference(api, torch, oracle, name):
    g = load_golden(name)
    N, n = int(g["N"]), int(g["n"])
    ch = api.make_channel(list(g["masses"]), float(g["M"]), int(g["seed"]), int(g["engine"]))
    och = oracle.make_channel(g["masses"], float(g["M"]), int(g["seed"]), int(g["engine"]))
    mo = torch.as_tensor(g["mothers"], device="cuda")
    four = torch.zeros((N, n, 4), dtype=torch.float64, device="cuda")
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    api.generate_mothers(ch, 0, mo, four, w)
    _, rw = oracle.generate_mothers(och, 0, g["mothers"])
    f = g["functor"]
    fn = api.HpsFunctor(int(f[0]), int(f[1]), int(f[2]), 0, float(f[3]), float(f[4]))
    ew = torch.zeros(n, dtype=torch.float64, device="cuda")
    ef = torch.zeros(n, dtype=torch.float64, device="cuda")
    api.evaluate_mothers(ch, 0, mo, [fn], ew, [ef])
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.average_on_mothers(ch, 0, mo, fn, out)
    torch.cuda.synchronize()
    assert enorm(four.cpu().numpy(), g["four"]) <= TOL
    assert np.array_equal(w.cpu().numpy(), rw)
    assert np.array_equal(ew.cpu().numpy(), g["eval_w"])
    assert np.allclose(ef.cpu().numpy(), g["eval_f"], rtol=TOL, atol=0)
    mean, m2, W = out.cpu().tolist()
    assert abs(mean - g["avg_mean"]) <= 1e-10 * abs(g["avg_mean"])
    # the spread is rounding noise when the functor is constant (N=2: m2(p1+p2) is the mother
    # mass squared), so the error also gets an absolute allowance at the scale of the mean
    assert abs(np.sqrt(m2) / W - g["avg_err"]) <= 1e-8 * abs(g["avg_err"]) + 1e-12 * abs(mean)


def test_decay_chain_from_daughter_column(api, torch, oracle):
    """B0 -> J/psi K pi, then J/psi -> mu mu with the J/psi column as the mothers."""
    n = 50_000
    b0 = api.make_channel([3.0969, 0.493677, 0.13957], 5.27955, 0x3039, "philox")
    jpsi = api.make_channel([0.1056583745, 0.1056583745], 3.0969, 0x3040, "philox")
    three = torch.zeros((3, n, 4), dtype=torch.float64, device="cuda")
    api.generate(b0, 0, three)
    two = torch.zeros((2, n, 4), dtype=torch.float64, device="cuda")
    api.generate_mothers(jpsi, 0, three[0], two)
    torch.cuda.synchronize()
    mothers = three[0].cpu().numpy()
    oj = oracle.make_channel([0.1056583745, 0.1056583745], 3.0969, 0x3040, oracle.ENGINE_PHILOX)
    rfour, _ = oracle.generate_mothers(oj, 0, mothers)
    got = two.cpu().numpy()
    assert enorm(got, rfour) <= TOL
    # the muons add up to their J/psi
    assert np.abs(got.sum(axis=0) - mothers).max() <= 1e-12 * np.abs(mothers[:, 0]).max()


FP32_TOL = 1e-6


@pytest.mark.parametrize("name", MOTHER_GOLDEN)
def test_evalmothers_fp32fix_within_tolerance(api, torch, name):
    """EvalMothers in FP32_FIX (each event's ECM and maximum weight from its own mother, stream
    hash(evt, seed)) against the reference fixtures: weights within 1e-6, and m^2 functor values
    within 1e-5 (a pair mass squared formed from float four-vectors)."""
    g = load_golden(name)
    n = int(g["n"])
    ch = api.make_channel(list(g["masses"]), float(g["M"]), int(g["seed"]), int(g["engine"]))
    mo = torch.as_tensor(g["mothers"], device="cuda")
    f = g["functor"]
    fn = api.HpsFunctor(int(f[0]), int(f[1]), int(f[2]), 0, float(f[3]), float(f[4]))
    ew = torch.zeros(n, dtype=torch.float64, device="cuda")
    ef = torch.zeros(n, dtype=torch.float64, device="cuda")
    api.evaluate_mothers(ch, 0, mo, [fn], ew, [ef], precision="fp32_fix")
    torch.cuda.synchronize()
    w = ew.cpu().numpy()
    ewe = float((np.abs(w - g["eval_w"]) / g["eval_w"]).max())
    efe = float(np.median(np.abs(ef.cpu().numpy() - g["eval_f"]) / np.abs(g["eval_f"])))
    print(f"\n[fp32_fix EvalMothers] {name}: weight {ewe:.3e}, functor (median) {efe:.3e}")
    assert ewe <= FP32_TOL
    assert efe <= 1e-5


@pytest.mark.parametrize("name", MOTHER_GOLDEN)
def test_mothers_fp32fix_within_tolerance(api, torch, oracle, name):
    """DecayMothers and AverageMothers in FP32_FIX against the reference fixtures (the mothers move
    with gamma up to about 1.03) within the precision contract of this form."""
    g = load_golden(name)
    N, n = int(g["N"]), int(g["n"])
    ch = api.make_channel(list(g["masses"]), float(g["M"]), int(g["seed"]), int(g["engine"]))
    mo = torch.as_tensor(g["mothers"], device="cuda")
    four = torch.zeros((N, n, 4), dtype=torch.float64, device="cuda")
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    api.generate_mothers(ch, 0, mo, four, w, precision="fp32_fix")
    torch.cuda.synchronize()
    och = oracle.make_channel(g["masses"], float(g["M"]), int(g["seed"]), int(g["engine"]))
    _, rw = oracle.generate_mothers(och, 0, g["mothers"])
    e4 = enorm(four.cpu().numpy(), g["four"])
    ew = float((np.abs(w.cpu().numpy() - rw) / rw).max())
    print(f"\n[fp32_fix mothers] {name}: four {e4:.3e}, weight {ew:.3e}")
    assert e4 <= FP32_TOL and ew <= FP32_TOL


@pytest.mark.parametrize("gamma_p", [0.0, 1.0, 5.0, 40.0])
def test_mothers_fp32fix_fast_mothers(api, torch, oracle, gamma_p):
    """Mothers of mass 3.0969 with momentum up to 40 GeV (gamma up to 13).  The float kinematics of
    the decay are done in the mother's rest frame, where their errors are about 5e-7 of the
    daughters' energies there; a daughter thrown backwards ends with a lab energy up to about
    gamma times smaller, so the contract for this form is 1e-6 times the largest mother gamma
    (1e-6 for the slow mothers of a decay chain, and FP64 for very fast ones)."""
    n = 1 << 16
    m = [0.1056583745, 0.1056583745, 0.13957]
    M = 3.0969
    rng = np.random.default_rng(7)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = d * gamma_p * rng.uniform(0.5, 1.0, size=(n, 1))
    mothers = np.concatenate([np.sqrt(M * M + (p * p).sum(axis=1, keepdims=True)), p], axis=1)
    ch = api.make_channel(m, M, 0x3039, "philox")
    och = oracle.make_channel(m, M, 0x3039, oracle.ENGINE_PHILOX)
    four = torch.zeros((3, n, 4), dtype=torch.float64, device="cuda")
    api.generate_mothers(ch, 0, torch.as_tensor(mothers, device="cuda"), four, None, precision="fp32_fix")
    torch.cuda.synchronize()
    rfour, _ = oracle.generate_mothers(och, 0, mothers)
    e4 = enorm(four.cpu().numpy(), rfour)
    gamma = float((mothers[:, 0] / M).max())
    print(f"\n[fp32_fix mothers] |p| up to {gamma_p} (gamma {gamma:.2f}): four {e4:.3e}")
    assert e4 <= FP32_TOL * max(1.0, gamma)


@pytest.mark.parametrize("engine", ["philox", "squares3"])
def test_average_mothers_fp32fix(api, torch, oracle, engine):
    n = 1 << 20
    m = [0.493677, 0.13957, 0.13957]
    M = 1.86484
    rng = np.random.default_rng(11)
    p = rng.normal(scale=0.8, size=(n, 3))
    mothers = np.concatenate([np.sqrt(M * M + (p * p).sum(axis=1, keepdims=True)), p], axis=1)
    ch = api.make_channel(m, M, 0x3039, engine)
    och = oracle.make_channel(m, M, 0x3039, oracle.ENGINE_PHILOX if engine == "philox" else oracle.ENGINE_SQUARES3)
    fn = api.functor_bw2(1, 2, 0.8955, 0.0473)     # K pi pair, indices count the mother as 0
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.average_on_mothers(ch, 0, torch.as_tensor(mothers, device="cuda"), fn, out, precision="fp32_fix")
    mean, m2, W = out.cpu().tolist()
    rmean, rm2, rW = oracle.average_mothers(och, oracle.make_functor(2, 1, 2, 0.8955, 0.0473), 0, mothers)
    sigma = np.sqrt(rm2) / rW
    print(f"\n[fp32_fix AverageMothers] {engine}: rel err mean {abs(mean - rmean) / abs(rmean):.3e}")
    assert abs(mean - rmean) <= FP32_TOL * abs(rmean)
    assert abs(mean - rmean) <= 3 * sigma


def heavy_mothers(n, seed, mass_lo, mass_hi, p_max):
    """n mother four-vectors with masses uniform in [mass_lo, mass_hi] and momenta up to p_max in
    random directions."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = d * rng.uniform(0.0, p_max, size=(n, 1))
    m = rng.uniform(mass_lo, mass_hi, size=(n, 1))
    return np.concatenate([np.sqrt(m * m + (p * p).sum(axis=1, keepdims=True)), p], axis=1)


@pytest.mark.parametrize("engine", ["philox", "squares3"])
def test_mothers_fp32fix_full_form(api, torch, oracle, engine):
    """The N >= 7 (full float-float) form with per-event mothers: eight pions from mothers of mass
    2.5..4 GeV (the channel's nominal 3 GeV) and momentum up to 1 GeV.  DecayMothers against the
    oracle; EvalMothers (each event's ECM and maximum weight from its own mother, so the float-float
    weight's fixed scalings are off by up to the mass ratio) in FP32_FIX against the FP64 form;
    AverageMothers against the oracle.  Four-vectors within 1e-6 x the mothers' largest gamma."""
    n = 1 << 14
    N, M = 8, 3.0
    m = [0.13957] * N
    mothers = heavy_mothers(n, 23, 2.5, 4.0, 1.0)
    eng = oracle.ENGINE_PHILOX if engine == "philox" else oracle.ENGINE_SQUARES3
    ch = api.make_channel(m, M, 0x3039, engine)
    och = oracle.make_channel(m, M, 0x3039, eng)
    mo = torch.as_tensor(mothers, device="cuda")
    gamma = float((mothers[:, 0] / np.sqrt(mothers[:, 0] ** 2 - (mothers[:, 1:] ** 2).sum(axis=1))).max())
    # DecayMothers (the channel's ECM; boost by each mother)
    four = torch.zeros((N, n, 4), dtype=torch.float64, device="cuda")
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    api.generate_mothers(ch, 0, mo, four, w, precision="fp32_fix")
    torch.cuda.synchronize()
    rfour, rw = oracle.generate_mothers(och, 0, mothers)
    e4 = enorm(four.cpu().numpy(), rfour)
    ew = float((np.abs(w.cpu().numpy() - rw) / rw).max())
    # EvalMothers: FP32_FIX against FP64 (pinned to the reference fixtures above)
    fn = api.functor_mass2(1, 2)
    w32, w64 = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(2))
    f32, f64 = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(2))
    api.evaluate_mothers(ch, 0, mo, [fn], w32, [f32], precision="fp32_fix")
    api.evaluate_mothers(ch, 0, mo, [fn], w64, [f64], precision="fp64")
    torch.cuda.synchronize()
    a, b = w32.cpu().numpy(), w64.cpu().numpy()
    ok = b > 0
    eew = float((np.abs(a[ok] - b[ok]) / b[ok]).max())
    # AverageMothers
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.average_on_mothers(ch, 0, mo, api.functor_mass2(1, 2), out, precision="fp32_fix")
    mean, m2, W = out.cpu().tolist()
    rmean, rm2, rW = oracle.average_mothers(och, oracle.make_functor(1, 1, 2), 0, mothers)
    print(f"\n[fp32_fix mothers N=8] {engine}: gamma {gamma:.2f}, DecayMothers four {e4:.3e} weight {ew:.3e}, "
          f"EvalMothers weight {eew:.3e}, AverageMothers mean {abs(mean - rmean) / abs(rmean):.3e}")
    assert e4 <= FP32_TOL * gamma and ew <= FP32_TOL
    assert eew <= FP32_TOL
    assert abs(mean - rmean) <= FP32_TOL * abs(rmean)
