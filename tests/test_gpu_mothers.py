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


def test_mothers_reject_fp32fix(api, torch, hps):
    ch = api.make_channel([0.1, 0.2], 1.0, 1)
    mo = torch.zeros((4, 4), dtype=torch.float64, device="cuda")
    four = torch.zeros((2, 4, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(hps.HpsError, match="FP64 only"):
        api.generate_mothers(ch, 0, mo, four, precision="fp32_fix")
