"""hps_generate_average: Generate and AverageOn of the same events in one pass must give exactly the
results of the two separate calls (same events, same tiles, same reduction order)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PI, K = 0.13957, 0.493677


@pytest.fixture(scope="module")
def api(hps, cuda):
    from hydra_gb300 import api as A
    return A


@pytest.fixture(scope="module")
def torch():
    import torch as T
    return T


@pytest.mark.parametrize("precision", ["fp32_fix", "fp64"])
@pytest.mark.parametrize("masses,M,engine,n,first", [
    ([K, PI, PI, PI, PI], 1.86484, "philox", 1 << 20, 0),
    ([3.0969, K, PI], 5.27934, "squares3", 100_003, 17),
    ([PI] * 10, 5.0, "philox", 50_000, 4095),
])
def test_fused_equals_separate_calls(api, torch, precision, masses, M, engine, n, first):
    N = len(masses)
    ch = api.make_channel(masses, M, 0x3039, engine)
    fn = api.functor_bw2(0, 1, 0.8955, 0.0473)
    f1 = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
    w1 = torch.empty(n, dtype=torch.float64, device="cuda")
    g1 = torch.empty(n, dtype=torch.uint8, device="cuda")
    s1 = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.generate(ch, first, f1, w1, g1, precision=precision)
    api.average_on(ch, first, n, fn, s1, None, precision)
    f2 = torch.empty_like(f1)
    w2 = torch.empty_like(w1)
    g2 = torch.empty_like(g1)
    s2 = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.generate_average(ch, first, f2, w2, g2, fn, s2, precision=precision)
    torch.cuda.synchronize()
    assert torch.equal(f1, f2) and torch.equal(w1, w2) and torch.equal(g1, g2)
    assert s1.tolist() == s2.tolist()


def test_fused_without_weights_and_flags(api, torch):
    ch = api.make_channel([K, PI, PI], 1.86484, 7, "philox")
    fn = api.functor_mass2(0, 1)
    n = 9000
    f = torch.empty((3, n, 4), dtype=torch.float64, device="cuda")
    s = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.generate_average(ch, 0, f, None, None, fn, s, precision="fp32_fix")
    f1 = torch.empty_like(f)
    s1 = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.generate(ch, 0, f1, None, None, precision="fp32_fix")
    api.average_on(ch, 0, n, fn, s1, None, "fp32_fix")
    torch.cuda.synchronize()
    assert torch.equal(f, f1) and s.tolist() == s1.tolist()


@pytest.mark.parametrize("pinned", [True, False])
def test_fused_host_equals_separate_calls(api, torch, pinned):
    ch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, "philox")
    fn = api.functor_bw2(0, 1, 0.8955, 0.0473)
    n = 300_001
    f1 = torch.empty((5, n, 4), dtype=torch.float64, device="cuda")
    w1 = torch.empty(n, dtype=torch.float64, device="cuda")
    g1 = torch.empty(n, dtype=torch.uint8, device="cuda")
    s1 = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.generate(ch, 5, f1, w1, g1, precision="fp32_fix")
    api.average_on(ch, 5, n, fn, s1, None, "fp32_fix")
    hf = torch.zeros((5, n, 4), dtype=torch.float64)
    hw = torch.zeros(n, dtype=torch.float64)
    hg = torch.zeros(n, dtype=torch.uint8)
    if pinned:
        hf, hw, hg = hf.pin_memory(), hw.pin_memory(), hg.pin_memory()
    s2 = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.generate_average_host(ch, 5, hf, hw, hg, fn, s2, precision="fp32_fix")
    torch.cuda.synchronize()
    assert torch.equal(f1.cpu(), hf) and torch.equal(w1.cpu(), hw) and torch.equal(g1.cpu(), hg)
    assert s1.tolist() == s2.tolist()
