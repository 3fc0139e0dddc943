"""Launch sizes past the 32-bit boundaries of the index arithmetic.

Every event depends only on its index (its random stream is keyed by seed and event number), so
the events of one large launch must equal, bit for bit, the same events produced by a small launch
that starts at them.  That checks a large launch at full size without an oracle run of its size:

  * Generate / Evaluate with n = 2^28 + 5: each Decays column spans 8 GiB, so the byte offsets of
    the stores cross 2^31 and 2^32 (at events 2^26 and 2^27); windows at those events, at the
    last events and at the first ones are compared with small launches at the same first event.
  * AverageOn with n = 2^32 + 4099 events, which passes the 32-bit event count itself (nothing is
    stored, so this costs no memory): the whole call against the same range in five calls merged
    with AddStatsPHSP (hydra/detail/functors/StatsPHSP.h:67-84).  The tile partials and the shift
    differ between the two, so the comparison is to rounding: relative 1e-10.

Channel: B0 -> J/psi K pi (M = 5.27934 GeV; 3.0969, 0.493677, 0.13957 GeV), Philox, seed 0x3039.
Memory held: about 28 GB for the Generate case.
"""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

MASSES = [3.0969, 0.493677, 0.13957]
M = 5.27934
N_GEN = (1 << 28) + 5
WINDOW = 4096 + 37
N_AVG = (1 << 32) + 4099


def windows(n: int):
    return [0, (1 << 26) - 1000, (1 << 27) - 1000, (1 << 27) + 12345, n - WINDOW]


@pytest.fixture(scope="module")
def api(hps):
    from hydra_gb300 import api as A
    return A


@pytest.mark.parametrize("precision", ["fp32_fix", "fp64"])
def test_generate_columns_past_4gib(api, cuda, precision):
    import torch

    ch = api.make_channel(MASSES, M, 0x3039, "philox")
    four = torch.empty((3, N_GEN, 4), dtype=torch.float64, device=cuda)
    w = torch.empty(N_GEN, dtype=torch.float64, device=cuda)
    fl = torch.empty(N_GEN, dtype=torch.uint8, device=cuda)
    api.generate(ch, 0, four, w, fl, precision=precision)
    f_s = torch.empty((3, WINDOW, 4), dtype=torch.float64, device=cuda)
    w_s = torch.empty(WINDOW, dtype=torch.float64, device=cuda)
    fl_s = torch.empty(WINDOW, dtype=torch.uint8, device=cuda)
    for a in windows(N_GEN):
        api.generate(ch, a, f_s, w_s, fl_s, precision=precision)
        assert torch.equal(four[:, a:a + WINDOW], f_s), f"four-vectors differ in the window at event {a}"
        assert torch.equal(w[a:a + WINDOW], w_s), f"weights differ in the window at event {a}"
        assert torch.equal(fl[a:a + WINDOW], fl_s), f"flags differ in the window at event {a}"
    del four, w, fl
    torch.cuda.empty_cache()


@pytest.mark.parametrize("precision", ["fp32_fix", "fp64"])
def test_evaluate_past_4gib(api, cuda, precision):
    import torch

    ch = api.make_channel(MASSES, M, 0x3039, "philox")
    fns = [api.functor_mass2(1, 2), api.functor_bw2(0, 1, 3.5, 0.2)]
    w = torch.empty(N_GEN, dtype=torch.float64, device=cuda)
    outs = [torch.empty(N_GEN, dtype=torch.float64, device=cuda) for _ in fns]
    api.evaluate(ch, 0, N_GEN, fns, w, outs, precision=precision)
    w_s = torch.empty(WINDOW, dtype=torch.float64, device=cuda)
    outs_s = [torch.empty(WINDOW, dtype=torch.float64, device=cuda) for _ in fns]
    for a in windows(N_GEN):
        api.evaluate(ch, a, WINDOW, fns, w_s, outs_s, precision=precision)
        assert torch.equal(w[a:a + WINDOW], w_s), f"weights differ in the window at event {a}"
        for big, small in zip(outs, outs_s):
            assert torch.equal(big[a:a + WINDOW], small), f"functor values differ in the window at event {a}"
    del w, outs
    torch.cuda.empty_cache()


@pytest.mark.parametrize("precision", ["fp32_fix", "fp64"])
def test_average_on_past_2_32_events(api, cuda, precision):
    import torch
    from hydra_gb300.shard import merge_in_order

    ch = api.make_channel(MASSES, M, 0x3039, "philox")
    fn = api.functor_mass2(1, 2)
    out = torch.zeros(3, dtype=torch.float64, device=cuda)
    api.average_on(ch, 0, N_AVG, fn, out, precision=precision)
    whole = out.tolist()
    cuts = [0, 1 << 30, 1 << 31, 3 << 30, 1 << 32, N_AVG]
    parts = []
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        out.zero_()
        api.average_on(ch, lo, hi - lo, fn, out, precision=precision)
        parts.append(out.tolist())
    merged = merge_in_order(parts)
    print(f"\n[large average_on {precision}] n={N_AVG}: whole {whole}, merged {list(merged)}")
    for k, name in enumerate(("mean", "M2", "W")):
        assert merged[k] == pytest.approx(whole[k], rel=1e-10), name
    # the count is past 2^32: W is the sum of that many positive weights
    assert whole[2] > 0.0 and whole[1] > 0.0
