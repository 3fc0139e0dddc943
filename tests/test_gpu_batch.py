"""Batched persistent kernel: many channels of uneven N and event counts in one graph launch.

The contract: each item's outputs are bit-identical to the same request made alone
(hps_generate / hps_average_on at FP32_FIX), whatever else is in the batch and whatever launch
shape the autotuner picks; and they meet the FP32_FIX precision bar against the oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MASS_MENU = [0.13957, 0.493677, 0.938272, 1.86484]


@pytest.fixture(scope="module")
def api(hps, cuda):
    from hydra_gb300 import api as A
    return A


@pytest.fixture(scope="module")
def torch():
    import torch as T
    return T


def make_mix(api, torch, n_channels, seed, n_lo=1e3, n_hi=2e5):
    """Channels drawn like the batched workload: N uniform in 2..10, masses from the menu,
    M uniform in [1.2 sum m, sum m + 6], events log-uniform, half store / half AverageOn."""
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n_channels):
        N = int(rng.integers(2, 11))
        m = list(rng.choice(MASS_MENU, size=N))
        sm = float(sum(m))
        M = float(rng.uniform(1.2 * sm, sm + 6.0))
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        engine = "philox" if c % 3 else "squares3"
        ch = api.make_channel(m, M, 0x3039 + c, engine)
        first = int(rng.integers(0, 1 << 40))
        if c % 2 == 0:
            four = torch.zeros((N, n, 4), dtype=torch.float64, device="cuda")
            w = torch.zeros(n, dtype=torch.float64, device="cuda")
            fl = torch.zeros(n, dtype=torch.uint8, device="cuda")
            out.append(("store", ch, first, n, four, w, fl))
        else:
            fn = api.functor_bw2(0, 1, 0.8955, 0.0473) if N >= 2 else api.functor_one()
            stats = torch.zeros(3, dtype=torch.float64, device="cuda")
            out.append(("avg", ch, first, n, fn, stats))
    return out


def items_of(api, mix):
    items = []
    for r in mix:
        if r[0] == "store":
            _, ch, first, n, four, w, fl = r
            items.append(api.store_item(ch, first, four, w, fl))
        else:
            _, ch, first, n, fn, stats = r
            items.append(api.average_item(ch, first, n, fn, stats))
    return items


def solo(api, torch, r):
    if r[0] == "store":
        _, ch, first, n, four, w, fl = r
        f2 = torch.zeros_like(four)
        w2 = torch.zeros_like(w)
        l2 = torch.zeros_like(fl)
        api.generate(ch, first, f2, w2, l2, precision="fp32_fix")
        return f2, w2, l2
    _, ch, first, n, fn, stats = r
    s2 = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.average_on(ch, first, n, fn, s2, None, precision="fp32_fix")
    return (s2,)


def assert_same_as_alone(api, torch, mix):
    torch.cuda.synchronize()
    for r in mix:
        ref = solo(api, torch, r)
        torch.cuda.synchronize()
        got = r[4:] if r[0] == "store" else (r[5],)
        for a, b in zip(got, ref):
            assert torch.equal(a, b), r[:4]


def test_batch_equals_alone(api, torch):
    mix = make_mix(api, torch, 40, seed=1)
    total_tiles = sum((r[3] + 4095) // 4096 for r in mix if r[0] == "avg")
    plan = api.BatchPlan(64, total_tiles)
    plan.set_items(items_of(api, mix))
    plan.launch()
    assert_same_as_alone(api, torch, mix)
    plan.close()


def test_batch_shapes_and_autotune_do_not_change_results(api, torch, tmp_path):
    mix = make_mix(api, torch, 24, seed=2)
    total_tiles = sum((r[3] + 4095) // 4096 for r in mix if r[0] == "avg")
    plan = api.BatchPlan(24, total_tiles, tuning=(1, 4096))
    plan.set_items(items_of(api, mix))
    plan.launch()
    torch.cuda.synchronize()
    first = [tuple(t.clone() for t in (r[4:] if r[0] == "store" else (r[5],))) for r in mix]
    cache = tmp_path / "tune.txt"
    chosen = plan.autotune(str(cache))
    assert chosen[0] >= 1 and chosen[1] % 256 == 0
    assert cache.read_text().strip()
    for r in mix:                       # clear outputs, rerun with the tuned shape
        for t in (r[4:] if r[0] == "store" else (r[5],)):
            t.zero_()
    plan.launch()
    torch.cuda.synchronize()
    for r, ref in zip(mix, first):
        for a, b in zip(r[4:] if r[0] == "store" else (r[5],), ref):
            assert torch.equal(a, b)
    # the cached choice is reused
    assert plan.autotune(str(cache)) == chosen
    # both kernel forms (one persistent kernel per N, one over every N) and two threads per event
    # give the same bytes
    for form, tpe in ((0, 1), (1, 1), (0, 2)):
        for r in mix:
            for t in (r[4:] if r[0] == "store" else (r[5],)):
                t.zero_()
        plan.set_tuning(3, 8192, form, tpe)
        assert plan.tuning() == (3, 8192, form, tpe)
        plan.launch()
        torch.cuda.synchronize()
        for r, ref in zip(mix, first):
            for a, b in zip(r[4:] if r[0] == "store" else (r[5],), ref):
                assert torch.equal(a, b)
    plan.close()


def test_batch_against_oracle(api, torch, oracle):
    mix = make_mix(api, torch, 12, seed=3, n_lo=2e3, n_hi=3e4)
    total_tiles = sum((r[3] + 4095) // 4096 for r in mix if r[0] == "avg")
    plan = api.BatchPlan(12, total_tiles)
    plan.set_items(items_of(api, mix))
    plan.launch()
    torch.cuda.synchronize()
    for r in mix:
        ch, first, n = r[1], r[2], r[3]
        och = oracle.Channel()
        for f in ("n_daughters", "engine", "seed", "ecm", "max_weight"):
            setattr(och, f, getattr(ch, f))
        for i in range(3):
            och.beta[i] = ch.beta[i]
        for i in range(10):
            och.masses[i] = ch.masses[i]
        if r[0] == "store":
            rfour, rw = oracle.generate(och, first, n)
            g4 = r[4].cpu().numpy()
            assert float((np.abs(g4 - rfour).max(axis=2) / rfour[:, :, 0]).max()) <= 1e-6
            gw = r[5].cpu().numpy()
            ok = rw > 0
            assert float((np.abs(gw[ok] - rw[ok]) / rw[ok]).max()) <= 1e-6
        else:
            fn = r[4]
            mean, m2, W = r[5].cpu().tolist()
            rmean, rm2, rW = oracle.average_on(och, oracle.make_functor(fn.kind, fn.i, fn.j, fn.a, fn.b), first, n, 0)
            assert abs(mean - rmean) <= 1e-6 * abs(rmean)
    plan.close()


def test_batch_rejects_bad_item(api, torch, hps):
    plan = api.BatchPlan(4, 4)
    ch = api.make_channel([0.13957] * 3, 1.0, 1)
    four = torch.zeros((3, 10, 4), dtype=torch.float64, device="cuda")
    bad = api.store_item(ch, 0, four)
    bad.cols[1] = None
    with pytest.raises(hps.HpsError, match="item 0: column 1"):
        plan.set_items([bad])
    stats = torch.zeros(3, dtype=torch.float64, device="cuda")
    big = api.average_item(ch, 0, 10 * 4096, api.functor_one(), stats)
    with pytest.raises(hps.HpsError, match="exceed"):
        plan.set_items([big])
    plan.close()


def test_batch_single_class_empty_and_reordered(api, torch):
    """Items of one N only (the other class kernels find no work and launch one CTA each), an
    empty item list, and a mix given in descending N (the table is reordered by N), on one plan
    whose class kernel grids follow each new table: every item equals its call alone."""
    mix = [r for r in make_mix(api, torch, 60, seed=4) if r[1].n_daughters == 5][:4]
    assert mix
    plan = api.BatchPlan(32, 512)
    plan.set_items(items_of(api, mix))
    plan.launch()
    assert_same_as_alone(api, torch, mix)
    plan.set_items([])
    plan.launch()
    torch.cuda.synchronize()
    mix2 = sorted(make_mix(api, torch, 16, seed=5, n_lo=500, n_hi=5e4), key=lambda r: -r[1].n_daughters)
    assert sum((r[3] + 4095) // 4096 for r in mix2 if r[0] == "avg") <= 512
    plan.set_items(items_of(api, mix2))
    plan.launch()
    assert_same_as_alone(api, torch, mix2)
    plan.close()


def test_config4_every_event_within_contract(api, torch):
    """The batched workload exactly as the bench runs it (256 seeded channels: N uniform in 2..10,
    daughter masses from the menu, mother mass uniform in [1.2 sum m, sum m + 6] GeV, events
    log-uniform 1e3..1e6, about 35 M in all): every event of the one-launch FP32_FIX batch against
    the FP64 form of the same events, within the 1e-6 contract (four-vectors max_k |dp_k| / E,
    weights |dw| / w)."""
    from hydra_gb300 import batch_bench as BB
    chans = BB.make_channels(256)
    outs, items, hch = [], [], []
    for N, m, M, n, seed in chans:
        ch = api.make_channel(m, M, seed, "philox")
        four = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        outs.append((four, w))
        hch.append(ch)
        items.append(api.store_item(ch, 0, four, w))
    plan = api.BatchPlan(len(items), 1)
    plan.set_items(items)
    plan.launch()
    torch.cuda.synchronize()
    e4 = ew = 0.0
    for ch, (four, w) in zip(hch, outs):
        f64, w64 = torch.empty_like(four), torch.empty_like(w)
        api.generate(ch, 0, f64, w64, None, precision="fp64")
        e4 = max(e4, float(((four - f64).abs().amax(dim=2) / f64[:, :, 0]).max()))
        ew = max(ew, float(((w - w64).abs() / w64).max()))
    plan.close()
    print(f"\n[batch config 4] {sum(c[3] for c in chans)} events: four {e4:.3e}, weight {ew:.3e}")
    assert e4 <= 1e-6 and ew <= 1e-6
