"""Serving loop (hps_server_*): continuous batching with admission by memory budget.

* every request's result is bit-identical to the same request run alone (hps_generate /
  hps_average_on at FP32_FIX), whatever it was batched with;
* requests that arrive while others run join later launches; admission is first-in
  first-admitted under the budget; a request that can never fit is refused at submit;
* failures are made on the host: an injected allocation failure, a cancelled request, a wait
  that times out -- no GPU fault is provoked.
"""
from __future__ import annotations

import threading
import time

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


def random_request(api, rng, c, n_lo=1e3, n_hi=2e5):
    N = int(rng.integers(2, 11))
    m = [float(x) for x in rng.choice(MASS_MENU, size=N)]
    M = float(rng.uniform(1.2 * sum(m), sum(m) + 6.0))
    n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
    ch = api.make_channel(m, M, 1000 + c, "philox" if c % 4 else "squares3")
    first = int(rng.integers(0, 1 << 32))
    if c % 2 == 0:
        return api.store_request(ch, first, n, want_flags=(c % 3 == 0))
    return api.average_request(ch, first, n, api.functor_bw2(0, 1, 0.8955, 0.0473))


def alone(api, torch, req):
    ch, first, n = req.channel, req.first_evt, req.n_events
    if req.mode == 0:
        four = torch.zeros((ch.n_daughters, n, 4), dtype=torch.float64, device="cuda")
        w = torch.zeros(n, dtype=torch.float64, device="cuda")
        fl = torch.zeros(n, dtype=torch.uint8, device="cuda") if req.want_flags else None
        api.generate(ch, first, four, w, fl, req.unweight_seed, precision="fp32_fix")
        torch.cuda.synchronize()
        return four, w, fl
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    api.average_on(ch, first, n, req.functor, out, None, precision="fp32_fix")
    torch.cuda.synchronize()
    return out.cpu().tolist()


def check_same(api, torch, req, res):
    assert res.status == 0
    ref = alone(api, torch, req)
    if req.mode == 0:
        four, w, fl = api.result_views(res, req.channel.n_daughters)
        assert torch.equal(four, ref[0]) and torch.equal(w, ref[1])
        if req.want_flags:
            assert torch.equal(fl, ref[2])
    else:
        s = res.stats
        assert [s.mean, s.m2, s.w] == ref


def test_mixed_requests_equal_alone(api, torch):
    server = api.Server(budget_bytes=8 << 30, slice_events=1 << 16, max_batch_items=64)
    rng = np.random.default_rng(7)
    reqs = [random_request(api, rng, c) for c in range(48)]
    tickets = [None] * len(reqs)

    def submitter(lo, hi):
        for i in range(lo, hi):
            tickets[i] = server.submit(reqs[i])
            time.sleep(0.0005)

    ths = [threading.Thread(target=submitter, args=(0, 24)), threading.Thread(target=submitter, args=(24, 48))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    results = [server.wait(t, 60.0) for t in tickets]
    for req, res in zip(reqs, results):
        check_same(api, torch, req, res)
    st = server.stats()
    assert st["completed"] == 48 and st["failed"] == 0 and st["launches"] >= 2
    for t in tickets:
        server.release(t)
    assert server.stats()["bytes_in_use"] == 0
    server.close()


def test_completion_queue_hands_out_each_once(api, torch):
    server = api.Server(budget_bytes=1 << 30)
    rng = np.random.default_rng(11)
    tickets = {server.submit(random_request(api, rng, c, 1e3, 2e4)) for c in range(20)}
    seen = set()
    while len(seen) < 20:
        got = server.next_done(10.0)
        assert got is not None
        t, res = got
        assert res.status == 0 and t in tickets and t not in seen
        seen.add(t)
        server.release(t)
    assert server.next_done(0.01) is None
    server.close()


def test_budget_admission_fifo_and_timeouts(api, torch, hps):
    ch = api.make_channel([0.13957] * 4, 2.0, 5)
    per_req = 4 * 32 * 100_000 + 8 * 100_000            # bytes of one 1e5-event store request
    server = api.Server(budget_bytes=int(per_req * 2.5))
    with pytest.raises(hps.HpsError, match="budget"):
        server.submit(api.store_request(ch, 0, 1_000_000))   # can never fit
    t1 = server.submit(api.store_request(ch, 0, 100_000))
    t2 = server.submit(api.store_request(ch, 100_000, 100_000))
    t3 = server.submit(api.store_request(ch, 200_000, 100_000))   # waits for budget
    r1 = server.wait(t1, 30.0)
    server.wait(t2, 30.0)
    assert r1.status == 0
    with pytest.raises(hps.HpsError, match="still running"):
        server.wait(t3, 0.2)                                # not admitted until a release
    server.release(t1)
    r3 = server.wait(t3, 30.0)
    assert r3.status == 0 and r3.t_admit > r1.t_done
    check_same(api, torch, api.store_request(ch, 200_000, 100_000), r3)
    server.release(t2)
    server.release(t3)
    server.close()


def test_cancel_queued_request(api, torch, hps):
    ch = api.make_channel([0.13957] * 3, 1.0, 9)
    per_req = 3 * 32 * 50_000 + 8 * 50_000
    server = api.Server(budget_bytes=int(per_req * 1.5))
    t1 = server.submit(api.store_request(ch, 0, 50_000))
    t2 = server.submit(api.store_request(ch, 0, 50_000))         # blocked behind t1's memory
    server.cancel(t2)
    res = server.wait(t2, 5.0)
    assert res.status == hps.ERR_BAD_ARG
    with pytest.raises(hps.HpsError, match="not queued"):
        server.cancel(t1 if server.wait(t1, 30.0).status == 0 else t1)
    assert server.stats()["cancelled"] == 1
    server.release(t1)
    server.release(t2)
    server.close()


def test_injected_allocation_failure(api, torch, hps):
    ch = api.make_channel([0.13957] * 3, 1.0, 3)
    server = api.Server(budget_bytes=1 << 30, fail_alloc_after=2)
    tickets = [server.submit(api.store_request(ch, 1000 * i, 10_000)) for i in range(4)]
    res = [server.wait(t, 30.0) for t in tickets]
    assert [r.status for r in res] == [0, hps.ERR_OOM, 0, 0]
    check_same(api, torch, api.store_request(ch, 3000, 10_000), res[3])
    for t in tickets:
        server.release(t)
    st = server.stats()
    assert st["failed"] == 1 and st["completed"] == 3 and st["bytes_in_use"] == 0
    server.close()
