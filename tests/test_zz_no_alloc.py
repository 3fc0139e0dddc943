"""hps_average_on_noalloc: AverageOn for callers that may not allocate device memory.

Some host programs reserve all device memory for their own pool when they start, or run under
a fixed quota on a shared GPU, and must not let a library call cudaMalloc later on.  The
allocation-free entry point keeps its scratch in a fixed device array inside libhps.so.  These
tests call it through the C ABI and compare it with hps_average_on (which allocates its scratch
or takes a workspace) on two calls in a row, and check that oversized requests are refused.

Collected last on purpose (file name), so a run that stops at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes

import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10          # the AverageOn tolerance of tests/test_gpu_parity.py
PI, K = 0.13957, 0.493677


@pytest.fixture(scope="module")
def api(hps, cuda):
    from hydra_gb300 import api as A
    return A


def _noalloc(hps, ch, first, n, fn, out, precision, stream):
    return hps.lib().hps_average_on_noalloc(ctypes.byref(ch), first, n, ctypes.byref(fn),
                                            ctypes.c_void_p(out.data_ptr()), precision, stream)


def _allocating(hps, ch, first, n, fn, out, precision, stream):
    return hps.lib().hps_average_on(ctypes.byref(ch), first, n, ctypes.byref(fn),
                                    ctypes.c_void_p(out.data_ptr()), None, 0, precision, stream)


def _close(a, b):
    return all(abs(x - y) <= TOL * max(abs(y), 1e-300) for x, y in zip(a, b))


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_average_on_two_calls(hps, api, precision):
    import torch
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # the second call covers fewer tiles than the first, so stale partials left in the shared
    # array by call 1 would show up if the call read anything it had not written
    calls = [
        (api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, "philox"), 0, 3_000_001,
         api.functor_bw2(0, 1, 0.8955, 0.0473)),
        (api.make_channel([3.0969, K, PI], 5.27934, 77, "squares3"), 12_345, 250_000,
         api.functor_mass2(1, 2)),
    ]
    for ch, first, n, fn in calls:
        got = torch.zeros(3, dtype=torch.float64, device="cuda")
        ref = torch.zeros(3, dtype=torch.float64, device="cuda")
        assert _noalloc(hps, ch, first, n, fn, got, precision, stream) == hps.OK, hps.lib().hps_last_error()
        assert _allocating(hps, ch, first, n, fn, ref, precision, stream) == hps.OK, hps.lib().hps_last_error()
        torch.cuda.synchronize()
        g, r = got.cpu().tolist(), ref.cpu().tolist()
        assert r[2] > 0 and _close(g, r), (g, r)


def test_noalloc_rejects_oversized_request(hps, api):
    import torch
    limit = 16384 * 4096
    ch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, "philox")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    st = _noalloc(hps, ch, 0, limit + 1, api.functor_one(), out, 0, None)
    assert st == hps.ERR_BAD_ARG
    assert b"allocation-free limit" in hps.lib().hps_last_error()
    torch.cuda.synchronize()
    assert out.cpu().tolist() == [0.0, 0.0, 0.0]       # nothing was launched


def test_noalloc_at_the_limit_and_empty(hps, api):
    """n exactly HPS_NOALLOC_MAX_EVENTS writes and reads the last entry of the array; n = 0
    launches no tile and returns an empty StatsPHSP."""
    import torch
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    limit = 16384 * 4096
    ch = api.make_channel([K, PI, PI, PI, PI], 1.86484, 0x3039, "philox")
    fn = api.functor_bw2(0, 1, 0.8955, 0.0473)
    got = torch.zeros(3, dtype=torch.float64, device="cuda")
    ref = torch.zeros(3, dtype=torch.float64, device="cuda")
    assert _noalloc(hps, ch, 7, limit, fn, got, 1, stream) == hps.OK, hps.lib().hps_last_error()
    assert _allocating(hps, ch, 7, limit, fn, ref, 1, stream) == hps.OK, hps.lib().hps_last_error()
    torch.cuda.synchronize()
    g, r = got.cpu().tolist(), ref.cpu().tolist()
    assert r[2] > 0 and _close(g, r), (g, r)
    for precision in (0, 1):
        out = torch.full((3,), 7.0, dtype=torch.float64, device="cuda")
        assert _noalloc(hps, ch, 0, 0, fn, out, precision, stream) == hps.OK, hps.lib().hps_last_error()
        torch.cuda.synchronize()
        assert out.cpu().tolist() == [0.0, 0.0, 0.0]
