"""Product kernels against the reference's OWN CUDA device code on the same GPU.

oracle/ref_gpu.py launches hydra::detail::DecayMother / AverageMother compiled by nvcc for
sm_103a from the unmodified Hydra headers (a cubin built where the Hydra tree is present;
the tests skip when it was not built).  This pins the product to what a user of the
reference's CUDA backend gets on this GPU, not only to the CPU build:
  FP64 form     four-vectors within 1e-12 of the reference's CUDA ones (energy-normalised;
                nvcc contracts the reference's mul+add pairs into FMAs, so the two differ
                by a few ulps), AverageOn mean within 1e-12 and error within 1e-9 relative
                (same events, different summation order);
  FP32_FIX form within its 1e-6 contract of the reference's CUDA output (AverageOn's error
                estimate within 1e-4).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PI, K = 0.13957, 0.493677

CASES = [
    ("n3_b0_jpsikpi", 3, "philox", 5.27934, [3.0969, K, PI], None, 0),
    ("n5_d0_kpipipipi", 5, "philox", 1.86484, [K, PI, PI, PI, PI], None, 0),
    ("n10_pions", 10, "philox", 5.0, [PI] * 10, None, 1 << 20),
    ("n2", 2, "philox", 3.0, [1.0, 0.5], None, 7),
    ("n4_sq", 4, "squares3", 3.0, [0.1, 0.2, 0.3, 0.4], None, 0),
    ("n7_sq_moving", 7, "squares3", 6.0, [PI, K, 0.938272, PI, PI, K, PI], [6.5, 1.0, -2.0, 1.5], 99),
]


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference cubin not built (oracle/build_ref.sh needs the Hydra sources)")
    return ref_gpu


@pytest.fixture(scope="module")
def api(hps, cuda):
    from hydra_gb300 import api as A
    return A


@pytest.fixture(scope="module")
def torch():
    import torch as T
    return T


def _rel4(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return float((np.abs(a - b).max(axis=2) / np.abs(b[:, :, 0])).max())


@pytest.mark.parametrize("name,N,engine,M,masses,mother,first", CASES, ids=[c[0] for c in CASES])
def test_generate_vs_reference_cuda(api, ref, torch, name, N, engine, M, masses, mother, first):
    n = 1 << 16
    ch = api.make_channel(masses, M, 0x3039, engine, mother=mother)
    want = ref.generate(ch, first, n)
    got = torch.empty((N, n, 4), dtype=torch.float64, device="cuda")
    api.generate(ch, first, got, precision="fp64")
    fast = torch.empty_like(got)
    api.generate(ch, first, fast, precision="fp32_fix")
    torch.cuda.synchronize()
    assert _rel4(got, want) <= 1e-12
    assert _rel4(fast, want) <= 1e-6


@pytest.mark.parametrize("first,n", [(0, 1 << 18), (12345, 100003)])
def test_average_on_vs_reference_cuda(api, ref, torch, first, n):
    masses, M = [K, PI, PI, PI, PI], 1.86484
    ch = api.make_channel(masses, M, 0x3039, "philox")
    want_mean, want_err = ref.average_bw(ch, 0, 1, 0.8955, 0.0473, first, n)
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    res = {}
    for prec in ("fp64", "fp32_fix"):
        api.average_on(ch, first, n, api.functor_bw2(0, 1, 0.8955, 0.0473), out, precision=prec)
        mean, m2, w = out.cpu().tolist()
        res[prec] = (mean, np.sqrt(m2) / w)
    assert abs(res["fp64"][0] - want_mean) <= 1e-12 * abs(want_mean)
    assert abs(res["fp64"][1] - want_err) <= 1e-9 * want_err
    assert abs(res["fp32_fix"][0] - want_mean) <= 1e-6 * abs(want_mean)
    # the error estimate sums squares of |BW|^2 values, whose float error is amplified
    # near the pole (same bound as the FP32_FIX AverageOn test against the CPU oracle)
    assert abs(res["fp32_fix"][1] - want_err) <= 1e-4 * want_err


def test_empty_and_ragged(api, ref, torch):
    ch = api.make_channel([K, PI, PI], 1.86484, 0x3039, "philox")
    empty = ref.generate(ch, 0, 0)
    assert empty.shape == (3, 0, 4)
    n = 257                       # one full block and one event in the next
    want = ref.generate(ch, 5, n)
    got = torch.empty((3, n, 4), dtype=torch.float64, device="cuda")
    api.generate(ch, 5, got, precision="fp64")
    torch.cuda.synchronize()
    assert _rel4(got, want) <= 1e-12


@pytest.mark.parametrize("name,N,engine,M,masses,mother,first", [CASES[0], CASES[1], CASES[2], CASES[5]],
                         ids=[CASES[k][0] for k in (0, 1, 2, 5)])
def test_evaluate_vs_reference_cuda(api, ref, torch, oracle, name, N, engine, M, masses, mother, first):
    """Evaluate (EvalMother) with |BW(m_01)|^2 and m^2(p_0 + p_1): the generation-time weight and
    both functor values per event.  The reference's CUDA build contracts the products and sums of
    pdk into FMAs, so its weights are not its CPU build's: near threshold, where a - b - c
    cancels, the two builds differ by up to about 1e-10 relative (the FP64 kernels here follow
    the CPU build bit for bit).  The weight bar against the CUDA build is therefore 1e-9, and
    the test checks that the CPU oracle sits at the same distance from it."""
    n = 1 << 16
    ch = api.make_channel(masses, M, 0x3039, engine, mother=mother)
    rw, rbw, rm2 = ref.evaluate(ch, first, n)
    fns = [api.functor_bw2(0, 1, 0.8955, 0.0473), api.functor_mass2(0, 1)]
    res = {}
    for prec in ("fp64", "fp32_fix"):
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        outs = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in fns]
        api.evaluate(ch, first, n, fns, w, outs, precision=prec)
        res[prec] = (w, *outs)
    torch.cuda.synchronize()
    rw, rbw, rm2 = (t.cpu().numpy() for t in (rw, rbw, rm2))
    scale = M * M                                  # m^2 errors measured against the mother's M^2
    w64, bw64, m264 = (t.cpu().numpy() for t in res["fp64"])
    ok = rw > 0
    och = oracle.make_channel(masses, M, 0x3039, oracle.ENGINE_PHILOX if engine == "philox" else oracle.ENGINE_SQUARES3,
                              mother=mother)
    cw, _ = oracle.evaluate(och, oracle.make_functor(0), first, n)
    assert np.array_equal(w64, cw)                 # FP64 weights: the reference's CPU arithmetic
    gap = float((np.abs(w64[ok] - rw[ok]) / rw[ok]).max())
    print(f"\n[reference CUDA vs CPU build] {name}: max weight difference {gap:.2e}")
    assert gap <= 1e-9
    assert float((np.abs(bw64 - rbw) / rbw).max()) <= 1e-9
    assert float(np.abs(m264 - rm2).max()) <= 1e-12 * scale
    w32, bw32, m232 = (t.cpu().numpy() for t in res["fp32_fix"])
    assert float((np.abs(w32[ok] - rw[ok]) / rw[ok]).max()) <= 1e-6
    assert float(np.abs(m232 - rm2).max()) <= 1e-6 * scale


def _mothers(torch, n, M, pscale, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(scale=pscale, size=(n, 3))
    m = np.concatenate([np.sqrt(M * M + (p * p).sum(axis=1, keepdims=True)), p], axis=1)
    return torch.as_tensor(m, device="cuda")


@pytest.mark.parametrize("engine", ["philox", "squares3"])
@pytest.mark.parametrize("N", [3, 5])
def test_mothers_vs_reference_cuda(api, ref, torch, engine, N):
    """DecayMothers and AverageMothers (one mother per event, moving): FP64 within 1e-12 of the
    reference's CUDA four-vectors, FP32_FIX within 1e-6 times the largest mother gamma."""
    masses = [0.493677] + [0.13957] * (N - 1)
    M = 1.86484
    n = 1 << 15
    mothers = _mothers(torch, n, M, 0.8, seed=N)
    ch = api.make_channel(masses, M, 0x3039, engine)
    want = ref.generate_mothers(ch, 17, mothers)
    got = torch.empty_like(want)
    api.generate_mothers(ch, 17, mothers, got, None, precision="fp64")
    fast = torch.empty_like(want)
    api.generate_mothers(ch, 17, mothers, fast, None, precision="fp32_fix")
    torch.cuda.synchronize()
    gamma = float((mothers[:, 0] / M).max())
    assert _rel4(got, want) <= 1e-12
    assert _rel4(fast, want) <= 1e-6 * max(1.0, gamma)
    rmean, rerr = ref.average_mothers_bw(ch, 1, 2, 0.8955, 0.0473, 17, mothers)
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    api.average_on_mothers(ch, 17, mothers, api.functor_bw2(1, 2, 0.8955, 0.0473), out, precision="fp64")
    mean, m2, w = out.cpu().tolist()
    assert abs(mean - rmean) <= 1e-12 * abs(rmean)
    assert abs(np.sqrt(m2) / w - rerr) <= 1e-9 * rerr
