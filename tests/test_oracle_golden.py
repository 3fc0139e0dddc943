"""The oracle (oracle/genbod_oracle.c) against fixtures produced by the reference itself.

Everything here is bit-exact: the fixtures come from Hydra's own PhaseSpace / Decays /
engines built with -ffp-contract=off (tests/golden/make_golden.py), and the oracle is
built the same way.  When the reference harness is built in this checkout
(oracle/_ref/, only where the Hydra sources exist) the oracle is also compared with it
live on fresh seeds.
"""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import AVG_GOLDEN, EXTRA_GOLDEN, GEN_GOLDEN, MOTHER_GOLDEN, REPO, RNG_GOLDEN, load_golden

REF = REPO / "oracle" / "_ref" / "ref_harness_cpp"


def _channel(O, g):
    seed = int(g["seed"])
    if seed == -1:
        seed = int(g["default_seed"])
    elif seed < 0 or seed >= 2**31:
        seed = seed & 0xFFFFFFFF
        seed = (seed - (1 << 32)) & (2**64 - 1) if seed >= (1 << 31) else seed
    return O.make_channel(g["masses"], float(g["M"]), seed, int(g["engine"]),
                          mother=g["mother"] if "mother" in g else None)


@pytest.mark.parametrize("name", RNG_GOLDEN)
def test_rng_words_bit_exact(oracle, name):
    g = load_golden(name)
    words = oracle.rng_words(int(g["N"]), int(g["engine"]), int(g["seed"]), 0, int(g["n"]))
    assert np.array_equal(words, g["words"])


@pytest.mark.parametrize("name", RNG_GOLDEN)
def test_rng_offset_consistency(oracle, name):
    """Event e's stream does not depend on where a call starts (counter-based streams)."""
    g = load_golden(name)
    n = int(g["n"])
    a = oracle.rng_words(int(g["N"]), int(g["engine"]), int(g["seed"]), 5, n - 5)
    assert np.array_equal(a, g["words"][5:])


@pytest.mark.parametrize("name", GEN_GOLDEN)
def test_generate_bit_exact(oracle, name):
    g = load_golden(name)
    ch = _channel(oracle, g)
    assert ch.max_weight == g["max_weight"] and ch.ecm == g["ecm"]
    four, w = oracle.generate(ch, 0, int(g["n"]), nthreads=1)
    assert np.array_equal(four, g["four"])
    assert np.array_equal(w, g["w_gen"])


@pytest.mark.parametrize("name", GEN_GOLDEN)
def test_evaluate_bit_exact(oracle, name):
    g = load_golden(name)
    ch = _channel(oracle, g)
    f = g["functor"]
    fn = oracle.make_functor(int(f[0]), int(f[1]), int(f[2]), float(f[3]), float(f[4]))
    w, fv = oracle.evaluate(ch, fn, 0, int(g["n"]), nthreads=1)
    assert np.array_equal(w, g["w_gen"])
    assert np.array_equal(fv, g["f_val"])


@pytest.mark.parametrize("name", GEN_GOLDEN)
def test_recomputed_weight_and_flags_bit_exact(oracle, name):
    g = load_golden(name)
    ch = _channel(oracle, g)
    wr = oracle.recompute_weights(ch, g["four"], g["decays_max_weight"])
    assert np.array_equal(wr, g["w_rec"])
    fl = oracle.flags(wr, float(g["decays_max_weight"]), int(g["useed"]))
    assert np.array_equal(fl, g["flags"])
    assert int(fl.sum()) == int(g["n_unweighted"])          # Decays::Unweight() kept exactly these


@pytest.mark.parametrize("name", AVG_GOLDEN)
def test_average_on_sequential_fold_bit_exact(oracle, name):
    """nthreads=1 folds events in index order, as the reference's cpp backend does."""
    g = load_golden(name)
    ch = oracle.make_channel(g["masses"], float(g["M"]), int(g["seed"]), int(g["engine"]))
    f = g["functor"]
    fn = oracle.make_functor(int(f[0]), int(f[1]), int(f[2]), float(f[3]), float(f[4]))
    mean, m2, w = oracle.average_on(ch, fn, 0, int(g["n"]), nthreads=1)
    assert mean == g["mean"]
    assert np.sqrt(m2) / w == g["err"]


def test_generate_threads_identical(oracle):
    g = load_golden("d0_kpipipipi_n5_philox")
    ch = _channel(oracle, g)
    a = oracle.generate(ch, 0, 3000, nthreads=1)
    b = oracle.generate(ch, 0, 3000, nthreads=0)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_quirk_moving_mother_not_boosted(oracle):
    """Q1: the reference's final-boost vector is (E,px,py)/E, |beta| >= 1, so no boost."""
    g = load_golden("n6_philox_moving")
    s = g["four"].sum(axis=0)
    assert np.allclose(s[:, 0], g["M"], rtol=0, atol=1e-12)
    assert np.allclose(s[:, 1:], 0.0, atol=1e-12)


def test_channel_errors(oracle):
    with pytest.raises(ValueError):
        oracle.make_channel([0.1, -0.2], 1.0, 1)
    with pytest.raises(ValueError):
        oracle.make_channel([0.1, 0.2], 0.0, 1)
    with pytest.raises(RuntimeError):
        oracle.make_channel([0.6, 0.5], 1.0, 1)


def _ref_gen(args, tmp_path):
    out = tmp_path / "o.bin"
    subprocess.run([str(REF)] + [str(a) for a in args] + [str(out)], check=True)
    return np.fromfile(out, dtype=np.float64)


@pytest.mark.skipif(not REF.exists(), reason="reference harness not built in this checkout")
@pytest.mark.parametrize("N,engine,seed", [(3, 0, 1), (5, 1, 77), (9, 0, 424242), (10, 1, 5)])
def test_oracle_against_live_reference(oracle, tmp_path, N, engine, seed):
    rng = np.random.default_rng(seed)
    masses = rng.choice([0.13957, 0.493677, 0.938272, 1.86484], size=N)
    M = float(1.2 * masses.sum() + rng.uniform(0, 3))
    n = 200
    args = ["gen", N, engine, seed, n, repr(M)] + [repr(float(x)) for x in masses] + \
           [1, 0, N - 1, "0.0", "0.0", hex(oracle.DEFAULT_UNWEIGHT_SEED), "0", "0", "0"]
    d = _ref_gen(args, tmp_path)
    ch = oracle.make_channel(masses, M, seed, engine)
    four, w = oracle.generate(ch, 0, n, nthreads=1)
    assert np.array_equal(four, d[:n * N * 4].reshape(n, N, 4).transpose(1, 0, 2))
    assert np.array_equal(w, d[n * N * 4:n * N * 4 + n])


@pytest.mark.parametrize("name", MOTHER_GOLDEN)
def test_mothers_variants_bit_exact(oracle, name):
    """DecayMothers (Generate), AverageMothers (AverageOn, sequential fold) and EvalMothers
    (Evaluate: hash(evt, seed) streams, per-event ECM from the mother's mass)."""
    g = load_golden(name)
    ch = oracle.make_channel(g["masses"], float(g["M"]), int(g["seed"]), int(g["engine"]))
    four, _ = oracle.generate_mothers(ch, 0, g["mothers"], nthreads=1)
    assert np.array_equal(four, g["four"])
    f = g["functor"]
    fn = oracle.make_functor(int(f[0]), int(f[1]), int(f[2]), float(f[3]), float(f[4]))
    w, fv, _ = oracle.evaluate_mothers(ch, fn, 0, g["mothers"], nthreads=1)
    assert np.array_equal(w, g["eval_w"]) and np.array_equal(fv, g["eval_f"])
    mean, m2, W = oracle.average_mothers(ch, fn, 0, g["mothers"])
    assert mean == g["avg_mean"] and np.sqrt(m2) / W == g["avg_err"]


# ------------------------------------------------ consumers of a stored sample, lazy range --

def _functor(O, g):
    f = g["functor"]
    return O.make_functor(int(f[0]), int(f[1]), int(f[2]), float(f[3]), float(f[4]))


@pytest.mark.parametrize("name", EXTRA_GOLDEN)
def test_reweight_and_unweight_functor_bit_exact(oracle, name):
    """PhaseSpaceReweight values and both Unweight(functor, w, seed) permutations."""
    g = load_golden(name)
    ch = oracle.make_channel(g["masses"], float(g["M"]), int(g["seed"]), int(g["engine"]))
    four, _ = oracle.generate(ch, 0, int(g["n"]))
    assert np.array_equal(four, g["four"])
    fn = _functor(oracle, g)
    assert np.array_equal(oracle.reweight(ch, fn, four), g["reweight"])
    for key, weight in (("unw_max", -1.0), ("unw_fixed", float(g["fmax"]))):
        _, _, fl, perm = oracle.unweight_functor(ch, fn, four, weight, int(g["fseed"]))
        assert int(fl.sum()) == int(g[key + "_kept"])
        assert np.array_equal(four[:, perm], g[key + "_four"])


@pytest.mark.parametrize("name", [n for n in EXTRA_GOLDEN if int(load_golden(n)["N"]) >= 3])
def test_dalitz_histogram_bit_exact(oracle, name):
    """DenseHistogram<double,2>::Fill of the Dalitz variables weighted by PhaseSpaceWeight."""
    g = load_golden(name)
    ch = oracle.make_channel(g["masses"], float(g["M"]), int(g["seed"]), int(g["engine"]))
    w = oracle.recompute_weights(ch, g["four"])
    bins = oracle.dalitz_histogram(g["four"], w, [0, 1, 1, 2], g["grid"], g["lower"], g["upper"])
    assert np.array_equal(bins, g["hist"])
    assert bins.sum() > 0


@pytest.mark.parametrize("name", EXTRA_GOLDEN)
def test_phase_space_range_bit_exact(oracle, name):
    """phase_space_range: GenerateDecay over thrust's minstd_rand, 32-bit seed, mother-mass ECM."""
    g = load_golden(name)
    ch = oracle.range_channel(g["masses"], g["range_mother"], int(g["rseed"]))
    four, w = oracle.generate(ch, 0, int(g["n"]))
    assert np.array_equal(w, g["range_w"])
    assert np.array_equal(four, g["range_four"])


def test_minstd_words_against_recurrence(oracle):
    """Event e of a minstd stream starts at seed * 48271^(e+3N+1) mod 2^31-1 (discard by modular
    exponentiation); check it against the plain recurrence x <- 48271 x mod 2^31-1."""
    m = 2**31 - 1
    for seed in (987654321, 0, m, m + 5, 2**32 - 1):
        N = 4
        x = (seed & 0xFFFFFFFF) % m or 1
        stream = []
        for _ in range(40 + 6 * N):
            x = x * 48271 % m
            stream.append(x)
        words = oracle.rng_words(N, oracle.ENGINE_MINSTD, seed, 0, 40)
        for e in range(40):
            assert list(words[e]) == stream[e + 3 * N:e + 3 * N + 3 * N - 4]


@pytest.mark.parametrize("name", EXTRA_GOLDEN)
def test_phase_space_integrator_sequential_fold(oracle, name):
    """PhaseSpaceIntegrator::Integrate = AverageOn with the generator's default seed."""
    g = load_golden(name)
    ch = oracle.make_channel(g["masses"], float(g["M"]), int(g["integ_seed"]), int(g["engine"]))
    mean, m2, w = oracle.average_on(ch, _functor(oracle, g), 0, int(g["n"]), nthreads=1)
    assert mean == g["integ_mean"]
    assert np.sqrt(m2) / w == g["integ_err"]
