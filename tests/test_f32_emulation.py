"""The FP32_FIX event body compiled for the CPU (tests/f32_emulation/) against the FP64 body of the
same events, on channels and event ranges beyond what the GPU tests sample.

The emulation is the kernels' own source (hydra_gb300/csrc/genbod_f32.cuh) with the CUDA intrinsics
replaced by the IEEE operations they name and the two hardware approximations (rcp.approx,
rsqrt.approx) by 1/x and 1/sqrt(x); each of those is followed by a Newton step in the body, so the
emulated events differ from the GPU's only in last bits.  The FP64 side is genbod.cuh, which the GPU
tests pin to the oracle (the reference's arithmetic) at 1e-12.

Tolerance: the precision contract of the FP32_FIX form, 1e-6, on
  four-vectors  max over daughters of max_k |dp_k| / E
  weights       |dw| / w
"""
from __future__ import annotations

import json
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent / "f32_emulation"
TOL = 1e-6
PI, K = 0.13957, 0.493677


@pytest.fixture(scope="module")
def emulator():
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    r = subprocess.run(["bash", str(HERE / "build.sh")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip().splitlines()[-1]


def run(exe, masses, M, n, first=0, engine=0, form=-1):
    args = [exe, str(len(masses)), repr(M), ",".join(repr(m) for m in masses), str(n), str(first), str(engine),
            "0x3039", str(form)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


CASES = [
    # the bench workload and the config-3 channels
    ("d0_kpipipipi", [K] + [PI] * 4, 1.86484, 0),
    ("b0_jpsikpi", [3.0969, K, PI], 5.27934, 0),
    ("ten_pions_M5", [PI] * 10, 5.0, 0),
    # the batched workloads' largest energy per N: mother mass sum(m) + 6 GeV, all pions
    ("four_pions_hard", [PI] * 4, 4 * PI + 6.0, 0),
    ("six_pions_hard", [PI] * 6, 6 * PI + 6.0, 0),
    ("seven_pions_hard", [PI] * 7, 7 * PI + 6.0, 1),
    ("ten_pions_hard", [PI] * 10, 10 * PI + 6.0, 0),
]


@pytest.mark.parametrize("name,masses,M,engine", CASES, ids=[c[0] for c in CASES])
def test_emulated_float_body_within_contract(emulator, name, masses, M, engine):
    d = run(emulator, masses, M, 1 << 18, engine=engine)
    print(f"\n[f32 emulation] {name}: four {d['four_vectors']:.3e} weight {d['weights']:.3e}")
    assert d["four_vectors"] <= TOL and d["weights"] <= TOL, d


def test_emulated_weight_product_range(emulator):
    """Event 13901751 of ten pions from 8 GeV: prod num of the float-float weight fell below float's
    normal range before each stage took an even power of two out of it (85% weight error)."""
    d = run(emulator, [PI] * 10, 8.0, 128, first=13901700)
    assert d["weights"] <= TOL and d["four_vectors"] <= TOL, d


def test_emulated_forms_of_a_hard_channel(emulator):
    """Six pions from 3 GeV (kinetic energy 15.5 pion masses, above the float-float boosts'
    threshold of 12): the library takes the float-float boosts; the plain form of the same events
    is within the contract too, with less margin."""
    masses, M = [PI] * 6, 3.0
    auto = run(emulator, masses, M, 1 << 18)
    plain = run(emulator, masses, M, 1 << 18, form=0)
    assert auto["float_float_form"] == 1 and plain["float_float_form"] == 0
    assert auto["four_vectors"] <= plain["four_vectors"] <= TOL, (auto, plain)
    assert auto["weights"] <= TOL and plain["weights"] <= TOL
