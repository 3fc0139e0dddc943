"""Functors outside the C ABI's menu through the drop-in headers (include/hydra/): the functor is
compiled by nvcc into the library's kernel templates (include/hydra/detail/hps_user_kernels.cuh),
as the reference compiles it into its Thrust functors.

* CPU: tests/cpp/phsp_user_functors.cu -- written as the reference's phase-space examples write
  their functors (wrap_lambda over declarg arguments, hydra::CosHelicityAngle, a multivector of
  named columns) -- compiles and links; where the reference's source tree is present (it is not
  on a GPU host), the reference's own examples/phase_space/phsp_averaging_functor.inl and
  phsp_evaluating_functor.inl compile against include/ with only the include path changed (their
  TCLAP argument parser stubbed by tests/cpp/stubs/tclap/CmdLine.h).
* GPU: the program's AverageOn / Evaluate / Unweight(functor) results against fixtures the
  reference itself produced for the same functors (oracle/ref_harness.cpp mode "functors",
  tests/golden/make_golden.py).

Tolerances: the FP64 events are the reference's arithmetic operation for operation, but nvcc
contracts the functors' own products into FMAs where the reference build does not, so functor
values are compared at 1e-12 (relative for masses, absolute for cos(theta)); weights bit for
bit; AverageOn mean / error at 1e-10 / 1e-8 of the error / relative (another reduction order);
the events Unweight keeps and their order exactly.  FP32_FIX: 1e-6 (the precision contract of
that form) for weights, masses to 1e-5 (m^2 differences of float four-vectors).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import FUNCTOR_GOLDEN, REPO, load_golden

SRC = REPO / "tests" / "cpp" / "phsp_user_functors.cu"
SRC_MOTHERS = REPO / "tests" / "cpp" / "phsp_user_mothers.cu"
STUBS = REPO / "tests" / "cpp" / "stubs"
# the reference's examples, read in place where its source tree sits beside this repository
REF_EXAMPLES = REPO.parent / "reference" / "examples" / "phase_space"


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    pytest.skip("nvcc not found")


NVCC_FLAGS = ["-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "--extended-lambda",
              "--expt-relaxed-constexpr"]


def build_program(hps, out, src=SRC):
    lib_dir = str(hps.library_path().parent)
    cmd = [nvcc(), *NVCC_FLAGS, "-I", str(REPO / "include"), str(src), "-L", lib_dir, "-lhps",
           f"-Xlinker=-rpath,{lib_dir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_user_functor_program_builds(hps, tmp_path):
    assert build_program(hps, tmp_path / "phsp_user_functors").exists()


def test_user_functor_mothers_program_builds(hps, tmp_path):
    assert build_program(hps, tmp_path / "phsp_user_mothers", SRC_MOTHERS).exists()


@pytest.mark.parametrize("example", ["phsp_averaging_functor.inl", "phsp_evaluating_functor.inl"])
def test_reference_examples_compile_against_dropin(tmp_path, example):
    src = REF_EXAMPLES / example
    if not src.exists():
        pytest.skip("the reference's source tree is not on this machine")
    cmd = [nvcc(), "-x", "cu", *NVCC_FLAGS, "-I", str(STUBS), "-I", str(REPO / "include"), "-c", str(src),
           "-o", str(tmp_path / "example.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def run_program(exe, g, precision, out):
    m = [repr(float(x)) for x in g["masses"]]
    args = [str(exe), str(int(g["engine"])), str(int(g["seed"])), str(int(g["n"])), repr(float(g["M"])), *m,
            hex(int(g["fseed"])), str(precision), str(out)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    n = int(g["n"])
    d = np.fromfile(out, dtype=np.float64)
    rows = d[2:2 + 4 * n].reshape(n, 4)
    o = 2 + 4 * n
    unw = d[o:o + 12 * n].reshape(n, 3, 4).transpose(1, 0, 2)
    return d[0], d[1], rows, unw, int(d[o + 12 * n]), r.stdout


@pytest.fixture(scope="module")
def program(hps, tmp_path_factory):
    return build_program(hps, tmp_path_factory.mktemp("functors") / "phsp_user_functors")


@pytest.mark.gpu
@pytest.mark.parametrize("name", FUNCTOR_GOLDEN)
def test_user_functors_fp64_match_reference(program, cuda, tmp_path, name):
    g = load_golden(name)
    mean, err, rows, unw, kept, stdout = run_program(program, g, 0, tmp_path / "out.bin")
    assert stdout.startswith("<0>: (")
    assert np.array_equal(rows[:, 0], g["eval_w"])
    assert np.allclose(rows[:, 1], g["eval_m13"], rtol=1e-12, atol=0)
    assert np.allclose(rows[:, 2], g["eval_m23"], rtol=1e-12, atol=0)
    assert np.allclose(rows[:, 3], g["eval_cos"], rtol=0, atol=1e-12)
    assert abs(mean - g["avg_mean"]) <= 1e-10 * max(abs(g["avg_mean"]), g["avg_err"])
    assert abs(err - g["avg_err"]) <= 1e-8 * g["avg_err"]
    assert kept == int(g["unw_kept"])
    e4 = float((np.abs(unw - g["unw_four"]).max(axis=2) / g["unw_four"][:, :, 0]).max())
    assert e4 <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", FUNCTOR_GOLDEN)
def test_user_functors_fp32fix_within_contract(program, cuda, tmp_path, name):
    g = load_golden(name)
    mean, err, rows, unw, kept, _ = run_program(program, g, 1, tmp_path / "out.bin")
    assert float((np.abs(rows[:, 0] - g["eval_w"]) / g["eval_w"]).max()) <= 1e-6
    assert np.allclose(rows[:, 1], g["eval_m13"], rtol=1e-5, atol=0)
    assert np.allclose(rows[:, 2], g["eval_m23"], rtol=1e-5, atol=0)
    # the mean of cos(theta) is near 0: compare against the statistical error of the sample
    assert abs(mean - g["avg_mean"]) <= 1e-3 * g["avg_err"]
    assert abs(err - g["avg_err"]) <= 1e-4 * g["avg_err"]


@pytest.fixture(scope="module")
def mothers_program(hps, tmp_path_factory):
    return build_program(hps, tmp_path_factory.mktemp("mothers") / "phsp_user_mothers", SRC_MOTHERS)


def run_mothers(exe, n, precision):
    import json
    r = subprocess.run([str(exe), str(n), str(precision)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    return {k: np.asarray(v) for k, v in d.items()}


# m^2(mu+ pi0) is E^2 - p^2 of lab-frame four-vectors, so its float rounding scales with the pair's
# energy squared, not with m^2 (which reaches down to (m_mu + m_pi0)^2 = 0.058 GeV^2).  A J/psi from
# B0 -> J/psi K pi has E <= (M_B^2 + M_J^2) / (2 M_B) = 3.55 GeV, so (E_mu + E_pi0)^2 < 12.6 GeV^2;
# the FP32_FIX bars below are 1e-6 and 4e-6 of 16 GeV^2 in absolute terms.
PAIR_E2 = 16.0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_fix"])
def test_user_functor_with_mothers_matches_menu(mothers_program, cuda, precision):
    """AverageOn(mothers, F) and Evaluate(mothers, result, F) with F = m^2(mu+ pi0) of
    J/psi -> mu+ mu- pi0 as a compiled-in lambda against the menu's Mass2(1, 3) on the same chain:
    the events are the same code in both (weights bit for bit); the functor values differ only by
    how m^2 is rounded (FP64: the menu's separately rounded operations against nvcc's contracted
    ones, 1e-12 relative; FP32_FIX: the menu's float m^2 in the mother's frame against the lambda's
    double m^2 of the widened four-vectors, 1e-6 of the pair energy squared)."""
    n = 3000
    d = run_mothers(mothers_program, n, precision)
    assert d["user_w"].shape == (n,)
    assert np.array_equal(d["user_w"], d["menu_w"])
    (mm, em), (mu, eu) = d["avg_menu"], d["avg_user"]
    if precision == 0:
        np.testing.assert_allclose(d["user_f"], d["menu_f"], rtol=1e-12, atol=0)
        assert abs(mu - mm) <= 1e-12 * abs(mm) and abs(eu - em) <= 1e-8 * em
    else:
        np.testing.assert_allclose(d["user_f"], d["menu_f"], rtol=0, atol=1e-6 * PAIR_E2)
        assert abs(mu - mm) <= 1e-6 * PAIR_E2 and abs(eu - em) <= 1e-4 * em


@pytest.mark.gpu
def test_user_functor_with_mothers_fp32fix_within_contract(mothers_program, cuda):
    """The FP32_FIX weights and functor values of the per-event-mother Evaluate against FP64: weights
    within the 1e-6 relative contract of that form; m^2(mu+ pi0) within 4e-6 of the pair energy
    squared (each four-vector is within 1e-6 x the mother's gamma, about 1.14, of its energy, and
    m^2 = E^2 - p^2 takes twice the error of each of the two)."""
    a, b = run_mothers(mothers_program, 3000, 0), run_mothers(mothers_program, 3000, 1)
    assert float(np.max(np.abs(b["user_w"] - a["user_w"]) / a["user_w"])) <= 1e-6
    np.testing.assert_allclose(b["user_f"], a["user_f"], rtol=0, atol=4e-6 * PAIR_E2)
