"""The C++ drop-in headers (include/hydra/*.h): reference-style user code compiles against them
(CPU test) and, on a GPU, produces the reference's numbers (tests/cpp/phsp_dropin.cpp)."""
from __future__ import annotations

import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_golden

SRC = REPO / "tests" / "cpp" / "phsp_dropin.cpp"
SRC_EXTRAS = REPO / "tests" / "cpp" / "phsp_extras.cpp"
SRC_CHAIN = REPO / "tests" / "cpp" / "phsp_chain.cpp"


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    pytest.skip("CUDA toolkit headers not found")


def compile_example(hps, out, src=SRC):
    cuda = cuda_home()
    lib_dir = str(hps.library_path().parent)
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", str(REPO / "include"),
           "-I", f"{cuda}/include", str(src), "-L", lib_dir, "-lhps", "-L", f"{cuda}/lib64", "-lcudart",
           f"-Wl,-rpath,{lib_dir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_dropin_example_compiles(hps, tmp_path):
    assert compile_example(hps, tmp_path / "phsp_dropin").exists()


@pytest.mark.gpu
def test_dropin_example_matches_reference(hps, cuda, tmp_path):
    exe = compile_example(hps, tmp_path / "phsp_dropin")
    r = subprocess.run([str(exe), "256", "20000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    g = load_golden("b0_jpsikpi_n3_philox")
    ga = load_golden("avg_b0_jpsikpi_m2")
    assert d["max_weight"] == g["max_weight"] and d["ecm"] == g["ecm"] and d["seed"] == 12345
    four = np.array(d["four"]).reshape(256, 3, 4).transpose(1, 0, 2)
    err = float((np.abs(four - g["four"]).max(axis=2) / g["four"][:, :, 0]).max())
    assert err <= 1e-12
    assert np.array_equal(np.array(d["w_gen"]), g["w_gen"])
    assert np.allclose(d["w_rec"], g["w_rec"], rtol=1e-12, atol=0)
    assert np.array_equal(np.array(d["eval_w"]), g["w_gen"])
    assert np.allclose(d["eval_f"], g["f_val"], rtol=1e-12, atol=0)
    assert d["unweighted"] == int(g["n_unweighted"])
    assert abs(d["avg_mean"] - ga["mean"]) <= 1e-10 * ga["mean"]
    assert abs(d["avg_err"] - ga["err"]) <= 1e-8 * ga["err"]
    assert d["host_equal"] is True and d["errors_ok"] == 2


def test_extras_example_compiles(hps, tmp_path):
    assert compile_example(hps, tmp_path / "phsp_extras", SRC_EXTRAS).exists()


@pytest.mark.gpu
def test_extras_example_matches_reference(hps, cuda, tmp_path):
    """Unweight(functor), GetEventWeightFunctor(functor), the Dalitz histogram,
    PhaseSpaceIntegrator and phase_space_range through the C++ headers, against the fixture the
    reference itself produced for the same calls."""
    g = load_golden("extras_b0_jpsikpi_n3_philox")
    n = int(g["n"])
    exe = compile_example(hps, tmp_path / "phsp_extras", SRC_EXTRAS)
    r = subprocess.run([str(exe), str(n), repr(float(g["fmax"]))], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)

    def four(key):
        return np.array(d[key]).reshape(n, 3, 4).transpose(1, 0, 2)
    # the events are this GPU's (four-vectors within 1e-12 of the reference's, through sin/cos),
    # so the values computed from them agree to that tolerance rather than bit for bit
    np.testing.assert_allclose(d["reweight"], g["reweight"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(d["hist"], g["hist"], rtol=1e-12, atol=0)
    assert d["unw_max_kept"] == int(g["unw_max_kept"]) and d["unw_fixed_kept"] == int(g["unw_fixed_kept"])
    for key in ("unw_max_four", "unw_fixed_four"):
        err = float((np.abs(four(key) - g[key]).max(axis=2) / np.abs(g[key][:, :, 0])).max())
        assert err <= 1e-12, key
    assert abs(d["integ_mean"] - g["integ_mean"]) <= 1e-10 * abs(g["integ_mean"])
    assert abs(d["integ_err"] - g["integ_err"]) <= 1e-8 * abs(g["integ_err"])
    assert np.array_equal(np.array(d["range_w"]), g["range_w"])
    rf = four("range_four")
    assert float((np.abs(rf - g["range_four"]).max(axis=2) / np.abs(g["range_four"][:, :, 0])).max()) <= 1e-12


def test_chain_example_compiles(hps, tmp_path):
    assert compile_example(hps, tmp_path / "phsp_chain", SRC_CHAIN).exists()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
def test_chain_example_matches_oracle(hps, cuda, oracle, tmp_path, precision, tol):
    """Generate(GetDaugtherRange(_0), events), AverageOn(mothers, f) and Evaluate(mothers, ...)
    through the C++ headers against the oracle's DecayMothers / AverageMothers / EvalMothers on the
    J/psi column the program produced."""
    n = 2048
    exe = compile_example(hps, tmp_path / "phsp_chain", SRC_CHAIN)
    r = subprocess.run([str(exe), str(n), str(precision)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    jpsi = np.array(d["jpsi"]).reshape(n, 4)
    mu = np.stack([np.array(d["mup"]).reshape(n, 4), np.array(d["mum"]).reshape(n, 4)])
    och = oracle.make_channel([0.1056583745, 0.1056583745], 3.0969, 0x3040, oracle.ENGINE_PHILOX)
    rfour, _ = oracle.generate_mothers(och, 0, jpsi)
    err = float((np.abs(mu - rfour).max(axis=2) / np.abs(rfour[:, :, 0])).max())
    assert err <= tol, err
    # the muons add up to their J/psi
    assert np.abs(mu.sum(axis=0) - jpsi).max() <= 10 * tol * np.abs(jpsi[:, 0]).max()
    rmean, rm2, rW = oracle.average_mothers(och, oracle.make_functor(1, 1, 2), 0, jpsi)
    assert abs(d["avg_mean"] - rmean) <= max(tol, 1e-10) * abs(rmean)
    rw, rf, _ = oracle.evaluate_mothers(och, oracle.make_functor(1, 0, 1), 0, jpsi)
    if precision == 0:
        assert np.array_equal(np.array(d["eval_w"]), rw)
        np.testing.assert_allclose(d["eval_f"], rf, rtol=1e-12, atol=0)
    else:
        # FP32_FIX EvalMothers: weights within the form's 1e-6; m^2(J/psi + mu+) from a muon that is
        # within 1e-6 x the J/psi's gamma (about 1.14) of the oracle's
        np.testing.assert_allclose(d["eval_w"], rw, rtol=1e-6, atol=0)
        np.testing.assert_allclose(d["eval_f"], rf, rtol=2e-6, atol=0)
