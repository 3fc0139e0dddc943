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


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    pytest.skip("CUDA toolkit headers not found")


def compile_example(hps, out):
    cuda = cuda_home()
    lib_dir = str(hps.library_path().parent)
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", str(REPO / "include"),
           "-I", f"{cuda}/include", str(SRC), "-L", lib_dir, "-lhps", "-L", f"{cuda}/lib64", "-lcudart",
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
    g = load_golden("cfg1_n3_philox")
    ga = load_golden("avg_cfg1_m2")
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
