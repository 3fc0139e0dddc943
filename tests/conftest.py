"""Shared test set-up: the `gpu` marker, golden fixtures, and build of the oracle / library."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
GOLDEN = REPO / "tests" / "golden"
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def golden_names(prefix: str = ""):
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if p.stem.startswith(prefix))


GEN_GOLDEN = [n for n in golden_names() if not n.startswith(("rng_", "avg_", "mothers_", "extras_", "functors_"))]
MOTHER_GOLDEN = golden_names("mothers_")
EXTRA_GOLDEN = golden_names("extras_")
FUNCTOR_GOLDEN = golden_names("functors_")
RNG_GOLDEN = golden_names("rng_")
AVG_GOLDEN = golden_names("avg_")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def hps():
    import hydra_gb300
    from hydra_gb300 import build
    build.build()
    return hydra_gb300


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    return torch.device("cuda:0")
