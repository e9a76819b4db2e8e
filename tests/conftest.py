"""Shared fixtures; registers the `gpu` and `slow` markers.

Tests marked `gpu` need a CUDA device and the built extension; everything else
runs on the CPU (oracle, golden vectors, host logic, library symbol checks).
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN_DIR = Path(__file__).resolve().parent / "golden"


def pytest_configure(config: pytest.Config) -> None:
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built sm_103a library")
    config.addinivalue_line("markers", "slow: large grids and long runs")


def two_phase(n: int, seed: int = 0, hi: float = 12.0, lo: float = 3.0) -> np.ndarray:
    """Thresholded-GRF permeability, the reference test suite's standard medium."""
    from darcy_cpp_gb300.fields import gaussian_random_field, two_phase_permeability

    return two_phase_permeability(gaussian_random_field(n, seed=seed), hi=hi, lo=lo)


@pytest.fixture(scope="session")
def golden() -> tuple[dict, dict]:
    arrays = dict(np.load(GOLDEN_DIR / "golden.npz"))
    meta = json.loads((GOLDEN_DIR / "golden.json").read_text())
    return arrays, meta


@pytest.fixture
def rng() -> np.random.Generator:
    return np.random.default_rng(20240724)


@pytest.fixture(params=["multigrid", "jacobi", "none"])
def preconditioner(request: pytest.FixtureRequest) -> str:
    return str(request.param)


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (ctypes over oracle/_build/liboracle.so), pinned to 1 thread."""
    import oracle

    oracle.lib()
    oracle.set_threads(1)
    return oracle
