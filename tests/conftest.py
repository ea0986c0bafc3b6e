"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs
on a CPU-only machine."""
import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLD = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def golden():
    return json.loads((GOLD / "golden.json").read_text())


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def native():
    """The built libla3g (built on first use)."""
    import la3_gb300.build as B
    B.build()
    import la3_gb300
    la3_gb300._native.lib()
    return la3_gb300


@pytest.fixture(scope="session")
def gpu(native):
    import torch  # noqa: F401  (only to report the device)
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return native
