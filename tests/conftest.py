"""Shared fixtures: builds the backend and the oracle once per session."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_built():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def backend_built():
    from exploringsycl_gb300 import build
    build.build_all()
    import exploringsycl_gb300
    return exploringsycl_gb300
