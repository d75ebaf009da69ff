"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on a CPU-only machine."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def am():
    import adaptivemesh_gb300 as pkg
    pkg.load()
    return pkg


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


def _ref(cfg: str):
    from oracle import reflib
    try:
        return reflib.load(cfg)
    except Exception as e:  # the reference-build library needs the staged reference headers
        pytest.skip(f"reference-build library {cfg} unavailable: {e}")


@pytest.fixture(scope="session")
def ref28():
    return _ref("n28p2")


@pytest.fixture(scope="session")
def ref16():
    return _ref("n16p3")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda")
