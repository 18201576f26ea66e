"""Shared test set-up: import paths, the `gpu` marker, and session fixtures
that build the product library and the CPU oracle once."""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "sycl-building-blocks_gb300"
for p in (ROOT, PKG, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    import ppbuild  # the package build recipe

    return ppbuild.build()


@pytest.fixture(scope="session")
def pp(built_lib):
    import ppgb300

    ppgb300.lib()
    return ppgb300


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
