"""Shared test set-up: the gpu marker, repo imports, one build per session."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from licenta_gb300 import _build
    from oracle import build_oracle
    _build.build()
    build_oracle.build()
    yield


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch


# Measured figures that parity tests report (largest errors, steps excused by
# the bend singularity, sizes checked), printed at the end of the run.
_REPORT: list[tuple[str, dict]] = []


@pytest.fixture
def parity_report(request):
    def add(**figures):
        _REPORT.append((request.node.nodeid, figures))
    return add


def pytest_terminal_summary(terminalreporter):
    if _REPORT:
        terminalreporter.section("parity report")
        for node, figures in _REPORT:
            terminalreporter.write_line(f"{node}: " + ", ".join(f"{k}={v}" for k, v in figures.items()))
