import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build libinfoli_gpu.so and the oracle once per session."""
    from infoli_gb300 import build
    from oracle import oracle

    build.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def conf():
    """The 42 default parameters (default.conf shipped with the CLI)."""
    from infoli_gb300 import capi

    return capi.read_parameters(os.path.join(ROOT, "infoli_gb300", "host", "default.conf"))


def pytest_sessionstart(session):
    # measured figures the at-size parity tests print in the terminal summary
    session.config._infoli_report = []


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    lines = getattr(config, "_infoli_report", [])
    if lines:
        terminalreporter.section("measured against the oracle")
        for line in lines:
            terminalreporter.write_line(line)
