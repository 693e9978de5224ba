import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "pflotran-elm-interface_gb300")
for p in (REPO, PKG, os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    """Prints the per-case parity report (tests/parity.py) collected by the
    GPU parity tests, so that it is part of the session's output."""
    mod = sys.modules.get("parity")
    if mod is None or not getattr(mod, "REPORT", None):
        return
    for line in mod.format_report():
        terminalreporter.write_line(line)
