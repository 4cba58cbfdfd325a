import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")
    return {name[:-4]: np.load(os.path.join(d, name)) for name in os.listdir(d) if name.endswith(".npz")}


@pytest.fixture(scope="session")
def port_lib():
    """The C restatement of the stock backend (built on demand; no GPU needed)."""
    from oracle import heffte_oracle as O
    if O.load_port() is None:
        import subprocess
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "port")], check=True)
    lib = O.load_port()
    assert lib is not None
    return lib


@pytest.fixture(scope="session")
def gb():
    """The product library (built on demand)."""
    import heffte_gb300
    from heffte_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    heffte_gb300.lib()
    return heffte_gb300


_REPORT = []


@pytest.fixture(scope="session")
def report():
    """Collects lines (e.g. measured errors) printed at the end of the run,
    also under -q."""
    return _REPORT


def pytest_terminal_summary(terminalreporter):
    if _REPORT:
        terminalreporter.section("measured")
        for line in _REPORT:
            terminalreporter.write_line(line)
