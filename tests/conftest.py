import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


# Tolerances the parity tests applied and the errors they measured (one line
# per check), printed at the end of the run so that a widened tolerance is
# visible in the log of a passing run.
TOLERANCE_REPORT = []


def pytest_terminal_summary(terminalreporter):
    if TOLERANCE_REPORT:
        terminalreporter.section("parity tolerances applied")
        for line in TOLERANCE_REPORT:
            terminalreporter.write_line(line)


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built():
    """Builds the native libraries (tracker, synth) and the oracle."""
    from slam_gb300 import _build
    from oracle import build as obuild
    _build.build()
    obuild.build_oracle()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch
    torch.cuda.init()
    return torch.device("cuda:0")


ANGLE_THRESH = float(np.float32(np.sin(np.float32(np.float32(20.0) * np.float32(3.14159254)) / np.float32(180.0))))
DIST_THRESH = float(np.float32(0.10))
