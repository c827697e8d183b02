import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def E():
    import eegraph_gb300

    return eegraph_gb300


@pytest.fixture(scope="session")
def gpu(E):
    if E.device_count() < 1:
        pytest.fail("GPU test collected on a machine without a CUDA device")
    E.lib().eeg_set_device(0)
    return E
