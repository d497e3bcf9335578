import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "lion-codes_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import lufqhe_oracle
    lufqhe_oracle.lib()
    return lufqhe_oracle


@pytest.fixture(scope="session")
def lufqhe_mod():
    import lufqhe
    lufqhe.lib()
    return lufqhe


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.set_device(0)
    return torch
