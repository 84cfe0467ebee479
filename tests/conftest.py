import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

REFERENCE = Path(os.environ.get("LMG_REFERENCE_SRC", "/root/reference"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as orc
    return orc


@pytest.fixture(scope="session")
def reference_tests_dir():
    d = REFERENCE / "tests" / "ref"
    if not d.exists():
        pytest.skip("reference checkout not present on this machine")
    return d


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import libmobility_gb300._build as b
    b.build()
    return True
