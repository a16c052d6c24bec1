import importlib
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def gm():
    return importlib.import_module("gales-multi-fluid_gb300")


@pytest.fixture(scope="session")
def syn():
    return importlib.import_module("gales-multi-fluid_gb300.synthetic")


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle


@pytest.fixture(scope="session")
def cuda_lib(gm):
    """Builds (if needed) and loads libgales_asm.so; GPU tests fail loudly without it."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    b = importlib.import_module("gales-multi-fluid_gb300.build")
    b.build()
    return gm.abi.lib()
