import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
PARAMS = os.path.join(ROOT, "params")
GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference source tree (UEPM_REFERENCE_ROOT), present only where fixtures are made
from oracle.oracle import REFERENCE_ROOT  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def _build_native():
    from ultimateepm_gb300 import build

    build.build()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def native():
    """The C ABI library, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    _build_native()
    from ultimateepm_gb300 import _native

    return _native.load()


def _gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(native):
    if not _gpu_available():
        pytest.skip("no CUDA device visible")
    import torch

    torch.cuda.init()
    return native


@pytest.fixture(scope="session")
def mats(oracle):
    """Oracle-side material structs from the committed parameter files."""
    out = {}
    out.update({"Si-CB": oracle.load_materials(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))["Si"]})
    out.update({"Si-d": oracle.load_materials(os.path.join(PARAMS, "si-nonlocal-d.yaml"))["Si"]})
    out.update(oracle.load_materials(os.path.join(PARAMS, "materials.yaml")))
    return out
