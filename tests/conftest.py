"""pytest configuration: the `gpu` marker and shared fixtures."""
import shutil
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """The native library, built in-tree if missing."""
    from vk_compute_mipmaps_gb300 import _build, _native
    if not _native.LIB_PATH.exists():
        _build.build()
    return _native.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture
def repo_tmp(request):
    """A scratch directory inside the repository (tests/.tmp/<test>), removed
    afterwards."""
    d = ROOT / "tests" / ".tmp" / request.node.name.replace("[", "_").replace("]", "")
    shutil.rmtree(d, ignore_errors=True)
    d.mkdir(parents=True)
    yield d
    shutil.rmtree(d, ignore_errors=True)
