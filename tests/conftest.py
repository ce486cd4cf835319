import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "webgpu-3dgs_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: full-size workload")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def built_lib():
    """Builds libgs3d.so in-tree if needed (nvcc cross-compiles without a GPU)."""
    sys.path.insert(0, str(PKG))
    import build as gsbuild  # webgpu-3dgs_gb300/build.py
    return gsbuild.build()


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return os.path.exists("/dev/nvidia0")
