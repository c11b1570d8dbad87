import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG_DIR = ROOT / "parallelparticleswarms.jl_gb300"
for p in (str(PKG_DIR), str(ROOT / "oracle"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libpps_cuda.so)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def orc():
    import pps_oracle

    pps_oracle.load()
    return pps_oracle


@pytest.fixture(scope="session")
def pps():
    """The package with its CUDA library built (GPU tests only)."""
    sys.path.insert(0, str(PKG_DIR / "csrc"))
    try:
        import build as cuda_build
    finally:
        sys.path.pop(0)
    cuda_build.build()
    import parallelparticleswarms

    return parallelparticleswarms
