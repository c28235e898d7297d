import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "gpu-domain-propagator_gb300"
for p in (str(ROOT), str(PKG), str(Path(__file__).resolve().parent)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _native_built():
    """Builds the oracle and the package libraries if they are missing."""
    if not (ROOT / "oracle" / "build" / "libgdporacle.so").exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    lib = PKG / "lib"
    if not (lib / "libgdp_gb300.so").exists() or not (lib / "libgdpgen.so").exists():
        import build as pkg_build
        pkg_build.build()
    yield
