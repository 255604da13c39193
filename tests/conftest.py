"""pytest configuration: the `gpu` marker and shared import paths.

`-m gpu` tests need a CUDA device and the built product library; everything
else runs on CPU (oracle vs golden fixtures, host logic, ABI exports)."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "paint-sim-3d_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")
