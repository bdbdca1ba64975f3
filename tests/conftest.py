import importlib.util
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu on a GB300)")


def _ensure_built():
    """Build the CUDA library and the oracle in-tree when they are missing (the build
    recipe is loaded from its file so that the package, which needs the library, is not
    imported first)."""
    if not (ROOT / "grid_gb300" / "libgbdwf.so").exists():
        spec = importlib.util.spec_from_file_location("_gb_build", ROOT / "grid_gb300" / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    if not (ROOT / "oracle" / "liboracle.so").exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)


_ensure_built()


@pytest.fixture(scope="session")
def gpu_available():
    import grid_gb300 as g
    n = g.device_count()
    if n < 1:
        pytest.fail("no CUDA device visible: GPU tests need a GB300 (the library has no CPU fallback)")
    return n
