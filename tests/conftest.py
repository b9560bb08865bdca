import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(ROOT / "tests") not in sys.path:
    sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            import torch
            return torch.cuda.is_available()
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def engine_lib():
    """The built engine library (built on demand)."""
    from sprout_gb300 import build
    build.build()
    import sprout_gb300
    return sprout_gb300.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    return O.lib()


def pytest_collection_modifyitems(config, items):
    if os.environ.get("SPROUT_FORCE_GPU_TESTS"):
        return
    if any("gpu" in item.keywords for item in items) and not gpu_available():
        skip = pytest.mark.skip(reason="no CUDA GPU here")
        for item in items:
            if "gpu" in item.keywords:
                item.add_marker(skip)
