import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "fluid-sim-lb_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def _have_gpu() -> bool:
    try:
        import ctypes

        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import torch

            return torch.cuda.is_available()
        except Exception:
            return False
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


HAVE_GPU = None


def pytest_collection_modifyitems(config, items):
    global HAVE_GPU
    gpu_items = [it for it in items if "gpu" in it.keywords]
    if not gpu_items:
        return
    if HAVE_GPU is None:
        HAVE_GPU = _have_gpu()
    if not HAVE_GPU:
        skip = pytest.mark.skip(reason="no CUDA device")
        for it in gpu_items:
            it.add_marker(skip)


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the libraries once per session (no-op when up to date)."""
    import build as fsim_build

    fsim_build.build_oracle()
    try:
        fsim_build.build_fsim()
    except Exception as e:  # nvcc missing: CPU-only runs still test the oracle
        print("libfsim build skipped:", e)
    yield
