import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


_gpu_state = {}


def _has_gpu():
    if "ok" not in _gpu_state:
        try:
            import torch
            _gpu_state["ok"] = torch.cuda.is_available()
        except Exception:
            _gpu_state["ok"] = False
    return _gpu_state["ok"]


def pytest_collection_modifyitems(config, items):
    for item in items:
        if "gpu" in item.keywords and not _has_gpu():
            item.add_marker(pytest.mark.skip(reason="no CUDA device"))


@pytest.fixture(scope="session")
def built():
    """Builds (if needed) and loads the CUDA library and the C oracle."""
    from gpurir_gb300 import _build, _lib
    import oracle
    _build.build()
    oracle.build()
    return _lib.load()


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
