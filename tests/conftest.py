import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import ctypes
        from flowunsteady_gb300 import _lib as L
        p = ctypes.c_void_p()
        rc = L.lib().vpm_ctx_create(0, 1, ctypes.byref(p))
        if rc == 0:
            L.lib().vpm_ctx_destroy(p)
            return True
    except Exception:
        return False
    return False


def pytest_collection_modifyitems(config, items):
    if any("gpu" in item.keywords for item in items):
        if not _has_gpu():
            skip = pytest.mark.skip(reason="no CUDA device")
            for item in items:
                if "gpu" in item.keywords:
                    item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
