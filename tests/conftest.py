import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device")


def gpu_available() -> bool:
    try:
        from persiansph_gb300 import abi
        import ctypes
        lib = abi.load_library()
        n = ctypes.c_int(0)
        return lib.psph_device_check(ctypes.byref(n)) == 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """Library handle; fails (does not skip) when the CUDA path is unavailable,
    so a GPU run cannot pass on a missing extension."""
    from persiansph_gb300 import abi
    lib = abi.load_library()
    import ctypes
    n = ctypes.c_int(0)
    st = lib.psph_device_check(ctypes.byref(n))
    assert st == 0, f"no usable sm_103 device (psph_device_check={st}, devices={n.value})"
    return lib
