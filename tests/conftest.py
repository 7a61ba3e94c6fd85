import ctypes
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu():
    """Device info through the product library.  A gpu-marked test on a
    machine without a usable GPU fails here, loudly."""
    import lisa_gb300 as L

    sm, cc, cm = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    L._native.check(L._native.lib().lisa_device_info(ctypes.byref(sm), ctypes.byref(cc), ctypes.byref(cm)))
    return {"sm_count": sm.value, "cc": (cc.value, cm.value)}


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O
