import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available():
    """True when the CUDA driver reports at least one device (no torch import needed)."""
    import ctypes
    try:
        cuda = ctypes.CDLL("libcuda.so.1")
        if cuda.cuInit(0) != 0:
            return False
        n = ctypes.c_int(0)
        return cuda.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


# tolerances of the parity contract: metric value within 1e-5 relative, derivative
# within 1e-4 relative (relative to the derivative's largest magnitude component)
VALUE_RTOL = 1e-5
DERIV_RTOL = 1e-4
# Mattes MI can be ~0 (e.g. 5 bins leave one central bin): there a relative bound is
# meaningless, so the value also passes within 1e-8 absolute (entropies are O(1) nats)
MATTES_VALUE_ATOL = 1e-8


def assert_value_close(got, want, rtol=VALUE_RTOL, what="value", atol=0.0):
    err = abs(got - want)
    assert err <= rtol * abs(want) + atol, \
        f"{what}: got {got!r} want {want!r} abs err {err:.3e} > {rtol:.1e} * |want| + {atol:.1e}"


def assert_deriv_close(got, want, rtol=DERIV_RTOL, what="derivative"):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    scale = max(np.max(np.abs(want)), 1e-300)
    err = np.max(np.abs(got - want)) / scale
    assert err <= rtol, f"{what}: max |diff| / max |want| = {err:.3e} > {rtol:.1e}\n got {got}\n want {want}"
