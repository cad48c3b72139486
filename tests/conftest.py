"""Shared fixtures. GPU tests carry @pytest.mark.gpu; the CPU suite runs with
-m "not gpu" and needs no device."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def lib():
    from nanofiller_gb300 import build
    build.build()
    import nanofiller_gb300 as nf
    return nf


@pytest.fixture(scope="session")
def oracle():
    from oracle import nf_oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu(lib):
    """The CUDA device; GPU tests fail loudly (no skip) when it is absent."""
    import ctypes as C
    p = lib.make_params(lib.configs.SMALL)
    h = C.c_void_p()
    st = lib.load().nf_create(C.byref(p), C.byref(h))
    assert st == 0, f"nf_create failed with status {st}: a GPU test ran without a usable CUDA device"
    lib.load().nf_destroy(h)
    return lib


def rods_struct(rods):
    """dict-of-arrays rods -> oracle record array."""
    from oracle import nf_oracle as O
    out = np.zeros(len(rods["x"]), O.ROD_DTYPE)
    for f in ("x", "y", "z", "cx", "cy", "cz", "l", "a"):
        out[f] = rods[f]
    return out


@pytest.fixture(scope="session")
def cfg():
    """The workload presets (no library or device needed)."""
    from nanofiller_gb300 import configs
    return configs
