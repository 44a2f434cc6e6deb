import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdftbgpu.so")


@pytest.fixture(scope="session")
def water_model():
    from dftbplus_gb300 import synth
    return synth.water_model()


@pytest.fixture(scope="session")
def tio2_model():
    from dftbplus_gb300 import synth
    return synth.tio2_model()


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load libdftbgpu.so; GPU tests skip only when no CUDA device exists."""
    import ctypes
    from dftbplus_gb300 import build, binding
    build.build()
    lib = binding.load_library()
    h = ctypes.c_void_p()
    rc = lib.dftbgpu_create(ctypes.byref(h), 0)
    if rc == 8:
        pytest.skip("no CUDA device")
    assert rc == 0, f"dftbgpu_create failed with {rc}"
    lib.dftbgpu_destroy(h)
    return lib


def small_water(n_mol, seed, radius=None):
    from dftbplus_gb300 import synth
    if radius is None:
        radius = 10.0 * (n_mol / 32.0) ** (1.0 / 3.0)
    return synth.water_cluster(n_mol, radius, seed)
