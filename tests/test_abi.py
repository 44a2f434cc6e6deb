"""CPU checks of the C-ABI boundary: the library builds, loads and exports every declared symbol."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "dftbgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dftbgpu_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    from dftbplus_gb300 import build
    return build.build()


def test_header_symbols_exported(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (dftbgpu_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_binding_covers_header():
    from dftbplus_gb300 import binding
    assert sorted(binding.SIGNATURES) == declared_symbols()


def test_library_loads_and_defaults(lib_path):
    from dftbplus_gb300 import binding
    lib = binding.load_library()
    o = binding.default_opts()
    # parser.F90:5786-5790 defaults
    assert (o.mix_alpha, o.mix_omega0, o.mix_min_weight, o.mix_max_weight, o.mix_weight_fac) == (0.2, 0.01, 1.0, 1e5, 1e-2)
    assert lib.dftbgpu_last_error(None) == b"null context"


def test_no_device_fails_loudly(lib_path):
    """Without a GPU the product path refuses to run (there is no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from dftbplus_gb300 import binding
    with pytest.raises(binding.DftbGpuError) as e:
        binding.Context(0)
    assert e.value.code == 8


def test_product_does_not_use_oracle():
    pkg = os.path.join(ROOT, "dftbplus_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
