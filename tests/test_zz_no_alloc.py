"""The allocation-free tridiagonal divide and conquer (dftbgpu_stedc_noalloc).

It is meant for callers that cannot allocate device memory (a step recorded into a CUDA graph, a
host whose device memory belongs to another allocator, a loop that must not synchronise the
device). The caller owns inputs and outputs; the routine's scratch is a file-scope device array
shared by all calls. This file is collected last so that a failure here does not hide the others.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same tolerance as the tridiagonal stage tests


def _noalloc(lib, d, e):
    import torch
    n = len(d)
    dd = torch.tensor(d, dtype=torch.float64, device="cuda")
    ee = torch.tensor(e if n > 1 else [0.0], dtype=torch.float64, device="cuda")
    qq = torch.empty(n * n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.dftbgpu_stedc_noalloc(n, dd.data_ptr(), ee.data_ptr(), qq.data_ptr(), None)
    torch.cuda.synchronize()
    return rc, dd.cpu().numpy(), qq.cpu().numpy().reshape(n, n, order="F")


def test_noalloc_matches_existing_entry_point(gpu_lib):
    """Two calls in a row (the second smaller, on the scratch the first left behind), each
    compared with dftbgpu_test_stedc on the same tridiagonal."""
    from dftbplus_gb300 import binding
    ctx = binding.Context(0)
    rng = np.random.default_rng(2024)
    for n in (256, 173):
        d = rng.normal(size=n)
        e = rng.normal(size=n - 1)
        w_ref, q_ref = ctx.test_stedc(d, e)
        rc, w, q = _noalloc(gpu_lib, d, e)
        assert rc == 0
        assert np.max(np.abs(w - w_ref)) < TOL
        assert np.max(np.abs(q - q_ref)) < TOL
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        assert np.max(np.abs(T @ q - q * w)) < TOL
    ctx.close()


def test_noalloc_rejects_oversize(gpu_lib):
    rc, _, _ = _noalloc(gpu_lib, np.zeros(257), np.zeros(256))
    assert rc == 1  # DFTBGPU_ERR_ARGS
