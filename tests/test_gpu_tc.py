"""Tensor-core (tcgen05) split-BF16 GEMM against a float64 reference of the same product.

Three BF16 pieces per operand and the six leading products keep about 22 significant bits; with the
FP32 accumulation in tensor memory the bound is 2e-6 * sum_k |a_ik| |b_kj| per element (FP32 FMA
products are within ~1e-6 of the same reference)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref(ta, tb, A, B):
    a = A.T if ta == "T" else A
    b = B.T if tb == "T" else B
    return a.astype(np.float64) @ b.astype(np.float64), np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64)


@pytest.mark.parametrize("m,n,k,ta,tb", [
    (128, 128, 64, "N", "N"),      # one tile, one K block
    (256, 256, 192, "N", "N"),     # several tiles, three K blocks (stage reuse)
    (300, 200, 100, "N", "T"),     # ragged edges, padding
    (384, 257, 640, "T", "N"),
    (129, 511, 77, "T", "T"),
])
def test_tc_gemm_products(gpu_lib, m, n, k, ta, tb):
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(m * 7 + n + k)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k)).astype(np.float32)
    B = rng.standard_normal((n, k) if tb == "T" else (k, n)).astype(np.float32)
    ctx = binding.Context(0)
    C = ctx.test_gemm_tc(ta, tb, A, B)
    ref, mag = _ref(ta, tb, A, B)
    assert np.all(np.abs(C - ref) <= 2e-6 * mag + 1e-6), np.max(np.abs(C - ref) / (mag + 1e-30))
    ctx.close()


def test_tc_gemm_flags_and_beta(gpu_lib):
    """Triangular operand hints, lower-only output and beta accumulation, as the mixed form uses."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(3)
    n = 320
    L = np.tril(rng.standard_normal((n, n))).astype(np.float32)
    junk = np.triu(rng.standard_normal((n, n)), 1).astype(np.float32)   # must be ignored
    X = rng.standard_normal((n, n)).astype(np.float32)
    C0 = rng.standard_normal((n, n)).astype(np.float32)
    ctx = binding.Context(0)
    kALower, kCLower = 1, 16
    C = ctx.test_gemm_tc("N", "N", L + junk, X, C=C0, alpha=0.5, beta=1.0, flags=kALower | kCLower)
    ref = 0.5 * L.astype(np.float64) @ X + C0
    mag = 0.5 * np.abs(L).astype(np.float64) @ np.abs(X) + np.abs(C0)
    low = np.tril(np.ones((n, n), dtype=bool))
    assert np.all(np.abs(C - ref)[low] <= 2e-6 * mag[low] + 1e-6)
    assert np.array_equal(C[~low], C0[~low])       # upper triangle untouched
    ctx.close()
