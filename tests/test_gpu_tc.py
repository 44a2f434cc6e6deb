"""Tensor-core (tcgen05) split-BF16 GEMM against a float64 reference of the same product.

Three BF16 pieces per operand and the six leading products keep about 22 significant bits; with the
FP32 accumulation in tensor memory the bound is 2e-6 * sum_k |a_ik| |b_kj| per element (FP32 FMA
products are within ~1e-6 of the same reference)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[0, 1], ids=["single-stage", "pipelined"])
def dg_kernel(request, gpu_lib):
    """Both kernels of the digit-slice product: the pipelined TMA kernel and the single-stage one."""
    from dftbplus_gb300 import binding
    prev = binding.set_digit_gemm_kernel(request.param)
    yield request.param
    binding.set_digit_gemm_kernel(prev)


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


# ------------------------------------------------------------------ FP64-class digit-slice products
def _dref(ta, tb, A, B):
    a = A.T if ta == "T" else A
    b = B.T if tb == "T" else B
    k = a.shape[1]
    # error bound of the digit-slice product (K max|a_i.| max|b_.j| (2^-53 + K 2^-65)) plus that of
    # the float64 reference itself (K 2^-53 sum |a||b| <= K^2 2^-53 max max, kept to the same form)
    scale = k * np.abs(a).max(1)[:, None] * np.abs(b).max(0)[None, :]
    return a @ b, scale * (2.0 ** -51 + k * 2.0 ** -64)


@pytest.mark.parametrize("m,n,k,ta,tb", [
    (128, 64, 64, "N", "N"),       # one tile, one K block
    (256, 192, 200, "N", "N"),     # several tiles and K blocks, ragged K
    (300, 200, 100, "N", "T"),     # ragged edges, padding
    (384, 257, 640, "T", "N"),
    (129, 511, 77, "T", "T"),
    (96, 40, 32, "N", "N"),        # smaller than one tile
    (64, 64, 2000, "T", "N"),      # one tile, long K: split over 8 CTAs along K
    (64, 512, 1500, "T", "N"),     # few tiles: split along K
])
def test_tc_dgemm_products(gpu_lib, dg_kernel, m, n, k, ta, tb):
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(m * 5 + n + k)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k))
    B = rng.standard_normal((n, k) if tb == "T" else (k, n))
    ctx = binding.Context(0)
    C = ctx.test_dgemm_tc(ta, tb, A, B)
    ref, tol = _dref(ta, tb, A, B)
    assert np.all(np.abs(C - ref) <= tol), np.max(np.abs(C - ref) / tol)
    ctx.close()


def test_tc_dgemm_scales_zeros_and_flags(gpu_lib, dg_kernel):
    """Rows and columns over 60 orders of magnitude, zero rows, triangular hints, lower-only output
    and beta accumulation; the untouched upper triangle keeps its bits."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(11)
    n = 320
    L = np.tril(rng.standard_normal((n, n))) * 10.0 ** rng.uniform(-30, 30, (n, 1))
    L[17] = 0.0
    junk = np.triu(rng.standard_normal((n, n)), 1)          # must be ignored (kALower)
    X = rng.standard_normal((n, n)) * 10.0 ** rng.uniform(-5, 5, (1, n))
    C0 = rng.standard_normal((n, n))
    ctx = binding.Context(0)
    kALower, kCLower = 1, 16
    C = ctx.test_dgemm_tc("N", "N", L + junk, X, C=C0, alpha=0.5, beta=1.0, flags=kALower | kCLower)
    ref, tol = _dref("N", "N", L, X)
    ref = 0.5 * ref + C0
    tol = 0.5 * tol + 2.0 ** -52 * np.abs(C0)
    low = np.tril(np.ones((n, n), dtype=bool))
    assert np.all(np.abs(C - ref)[low] <= tol[low]), np.max((np.abs(C - ref) / tol)[low])
    assert np.array_equal(C[~low], C0[~low])
    assert np.array_equal(C[17, :18], C0[17, :18])          # zero row: alpha * 0 + beta * C0
    ctx.close()


def test_tc_dgemm_split_lower_beta(gpu_lib, dg_kernel):
    """Split-K with a lower-only output and beta accumulation (int64 partials summed exactly): the
    same product split and unsplit agree bit for bit."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(21)
    m, k = 256, 1200                 # 4 x 4 tiles (lower half computed), 19 K blocks: split 4 ways
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, m))
    C0 = rng.standard_normal((m, m))
    ctx = binding.Context(0)
    kCLower = 16
    C = ctx.test_dgemm_tc("N", "N", A, B, C=C0, alpha=-1.0, beta=1.0, flags=kCLower)
    ref, tol = _dref("N", "N", A, B)
    ref = C0 - ref
    tol = tol + 2.0 ** -52 * np.abs(C0)
    low = np.tril(np.ones((m, m), dtype=bool))
    assert np.all(np.abs(C - ref)[low] <= tol[low])
    assert np.array_equal(C[~low], C0[~low])
    # the same product computed as two K halves added by beta reproduces the result to rounding
    C2 = ctx.test_dgemm_tc("N", "N", A[:, :600], B[:600], C=C0, alpha=-1.0, beta=1.0, flags=kCLower)
    C2 = ctx.test_dgemm_tc("N", "N", A[:, 600:], B[600:], C=C2, alpha=-1.0, beta=1.0, flags=kCLower)
    assert np.all(np.abs(C2 - C)[low] <= 2 * tol[low])
    ctx.close()


def test_tc_dgemm_largest_digit_sums(gpu_lib, dg_kernel):
    """Every digit 63 but the last: group sums near their bound must stay exact in the tensor-memory
    FP32 accumulators (K = 1,024: 16 blocks of 64 read back, sums near 2^21, in the single-stage
    kernel; 4 windows of 256, sums near 2^23, in the pipelined one)."""
    from dftbplus_gb300 import binding
    Y = 63 * sum(128 ** j for j in range(1, 8))
    x = Y * 2.0 ** -54
    k = 1024
    A = np.full((128, k), x)
    B = np.full((k, 64), -x)
    ctx = binding.Context(0)
    C = ctx.test_dgemm_tc("N", "N", A, B)
    exact = -k * x * x
    assert np.all(np.abs(C - exact) <= abs(exact) * 2.0 ** -50)
    ctx.close()


# ------------------------------------------------------------------ FP32 FMA products (128 x 128 tiles)
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_sgemm_large_tiles(gpu_lib, ta, tb):
    """Products with enough 128 x 128 tiles to fill the GPU take the large-tile FP32 kernel (ragged
    edges, K not a multiple of the K step); FP32 FMA bound 1e-6 sum_k |a_ik| |b_kj|."""
    from dftbplus_gb300 import binding
    m, n, k = 2500, 2437, 301
    rng = np.random.default_rng(len(ta + tb) + (ta == "T") * 3 + (tb == "T"))
    A = rng.standard_normal((k, m) if ta == "T" else (m, k)).astype(np.float32)
    B = rng.standard_normal((n, k) if tb == "T" else (k, n)).astype(np.float32)
    ctx = binding.Context(0)
    C = ctx.test_sgemm(ta, tb, A, B)
    ref, mag = _ref(ta, tb, A, B)
    assert np.all(np.abs(C - ref) <= 1e-6 * mag + 1e-6), np.max(np.abs(C - ref) / (mag + 1e-30))
    ctx.close()


def test_sgemm_large_tiles_flags_beta(gpu_lib):
    """Triangular hints, lower-only output (elements above the diagonal keep their bits) and beta, as
    the FP32 iterations use them (reduced transform, tridiagonalisation updates, density)."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(8)
    n = 2304
    L = np.tril(rng.standard_normal((n, n))).astype(np.float32)   # the hints promise these zeros
    X = np.tril(rng.standard_normal((n, n))).astype(np.float32)
    C0 = rng.standard_normal((n, n)).astype(np.float32)
    kALower, kBLower, kCLower = 1, 4, 16
    ctx = binding.Context(0)
    C = ctx.test_sgemm("N", "N", L, X, C=C0, alpha=-0.5, beta=1.0, flags=kALower | kBLower | kCLower)
    ref = -0.5 * (L.astype(np.float64) @ X) + C0
    mag = 0.5 * (np.abs(L).astype(np.float64) @ np.abs(X)) + np.abs(C0)
    low = np.tril(np.ones((n, n), dtype=bool))
    assert np.all(np.abs(C - ref)[low] <= 1e-6 * mag[low] + 1e-6)
    assert np.array_equal(C[~low], C0[~low])
    ctx.close()


# ------------------------------------------------------------------ FP32-class digit-slice products
def _fref(ta, tb, A, B):
    a = (A.T if ta == "T" else A).astype(np.float64)
    b = (B.T if tb == "T" else B).astype(np.float64)
    k = a.shape[1]
    # operand rounding (2^-25 of the row / column maxima), the dropped digit groups (2^-24) and the
    # final rounding to FP32
    scale = k * np.abs(a).max(1)[:, None] * np.abs(b).max(0)[None, :]
    ref = a @ b
    return ref, scale * 2.0 ** -22 + np.abs(ref) * 2.0 ** -23


@pytest.mark.parametrize("m,n,k,ta,tb", [
    (128, 64, 64, "N", "N"),       # one tile, one K block
    (256, 192, 200, "N", "N"),     # several tiles and K blocks (both stages), ragged K
    (300, 200, 130, "N", "T"),     # ragged edges, padding
    (384, 257, 640, "T", "N"),
    (129, 511, 77, "T", "T"),
    (64, 512, 1500, "T", "N"),     # few tiles: split along K
    (1000, 900, 3000, "N", "T"),
])
def test_fp32_digit_products(gpu_lib, m, n, k, ta, tb):
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(m * 7 + n + k)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k)).astype(np.float32)
    B = rng.standard_normal((n, k) if tb == "T" else (k, n)).astype(np.float32)
    ctx = binding.Context(0)
    C = ctx.test_sgemm_digits(ta, tb, A, B)
    ref, tol = _fref(ta, tb, A, B)
    assert np.all(np.abs(C - ref) <= tol), np.max(np.abs(C - ref) / tol)
    ctx.close()


def test_fp32_digit_scales_zeros_and_flags(gpu_lib):
    """Rows and columns over 20 orders of magnitude, a zero row, triangular hints, lower-only output
    and beta accumulation; the untouched upper triangle keeps its bits."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(12)
    n = 320
    L = (np.tril(rng.standard_normal((n, n))) * 10.0 ** rng.uniform(-10, 10, (n, 1))).astype(np.float32)
    L[17] = 0.0
    junk = np.triu(rng.standard_normal((n, n)), 1).astype(np.float32)   # must be ignored (kALower)
    X = (rng.standard_normal((n, n)) * 10.0 ** rng.uniform(-3, 3, (1, n))).astype(np.float32)
    C0 = rng.standard_normal((n, n)).astype(np.float32)
    ctx = binding.Context(0)
    kALower, kCLower = 1, 16
    C = ctx.test_sgemm_digits("N", "N", L + junk, X, C=C0, alpha=0.5, beta=1.0, flags=kALower | kCLower)
    ref, tol = _fref("N", "N", L, X)
    ref = 0.5 * ref + C0
    tol = 0.5 * tol + 2.0 ** -22 * np.abs(C0) + np.abs(ref) * 2.0 ** -23
    low = np.tril(np.ones((n, n), dtype=bool))
    assert np.all(np.abs(C - ref)[low] <= tol[low]), np.max((np.abs(C - ref) / tol)[low])
    assert np.array_equal(C[~low], C0[~low])
    assert np.array_equal(C[17, :18], C0[17, :18])          # zero row: alpha * 0 + beta * C0
    ctx.close()


def test_fp32_digit_split_lower_beta(gpu_lib):
    """Split-K with a lower-only output and beta accumulation (int64 partials summed exactly)."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(22)
    m, k = 256, 1200                 # 4 x 4 tiles (lower half computed), 19 K blocks: split 4 ways
    A = rng.standard_normal((m, k)).astype(np.float32)
    B = rng.standard_normal((k, m)).astype(np.float32)
    C0 = rng.standard_normal((m, m)).astype(np.float32)
    ctx = binding.Context(0)
    kCLower = 16
    C = ctx.test_sgemm_digits("N", "N", A, B, C=C0, alpha=-1.0, beta=1.0, flags=kCLower)
    ref, tol = _fref("N", "N", A, B)
    ref = C0 - ref
    tol = tol + 2.0 ** -22 * np.abs(C0)
    low = np.tril(np.ones((m, m), dtype=bool))
    assert np.all(np.abs(C - ref)[low] <= tol[low])
    assert np.array_equal(C[~low], C0[~low])
    ctx.close()


def test_fp32_digit_largest_group_sums(gpu_lib):
    """x = 1 - 2^-24 has the digits (256, 0, -1): the leading group sum of a 64-wide K block is 2^22,
    next to its bound, and must stay exact in the tensor-memory FP32 accumulators (K = 1,024)."""
    from dftbplus_gb300 import binding
    x = np.float32(1.0) - np.float32(2.0 ** -24)
    k = 1024
    A = np.full((128, k), x, dtype=np.float32)
    B = np.full((k, 64), -x, dtype=np.float32)
    ctx = binding.Context(0)
    C = ctx.test_sgemm_digits("N", "N", A, B)
    exact = -k * float(x) * float(x)
    assert np.all(np.abs(C.astype(np.float64) - exact) <= abs(exact) * 2.0 ** -23)
    ctx.close()
