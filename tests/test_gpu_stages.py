"""Stage-level GPU checks of the FP64 eigensolver pieces (GEMM, tridiagonalisation, D&C)."""
import numpy as np
import pytest
import scipy.linalg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    from dftbplus_gb300 import binding
    c = binding.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("ta,tb,m,n,k", [("N", "N", 37, 41, 29), ("N", "T", 130, 70, 200), ("T", "N", 65, 129, 64),
                                         ("T", "T", 100, 3, 77)])
def test_dgemm(ctx, ta, tb, m, n, k):
    rng = np.random.default_rng(m * n + k)
    a = rng.normal(size=(m, k) if ta == "N" else (k, m))
    b = rng.normal(size=(k, n) if tb == "N" else (n, k))
    c = rng.normal(size=(m, n))
    opa = a if ta == "N" else a.T
    opb = b if tb == "N" else b.T
    out = ctx.test_dgemm(ta, tb, a, b, c, alpha=1.5, beta=-0.5)
    np.testing.assert_allclose(out, 1.5 * opa @ opb - 0.5 * c, atol=1e-12, rtol=1e-12)


@pytest.mark.parametrize("n", [3, 33, 37, 70, 200])
def test_tridiag(ctx, n):
    rng = np.random.default_rng(n)
    a = rng.normal(size=(n, n)); a = a + a.T
    d, e = ctx.test_tridiag(a)
    w = scipy.linalg.eigh_tridiagonal(d, e, eigvals_only=True)
    assert np.max(np.abs(w - np.linalg.eigvalsh(a))) < 1e-11


@pytest.fixture(params=[True, False], ids=["staged", "global"])
def dc_staging(request):
    """Deflation of the divide-and-conquer merges in shared memory (the default) or global memory."""
    from dftbplus_gb300 import binding
    prev = binding.set_dc_staging(request.param)
    yield request.param
    binding.set_dc_staging(prev)


def _check_stedc(ctx, d, e, tol=1e-12):
    n = len(d)
    w, q = ctx.test_stedc(d, e)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    scale = max(1.0, np.max(np.abs(np.linalg.eigvalsh(T))))
    assert np.max(np.abs(w - np.linalg.eigvalsh(T))) < tol * scale
    assert np.max(np.abs(T @ q - q * w)) < tol * scale
    assert np.max(np.abs(q.T @ q - np.eye(n))) < tol
    return w, q


@pytest.mark.parametrize("n", [2, 3, 5, 37, 130, 300])
def test_stedc(ctx, dc_staging, n):
    rng = np.random.default_rng(n + 1)
    d = rng.normal(size=n); e = rng.normal(size=n - 1)
    _check_stedc(ctx, d, e)


@pytest.mark.parametrize("n", [300, 1500])
def test_stedc_heavy_deflation(ctx, dc_staging, n):
    """Both kinds of deflation: clusters of equal diagonal entries (pairs deflated by a rotation),
    couplings at round-off size (negligible z entries) and couplings of zero, mixed with ordinary
    entries; the staged and the global-memory scans run the same arithmetic and agree to rounding."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(7 * n)
    d = np.round(rng.normal(size=n) * 4) / 4          # many repeated values
    e = rng.normal(size=n - 1)
    e[rng.random(n - 1) < 0.3] *= 1e-17
    e[rng.random(n - 1) < 0.1] = 0.0
    w, q = _check_stedc(ctx, d, e)
    binding.set_dc_staging(not dc_staging)
    try:
        w2, _ = _check_stedc(ctx, d, e)
    finally:
        binding.set_dc_staging(dc_staging)
    assert np.max(np.abs(w - w2)) <= 1e-14 * max(1.0, np.max(np.abs(w)))
