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


@pytest.mark.parametrize("n", [2, 3, 5, 37, 130, 300])
def test_stedc(ctx, n):
    rng = np.random.default_rng(n + 1)
    d = rng.normal(size=n); e = rng.normal(size=n - 1)
    w, q = ctx.test_stedc(d, e)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.max(np.abs(w - np.linalg.eigvalsh(T))) < 1e-12
    assert np.max(np.abs(T @ q - q * w)) < 1e-12
    assert np.max(np.abs(q.T @ q - np.eye(n))) < 1e-12
