"""One-stage tridiagonal reduction A = Q T Q^T (sytrd_lower) with both panel kernels, in FP64 and
FP32, against LAPACK eigenvalues: eigenvalues of T, A = Q T Q^T and orthogonality of Q.

Panel mode 0 re-reads the trailing matrix for every column; mode 1 keeps the panel's trailing tiles
in shared memory (TMA loads where the leading dimension is a multiple of 16 bytes, element-wise
asynchronous copies where it is not); mode 2 is mode 1 with at most 64 CTAs and 8 tile slots, so
that sizes around 2,000 run the streaming ring (tiles re-loaded every column, across column and
panel boundaries). The strict upper triangle is never read: some matrices carry NaN there."""
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


@pytest.fixture
def panel_mode():
    from dftbplus_gb300 import binding
    prev = binding.set_panel_mode(1)
    yield binding.set_panel_mode
    binding.set_panel_mode(prev)


def _check(ctx, a, fp32):
    n = a.shape[0]
    sym = np.tril(a) + np.tril(a, -1).T
    d, e, q = ctx.test_onestage(a, fp32=fp32)
    ev = np.linalg.eigvalsh(sym)
    scale = max(1.0, np.max(np.abs(ev)))
    tol = (2e-5 if fp32 else 1e-12) * scale * max(1.0, np.sqrt(n) / 8)
    w = scipy.linalg.eigh_tridiagonal(d, e, eigvals_only=True) if n > 1 else d
    assert np.all(np.isfinite(d)) and np.all(np.isfinite(e)) and np.all(np.isfinite(q))
    assert np.max(np.abs(w - ev)) < tol
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.max(np.abs(q @ T @ q.T - sym)) < 10 * tol
    assert np.max(np.abs(q.T @ q - np.eye(n))) < (2e-5 if fp32 else 1e-12) * max(1.0, np.sqrt(n) / 8)
    return w


def _sym(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(n, n))
    return a + a.T


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 33, 64, 65, 97, 130, 256, 258, 700])
def test_onestage_random(ctx, panel_mode, n, fp32, mode):
    panel_mode(mode)
    _check(ctx, _sym(n, 11 * n + fp32), fp32)


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("n", [2000, 2001, 2002])
def test_onestage_streaming_ring(ctx, panel_mode, n, fp32):
    """64 CTAs with at most 8 tile slots (one or two per tile group): the groups with more tiles than
    slots stream them through their ring every column. n = 2000 runs TMA in both precisions, 2001
    element copies in both, 2002 TMA in FP64 only."""
    panel_mode(2)
    a = _sym(n, n)
    w2 = _check(ctx, a, fp32)
    panel_mode(0)
    w0 = _check(ctx, a, fp32)
    assert np.max(np.abs(w2 - w0)) < (5e-4 if fp32 else 1e-11)


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("n", [130, 258])
def test_onestage_ignores_upper_triangle(ctx, panel_mode, n, fp32, mode):
    panel_mode(mode)
    a = np.tril(_sym(n, 5 * n))
    a[np.triu_indices(n, 1)] = np.nan
    _check(ctx, a, fp32)


@pytest.mark.parametrize("fp32", [False, True])
def test_onestage_block_diagonal(ctx, panel_mode, fp32):
    """Exactly zero columns below the subdiagonal (tau = 0 reflectors) inside resident panels."""
    rng = np.random.default_rng(4)
    n, nb = 300, 45
    a = np.zeros((n, n))
    for i in range(0, n, nb):
        x = rng.normal(size=(min(nb, n - i), min(nb, n - i)))
        a[i:i + nb, i:i + nb] = x + x.T
    _check(ctx, a, fp32)


def test_panel_mode_switch(gpu_lib):
    from dftbplus_gb300 import binding
    prev = binding.set_panel_mode(0)
    assert binding.set_panel_mode(prev) == 0
    with pytest.raises(ValueError):
        binding.set_panel_mode(3)
