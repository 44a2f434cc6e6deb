"""Two-stage tridiagonal reduction (dense -> band of width 32 -> tridiagonal) and its accumulated
transformation Q = Q1 Q2, in FP64 and FP32, against LAPACK eigenvalues: eigenvalues of the
tridiagonal, A = Q T Q^T and orthogonality of Q. Sizes cover a single band block (n <= 33), partial
last panels and blocks, sweep groups, and a matrix with exactly zero panels (block diagonal: the
reflectors with tau = 0)."""
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


def _check(ctx, a, fp32):
    n = a.shape[0]
    d, e, q = ctx.test_twostage(a, fp32=fp32)
    scale = max(1.0, np.max(np.abs(np.linalg.eigvalsh(a))))
    tol = (2e-5 if fp32 else 1e-12) * scale * max(1.0, np.sqrt(n) / 8)
    w = scipy.linalg.eigh_tridiagonal(d, e, eigvals_only=True) if n > 1 else d
    assert np.max(np.abs(w - np.linalg.eigvalsh(a))) < tol
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.max(np.abs(q @ T @ q.T - a)) < 10 * tol
    assert np.max(np.abs(q.T @ q - np.eye(n))) < (2e-5 if fp32 else 1e-12) * max(1.0, np.sqrt(n) / 8)


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("n", [1, 2, 5, 33, 34, 35, 70, 97, 257, 1000])
def test_twostage_random(ctx, n, fp32):
    rng = np.random.default_rng(7 * n + fp32)
    a = rng.normal(size=(n, n))
    a = a + a.T
    _check(ctx, a, fp32)


@pytest.mark.parametrize("fp32", [False, True])
def test_twostage_block_diagonal(ctx, fp32):
    """Blocks of 40 with nothing between them: whole panels and band columns are already zero."""
    rng = np.random.default_rng(3)
    n, nb = 200, 40
    a = np.zeros((n, n))
    for i in range(0, n, nb):
        x = rng.normal(size=(nb, nb))
        a[i:i + nb, i:i + nb] = x + x.T
    _check(ctx, a, fp32)


def test_twostage_graded_spectrum(ctx):
    """A = U diag(lambda) U^T with eigenvalues over 12 decades and a 50-fold degenerate cluster."""
    rng = np.random.default_rng(11)
    n = 300
    lam = np.concatenate([np.logspace(-6, 6, 250), np.full(50, 0.5)])
    u, _ = np.linalg.qr(rng.normal(size=(n, n)))
    a = (u * lam) @ u.T
    a = 0.5 * (a + a.T)
    _check(ctx, a, False)


@pytest.mark.parametrize("mode", [0, 1])
def test_mixed_scc_through_either_reduction(gpu_lib, water_model, mode):
    """The mixed form's FP32 eigensolves through the one-stage (0) and the two-stage (1) reduction:
    (H2O)128 against its oracle fixture at the mixed form's tolerances."""
    import os
    from dftbplus_gb300 import binding, synth
    from bench import CONFIGS
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scc_h2o128.npz"))
    c, s = synth.water_cluster(*CONFIGS["h2o128"])
    prev = binding.set_two_stage(mode)
    try:
        ctx = binding.Context(0)
        ctx.set_model(water_model)
        ctx.set_geometry(c, s)
        res = ctx.scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, precision=binding.PREC_MIXED))
        g = ctx.gradients()
        hist = ctx.scc_history()
        ctx.close()
    finally:
        binding.set_two_stage(prev)
    assert res["converged"] and binding.PREC_MIXED in set(hist["precision"].tolist())
    keys = [str(k) for k in z["energy_keys"]]
    assert abs(res["energies"]["EMermin"] - z["energies"][keys.index("EMermin")]) / len(s) < 1e-8
    assert np.max(np.abs(res["q_out"] - z["q_out_atom"])) < 1e-6
    assert np.max(np.abs(g - z["grad"])) < 1e-6


def test_two_stage_mode_switch(gpu_lib):
    from dftbplus_gb300 import binding
    prev = binding.set_two_stage(2)
    assert binding.set_two_stage(prev) == 2
    with pytest.raises(ValueError):
        binding.set_two_stage(3)
