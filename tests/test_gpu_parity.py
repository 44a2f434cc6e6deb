"""GPU parity tests: the CUDA path through the C-ABI against the CPU oracle on the same inputs.

Tolerances (plain FP64 form): total energy 1e-9 Ha, charges 1e-8 e, gradients 1e-8 Ha/Bohr;
H0/S elements 1e-13 (same interpolation and rotation arithmetic); eigenvalues 1e-10 * ||A||.
"""
import numpy as np
import pytest
import scipy.linalg

from oracle import dftb_oracle as O

pytestmark = pytest.mark.gpu

E_TOL = 1e-9
Q_TOL = 1e-8
G_TOL = 1e-8


def _ctx(model, coords, species):
    from dftbplus_gb300 import binding
    ctx = binding.Context(0)
    ctx.set_model(model)
    ctx.set_geometry(coords, species)
    return ctx


def test_h0_s_water(gpu_lib, water_model):
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(8, 6.3, 21)
    ctx = _ctx(water_model, c, s)
    H0, S = O.build_h0_s(O.System(water_model, c, s))
    assert np.max(np.abs(ctx.matrix(0) - H0)) < 1e-13
    assert np.max(np.abs(ctx.matrix(1) - S)) < 1e-13
    ctx.close()


def test_h0_s_spd_and_tail(gpu_lib, tio2_model):
    """s/p/d blocks (Ti) and pairs inside the 5th-order tail region (12..13 Bohr)."""
    rng = np.random.default_rng(3)
    c = rng.uniform(-7, 7, (3, 10))
    c[:, 9] = c[:, 0] + np.array([12.4, 0.3, 0.2])   # a pair in the tail window
    s = np.array([0, 1, 1, 0, 1, 1, 0, 1, 1, 1])
    ctx = _ctx(tio2_model, c, s)
    H0, S = O.build_h0_s(O.System(tio2_model, c, s))
    assert np.max(np.abs(ctx.matrix(0) - H0)) < 1e-13
    assert np.max(np.abs(ctx.matrix(1) - S)) < 1e-13
    ctx.close()


@pytest.mark.parametrize("n", [1, 2, 37, 200, 517])
def test_sygvd_random(gpu_lib, n):
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)); A = A + A.T
    X = rng.normal(size=(n, n)); B = X @ X.T / n + np.eye(n)
    ctx = binding.Context(0)
    w, V, L = ctx.sygvd(A, B)
    wr = scipy.linalg.eigh(A, B, eigvals_only=True)
    scale = max(1.0, np.max(np.abs(wr)))
    assert np.max(np.abs(w - wr)) < 1e-10 * scale
    assert np.max(np.abs(A @ V - B @ V * w)) < 1e-9 * scale
    assert np.max(np.abs(V.T @ B @ V - np.eye(n))) < 1e-10
    np.testing.assert_allclose(np.tril(L), np.linalg.cholesky(B), atol=1e-12)
    ctx.close()


def test_sygvd_degenerate_clusters(gpu_lib):
    """Many exactly/nearly degenerate eigenvalues (deflation path of the divide and conquer)."""
    from dftbplus_gb300 import binding
    n = 300
    rng = np.random.default_rng(9)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    lam = np.repeat(np.array([-1.0, -0.5, 0.0, 0.25, 2.0]), n // 5) + 1e-14 * rng.normal(size=n)
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    B = np.eye(n)
    ctx = binding.Context(0)
    w, V, _ = ctx.sygvd(A, B)
    assert np.max(np.abs(w - np.sort(lam))) < 1e-12
    assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-11
    assert np.max(np.abs(A @ V - V * w)) < 1e-11
    ctx.close()


def _scc_parity(model, c, s, kT=1e-3, tol=1e-7, check_grad=True):
    from dftbplus_gb300 import binding
    sys_ = O.System(model, c, s)
    ref = O.run_scc(sys_, kt=kT, scc_tol=tol)
    ctx = _ctx(model, c, s)
    res = ctx.scc(binding.default_opts(kT=kT, scc_tol=tol))
    assert res["converged"] and ref.converged
    assert res["n_iter"] == ref.n_iter
    for k in ("EnonSCC", "Escc", "Erep", "Etotal", "EMermin", "TS", "Eband"):
        assert abs(res["energies"][k] - ref.energies[k]) < E_TOL, (k, res["energies"][k], ref.energies[k])
    assert np.max(np.abs(res["q_out"] - ref.q_out_atom)) < Q_TOL
    assert np.max(np.abs(res["eig"] - ref.eig)) < 1e-9
    assert abs(res["ef"] - ref.ef) < 1e-9
    assert np.max(np.abs(ctx.matrix(2) - ref.rho)) < 1e-8
    if check_grad:
        g = ctx.gradients()
        gref = O.gradients(sys_, ref)
        assert np.max(np.abs(g - gref)) < G_TOL, np.max(np.abs(g - gref))
    ctx.close()
    return res


def test_scc_water8(gpu_lib, water_model):
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(8, 6.3, 11)
    _scc_parity(water_model, c, s)


def test_scc_water32_config0(gpu_lib, water_model):
    """(H2O)32, 192 orbitals, 256 electrons: the reference's CPU-runnable configuration."""
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(32, 10.0, 1)
    _scc_parity(water_model, c, s)


def test_scc_fractional_filling(gpu_lib, water_model):
    """Charged cluster with small gap at high kT: Fermi bisection path and fractional fillings."""
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(6, 5.7, 5)
    sys_ = O.System(water_model, c, s)
    ref = O.run_scc(sys_, kt=0.05, scc_tol=1e-7, net_charge=0.5)
    ctx = _ctx(water_model, c, s)
    res = ctx.scc(binding.default_opts(kT=0.05, scc_tol=1e-7, net_charge=0.5))
    assert abs(res["energies"]["EMermin"] - ref.energies["EMermin"]) < E_TOL
    assert abs(res["energies"]["TS"] - ref.energies["TS"]) < E_TOL
    assert np.max(np.abs(res["q_out"] - ref.q_out_atom)) < Q_TOL
    g = ctx.gradients()
    assert np.max(np.abs(g - O.gradients(sys_, ref))) < G_TOL
    ctx.close()


def test_spd_scc(gpu_lib, tio2_model):
    """Small Ti/O cluster with d shells through the whole SCC + gradient path."""
    rng = np.random.default_rng(12)
    pts = []
    while len(pts) < 9:
        p = rng.uniform(-4.5, 4.5, 3)
        if all(np.linalg.norm(p - q) > 3.3 for q in pts):
            pts.append(p)
    c = np.array(pts).T
    s = np.array([0, 1, 1, 0, 1, 1, 0, 1, 1])
    sys_ = O.System(tio2_model, c, s)
    _, S = O.build_h0_s(sys_)
    if np.linalg.eigvalsh(S)[0] < 0.05:
        pytest.skip("random geometry gives an ill-conditioned overlap")
    _scc_parity(tio2_model, c, s, kT=5e-3)


@pytest.mark.parametrize("n_mol,radius,seed", [(32, 10.0, 1), (128, 20.0, 128)])
def test_mixed_precision_matches_fp64(gpu_lib, water_model, n_mol, radius, seed):
    """Mixed form: FP32 eigensolves early, one FP64 reference eigensolve, perturbative FP32 updates
    around it, and a converged FP64 iteration at the end. Errors against the FP64 oracle must meet
    the mixed targets (|dE| <= 1e-6 Ha/atom, max|dF| <= 1e-5 Ha/Bohr); the test holds them to the
    SCC-tolerance level, which the form reaches."""
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(n_mol, radius, seed)
    sys_ = O.System(water_model, c, s)
    ref = O.run_scc(sys_, kt=1e-3, scc_tol=1e-7)
    ctx = _ctx(water_model, c, s)
    ctx.profile(True)
    res = ctx.scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, precision=binding.PREC_MIXED))
    prof = ctx.profile_read()
    ctx.profile(False)
    hist = ctx.scc_history()
    assert res["converged"]
    assert prof["gemm_fp32"]["calls"] > 0, "no reduced-precision iteration ran"
    kinds = set(hist["precision"].tolist())
    assert {binding.PREC_MIXED, binding.PREC_FP64, binding.ITER_PERTURB} <= kinds, kinds
    assert hist["precision"][-1] == binding.PREC_FP64 and hist["error"][-1] < 1e-7
    assert len(hist["error"]) == res["n_iter"]
    natom = len(s)
    de = abs(res["energies"]["EMermin"] - ref.energies["EMermin"])
    assert de / natom < 1e-8
    assert np.max(np.abs(res["q_out"] - ref.q_out_atom)) < 1e-6
    g = ctx.gradients()
    gref = O.gradients(sys_, ref)
    assert np.max(np.abs(g - gref)) < 1e-6
    ctx.close()


def test_mixed_fp64_products_on_tensor_cores(gpu_lib, water_model):
    """The mixed form's FP64 iterations with their GEMMs as exact digit-slice products on the tensor
    cores (default) and with FP64 arithmetic: both meet the oracle, and agree with each other."""
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(128, 20.0, 128)
    sys_ = O.System(water_model, c, s)
    ref = O.run_scc(sys_, kt=1e-3, scc_tol=1e-7)
    gref = O.gradients(sys_, ref)
    out = {}
    prev = binding.set_fp64_emulation(True)
    try:
        for emulate in (True, False):
            binding.set_fp64_emulation(emulate)
            ctx = _ctx(water_model, c, s)
            ctx.profile(True)
            res = ctx.scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, precision=binding.PREC_MIXED))
            prof = ctx.profile_read()
            ctx.profile(False)
            assert res["converged"]
            # the route is what the test is about: on, some FP64 products ran on the tensor cores;
            # off, none did
            if emulate:
                assert prof["gemm_tc_fp64"]["calls"] > 0, "no FP64 product ran on the tensor cores"
            else:
                assert prof["gemm_tc_fp64"]["calls"] == 0
            out[emulate] = (res["energies"]["EMermin"], res["q_out"], ctx.gradients())
            ctx.close()
    finally:
        binding.set_fp64_emulation(prev)
    for e, q, g in out.values():
        assert abs(e - ref.energies["EMermin"]) / len(s) < 1e-8
        assert np.max(np.abs(q - ref.q_out_atom)) < 1e-6
        assert np.max(np.abs(g - gref)) < 1e-6
    assert abs(out[True][0] - out[False][0]) / len(s) < 1e-9


def test_not_positive_definite_reports_status(gpu_lib):
    """A table draw with an indefinite overlap: the Cholesky reports the status, no fault."""
    from dftbplus_gb300 import binding, synth
    bad = synth.water_model(draw=3)
    c, s = synth.water_cluster(32, 10.0, 1)
    ctx = binding.Context(0)
    ctx.set_model(bad)
    with pytest.raises(binding.DftbGpuError) as e:
        ctx.set_geometry(c, s)
    assert e.value.code == 3
    ctx.close()


def test_not_converged_status(gpu_lib, water_model):
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(8, 6.3, 11)
    ctx = _ctx(water_model, c, s)
    with pytest.raises(binding.DftbGpuError) as e:
        ctx.scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, max_iter=2, convergent_only=1))
    assert e.value.code == 4
    res = ctx.scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, max_iter=2))
    assert not res["converged"] and res["n_iter"] == 2
    ctx.close()


def test_deterministic(gpu_lib, water_model):
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(16, 8.0, 4)
    out = []
    for _ in range(2):
        ctx = _ctx(water_model, c, s)
        r = ctx.scc(binding.default_opts(kT=1e-3, scc_tol=1e-7))
        out.append((r["energies"]["EMermin"], r["q_out"].copy(), ctx.gradients()))
        ctx.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])


def test_calculator_api(gpu_lib, water_model):
    """DftbGpu mirrors DftbPlus: energy, gradients (natom, 3), gross charges."""
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(4, 3.5, 3)
    calc = binding.DftbGpu(water_model, c, s)
    ref = O.run_scc(O.System(water_model, c, s))
    assert abs(calc.get_energy() - ref.energies["EMermin"]) < E_TOL
    assert calc.get_gradients().shape == (calc.get_nr_atoms(), 3)
    q0 = O.System(water_model, c, s).q0_atom
    assert np.max(np.abs(calc.get_gross_charges() - (q0 - ref.q_out_atom))) < Q_TOL
    calc.close()


def test_mixed_precision_fractional_spd(gpu_lib, tio2_model):
    """Mixed form on a Ti/O cluster at high kT: fractional fillings through the perturbative updates
    (Fermi divided differences, the Fermi-level shift), against the FP64 oracle."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(12)
    pts = []
    while len(pts) < 9:
        p = rng.uniform(-4.5, 4.5, 3)
        if all(np.linalg.norm(p - q) > 3.3 for q in pts):
            pts.append(p)
    c = np.array(pts).T
    s = np.array([0, 1, 1, 0, 1, 1, 0, 1, 1])
    sys_ = O.System(tio2_model, c, s)
    _, S = O.build_h0_s(sys_)
    if np.linalg.eigvalsh(S)[0] < 0.05:
        pytest.skip("random geometry gives an ill-conditioned overlap")
    ref = O.run_scc(sys_, kt=5e-3, scc_tol=1e-7)
    ctx = _ctx(tio2_model, c, s)
    res = ctx.scc(binding.default_opts(kT=5e-3, scc_tol=1e-7, precision=binding.PREC_MIXED,
                                       mixed_switch_tol=1e-2))
    hist = ctx.scc_history()
    assert res["converged"] and hist["precision"][-1] == binding.PREC_FP64
    assert abs(res["energies"]["EMermin"] - ref.energies["EMermin"]) / len(s) < 1e-8
    assert np.max(np.abs(ctx.gradients() - O.gradients(sys_, ref))) < 1e-6
    ctx.close()
