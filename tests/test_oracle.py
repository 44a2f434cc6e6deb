"""CPU checks of the oracle against the reference's golden vectors and physical identities."""
import json
import os

import numpy as np
import pytest

from oracle import dftb_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_broyden_golden_sequence():
    """mixer/broydenmixer.F90 against test/src/dftbp/unit/mixer/broyden.F90 (atol 100 eps)."""
    g = json.load(open(os.path.join(GOLDEN, "broyden_h2o.json")))
    mix = O.BroydenMixer(alpha=g["mix_param"], omega0=g["omega0"], min_weight=g["min_weight"],
                         max_weight=g["max_weight"], weight_fac=g["weight_fac"], max_iter=g["max_scc_iter"])
    q = np.array(g["charges"][0])
    atol = g["atol_eps_multiple"] * np.finfo(float).eps
    for i in range(4):
        q = mix.mix(q, np.array(g["differences"][i]))
        np.testing.assert_allclose(q, g["charges"][i + 1], rtol=0, atol=atol)


def test_coulomb_cluster_derivative_golden():
    """dV/dR of the cluster 1/r potential against test/src/dftbp/unit/dftb/coulomb.F90:31-101."""
    g = json.load(open(os.path.join(GOLDEN, "coulomb_cluster.json")))
    coords = np.array(g["coords_bohr"]).T
    out = O.coulomb_potential_prime(coords, np.array(g["charges"]))
    expected = np.array(g["expected_fortran_order"], dtype=float).reshape(g["expected_shape"], order="F")
    assert np.max(np.abs(out - expected)) < np.finfo(float).eps


def test_sk_rotation_invariance_spd(tio2_model):
    """Spectrum of (H0, S) is invariant under a rigid rotation (pins s/p/d rotation formulas)."""
    import scipy.linalg
    from dftbplus_gb300 import synth
    rng = np.random.default_rng(5)
    c = rng.uniform(-4, 4, (3, 6))
    s = np.array([0, 1, 1, 0, 1, 1])
    H0, S = O.build_h0_s(O.System(tio2_model, c, s))
    assert np.linalg.eigvalsh(S)[0] > 0.05
    e1 = scipy.linalg.eigh(H0, S, eigvals_only=True)
    R = synth._rotation_from_quaternion(rng.normal(size=4))
    H0b, Sb = O.build_h0_s(O.System(tio2_model, R @ c + 1.3, s))
    e2 = scipy.linalg.eigh(H0b, Sb, eigvals_only=True)
    assert np.max(np.abs(e1 - e2)) < 1e-13


def test_gradients_match_finite_differences(water_model):
    """Oracle gradient (FD SK blocks + DC + repulsive) vs central differences of E_Mermin."""
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(4, 3.5, 3)
    sys_ = O.System(water_model, c, s)
    res = O.run_scc(sys_, scc_tol=1e-11)
    g = O.gradients(sys_, res)
    h = 1e-4
    for (a, k) in [(0, 0), (4, 1), (7, 2)]:
        e = []
        for sg in (+1, -1):
            cp = c.copy()
            cp[k, a] += sg * h
            e.append(O.run_scc(O.System(water_model, cp, s), scc_tol=1e-11).energies["EMermin"])
        fd = (e[0] - e[1]) / (2 * h)
        assert abs(g[k, a] - fd) < 5e-8, (a, k, g[k, a], fd)
    assert np.max(np.abs(g.sum(axis=1))) < 1e-12


def test_water_tables_positive_definite(water_model):
    """The accepted synthetic table draw keeps S well conditioned on the water workloads."""
    from dftbplus_gb300 import synth
    for n_mol, radius, seed in [(32, 10.0, 1), (8, 10.0 * 0.25 ** (1 / 3), 7)]:
        c, s = synth.water_cluster(n_mol, radius, seed)
        _, S = O.build_h0_s(O.System(water_model, c, s))
        assert np.linalg.eigvalsh(S)[0] > 0.2


def test_fermi_bisection_fractional_electrons():
    """Non-integer electron count takes the bisection path (etemp.F90:140-190)."""
    eig = np.linspace(-1.0, 1.0, 41)
    f, ef, eb, ts, e0 = O.fermi_filling(eig, 20.5, 0.01)
    assert abs(f.sum() - 20.5) < 1e-12
    assert ts > 0


def test_skf_roundtrip(tmp_path, water_model):
    from dftbplus_gb300 import skf, synth
    sset = synth.make_skf_set([synth.SPECIES_O, synth.SPECIES_H], synth.WATER_SEED, synth.WATER_DRAW)
    names = ["O", "H"]
    for (a, b), d in sset.items():
        h10, s10 = synth.skf_columns10(d)
        homo = (d.onsite, d.hubbu, d.occ, d.mass) if a == b else None
        skf.write_skf(str(tmp_path / f"{names[a]}-{names[b]}.skf"), d.dist, h10, s10, homo=homo,
                      repulsive=d.repulsive)
    from dftbplus_gb300.model import Model
    m2 = Model.from_files([synth.SPECIES_O, synth.SPECIES_H], str(tmp_path / "{A}-{B}.skf"))
    for key, t in water_model.tables.items():
        np.testing.assert_allclose(m2.tables[key].ham, t.ham, rtol=1e-15, atol=0)
        np.testing.assert_allclose(m2.tables[key].over, t.over, rtol=1e-15, atol=0)
    for a in range(2):
        assert m2.species[a].onsite == water_model.species[a].onsite
        assert m2.species[a].hubbu == water_model.species[a].hubbu


def test_scc_charge_conservation(water_model):
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(8, 6.3, 11)
    sys_ = O.System(water_model, c, s)
    res = O.run_scc(sys_)
    assert res.converged
    assert abs(res.q_out_atom.sum() - sys_.q0_atom.sum()) < 1e-9


def test_scc_golden_fixtures_reproduce():
    """The committed end-to-end fixtures of the benchmark workloads belong to the current workload
    generator (geometry digest), and the (H2O)128 one is reproduced by the oracle to rounding."""
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    from make_scc_golden import geometry_digest, ENERGY_KEYS
    from bench import CONFIGS
    from dftbplus_gb300 import synth
    for name in ("h2o128", "h2o1024"):
        z = np.load(os.path.join(here, f"scc_{name}.npz"))
        n_mol, radius, seed = CONFIGS[name]
        c, s = synth.water_cluster(n_mol, radius, seed)
        assert str(z["geometry_sha256"]) == geometry_digest(c, s)
        assert bool(z["converged"]) and z["errors"][-1] < 1e-7
        assert z["grad"].shape == (3, len(s)) and z["q_out_atom"].shape == (len(s),)
    z = np.load(os.path.join(here, "scc_h2o128.npz"))
    c, s = synth.water_cluster(*CONFIGS["h2o128"])
    sys_ = O.System(synth.water_model(), c, s)
    res = O.run_scc(sys_, kt=1e-3, scc_tol=1e-7)
    assert res.n_iter == int(z["n_iter"])
    assert np.allclose([res.energies[k] for k in ENERGY_KEYS], z["energies"], atol=1e-10, rtol=0)
    assert np.allclose(res.q_out_atom, z["q_out_atom"], atol=1e-10, rtol=0)


def test_density_idempotent_and_traced_at_low_temperature(water_model):
    """Internal consistency of the oracle's converged state (no reference data needed): with a gap
    far above kT every level is filled with 2 or 0 electrons, so rho S rho = 2 rho (spin-unpolarised
    idempotency in the S metric) and Tr(rho S) = N_el; the eigenvectors are S-orthonormal."""
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(8, 6.3, 11)
    sys_ = O.System(water_model, c, s)
    res = O.run_scc(sys_, kt=1e-5)
    assert res.converged
    H0, S = O.build_h0_s(sys_)
    n_el = water_model.n_electrons(sys_.species, 0.0)
    assert np.all((np.abs(res.filling - 2.0) < 1e-12) | (np.abs(res.filling) < 1e-12))
    assert abs(np.trace(res.rho @ S) - n_el) < 1e-10
    assert np.max(np.abs(res.rho @ S @ res.rho - 2.0 * res.rho)) < 1e-10
    assert np.max(np.abs(res.C.T @ S @ res.C - np.eye(S.shape[0]))) < 1e-10
