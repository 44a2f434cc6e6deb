"""CPU checks of the synthetic workloads the configurations name (no GPU): the anatase TiO2 sphere of
the large spd configuration and the seeded water clusters."""
import numpy as np
import pytest

from oracle import dftb_oracle as O


def _nearest(x):
    d = np.linalg.norm(x[:, None, :] - x[None, :, :], axis=-1)
    np.fill_diagonal(d, np.inf)
    return d


def test_anatase_full_size_counts_and_bonds():
    """~1,700 Ti + 3,400 O, Ti spd (9) + O sp (4) = 28,900 orbitals; anatase bond lengths."""
    from dftbplus_gb300 import synth
    c, s = synth.anatase_cluster(1700)
    n_ti, n_o = int((s == 0).sum()), int((s == 1).sum())
    assert (n_ti, n_o) == (1700, 3400)
    assert 9 * n_ti + 4 * n_o == 28900
    x = c.T * synth.BOHR_AA
    ti, ox = x[s == 0], x[s == 1]
    # the Ti nearest the centre: four equatorial O at 1.93 A and two apical O at 1.98 A
    t0 = ti[np.argmin(np.linalg.norm(ti, axis=1))]
    d = np.sort(np.linalg.norm(ox - t0, axis=1))[:6]
    assert np.allclose(d[:4], 1.934, atol=2e-3) and np.allclose(d[4:], 1.979, atol=2e-3)
    # no two atoms closer than the Ti-O bond anywhere (the carving keeps whole lattice sites)
    sub = x[np.linalg.norm(x, axis=1) < 8.0]
    assert _nearest(sub).min() > 1.9


@pytest.mark.parametrize("n_ti", [40, 100])
def test_anatase_overlap_rule(n_ti):
    """The specified overlap prefactor range gives an indefinite overlap on anatase; the workload's
    model scales it by 1/4, which keeps S positive definite (the Cholesky of the eigensolver needs it)."""
    from dftbplus_gb300 import synth
    c, s = synth.anatase_cluster(n_ti)
    _, S_spec = O.build_h0_s(O.System(synth.tio2_model(), c, s))
    _, S = O.build_h0_s(O.System(synth.anatase_model(), c, s))
    assert np.linalg.eigvalsh(S_spec)[0] < 0.0
    assert np.linalg.eigvalsh(S)[0] > 0.2


def test_water_cluster_geometry():
    """Seeded (H2O)32 as configured: O-H 0.96 A, H-O-H 104.5 deg, O-O >= 2.6 A, inside a 10 A sphere."""
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(32, 10.0, 1)
    x = c.T * synth.BOHR_AA
    o, h = x[s == 0], x[s == 1]
    assert len(o) == 32 and len(h) == 64
    assert _nearest(o).min() >= 2.6 - 1e-9
    assert np.all(np.linalg.norm(o, axis=1) <= 10.0 + 1e-9)
    for i in range(32):
        v1, v2 = h[2 * i] - o[i], h[2 * i + 1] - o[i]
        assert np.allclose([np.linalg.norm(v1), np.linalg.norm(v2)], 0.96, atol=1e-9)
        ang = np.degrees(np.arccos(v1 @ v2 / (np.linalg.norm(v1) * np.linalg.norm(v2))))
        assert abs(ang - 104.5) < 1e-6
    c2, _ = synth.water_cluster(32, 10.0, 1)
    assert np.array_equal(c, c2)            # seeded: the same cluster every time


def test_water_table_draw_criteria(water_model):
    """The accepted water table draw: lambda_min(S) >= 0.2 on the (H2O)32 and (H2O)128 clusters and an
    (H2O)32 SCC HOMO-LUMO gap above 0.1 Ha; the preceding draw 1 (the only other definite one) has a
    gap below 0.1 Ha."""
    from dftbplus_gb300 import synth
    for n_mol, radius, seed in [(32, 10.0, 1), (128, 20.0, 128)]:
        c, s = synth.water_cluster(n_mol, radius, seed)
        _, S = O.build_h0_s(O.System(water_model, c, s))
        assert np.linalg.eigvalsh(S)[0] >= 0.2
    c, s = synth.water_cluster(32, 10.0, 1)
    nocc = int(round(water_model.n_electrons(s) / 2))
    res = O.run_scc(O.System(water_model, c, s))
    assert res.converged and res.eig[nocc] - res.eig[nocc - 1] > 0.1
    res1 = O.run_scc(O.System(synth.water_model(draw=1), c, s))
    assert res1.eig[nocc] - res1.eig[nocc - 1] < 0.1
