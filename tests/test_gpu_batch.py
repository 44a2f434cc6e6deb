"""Batched form: many ragged molecules in one call, each checked against the CPU oracle run on that
molecule alone (same tolerances as the single-system FP64 parity: 1e-9 Ha, 1e-8 e, 1e-8 Ha/Bohr)."""
import numpy as np
import pytest

from oracle import dftb_oracle as O

pytestmark = pytest.mark.gpu


def _water_set(n, seed, lo=1, hi=6):
    from dftbplus_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nm = int(rng.integers(lo, hi + 1))
        c, s = synth.water_cluster(nm, 3.5 * (nm / 2.0) ** (1.0 / 3.0) + 2.0, 1000 + 17 * seed + i)
        out.append((c, s))
    return out


def _ctx(model):
    from dftbplus_gb300 import binding
    ctx = binding.Context(0)
    ctx.set_model(model)
    return ctx


@pytest.mark.parametrize("nmol,seed", [(12, 1), (40, 2)])
def test_batch_fp64_matches_oracle(gpu_lib, water_model, nmol, seed):
    from dftbplus_gb300 import binding
    mols = _water_set(nmol, seed)
    ctx = _ctx(water_model)
    ctx.batch_set_geometries([m[0] for m in mols], [m[1] for m in mols])
    res = ctx.batch_scc(binding.default_opts(kT=1e-3, scc_tol=1e-7))
    grads = ctx.batch_gradients()
    off = ctx.batch_atom_off
    for i, (c, s) in enumerate(mols):
        sys_ = O.System(water_model, c, s)
        ref = O.run_scc(sys_, kt=1e-3, scc_tol=1e-7)
        assert res["converged"][i] and ref.converged
        assert res["n_iter"][i] == ref.n_iter, (i, res["n_iter"][i], ref.n_iter)
        e = res["energies"][i]
        for k in ("EnonSCC", "Escc", "Erep", "Etotal", "EMermin", "TS", "Eband"):
            assert abs(e[k] - ref.energies[k]) < 1e-9, (i, k, e[k], ref.energies[k])
        q = res["q_out"][off[i]:off[i + 1]]
        assert np.max(np.abs(q - ref.q_out_atom)) < 1e-8
        gref = O.gradients(sys_, ref)
        assert np.max(np.abs(grads[i] - gref)) < 1e-8, (i, np.max(np.abs(grads[i] - gref)))
    ctx.close()


def test_batch_spd_fractional(gpu_lib, tio2_model):
    """Ti/O molecules (d shells) at high kT: fractional fillings through the per-molecule Fermi search."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(5)
    mols = []
    while len(mols) < 6:
        nat = int(rng.integers(2, 7))
        pts = []
        while len(pts) < nat:
            p = rng.uniform(-3.5, 3.5, 3)
            if all(np.linalg.norm(p - q) > 3.3 for q in pts):
                pts.append(p)
        c = np.array(pts).T
        s = rng.integers(0, 2, nat)
        _, S = O.build_h0_s(O.System(tio2_model, c, s))
        if np.linalg.eigvalsh(S)[0] > 0.05:
            mols.append((c, s))
    ctx = _ctx(tio2_model)
    ctx.batch_set_geometries([m[0] for m in mols], [m[1] for m in mols])
    res = ctx.batch_scc(binding.default_opts(kT=5e-3, scc_tol=1e-7))
    grads = ctx.batch_gradients()
    for i, (c, s) in enumerate(mols):
        sys_ = O.System(tio2_model, c, s)
        ref = O.run_scc(sys_, kt=5e-3, scc_tol=1e-7)
        assert res["converged"][i] == ref.converged
        assert abs(res["energies"][i]["EMermin"] - ref.energies["EMermin"]) < 1e-9
        assert np.max(np.abs(grads[i] - O.gradients(sys_, ref))) < 1e-8
    ctx.close()


def test_batch_mixed_precision(gpu_lib, water_model):
    """Mixed batched form: FP32 eigensolves per molecule until close, FP64 to convergence."""
    from dftbplus_gb300 import binding
    mols = _water_set(16, 3, 2, 8)
    ctx = _ctx(water_model)
    ctx.batch_set_geometries([m[0] for m in mols], [m[1] for m in mols])
    res = ctx.batch_scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, precision=binding.PREC_MIXED))
    grads = ctx.batch_gradients()
    for i, (c, s) in enumerate(mols):
        sys_ = O.System(water_model, c, s)
        ref = O.run_scc(sys_, kt=1e-3, scc_tol=1e-7)
        assert res["converged"][i]
        assert abs(res["energies"][i]["EMermin"] - ref.energies["EMermin"]) / len(s) < 1e-8
        assert np.max(np.abs(grads[i] - O.gradients(sys_, ref))) < 1e-6
    ctx.close()


def test_batch_not_posdef_names_molecule(gpu_lib, water_model):
    from dftbplus_gb300 import binding, synth
    bad = synth.water_model(draw=3)
    mols = _water_set(3, 4)
    c, s = synth.water_cluster(32, 10.0, 1)
    mols.insert(1, (c, s))
    ctx = _ctx(bad)
    with pytest.raises(binding.DftbGpuError) as e:
        ctx.batch_set_geometries([m[0] for m in mols], [m[1] for m in mols])
    assert e.value.code == 3
    ctx.close()


def test_batch_state_errors(gpu_lib, water_model):
    from dftbplus_gb300 import binding
    ctx = _ctx(water_model)
    ctx.batch_atom_off = np.array([0, 3])
    with pytest.raises(binding.DftbGpuError) as e:
        ctx.batch_scc(binding.default_opts(kT=1e-3, scc_tol=1e-7))
    assert e.value.code == 7
    ctx.close()


def test_batch_mixed_spd_fractional(gpu_lib, tio2_model):
    """Mixed batched form (FP32, FP64 reference, perturbative updates) on Ti/O molecules at high kT."""
    from dftbplus_gb300 import binding
    rng = np.random.default_rng(8)
    mols = []
    while len(mols) < 6:
        nat = int(rng.integers(3, 8))
        pts = []
        while len(pts) < nat:
            p = rng.uniform(-4.0, 4.0, 3)
            if all(np.linalg.norm(p - q) > 3.3 for q in pts):
                pts.append(p)
        c = np.array(pts).T
        s = rng.integers(0, 2, nat)
        _, S = O.build_h0_s(O.System(tio2_model, c, s))
        if np.linalg.eigvalsh(S)[0] > 0.05:
            mols.append((c, s))
    ctx = _ctx(tio2_model)
    ctx.batch_set_geometries([m[0] for m in mols], [m[1] for m in mols])
    res = ctx.batch_scc(binding.default_opts(kT=5e-3, scc_tol=1e-7, precision=binding.PREC_MIXED,
                                             mixed_switch_tol=1e-2))
    grads = ctx.batch_gradients()
    for i, (c, s) in enumerate(mols):
        sys_ = O.System(tio2_model, c, s)
        ref = O.run_scc(sys_, kt=5e-3, scc_tol=1e-7)
        if not ref.converged:
            continue
        assert res["converged"][i]
        assert abs(res["energies"][i]["EMermin"] - ref.energies["EMermin"]) / len(s) < 1e-8
        assert np.max(np.abs(grads[i] - O.gradients(sys_, ref))) < 1e-6
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_largest_molecules_of_benchmark_set(gpu_lib, water_model, precision):
    """The largest molecules of the 4,096-molecule benchmark set (40-48 waters, 240-288 orbitals, the
    regime of long QL sweeps, large merges and slabs beyond shared memory), batched together with a
    few small ones: every molecule against the oracle run on it alone (FP64 at the single-system FP64
    tolerances, mixed at 1e-8 Ha/atom and 1e-6 Ha/Bohr)."""
    from dftbplus_gb300 import binding
    from bench import batch_sizes, batch_molecule
    ns = batch_sizes()
    big = [i for i, n in enumerate(ns) if n >= 40]
    pick = sorted(set([i for i in big if ns[i] == 48][:2] + big[:6] + [int(np.argmin(ns)), 7]))
    mols = [batch_molecule(i, ns[i]) for i in pick]
    assert max(len(m[1]) for m in mols) == 144 and min(len(m[1]) for m in mols) == 6
    ctx = _ctx(water_model)
    ctx.batch_set_geometries([m[0] for m in mols], [m[1] for m in mols])
    prec = binding.PREC_MIXED if precision == "mixed" else binding.PREC_FP64
    res = ctx.batch_scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, precision=prec))
    grads = ctx.batch_gradients()
    off = ctx.batch_atom_off
    for i, (c, s) in enumerate(mols):
        sys_ = O.System(water_model, c, s)
        ref = O.run_scc(sys_, kt=1e-3, scc_tol=1e-7)
        assert res["converged"][i] and ref.converged
        gref = O.gradients(sys_, ref)
        e = res["energies"][i]
        q = res["q_out"][off[i]:off[i + 1]]
        if precision == "fp64":
            assert res["n_iter"][i] == ref.n_iter, (pick[i], res["n_iter"][i], ref.n_iter)
            for k in ("EnonSCC", "Escc", "Erep", "Etotal", "EMermin", "TS", "Eband"):
                assert abs(e[k] - ref.energies[k]) < 1e-9, (pick[i], k, e[k], ref.energies[k])
            assert np.max(np.abs(q - ref.q_out_atom)) < 1e-8
            assert np.max(np.abs(grads[i] - gref)) < 1e-8, (pick[i], np.max(np.abs(grads[i] - gref)))
        else:
            assert abs(e["EMermin"] - ref.energies["EMermin"]) / len(s) < 1e-8
            assert np.max(np.abs(q - ref.q_out_atom)) < 1e-6
            assert np.max(np.abs(grads[i] - gref)) < 1e-6
    ctx.close()
