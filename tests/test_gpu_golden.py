"""The benchmark configurations against committed oracle fixtures (tests/golden/scc_<workload>.npz,
made by tests/golden/make_scc_golden.py): (H2O)1024, the workload the benchmark line is measured on
(3,072 atoms, 6,144 orbitals), and (H2O)128 (768 orbitals), each through the C-ABI in the plain FP64
form (held to 1e-9 Ha in every energy term, 1e-8 e, 1e-8 Ha/Bohr and the same SCC iteration count)
and in the mixed form (held to 1e-8 Ha/atom, 1e-6 e and 1e-6 Ha/Bohr, inside the form's targets of
1e-6 Ha/atom and 1e-5 Ha/Bohr)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture(name):
    from golden.make_scc_golden import geometry_digest
    from bench import CONFIGS
    from dftbplus_gb300 import synth
    z = dict(np.load(os.path.join(HERE, "golden", f"scc_{name}.npz")))
    n_mol, radius, seed = CONFIGS[name]
    c, s = synth.water_cluster(n_mol, radius, seed)
    assert str(z["geometry_sha256"]) == geometry_digest(c, s), "workload generator changed"
    return z, c, s


@pytest.mark.parametrize("name", ["h2o128", "h2o1024"])
@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_benchmark_workload_matches_oracle_fixture(gpu_lib, water_model, name, form):
    from dftbplus_gb300 import binding
    z, c, s = _fixture(name)
    keys = [str(k) for k in z["energy_keys"]]
    ctx = binding.Context(0)
    ctx.set_model(water_model)
    ctx.set_geometry(c, s)
    prec = binding.PREC_MIXED if form == "mixed" else binding.PREC_FP64
    res = ctx.scc(binding.default_opts(kT=1e-3, scc_tol=1e-7, precision=prec))
    g = ctx.gradients()
    ctx.close()
    assert res["converged"]
    natom = len(s)
    dq = np.max(np.abs(res["q_out"] - z["q_out_atom"]))
    dg = np.max(np.abs(g - z["grad"]))
    if form == "fp64":
        assert res["n_iter"] == int(z["n_iter"])
        for k, ref in zip(keys, z["energies"]):
            assert abs(res["energies"][k] - ref) < 1e-9, (k, res["energies"][k], ref)
        assert abs(res["ef"] - float(z["ef"])) < 1e-9
        assert np.max(np.abs(res["eig"] - z["eig"])) < 1e-9
        assert dq < 1e-8, dq
        assert dg < 1e-8, dg
    else:
        i = keys.index("EMermin")
        assert abs(res["energies"]["EMermin"] - z["energies"][i]) / natom < 1e-8
        assert dq < 1e-6, dq
        assert dg < 1e-6, dg
