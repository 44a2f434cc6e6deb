"""Generate end-to-end golden fixtures of the benchmark workloads with the CPU oracle.

    python tests/golden/make_scc_golden.py [h2o1024] [h2o128] ...

For each named water workload of ``bench.CONFIGS`` (seeded geometry, the synthetic SK tables of
``synth.water_model``) the oracle runs the full evaluation the GPU path is measured on: SCC from the
neutral reference charges to 1e-7 e (kT = 1e-3 Ha, Broyden 0.2), energies and energy gradients.
The results are stored compressed as ``scc_<workload>.npz`` next to this script: the eight energy
terms, the Fermi level, the eigenvalues, the Mulliken populations per atom, the gradient (3 x N),
the SCC iteration count and the geometry checksum, so that the GPU parity tests can hold the
(H2O)1024 benchmark configuration to the oracle without running it (minutes of CPU time) on the GPU
host. The oracle is test infrastructure; nothing in the product imports this script.
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

ENERGY_KEYS = ("EnonSCC", "Escc", "Erep", "Eband", "TS", "E0", "Etotal", "EMermin")


def geometry_digest(coords, species):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(coords, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(species, dtype=np.int32).tobytes())
    return h.hexdigest()


def generate(name):
    from bench import CONFIGS, KT, SCC_TOL, MIX
    from dftbplus_gb300 import synth
    from oracle import dftb_oracle as O
    n_mol, radius, seed = CONFIGS[name]
    coords, species = synth.water_cluster(n_mol, radius, seed)
    model = synth.water_model()
    sys_ = O.System(model, coords, species)
    t0 = time.perf_counter()
    res = O.run_scc(sys_, kt=KT, scc_tol=SCC_TOL, mixer=O.BroydenMixer(max_iter=100, alpha=MIX))
    t_scc = time.perf_counter() - t0
    grad = O.gradients(sys_, res, kt=KT)
    t_all = time.perf_counter() - t0
    out = os.path.join(HERE, f"scc_{name}.npz")
    np.savez_compressed(
        out, energies=np.array([res.energies[k] for k in ENERGY_KEYS]), energy_keys=np.array(ENERGY_KEYS),
        ef=np.array(res.ef), eig=res.eig, q_out_atom=res.q_out_atom, grad=grad,
        n_iter=np.array(res.n_iter), converged=np.array(res.converged),
        errors=np.array([h["err"] for h in res.history]),
        geometry_sha256=np.array(geometry_digest(coords, species)),
        settings=np.array([KT, SCC_TOL, MIX]))
    print(f"{name}: {sys_.n_atom} atoms, {sys_.n_orb} orbitals, {res.n_iter} SCC iterations, "
          f"EMermin {res.energies['EMermin']:.12f} Ha, SCC {t_scc:.0f} s, total {t_all:.0f} s -> {out}")


if __name__ == "__main__":
    for nm in (sys.argv[1:] or ["h2o128", "h2o1024"]):
        generate(nm)
