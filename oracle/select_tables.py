"""Search for the synthetic SK-table draw used by the water workloads (test infrastructure).

The BASELINE functional forms with the given parameter ranges often give an indefinite overlap
matrix, which the reference would reject (Cholesky failure). Draws are tried in order
k = 0, 1, 2, ... from ``default_rng([seed, k])`` and the first one is accepted whose overlap has
lambda_min >= 0.2 on the (H2O)32 and (H2O)128 workloads and whose (H2O)32 SCC HOMO-LUMO gap
exceeds 0.1 Ha (well above kT = 1e-3 Ha). The accepted index is recorded in
``dftbplus_gb300/synth.py`` (WATER_DRAW).

    python oracle/select_tables.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from dftbplus_gb300 import synth  # noqa: E402
from oracle import dftb_oracle as O  # noqa: E402


def accept(draw):
    model = synth.water_model(draw=draw)
    for n_mol, radius, seed in [(32, 10.0, 1), (128, 20.0, 128)]:
        c, s = synth.water_cluster(n_mol, radius, seed)
        _, S = O.build_h0_s(O.System(model, c, s))
        if np.linalg.eigvalsh(S)[0] < 0.2:
            return False
    c, s = synth.water_cluster(32, 10.0, 1)
    res = O.run_scc(O.System(model, c, s))
    nocc = int(round(model.n_electrons(s) / 2))
    return res.converged and res.eig[nocc] - res.eig[nocc - 1] > 0.1


if __name__ == "__main__":
    for k in range(100):
        if accept(k):
            print("accepted draw", k)
            break
        print("rejected draw", k)
