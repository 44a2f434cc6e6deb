"""Geometry drivers over the GPU calculator: velocity Verlet MD and XLBOMD on (H2O)2 with
binding.DftbGpu (plain FP64 path through the C-ABI) against the same drivers over the CPU oracle."""
import numpy as np
import pytest

from dftbplus_gb300 import drivers

pytestmark = pytest.mark.gpu


def _pair(water_model, gpu_lib):
    from dftbplus_gb300 import binding, synth
    from test_drivers import _OracleCalc
    c, s = synth.water_cluster(2, 4.0, 3)
    gpu = binding.DftbGpu(water_model, c, s, kT=1e-3, scc_tol=1e-9)
    ora = _OracleCalc(water_model, c, s)
    masses = np.array([water_model.species[q].mass for q in s])
    v0 = np.random.default_rng(0).normal(0.0, 2e-4, c.shape)
    return c, gpu, ora, masses, v0


def test_md_gpu_matches_oracle(water_model, gpu_lib):
    """Six velocity Verlet steps (dt = 10 a.u.), each SCC started from the previous step's charges:
    positions, velocities and energies follow the oracle's trajectory."""
    c, gpu, ora, masses, v0 = _pair(water_model, gpu_lib)
    x_g, v_g, en_g = drivers.run_md(gpu, c, masses, 10.0, 6, velocities=v0)
    x_o, v_o, en_o = drivers.run_md(ora, c, masses, 10.0, 6, velocities=v0)
    assert np.max(np.abs(x_g - x_o)) < 1e-9
    assert np.max(np.abs(v_g - v_o)) < 1e-11
    assert np.max(np.abs(np.array(en_g) - np.array(en_o))) < 1e-9


def test_xlbomd_gpu_matches_oracle(water_model, gpu_lib):
    """XLBOMD with the default iteration bound (200, above the engine's 150-iteration limit: the
    driver clamps it) runs past the filled history on the GPU and stays on the oracle's trajectory."""
    c, gpu, ora, masses, v0 = _pair(water_model, gpu_lib)
    x_g, _, en_g = drivers.run_xlbomd(gpu, c, masses, 10.0, 10, velocities=v0, scc_tol=1e-5)
    x_o, _, en_o = drivers.run_xlbomd(ora, c, masses, 10.0, 10, velocities=v0, scc_tol=1e-5)
    assert np.max(np.abs(x_g - x_o)) < 1e-7
    assert np.max(np.abs(np.array(en_g) - np.array(en_o))) < 1e-7
    assert gpu.opts.max_iter == 100 and gpu.opts.scc_tol == 1e-9      # settings restored
