"""CPU checks of the geometry drivers (dftbplus_gb300/drivers.py): the velocity Verlet split form of
md/velocityverlet.F90 and the FIRE steps of geoopt/fire.F90, on analytic potentials and on the CPU
oracle standing in for the GPU calculator (same set_geometry / get_energy / get_gradients protocol,
with the previous step's charges as the next start)."""
import numpy as np
import pytest

from dftbplus_gb300 import drivers
from oracle import dftb_oracle as O


class _Harmonic:
    """E = k/2 |x - x0|^2 per atom (3 x N coordinates), gradients (N, 3) like DftbGpu."""

    def __init__(self, x0, k=0.3):
        self.x0, self.k = np.array(x0, dtype=np.float64), k

    def set_geometry(self, x):
        self.x = np.array(x, dtype=np.float64)

    def get_energy(self):
        return 0.5 * self.k * float(np.sum((self.x - self.x0) ** 2))

    def get_gradients(self):
        return (self.k * (self.x - self.x0)).T


class _OracleCalc:
    """The CPU oracle behind the calculator protocol of binding.DftbGpu (test infrastructure)."""

    def __init__(self, model, coords, species):
        from dftbplus_gb300 import binding
        self.model, self.species = model, np.asarray(species)
        self._q_init, self.iters = None, []
        self.opts = binding.SccOpts()           # the calculator's SCC settings, as DftbGpu.opts
        self.opts.min_iter, self.opts.max_iter, self.opts.scc_tol = 1, 100, 1e-9
        self.set_geometry(coords)

    def set_geometry(self, x):
        self.sys = O.System(self.model, np.array(x, dtype=np.float64), self.species)
        self._res, self._grad = None, None

    def _ensure(self):
        if self._res is None:
            r = O.run_scc(self.sys, kt=1e-3, scc_tol=self.opts.scc_tol, max_iter=self.opts.max_iter,
                          q_init_atom=self._q_init)
            self.iters.append(r.n_iter)
            self._ref = r
            self._res = {"q_out": r.q_out_atom, "energies": r.energies}

    def get_energy(self):
        self._ensure()
        return self._res["energies"]["EMermin"]

    def get_gradients(self):
        self._ensure()
        if self._grad is None:
            self._grad = O.gradients(self.sys, self._ref).T.copy()
        return self._grad


def test_velocity_verlet_split_form():
    """First call returns v(0) and r(dt) = r0 + (v0 + a0 dt/2) dt; later calls v(t) = v(t-dt/2) + a dt/2."""
    r0, v0, a0, a1, dt = np.array([[1.0]]), np.array([[0.5]]), np.array([[-2.0]]), np.array([[-1.0]]), 0.1
    vv = drivers.VelocityVerlet(dt, r0, v0)
    r1, v_now = vv.next(a0)
    assert v_now[0, 0] == 0.5 and np.isclose(r1[0, 0], 1.0 + (0.5 - 1.0 * dt) * dt)
    r2, v1 = vv.next(a1)
    assert np.isclose(v1[0, 0], 0.5 - 0.1 - 0.05)
    assert np.isclose(r2[0, 0], r1[0, 0] + (v1[0, 0] - 0.05) * dt)


def test_md_harmonic_matches_analytic():
    x0 = np.zeros((3, 1))
    calc = _Harmonic(x0, k=1.0 * drivers.AMU_AU)        # omega = 1 for a 1 amu particle
    start = np.array([[1.0], [0.0], [0.0]])
    calc.set_geometry(start)
    dt, n = 0.01, 628                                    # about one period
    xs = []
    drivers.run_md(calc, start, np.array([1.0]), dt, n, reuse_charges=False,
                   callback=lambda i, x, v, ep, ek: xs.append(x[0, 0]))
    t = dt * np.arange(n + 1)
    assert np.max(np.abs(np.array(xs) - np.cos(t))) < 1e-3


def test_md_oracle_energy_conservation_and_charge_reuse(water_model):
    """(H2O)2 relaxed with FIRE, then NVE from it with the oracle: the total energy is conserved to
    second order in the time step (3e-7 Ha over 200 a.u. at dt = 10, about 4x less at dt = 5), and
    starting each SCC from the previous charges takes fewer SCC iterations than starting from
    neutral atoms, with the same trajectory."""
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(2, 4.0, 3)
    calc = _OracleCalc(water_model, c, s)
    x, _, _, conv = drivers.relax(calc, c, tol=1e-5, max_steps=2000, dt_max=20.0)
    assert conv
    masses = np.array([water_model.species[q].mass for q in s])
    v0 = np.random.default_rng(0).normal(0.0, 2e-4, c.shape)
    spread, iters, traj = {}, {}, {}
    for dt, n, reuse in ((10.0, 20, True), (10.0, 20, False), (5.0, 40, True)):
        calc = _OracleCalc(water_model, x, s)
        xe, _, en = drivers.run_md(calc, x, masses, dt, n, velocities=v0, reuse_charges=reuse)
        tot = np.array([a + b for a, b in en])
        spread[(dt, reuse)], iters[(dt, reuse)], traj[(dt, reuse)] = np.ptp(tot), sum(calc.iters[1:]), xe
    assert spread[(10.0, True)] < 3e-7
    assert spread[(10.0, True)] / spread[(5.0, True)] > 3.0
    assert iters[(10.0, True)] < iters[(10.0, False)]
    assert np.allclose(traj[(10.0, True)], traj[(10.0, False)], atol=1e-8)


def test_fire_quadratic_and_oracle_relaxation(water_model):
    # anisotropic quadratic: converges to the minimum
    x0 = np.array([[0.5, -1.0], [2.0, 0.0], [0.0, 1.0]])
    calc = _Harmonic(x0, k=0.7)
    x, e, steps, conv = drivers.relax(calc, np.zeros((3, 2)), tol=1e-6, max_steps=2000, reuse_charges=False)
    assert conv and np.allclose(x, x0, atol=1e-5)
    # a distorted water molecule relaxes with the oracle's forces
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(1, 1.0, 5)
    c = c.copy()
    c[:, 1] += np.array([0.15, -0.1, 0.05])
    calc = _OracleCalc(water_model, c, s)
    e0 = calc.get_energy()
    x, e, steps, conv = drivers.relax(calc, c, tol=1e-4, max_steps=600, dt_max=20.0)
    assert conv and e < e0
    assert np.max(np.abs(calc.get_gradients())) < 1e-4


def test_fire_reference_steps():
    """FIRE bookkeeping as fire.F90: dt grows by f_inc after nMin uphill-free steps, an uphill step
    zeroes the velocity, cuts dt by f_dec and resets a."""
    f = drivers.Fire(1, tol=1e-12, dt_max=1.0)
    assert f.dt == pytest.approx(0.1) and f.a == 0.1
    for _ in range(7):
        f.step(np.array([1.0]))                          # steady downhill: velocity along -grad
    assert f.dt > 0.1 and f.a < 0.1
    f.step(np.array([-1.0]))                             # the velocity now points uphill
    assert f.a == 0.1 and f.reset_step == f.iter - 1


def test_ext_lagrangian_phases_and_fixed_point():
    """md/extlagrangian.F90: after turnOn the integrator wants K + 1 converged outputs, then predicts;
    a constant output is a fixed point (the dissipation coefficients sum to zero)."""
    for k in (5, 6, 7):
        xl = drivers.ExtLagrangian(3, n_kappa=k)
        assert abs(sum(xl.coeffs)) < 1e-12
        q = np.array([6.1, 0.95, 0.95])
        assert np.array_equal(xl.next_input(q), q) and xl.needs_converged()      # off
        xl.turn_on(0)
        for _ in range(k + 1):
            assert xl.needs_converged()
            assert np.array_equal(xl.next_input(q), q)
        assert not xl.needs_converged()
        for _ in range(5):
            assert np.allclose(xl.next_input(q), q, atol=1e-13)
    with pytest.raises(ValueError):
        drivers.ExtLagrangian(3, n_kappa=4)


def test_xlbomd_oracle(water_model):
    """XLBOMD on relaxed (H2O)2 with the oracle: SCC cycles started from the propagated charges and
    stopped at 1e-5 e take far fewer iterations than converged cycles started from the previous
    charges, with the same energy conservation and a trajectory within 1e-5 Bohr."""
    from dftbplus_gb300 import synth
    c, s = synth.water_cluster(2, 4.0, 3)
    calc = _OracleCalc(water_model, c, s)
    x, _, _, _ = drivers.relax(calc, c, tol=1e-5, max_steps=2000, dt_max=20.0)
    masses = np.array([water_model.species[q].mass for q in s])
    v0 = np.random.default_rng(0).normal(0.0, 2e-4, c.shape)
    ref = _OracleCalc(water_model, x, s)
    x_ref, _, en_ref = drivers.run_md(ref, x, masses, 10.0, 30, velocities=v0)
    xl = _OracleCalc(water_model, x, s)
    x_xl, _, en_xl = drivers.run_xlbomd(xl, x, masses, 10.0, 30, velocities=v0, scc_tol=1e-5)
    assert sum(xl.iters) < 0.7 * sum(ref.iters)
    spread = lambda en: np.ptp([a + b for a, b in en])
    assert spread(en_xl) < 1.2 * spread(en_ref) + 1e-9
    assert np.max(np.abs(x_xl - x_ref)) < 1e-5
    assert xl.opts.scc_tol == 1e-9 and xl.opts.max_iter == 100        # settings restored
