"""Geometry drivers with resident state: velocity Verlet molecular dynamics (also with
extended-Lagrangian charge propagation, XLBOMD) and FIRE relaxation over a calculator
(``binding.DftbGpu`` on the GPU).

Between geometry steps the SCC cycle starts from the previous step's converged charges, as the
reference carries ``qInput`` over from one geometry to the next, and the device keeps its model,
buffers and pair arrays, so a step pays only for the geometry-dependent work.

* ``VelocityVerlet`` follows ``md/velocityverlet.F90:280-336`` (``VelocityVerlet_next``): the step
  is cut as v(t) = v(t - dt/2) + a(t) dt/2, v(t + dt/2) = v(t) + a(t) dt/2, r(t + dt) = r(t) +
  v(t + dt/2) dt, so the returned velocity lags the returned positions by one step; no thermostat
  (NVE).
* ``Fire`` follows ``geoopt/fire.F90`` (``TFire_init_old``, ``step``, ``next``,
  ``fireModifyVelocity``): unit masses, the defaults of the FIRE paper that the reference uses (nMin
  5, a_start 0.1, f_inc 1.1, f_dec 0.5, f_alpha 0.99), dt starting at dt_max / 10, converged when the
  largest gradient component drops below the tolerance.

Units are atomic (Bohr, Hartree, electron masses, time in atomic units); masses are given in amu
and converted with ``amu__au = 1 / 0.00054857990945`` (``common/constants.F90:49-52``).
"""
from __future__ import annotations

from typing import Callable, List, Optional

import numpy as np

AMU_AU = 1.0 / 0.00054857990945     # electron masses per amu (common/constants.F90:49-52)
FS_AU = 1.0 / 0.02418884326505      # atomic time units per fs (common/constants.F90:55-58)


class VelocityVerlet:
    """Velocity Verlet in the reference's split form (positions and half-step velocities stored)."""

    def __init__(self, dt: float, positions: np.ndarray, velocities: Optional[np.ndarray] = None):
        self.dt = float(dt)
        self.positions = np.array(positions, dtype=np.float64)
        self.velocities = (np.zeros_like(self.positions) if velocities is None
                           else np.array(velocities, dtype=np.float64))
        self.v_half = False

    def next(self, accel: np.ndarray):
        """(new positions, velocity at the current positions) from the accelerations there."""
        if self.v_half:
            v_now = self.velocities + 0.5 * accel * self.dt
        else:
            v_now = self.velocities.copy()
            self.v_half = True
        self.velocities = v_now + 0.5 * accel * self.dt
        self.positions = self.positions + self.velocities * self.dt
        return self.positions.copy(), v_now


def _start_from_previous(calc) -> None:
    """Next SCC starts from the converged atomic populations of the last one (if the calculator
    supports it and has converged once)."""
    res = getattr(calc, "_res", None)
    if res is not None and hasattr(calc, "_q_init"):
        calc._q_init = np.array(res["q_out"], dtype=np.float64)


def run_md(calc, coords: np.ndarray, masses_amu: np.ndarray, dt: float, n_steps: int,
           velocities: Optional[np.ndarray] = None, reuse_charges: bool = True,
           callback: Optional[Callable[[int, np.ndarray, np.ndarray, float, float], None]] = None):
    """NVE molecular dynamics: ``n_steps`` velocity Verlet steps of ``dt`` (atomic time units) from
    ``coords`` (3 x N, Bohr). Returns (coords, velocities, energies) where energies[i] = (potential
    EMermin, kinetic) at step i, both in Hartree. ``callback(step, coords, velocity, epot, ekin)``
    sees every step."""
    m = np.asarray(masses_amu, dtype=np.float64) * AMU_AU
    x = np.array(coords, dtype=np.float64)
    vv = VelocityVerlet(dt, x, velocities)
    energies: List[tuple] = []
    v = vv.velocities.copy()
    for step in range(n_steps + 1):
        if step > 0 and reuse_charges:
            _start_from_previous(calc)
        calc.set_geometry(x)
        epot = calc.get_energy()
        grad = np.asarray(calc.get_gradients(), dtype=np.float64).T     # (3, N)
        accel = -grad / m[None, :]
        x_new, v = vv.next(accel)
        ekin = 0.5 * float(np.sum(m[None, :] * v * v))
        energies.append((epot, ekin))
        if callback is not None:
            callback(step, x, v, epot, ekin)
        x = x_new
    return x, v, energies


# Dissipation coefficients of the extended-Lagrangian integrator for K = 5, 6, 7 auxiliary
# generations (md/extlagrangian.F90:80-96; Niklasson et al., J. Chem. Phys. 130, 214109 (2009)),
# kept identical because they define the integrator: (coefficients c_0..c_K, alpha, kappa). The
# reference declares the K = 7 alpha without a kind suffix, so Fortran stores the single-precision
# value of 1.6e-3; np.float32 reproduces that value bit for bit.
_XL_COEFFS = {
    5: ([-6.0, 14.0, -8.0, -3.0, 4.0, -1.0], 18e-3, 1.82),
    6: ([-14.0, 36.0, -27.0, -2.0, 12.0, -6.0, 1.0], 5.5e-3, 1.84),
    7: ([-36.0, 99.0, -88.0, 11.0, 32.0, -25.0, 8.0, -1.0], float(np.float32(1.6e-3)), 1.86),
}


class ExtLagrangian:
    """Extended-Lagrangian propagation of the SCC input charges (md/extlagrangian.F90): off (the next
    input is the last output), filling the history with K + 1 converged outputs, then for each step
    n(t + dt) = 2 n(t) - n(t - dt) + kappa s (q(t) - n(t)) + alpha sum_i c_i n(t - i dt), where q(t)
    is the SCC output at t and the n are the auxiliary charges kept in a ring of K + 1."""

    OFF, FILLING, INTERPOLATING, ON = 1, 2, 3, 4

    def __init__(self, n_elems: int, n_kappa: int = 5, scale: float = 1.0):
        if n_kappa not in _XL_COEFFS:
            raise ValueError("the number of integration steps must be 5, 6 or 7")
        coeffs, self.alpha, self.kappa = _XL_COEFFS[n_kappa]
        self.coeffs = np.array(coeffs)
        self.k = n_kappa
        self.scale = scale
        self.aux = np.zeros((n_elems, n_kappa + 1))
        self.ind = 0                  # 1-based slot of the newest vector (0 before the first)
        self.phase = self.OFF
        self.i_step, self.n_steps, self.n_transient = 1, 0, 0

    def _mod(self, ind: int) -> int:
        return (ind - 1) % (self.k + 1) + 1

    def turn_on(self, n_transient: int = 0) -> None:
        self.phase = self.FILLING
        self.i_step = 1
        self.n_steps = self.k + 1
        self.n_transient = n_transient

    def needs_converged(self) -> bool:
        return self.phase in (self.OFF, self.FILLING, self.INTERPOLATING)

    def next_input(self, q_out: np.ndarray) -> np.ndarray:
        q_out = np.asarray(q_out, dtype=np.float64)
        if self.phase == self.OFF:
            nxt = q_out.copy()
        elif self.phase == self.FILLING:
            self.ind = self._mod(self.ind + 1)
            self.aux[:, self.ind - 1] = q_out
            nxt = q_out.copy()
        else:
            i0 = self.ind
            if self.phase == self.INTERPOLATING:
                cc = self.i_step / (self.n_steps + 1)
                self.aux[:, i0 - 1] = cc * self.aux[:, i0 - 1] + (1.0 - cc) * q_out
            i1 = self._mod(i0 - 1)
            nxt = 2.0 * self.aux[:, i0 - 1] - self.aux[:, i1 - 1]
            nxt = nxt + self.kappa * self.scale * (q_out - self.aux[:, i0 - 1])
            for i in range(self.k + 1):
                nxt = nxt + self.alpha * self.coeffs[i] * self.aux[:, self._mod(i0 - i) - 1]
            self.ind = self._mod(self.ind + 1)
            self.aux[:, self.ind - 1] = nxt
        self._advance()
        return nxt

    def _advance(self) -> None:
        if self.phase in (self.OFF, self.ON):
            return
        self.i_step += 1
        if self.phase == self.FILLING and self.i_step > self.n_steps:
            self.phase, self.i_step, self.n_steps = self.INTERPOLATING, 1, self.n_transient
        if self.phase == self.INTERPOLATING and self.i_step > self.n_steps:
            self.phase = self.ON


def run_xlbomd(calc, coords: np.ndarray, masses_amu: np.ndarray, dt: float, n_steps: int,
               velocities: Optional[np.ndarray] = None, n_kappa: int = 5, pre_steps: int = 0,
               min_scc_iter: int = 1, max_scc_iter: int = 200, scc_tol: float = 1e-5):
    """Velocity Verlet MD whose SCC input charges are propagated by the extended Lagrangian
    (md/xlbomd.F90, the ``Xlbomd`` block): fully converged SCC cycles until K + 1 outputs fill the
    history (started after ``pre_steps``), then each step starts from the propagated charges and
    stops at ``scc_tol`` within ``min_scc_iter``..``max_scc_iter`` iterations. ``calc.opts`` carries
    the calculator's own SCC settings for the converged steps. A calculator that bounds its SCC
    iterations (``calc.MAX_SCC_ITER``, the GPU engine's 150) gets ``max_scc_iter`` clamped to that
    bound. Returns what ``run_md`` returns."""
    max_scc_iter = min(int(max_scc_iter), int(getattr(calc, "MAX_SCC_ITER", max_scc_iter)))
    if max_scc_iter < min_scc_iter:
        raise ValueError(f"max_scc_iter {max_scc_iter} < min_scc_iter {min_scc_iter}")
    m = np.asarray(masses_amu, dtype=np.float64) * AMU_AU
    x = np.array(coords, dtype=np.float64)
    vv = VelocityVerlet(dt, x, velocities)
    xl = None
    start_xl = pre_steps + 1          # nPreSteps + nFullSccSteps - nKappa, nFullSccSteps = K + 1
    full = (calc.opts.min_iter, calc.opts.max_iter, calc.opts.scc_tol)
    energies: List[tuple] = []
    v = vv.velocities.copy()
    try:
        for step in range(n_steps + 1):
            if xl is not None and not xl.needs_converged():
                calc.opts.min_iter, calc.opts.max_iter, calc.opts.scc_tol = min_scc_iter, max_scc_iter, scc_tol
            else:
                calc.opts.min_iter, calc.opts.max_iter, calc.opts.scc_tol = full
            calc.set_geometry(x)
            epot = calc.get_energy()
            grad = np.asarray(calc.get_gradients(), dtype=np.float64).T
            q_out = np.array(calc._res["q_out"], dtype=np.float64)
            if xl is None:
                xl = ExtLagrangian(len(q_out), n_kappa)
            if step + 1 == start_xl:
                xl.turn_on(0)
            calc._q_init = xl.next_input(q_out)
            x_new, v = vv.next(-grad / m[None, :])
            energies.append((epot, 0.5 * float(np.sum(m[None, :] * v * v))))
            x = x_new
    finally:
        calc.opts.min_iter, calc.opts.max_iter, calc.opts.scc_tol = full
    return x, v, energies


class Fire:
    """FIRE minimiser on a flat coordinate vector (unit masses, the reference's defaults)."""

    def __init__(self, n: int, tol: float, dt_max: float = 1.0, n_min: int = 5, a_start: float = 0.1,
                 f_inc: float = 1.1, f_dec: float = 0.5, f_alpha: float = 0.99):
        self.tol = float(tol)
        self.n_min, self.a_start, self.f_inc, self.f_dec, self.f_alpha = n_min, a_start, f_inc, f_dec, f_alpha
        self.dt_max = float(dt_max)
        self.dt = 0.1 * self.dt_max
        self.a = a_start
        self.iter = 0
        self.reset_step = 0
        self.velocity = np.zeros(n)

    def _modify_velocity(self, grad: np.ndarray) -> None:
        p = -float(np.dot(self.velocity, grad))
        ng = float(np.sqrt(np.sum(grad * grad)))
        nv = float(np.sqrt(np.sum(self.velocity * self.velocity)))
        mix = grad * (nv / ng) if ng > 0.0 else np.zeros_like(grad)
        self.velocity = (1.0 - self.a) * self.velocity - self.a * mix
        if p < 0.0:
            self.velocity[:] = 0.0
            self.reset_step = self.iter
            self.dt *= self.f_dec
            self.a = self.a_start
        elif self.iter - self.reset_step > self.n_min:
            self.dt = min(self.dt * self.f_inc, self.dt_max)
            self.a *= self.f_alpha

    def step(self, grad: np.ndarray) -> tuple:
        """(displacement, converged) for the gradient at the current point."""
        grad = np.asarray(grad, dtype=np.float64)
        if float(np.max(np.abs(grad))) < self.tol:
            return np.zeros_like(grad), True
        self._modify_velocity(grad)
        self.velocity = self.velocity - self.dt * grad
        self.iter += 1
        return self.velocity * self.dt, False


def relax(calc, coords: np.ndarray, tol: float = 1e-4, max_steps: int = 500, dt_max: float = 1.0,
          reuse_charges: bool = True):
    """FIRE relaxation until max |dE/dR| < ``tol`` (Ha/Bohr). Returns (coords, energy, steps,
    converged)."""
    x = np.array(coords, dtype=np.float64)
    opt = Fire(x.size, tol, dt_max=dt_max)
    energy = None
    for it in range(max_steps + 1):
        if it > 0 and reuse_charges:
            _start_from_previous(calc)
        calc.set_geometry(x)
        energy = calc.get_energy()
        grad = np.asarray(calc.get_gradients(), dtype=np.float64).T.reshape(-1)   # (3, N) flattened
        dx, conv = opt.step(grad)
        if conv:
            return x, energy, it, True
        x = x + dx.reshape(x.shape)
    return x, energy, max_steps, False
