"""Geometry drivers with resident state: velocity Verlet molecular dynamics and FIRE relaxation over
a calculator (``binding.DftbGpu`` on the GPU).

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
