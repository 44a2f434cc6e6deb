"""Slater-Koster file (.skf) reader/writer and per-species-pair table assembly.

This is host-side input handling, identical in meaning to the reference's SKF reader so that the
GPU engine receives exactly the tables DFTB+ would build:

* ``read_skf`` follows ``type/oldskdata.F90:83-202`` (``TOldSKData_readFromFile``): grid spacing and
  point count on line 1 (``nGrid - 1`` rows follow, row ``j`` belongs to ``r = j * dist``), the
  homonuclear line ``Ed Ep Es SPE Ud Up Us fd fp fs``, the mass/polynomial line, then 10 H and 10 S
  columns in the order ``dd0 dd1 dd2 pd0 pd1 pp0 pp1 sd0 sp0 ss0`` (slots 8,9,10,13,14,15,16,18,19,20
  of the 20-slot spdf layout, ``oldskdata.F90:77``), and the ``Spline`` repulsive block
  (``oldskdata.F90:206-280``).
* ``full_table`` follows ``dftbplus/parser.F90:4061-4130`` (``getFullTable``): one column per
  (shell on species 1, shell on species 2, m <= min(l1, l2)); for ``l1 <= l2`` the column comes from
  the A-B file, else from the B-A file, through the ``skMap(m, lMax, lMin)`` slot table.
"""
from __future__ import annotations

import dataclasses
import io
from typing import Dict, List, Sequence, Tuple

import numpy as np

from .fortran_io import ListDirected

# Slot (1-based, 20-slot spdf layout) of the integral (m, lMax, lMin); 0 = unused.
# Same table as parser.F90:4088-4094 (reshaped column-major over (m, lMax, lMin)).
_SLOT = {}
for (lmin, lmax, ms) in [
    (0, 0, [20]), (0, 1, [19]), (0, 2, [18]), (0, 3, [17]),
    (1, 1, [15, 16]), (1, 2, [13, 14]), (1, 3, [11, 12]),
    (2, 2, [8, 9, 10]), (2, 3, [5, 6, 7]),
    (3, 3, [1, 2, 3, 4]),
]:
    for m, slot in enumerate(ms):
        _SLOT[(m, lmax, lmin)] = slot

# Slots filled by the 10-column (s, p, d) file format, oldskdata.F90:77.
OLD_SLOTS = [8, 9, 10, 13, 14, 15, 16, 18, 19, 20]


@dataclasses.dataclass
class SplineRepulsive:
    """Spline pair repulsive as read from the ``Spline`` block of an SKF file.

    Evaluation follows ``dftb/repulsive/splinerep.F90:136-266``: exponential head below
    ``x_start[0]``, cubic segments, a 5th-order last segment, zero at and beyond ``cutoff``.
    """
    cutoff: float
    exp_coeffs: np.ndarray          # (3,)
    x_start: np.ndarray             # (nSpline,)
    sp_coeffs: np.ndarray           # (nSpline-1, 4)
    last_coeffs: np.ndarray         # (6,)

    def pack(self) -> np.ndarray:
        """Flat layout used across the C-ABI: [cutoff, a1, a2, a3, x_start..., cubic(4 per seg)..., last(6)]."""
        return np.concatenate([[self.cutoff], self.exp_coeffs, self.x_start,
                               self.sp_coeffs.reshape(-1), self.last_coeffs]).astype(np.float64)

    @classmethod
    def unpack(cls, flat: np.ndarray, n_spline: int) -> "SplineRepulsive":
        """Inverse of ``pack`` for a spline of ``n_spline`` segments."""
        f = np.asarray(flat, dtype=np.float64)
        x0 = 4
        c0 = x0 + n_spline
        l0 = c0 + 4 * (n_spline - 1)
        return cls(cutoff=float(f[0]), exp_coeffs=f[1:4].copy(), x_start=f[x0:c0].copy(),
                   sp_coeffs=f[c0:l0].reshape(n_spline - 1, 4).copy(), last_coeffs=f[l0:l0 + 6].copy())


@dataclasses.dataclass
class SkfData:
    dist: float
    ham: np.ndarray                 # (nRows, 20) in the spdf slot layout (slot k at column k-1)
    over: np.ndarray                # (nRows, 20)
    onsite: np.ndarray | None       # (3,) s, p, d (homonuclear only)
    hubbu: np.ndarray | None        # (3,) s, p, d
    occ: np.ndarray | None          # (3,) s, p, d
    mass: float | None
    repulsive: SplineRepulsive | None


def _fmt(vals: Sequence[float]) -> str:
    return " ".join(f"{v:.17e}" for v in vals)


def write_skf(path_or_buf, dist: float, ham10: np.ndarray, over10: np.ndarray, *,
              homo: Tuple[np.ndarray, np.ndarray, np.ndarray, float] | None,
              repulsive: SplineRepulsive) -> None:
    """Write a 10-column (s, p, d) SKF file.

    ``ham10``/``over10`` are (nRows, 10) in file column order dd0 dd1 dd2 pd0 pd1 pp0 pp1 sd0 sp0 ss0.
    ``homo`` = (onsite[s,p,d], U[s,p,d], occ[s,p,d], mass) for homonuclear files.
    """
    n_rows = ham10.shape[0]
    out = io.StringIO()
    out.write(f"{dist:.17e} {n_rows + 1}\n")
    if homo is not None:
        ons, hub, occ, mass = homo
        # Ed Ep Es SPE Ud Up Us fd fp fs
        out.write(_fmt([ons[2], ons[1], ons[0], 0.0, hub[2], hub[1], hub[0], occ[2], occ[1], occ[0]]) + "\n")
        out.write(_fmt([mass] + [0.0] * 19) + "\n")
    else:
        out.write(_fmt([0.0] * 20) + "\n")
    for i in range(n_rows):
        out.write(_fmt(list(ham10[i]) + list(over10[i])) + "\n")
    rep = repulsive
    n_spl = len(rep.x_start)
    out.write("Spline\n")
    out.write(f"{n_spl} {rep.cutoff:.17e}\n")
    out.write(_fmt(rep.exp_coeffs) + "\n")
    x_end = list(rep.x_start[1:]) + [rep.cutoff]
    for j in range(n_spl - 1):
        out.write(_fmt([rep.x_start[j], x_end[j]] + list(rep.sp_coeffs[j])) + "\n")
    out.write(_fmt([rep.x_start[-1], x_end[-1]] + list(rep.last_coeffs)) + "\n")
    text = out.getvalue()
    if hasattr(path_or_buf, "write"):
        path_or_buf.write(text)
    else:
        with open(path_or_buf, "w") as fh:
            fh.write(text)


def _num(v, default: float = 0.0) -> float:
    return default if v is None else float(v)


def read_skf(path_or_text, homo: bool, read_repulsive: bool = True) -> SkfData:
    """Parse an SKF file (10-column or '@' extended 20-column format) with the reference's
    list-directed reads: dist and nGrid, the homonuclear line (nShell on-site energies from d (f) down
    to s, SPE, Hubbard U and occupations in the same order), the mass/polynomial record (20 values),
    nGrid - 1 rows of 2 x 10 (2 x 20) integrals, then the records after the line ``Spline``.
    ``mass`` is the file's value (amu)."""
    if isinstance(path_or_text, str) and "\n" in path_or_text:
        lines = path_or_text.splitlines()
    else:
        with open(path_or_text) as fh:
            lines = fh.read().splitlines()
    extended = bool(lines) and lines[0][:1] == "@"
    rd = ListDirected(lines, 1 if extended else 0)
    head = rd.read(2)
    dist = _num(head[0])
    n_rows = int(_num(head[1])) - 1
    onsite = hubbu = occ = None
    mass = None
    n_shell = 4 if extended else 3
    if homo:
        v = [_num(x) for x in rd.read(3 * n_shell + 1)]
        onsite = np.array(v[0:n_shell][::-1])
        hubbu = np.array(v[n_shell + 1:2 * n_shell + 1][::-1])
        occ = np.array(v[2 * n_shell + 1:3 * n_shell + 1][::-1])
        mass = _num(rd.read(20)[0])
    else:
        rd.read(20)
    ham = np.zeros((n_rows, 20))
    over = np.zeros((n_rows, 20))
    n_int = 20 if extended else 10
    for i in range(n_rows):
        v = [_num(x) for x in rd.read(2 * n_int)]
        if extended:
            ham[i, :] = v[:20]
            over[i, :] = v[20:40]
        else:
            for k, slot in enumerate(OLD_SLOTS):
                ham[i, slot - 1] = v[k]
                over[i, slot - 1] = v[10 + k]
    rep = None
    if read_repulsive:
        # the record must read "Spline" (trailing blanks allowed, as Fortran compares strings)
        pos = 0
        while pos < len(lines) and lines[pos].rstrip() != "Spline":
            pos += 1
        if pos >= len(lines):
            raise ValueError("No spline repulsive found in SKF data")
        rd = ListDirected(lines, pos + 1)
        t = rd.read(2)
        n_spl = int(_num(t[0]))
        exp_c = np.array([_num(x) for x in rd.read(3)])
        xs, xe, cub = [], [], []
        for _ in range(n_spl - 1):
            v = [_num(x) for x in rd.read(6)]
            xs.append(v[0]); xe.append(v[1]); cub.append(v[2:6])
        v = [_num(x) for x in rd.read(8)]
        xs.append(v[0]); xe.append(v[1])
        last = np.array(v[2:8])
        for j in range(1, n_spl):
            if abs(xe[j - 1] - xs[j]) > 1e-8:
                raise ValueError("Repulsive not continuous")
        rep = SplineRepulsive(cutoff=xe[-1], exp_coeffs=exp_c, x_start=np.array(xs),
                              sp_coeffs=np.array(cub).reshape(n_spl - 1, 4), last_coeffs=last)
    return SkfData(dist=dist, ham=ham, over=over, onsite=onsite, hubbu=hubbu, occ=occ, mass=mass,
                   repulsive=rep)


def n_integrals(shells1: Sequence[int], shells2: Sequence[int]) -> int:
    return sum(min(l1, l2) + 1 for l1 in shells1 for l2 in shells2)


def full_table(d12: SkfData, d21: SkfData, shells1: Sequence[int], shells2: Sequence[int]):
    """Assemble the (nRows, nInt) H and S tables of the ordered pair (species1, species2)."""
    cols_h, cols_s = [], []
    for l1 in shells1:
        for l2 in shells2:
            if l1 <= l2:
                src, lmin, lmax = d12, l1, l2
            else:
                src, lmin, lmax = d21, l2, l1
            for m in range(lmin + 1):
                slot = _SLOT[(m, lmax, lmin)]
                cols_h.append(src.ham[:, slot - 1])
                cols_s.append(src.over[:, slot - 1])
    return np.stack(cols_h, axis=1), np.stack(cols_s, axis=1)
