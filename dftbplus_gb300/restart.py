"""Charge restart files of the reference (``charges.dat`` / ``charges.bin``), read and written on the
host so that a run of this engine can start from charges DFTB+ wrote and the other way round.

Layout (``dftb/sccinit.F90``, ``writeQToFile`` :619-905 writes format 8, ``initQFromFile``
:185-615 reads formats 4 to 8):

* record 1: the format number;
* record 2: presence flags and sizes. Format 4: ``tBlock, tiBlock, tRho, nSpin, checksum(nSpin)``;
  5: ``tBlock, tiBlock, tRho, nAtom, nSpin, checksum``; 6: ``tBlock, tiBlock, tRho, multipolar,
  nAtom, nSpin, checksum``; 7 and 8: ``tBlock, tiBlock, tRho, kpointInfo, multipolar, nAtom, nSpin,
  checksum`` (format 4 has no atom count: it covers all atoms of the system);
* then per spin channel, per atom, one record with the atom's orbital populations (s; p as y, z, x;
  d ...). Multipoles, block populations, density matrices and k-point data follow when flagged.

This path is spin-unpolarised without block populations, density-matrix restart or multipoles, so
those trailing sections are neither written nor needed: like the reference when it is not asked for
them, the reader reads the populations and leaves the rest of the file alone. The checksum (the
total population per spin channel) must match the populations read to 1e-7 (``elecTolMax``,
``common/accuracy.F90:60``), and, when the electron count is given, the total to 1e-3 as the
reference requires.
"""
from __future__ import annotations

import struct
from typing import Optional, Sequence

import numpy as np

from .fortran_io import (ListDirected, fortran_int, fortran_logical, fortran_real, read_records,
                         write_records)

RESTART_FORMAT = 8
ELEC_TOL_MAX = 1e-7
_HEADER = {  # format -> fields of record 2 before the checksum (logicals, then the integer sizes)
    4: ["tBlock", "tiBlock", "tRho", "nSpin"],
    5: ["tBlock", "tiBlock", "tRho", "nAtom", "nSpin"],
    6: ["tBlock", "tiBlock", "tRho", "multipolar", "nAtom", "nSpin"],
    7: ["tBlock", "tiBlock", "tRho", "kpoint", "multipolar", "nAtom", "nSpin"],
    8: ["tBlock", "tiBlock", "tRho", "kpoint", "multipolar", "nAtom", "nSpin"],
}
_INT_FIELDS = {"nAtom", "nSpin"}


def _check(q_atoms, checksum, n_el):
    total = float(sum(float(np.sum(q)) for q in q_atoms))
    if abs(checksum - total) > ELEC_TOL_MAX:
        raise ValueError("charge restart file: internal checksum failure, probably a damaged file")
    if n_el is not None and abs(n_el - total) >= 1e-3:
        raise ValueError(f"charge restart file has a total charge {total:.6f} instead of {n_el:.6f}")


def read_charges(path: str, n_orb_per_atom: Sequence[int], n_el: Optional[float] = None,
                 binary: Optional[bool] = None) -> np.ndarray:
    """Orbital populations (concatenated in atom order, len = sum(n_orb_per_atom)) from a reference
    charge file; atoms beyond those in the file get zero populations, as in the reference. ``binary``
    defaults to the extension (.bin binary, anything else ASCII)."""
    if binary is None:
        binary = str(path).endswith(".bin")
    n_orb = [int(x) for x in n_orb_per_atom]
    n_atom = len(n_orb)
    if binary:
        with open(path, "rb") as fh:
            recs = read_records(fh.read())
        if not recs:
            raise ValueError("empty charge restart file")
        (fmt,) = struct.unpack("<i", recs[0][:4])
        if fmt not in _HEADER:
            raise ValueError(f"incompatible charge restart format {fmt}")
        fields, off, hdr = _HEADER[fmt], 0, {}
        for name in fields:
            (v,) = struct.unpack_from("<i", recs[1], off)
            hdr[name] = v if name in _INT_FIELDS else bool(v)
            off += 4
        n_spin = hdr["nSpin"]
        checksum = struct.unpack_from("<d", recs[1], off)
        rows = recs[2:]
    else:
        with open(path) as fh:
            lines = fh.read().splitlines()
        rd = ListDirected(lines)
        fmt = rd.read(1, conv=fortran_int)[0]
        if fmt not in _HEADER:
            raise ValueError(f"incompatible charge restart format {fmt}")
        fields = _HEADER[fmt]
        # one read of the flags, the sizes and as many checksums as the system has spin channels
        # (one here), as the reference reads checkSum(size(qq, dim=3))
        convs = [fortran_int if f in _INT_FIELDS else fortran_logical for f in fields] + [fortran_real]
        vals = rd.read_mixed(convs)
        hdr = dict(zip(fields, vals))
        n_spin = hdr["nSpin"]
        checksum = [0.0 if vals[-1] is None else vals[-1]]
        rows = None
    if n_spin != 1:
        raise ValueError("incorrect number of spins in the restart file (this path is spin-unpolarised)")
    n_file = hdr.get("nAtom", n_atom)
    if n_file > n_atom:
        raise ValueError("the charge restart file has more atoms than the system")
    q_atoms = []
    for a in range(n_file):
        if binary:
            qa = struct.unpack(f"<{n_orb[a]}d", rows[a][:8 * n_orb[a]])
        else:
            qa = [0.0 if v is None else v for v in rd.read(n_orb[a])]
        q_atoms.append(np.array(qa, dtype=np.float64))
    _check(q_atoms, checksum[0], n_el)
    q_atoms += [np.zeros(n_orb[a]) for a in range(n_file, n_atom)]
    return np.concatenate(q_atoms) if q_atoms else np.zeros(0)


def write_charges(path: str, q_orb: np.ndarray, n_orb_per_atom: Sequence[int],
                  binary: Optional[bool] = None) -> None:
    """Write orbital populations (concatenated in atom order) as a format-8 reference charge file
    (spin-unpolarised, no block populations, density matrix, k-point data or multipoles)."""
    if binary is None:
        binary = str(path).endswith(".bin")
    n_orb = [int(x) for x in n_orb_per_atom]
    q = np.asarray(q_orb, dtype=np.float64)
    if q.shape != (sum(n_orb),):
        raise ValueError("q_orb must hold sum(n_orb_per_atom) orbital populations")
    offs = np.concatenate([[0], np.cumsum(n_orb)])
    total = float(np.sum(q))
    n_atom = len(n_orb)
    if binary:
        recs = [struct.pack("<i", RESTART_FORMAT),
                struct.pack("<5i2id", 0, 0, 0, 0, 0, n_atom, 1, total)]
        recs += [struct.pack(f"<{n_orb[a]}d", *q[offs[a]:offs[a + 1]]) for a in range(n_atom)]
        with open(path, "wb") as fh:
            fh.write(write_records(recs))
    else:
        lines = [f"{RESTART_FORMAT:12d}", f" F F F F F {n_atom:11d} {1:11d}  {total!r}"]
        lines += ["  " + "  ".join(repr(float(x)) for x in q[offs[a]:offs[a + 1]]) for a in range(n_atom)]
        with open(path, "w") as fh:
            fh.write("\n".join(lines) + "\n")
