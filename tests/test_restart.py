"""CPU checks of the charge restart files (dftb/sccinit.F90 formats): the reference's own
charges.dat fixtures (golden, tests/golden/charge_restart.json) read back exactly, format-8 files
written here read back bit for bit in ASCII and binary, and the reference's consistency checks."""
import json
import os
import struct

import numpy as np
import pytest

from dftbplus_gb300 import restart
from dftbplus_gb300.fortran_io import read_records

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "charge_restart.json")


def _fixtures():
    with open(GOLDEN) as fh:
        return json.load(fh)


@pytest.mark.parametrize("i", range(3))
def test_reference_files_read(tmp_path, i):
    fx = _fixtures()[i]
    p = tmp_path / "charges.dat"
    p.write_text(fx["text"])
    q = restart.read_charges(str(p), fx["n_orb_per_atom"])
    assert q.tolist() == fx["populations"]
    # the reference's total-charge check (1e-3) against the electron count
    restart.read_charges(str(p), fx["n_orb_per_atom"], n_el=round(fx["checksum"]))
    with pytest.raises(ValueError):
        restart.read_charges(str(p), fx["n_orb_per_atom"], n_el=round(fx["checksum"]) + 1)


def test_format4_covers_all_atoms_and_checksum(tmp_path):
    """Format 4 has no atom count: every atom of the system is read; a damaged population fails the
    checksum (1e-7)."""
    fx = _fixtures()[1]
    p = tmp_path / "charges.dat"
    p.write_text(fx["text"])
    with pytest.raises(ValueError):                       # fewer atoms than records needs
        restart.read_charges(str(p), fx["n_orb_per_atom"] + [1])
    lines = fx["text"].splitlines()
    lines[2] = lines[2].replace("6.7277403366336541", "6.7277413366336541")
    p.write_text("\n".join(lines))
    with pytest.raises(ValueError, match="checksum"):
        restart.read_charges(str(p), fx["n_orb_per_atom"])


@pytest.mark.parametrize("binary", [False, True])
def test_format8_round_trip(tmp_path, binary):
    rng = np.random.default_rng(7)
    n_orb = [4, 1, 1, 9, 4, 1]
    q = rng.uniform(0.0, 2.0, sum(n_orb))
    p = str(tmp_path / ("charges.bin" if binary else "charges.dat"))
    restart.write_charges(p, q, n_orb)
    q2 = restart.read_charges(p, n_orb)
    assert np.array_equal(q, q2)
    # a file written for fewer atoms restarts a larger system with zero populations beyond it
    restart.write_charges(p, q[:6], n_orb[:3])
    q3 = restart.read_charges(p, n_orb)
    assert np.array_equal(q3[:6], q[:6]) and not q3[6:].any()
    with pytest.raises(ValueError):
        restart.read_charges(p, n_orb[:2])               # more atoms in the file than the system


def test_binary_layout(tmp_path):
    """gfortran unformatted sequential records: format number; 5 logicals, nAtom, nSpin, checksum;
    one record of populations per atom."""
    p = str(tmp_path / "charges.bin")
    restart.write_charges(p, np.array([1.5, 0.5, 0.25, 0.75, 1.0]), [4, 1])
    recs = read_records(open(p, "rb").read())
    assert len(recs) == 4
    assert struct.unpack("<i", recs[0]) == (8,)
    assert struct.unpack("<5i2id", recs[1]) == (0, 0, 0, 0, 0, 2, 1, 4.0)
    assert struct.unpack("<4d", recs[2]) == (1.5, 0.5, 0.25, 0.75)
    assert struct.unpack("<d", recs[3]) == (1.0,)


def test_spin_polarised_file_rejected(tmp_path):
    p = tmp_path / "charges.dat"
    p.write_text("8\n F F F F F 1 2 1.0 0.0\n 1.0\n 0.0\n")
    with pytest.raises(ValueError, match="spin"):
        restart.read_charges(str(p), [1])


def test_calculator_restart_hooks(tmp_path, water_model):
    """DftbGpu.read_charges turns a reference charge file into the per-atom start populations of the
    next SCC call, write_charges writes the converged orbital populations (a stand-in context gives
    the populations: the library itself needs a GPU)."""
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(2, 4.0, 3)

    class _Ctx:
        def __init__(self):
            self.calls = []

        def scc(self, opts, q_init=None):
            self.calls.append(None if q_init is None else np.array(q_init))
            return {"energies": {"EMermin": 0.0}, "q_out": np.zeros(len(s))}

        def orbital_populations(self):
            return np.arange(12, dtype=np.float64) / 10.0

    calc = object.__new__(binding.DftbGpu)        # no device: the context is the stand-in above
    calc.ctx, calc.model, calc.species = _Ctx(), water_model, np.asarray(s, dtype=np.int32)
    calc.opts = binding.SccOpts()
    calc.opts.net_charge = 0.0
    calc._q_init, calc._res, calc._grad = None, None, None
    n_orb = [water_model.species[x].n_orb for x in s]
    assert n_orb == [4, 1, 1, 4, 1, 1]                     # O H H O H H
    q = np.array([1.9, 1.5, 1.6, 1.6, 0.7, 0.7, 1.8, 1.6, 1.6, 1.6, 0.6, 0.8])   # 16 electrons
    p = str(tmp_path / "charges.dat")
    restart.write_charges(p, q, n_orb)
    calc.read_charges(p)
    calc.get_energy()
    np.testing.assert_allclose(calc.ctx.calls[-1], [6.6, 0.7, 0.7, 6.6, 0.6, 0.8], rtol=0, atol=1e-14)
    with pytest.raises(ValueError):                         # a file for another electron count
        restart.write_charges(p, q * 1.1, n_orb)
        calc.read_charges(p)
    out = str(tmp_path / "out.bin")
    calc.write_charges(out)
    assert np.array_equal(restart.read_charges(out, n_orb), np.arange(12) / 10.0)
