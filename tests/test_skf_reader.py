"""CPU checks of the SKF reader against the reference's list-directed input rules
(type/oldskdata.F90:139-202 reads every data record with read(unit, *)): real Slater-Koster sets
write repeat counts (``19*0.0``), commas, D exponents and rows split over several lines."""
import io

import numpy as np
import pytest

from dftbplus_gb300 import skf


def _plain_file(rng, n_rows=6, homo=True):
    """A 10-column homonuclear (or heteronuclear) file written one record per line, and its values."""
    ham = rng.standard_normal((n_rows, 10))
    over = rng.standard_normal((n_rows, 10))
    rep = skf.SplineRepulsive(cutoff=3.0, exp_coeffs=np.array([1.5, 2.0, -0.3]),
                              x_start=np.array([1.0, 2.0]),
                              sp_coeffs=np.array([[0.1, -0.2, 0.03, -0.004]]),
                              last_coeffs=np.array([0.01, -0.02, 0.003, 0.0, 0.0, 0.0]))
    buf = io.StringIO()
    h = ((np.array([-0.5, -0.2, 0.0]), np.array([0.4, 0.4, 0.4]), np.array([2.0, 4.0, 0.0]), 15.999)
         if homo else None)
    skf.write_skf(buf, 0.02, ham, over, homo=h, repulsive=rep)
    return buf.getvalue(), ham, over, rep


def test_repeat_counts_commas_and_d_exponents():
    rng = np.random.default_rng(1)
    text, ham, over, rep = _plain_file(rng)
    lines = text.splitlines()
    # header: dist, nGrid with a comma; the homonuclear line with D exponents; mass record with 19*0.0
    lines[0] = "0.2D-01, 7"
    lines[1] = "0.0D0 -0.2D0 -0.5D0 0.0 0.4 0.4 0.4 0.0 4.0 2.0"
    lines[2] = "15.999, 19*0.0"
    # first grid row: the 20 values split over three records, separators mixed
    v = list(ham[0]) + list(over[0])
    lines[3] = " ".join(f"{x:.17e}" for x in v[:7]) + ","
    lines.insert(4, ", ".join(f"{x:.17e}" for x in v[7:15]))
    lines.insert(5, " ".join(f"{x:.17E}".replace("E", "D") for x in v[15:]) + "   trailing text ignored")
    d = skf.read_skf("\n".join(lines), homo=True)
    assert d.dist == 0.02 and d.ham.shape[0] == 6
    np.testing.assert_array_equal(d.onsite, [-0.5, -0.2, 0.0])
    np.testing.assert_array_equal(d.occ, [2.0, 4.0, 0.0])
    assert d.mass == 15.999
    cols = skf.OLD_SLOTS
    for i in range(6):
        np.testing.assert_array_equal(d.ham[i, [c - 1 for c in cols]], ham[i])
        np.testing.assert_array_equal(d.over[i, [c - 1 for c in cols]], over[i])
    np.testing.assert_array_equal(d.repulsive.x_start, rep.x_start)
    assert d.repulsive.cutoff == 3.0


def test_repeated_rows_and_slash():
    """``20*1.0`` rows (placeholder rows below the shortest distance in real sets) and a slash that
    ends a read early: the items not read keep their initial value (zero)."""
    rng = np.random.default_rng(2)
    text, ham, over, _ = _plain_file(rng, homo=False)
    lines = text.splitlines()
    lines[1] = "20*0.0"                       # heteronuclear dummy record
    lines[2] = "20*1.0"                       # grid row 1
    lines[3] = "3*0.5 /  the rest of this row is zero"
    d = skf.read_skf("\n".join(lines), homo=False)
    assert np.all(d.ham[0, [c - 1 for c in skf.OLD_SLOTS]] == 1.0)
    assert np.all(d.over[0, [c - 1 for c in skf.OLD_SLOTS]] == 1.0)
    row = np.concatenate([d.ham[1, [c - 1 for c in skf.OLD_SLOTS]], d.over[1, [c - 1 for c in skf.OLD_SLOTS]]])
    np.testing.assert_array_equal(row, [0.5] * 3 + [0.0] * 17)
    np.testing.assert_array_equal(d.ham[2, [c - 1 for c in skf.OLD_SLOTS]], ham[2])


def test_nulls_and_spline_record():
    rng = np.random.default_rng(3)
    text, _, _, rep = _plain_file(rng)
    lines = text.splitlines()
    lines[2] = "15.999,,, 17*"                # null values in the mass record
    i = lines.index("Spline")
    lines[i] = "Spline   "                     # trailing blanks still match the record
    d = skf.read_skf("\n".join(lines), homo=True)
    assert d.mass == 15.999
    np.testing.assert_array_equal(d.repulsive.exp_coeffs, rep.exp_coeffs)
    lines[i] = "  Spline"                      # a leading blank does not (Fortran string compare)
    with pytest.raises(ValueError):
        skf.read_skf("\n".join(lines), homo=True)


def test_truncated_file_reports():
    rng = np.random.default_rng(4)
    text, *_ = _plain_file(rng)
    lines = text.splitlines()[:5]
    with pytest.raises(ValueError):
        skf.read_skf("\n".join(lines), homo=True, read_repulsive=False)


def test_binary_table_cache(tmp_path, monkeypatch, water_model):
    """Model.from_files(cache=...) parses once and writes an .npz keyed by the SKF bytes; a matching
    cache is loaded without parsing and packs to the same C-ABI arrays; a changed file is reparsed."""
    from dftbplus_gb300 import synth
    from dftbplus_gb300 import model as model_mod
    sset = synth.make_skf_set([synth.SPECIES_O, synth.SPECIES_H], synth.WATER_SEED, synth.WATER_DRAW)
    names = ["O", "H"]
    for (a, b), d in sset.items():
        h10, s10 = synth.skf_columns10(d)
        homo = (d.onsite, d.hubbu, d.occ, d.mass) if a == b else None
        skf.write_skf(str(tmp_path / f"{names[a]}-{names[b]}.skf"), d.dist, h10, s10, homo=homo,
                      repulsive=d.repulsive)
    fmt = str(tmp_path / "{A}-{B}.skf")
    cache = str(tmp_path / "tables.npz")
    sp = [synth.SPECIES_O, synth.SPECIES_H]
    m1 = model_mod.Model.from_files(sp, fmt, cache=cache)
    parsed = []
    real_read = model_mod.read_skf
    monkeypatch.setattr(model_mod, "read_skf", lambda *a, **k: parsed.append(a) or real_read(*a, **k))
    m2 = model_mod.Model.from_files(sp, fmt, cache=cache)
    assert not parsed                                   # served from the cache
    p1, p2 = m1.pack(), m2.pack()
    for k in p1:
        assert np.array_equal(np.asarray(p1[k]), np.asarray(p2[k])), k
    assert [x.mass for x in m2.species] == [x.mass for x in m1.species]
    with open(str(tmp_path / "O-H.skf"), "a") as fh:     # any change of the bytes invalidates it
        fh.write("\n")
    model_mod.Model.from_files(sp, fmt, cache=cache)
    assert parsed


def test_table_cache_format_mismatch_is_a_miss(tmp_path, monkeypatch):
    """A cache written in another layout version is not loaded (treated as a miss and rewritten)."""
    from dftbplus_gb300 import synth
    from dftbplus_gb300 import model as model_mod
    sset = synth.make_skf_set([synth.SPECIES_O, synth.SPECIES_H], synth.WATER_SEED, synth.WATER_DRAW)
    names = ["O", "H"]
    for (a, b), d in sset.items():
        h10, s10 = synth.skf_columns10(d)
        homo = (d.onsite, d.hubbu, d.occ, d.mass) if a == b else None
        skf.write_skf(str(tmp_path / f"{names[a]}-{names[b]}.skf"), d.dist, h10, s10, homo=homo,
                      repulsive=d.repulsive)
    fmt = str(tmp_path / "{A}-{B}.skf")
    cache = str(tmp_path / "tables.npz")
    sp = [synth.SPECIES_O, synth.SPECIES_H]
    model_mod.Model.from_files(sp, fmt, cache=cache)
    monkeypatch.setattr(model_mod, "CACHE_FORMAT", model_mod.CACHE_FORMAT + 1)
    parsed = []
    real_read = model_mod.read_skf
    monkeypatch.setattr(model_mod, "read_skf", lambda *a, **k: parsed.append(a) or real_read(*a, **k))
    model_mod.Model.from_files(sp, fmt, cache=cache)
    assert parsed                                        # stale layout: reparsed
    with np.load(cache) as z:
        assert int(z["format"]) == model_mod.CACHE_FORMAT
