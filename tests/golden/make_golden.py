"""Generate golden fixtures from the reference's own unit tests (read as text, nothing executed).

    python tests/golden/make_golden.py /root/reference

* broyden_h2o.json   <- test/src/dftbp/unit/mixer/broyden.F90 (``broyden_mixer_H20``): the mixer
                        settings, 5 charge vectors and 4 difference vectors, tolerance 100 eps.
* coulomb_cluster.json <- test/src/dftbp/unit/dftb/coulomb.F90:31-101 (``coulombderivcluster``):
                        2 atoms on the x axis 1 Bohr apart, charges +1/-1, expected dV/dR array.
* charge_restart.json <- three charges.dat restart files of test/app/dftb+ (format 4, one spin
                        channel, no block populations), their text and populations.
"""
import json
import os
import re
import sys


def _floats(text):
    return [float(x.replace("_dp", "").replace("E", "e")) for x in
            re.findall(r"[-+]?\d+\.\d*(?:[eE][-+]?\d+)?(?:_dp)?", text)]


def broyden(ref):
    path = os.path.join(ref, "test/src/dftbp/unit/mixer/broyden.F90")
    src = open(path).read()
    m_q = re.search(r"expectedCharges\(3, 5\) = reshape\(\[(.*?)\], \[3,5\]\)", src, re.S)
    m_d = re.search(r"difference\(3, 4\) = reshape\(\[(.*?)\],[\s&]*\[3,4\]\)", src, re.S)
    q = _floats(m_q.group(1).replace("&", " "))
    d = _floats(m_d.group(1).replace("&", " "))
    assert len(q) == 15 and len(d) == 12, (len(q), len(d))

    def param(name):
        return float(re.search(rf"inp%{name}\s*=\s*([0-9.eE+-]+)_dp", src).group(1))

    return {
        "source": "test/src/dftbp/unit/mixer/broyden.F90 (broyden_mixer_H20)",
        "mix_param": param("mixParam"), "omega0": param("omega0"), "min_weight": param("minWeight"),
        "max_weight": param("maxWeight"), "weight_fac": param("weightFac"),
        "max_scc_iter": int(re.search(r"inp%maxSccIter\s*=\s*(\d+)", src).group(1)),
        "atol_eps_multiple": 100.0,
        "charges": [q[3 * i:3 * i + 3] for i in range(5)],
        "differences": [d[3 * i:3 * i + 3] for i in range(4)],
    }


def coulomb(ref):
    path = os.path.join(ref, "test/src/dftbp/unit/dftb/coulomb.F90")
    src = open(path).read()
    blk = src[src.index('TEST("coulombderivcluster")'):src.index('TEST("coulombderivperiodic")')]
    coords = [float(x) for x in re.search(r"coords0\(3,nAtom\) = reshape\(\[([^\]]*)\]", blk).group(1).split(",")]
    q = _floats(re.search(r"qAtom\(nAtom\) = \[([^\]]*)\]", blk).group(1))
    exp = [int(x) for x in re.search(r"reshape\(\[(-1,\+1[^\]]*)\],\[nAtom, 3,nAtom\]\)", blk).group(1).split(",")]
    return {"source": "test/src/dftbp/unit/dftb/coulomb.F90:31-101 (coulombderivcluster)",
            "coords_bohr": [coords[0:3], coords[3:6]], "charges": q,
            "expected_shape": [2, 3, 2], "expected_fortran_order": exp, "tol_eps_multiple": 1.0}


CHARGE_FILES = ["test/app/dftb+/scc/H3_skipcheck/charges.dat",
                "test/app/dftb+/scc/2H2O-3rdorder_read/charges.dat",
                "test/app/dftb+/transport/deph_CH4-poisson/charges.dat"]


def charges(ref):
    """Spin-unpolarised, block-free ASCII charge restart files of the reference's application tests:
    the text as it is, the orbital count of each atom (one record per atom in these files) and the
    populations (records 3..) read with a plain split."""
    out = []
    for rel in CHARGE_FILES:
        text = open(os.path.join(ref, rel)).read()
        recs = [r for r in text.splitlines() if r.strip()]
        rows = [[float(x) for x in r.split()] for r in recs[2:]]
        out.append({"source": rel, "text": text, "n_orb_per_atom": [len(r) for r in rows],
                    "populations": [x for r in rows for x in r],
                    "checksum": float(recs[1].split()[-1])})
    return out


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(out, "broyden_h2o.json"), "w") as fh:
        json.dump(broyden(ref), fh, indent=1)
    with open(os.path.join(out, "coulomb_cluster.json"), "w") as fh:
        json.dump(coulomb(ref), fh, indent=1)
    with open(os.path.join(out, "charge_restart.json"), "w") as fh:
        json.dump(charges(ref), fh, indent=1)
    print("wrote", out)
