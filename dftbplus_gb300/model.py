"""Host-side DFTB model: species, orbitals, Slater-Koster tables and pair repulsives.

Mirrors what the reference's init layer hands to the hot path (``dftbplus/parser.F90:3668-3886``
``readSKFiles``; ``type/commontypes.F90`` ``TOrbitals``): per species the shells (angular momenta),
on-site energies, Hubbard U and reference shell occupations; per ordered species pair the H and S
integral tables on an equidistant grid and the spline repulsive.
"""
from __future__ import annotations

import dataclasses
import hashlib
import json
import os
from typing import Dict, List, Sequence, Tuple

import numpy as np

from .skf import SkfData, SplineRepulsive, full_table, n_integrals, read_skf

MAX_SHELL = 4  # slots per species in the packed shell arrays (s, p, d, f)

# Layout version of the binary table cache (the .npz written by Model.save). It enters the cache
# key and is stored in the file; a cache of another version is treated as a miss and rewritten, so
# a change to full_table, SplineRepulsive.pack/unpack or the .npz layout must bump it.
CACHE_FORMAT = 2


def _files_key(species: Sequence[Species], paths: Sequence[str]) -> str:
    """SHA-256 over the cache format, the requested shells and the bytes of every SKF file, in order."""
    h = hashlib.sha256()
    h.update(f"dftbgpu-table-cache-v{CACHE_FORMAT}".encode())
    h.update(json.dumps([[x.name, list(x.shells)] for x in species]).encode())
    for p in paths:
        with open(p, "rb") as fh:
            h.update(hashlib.sha256(fh.read()).digest())
    return h.hexdigest()


@dataclasses.dataclass
class Species:
    name: str
    shells: List[int]               # angular momentum of each shell, e.g. [0, 1] for O (s, p)
    onsite: List[float]             # on-site energy per shell (Ha)
    hubbu: float                    # Hubbard U (Ha), same for all shells (no orbital-resolved SCC)
    occ: List[float]                # reference (neutral atom) occupation per shell
    mass: float = 1.0

    @property
    def n_orb(self) -> int:
        return sum(2 * l + 1 for l in self.shells)


@dataclasses.dataclass
class PairTable:
    dist: float
    ham: np.ndarray                 # (nRows, nInt)
    over: np.ndarray                # (nRows, nInt)

    @property
    def n_rows(self) -> int:
        return self.ham.shape[0]

    @property
    def n_int(self) -> int:
        return self.ham.shape[1]


class Model:
    """Species + SK tables + repulsives for an SCC-DFTB calculation (spin unpolarised, s/p/d)."""

    def __init__(self, species: Sequence[Species], tables: Dict[Tuple[int, int], PairTable],
                 repulsives: Dict[Tuple[int, int], SplineRepulsive]):
        self.species = list(species)
        self.tables = tables
        self.repulsives = repulsives
        ns = len(self.species)
        for a in range(ns):
            for b in range(ns):
                t = tables[(a, b)]
                want = n_integrals(self.species[a].shells, self.species[b].shells)
                if t.n_int != want:
                    raise ValueError(f"pair {a},{b}: {t.n_int} integrals, expected {want}")
                if (a, b) not in repulsives:
                    raise ValueError(f"missing repulsive for pair {a},{b}")

    @property
    def n_species(self) -> int:
        return len(self.species)

    @property
    def m_orb(self) -> int:
        return max(s.n_orb for s in self.species)

    def sk_cutoff(self) -> float:
        """Largest SK interaction range: nRows * dist + 1 Bohr tail (slakoeqgrid.F90:168-183)."""
        return max(t.n_rows * t.dist + 1.0 for t in self.tables.values())

    def rep_cutoff(self) -> float:
        return max(r.cutoff for r in self.repulsives.values())

    @classmethod
    def from_skf(cls, species: Sequence[Species], skf: Dict[Tuple[int, int], SkfData]) -> "Model":
        """Build from parsed SKF data keyed by ordered species pair (A, B) = file ``A-B.skf``."""
        tables, reps = {}, {}
        ns = len(species)
        for a in range(ns):
            for b in range(ns):
                h, s = full_table(skf[(a, b)], skf[(b, a)], species[a].shells, species[b].shells)
                tables[(a, b)] = PairTable(dist=skf[(a, b)].dist, ham=h, over=s)
                reps[(a, b)] = skf[(a, b)].repulsive
        return cls(species, tables, reps)

    @classmethod
    def from_files(cls, species: Sequence[Species], path_fmt: str, cache: str | None = None) -> "Model":
        """``path_fmt`` like ``"skf/{A}-{B}.skf"``; on-site/U/occ are taken from the homonuclear files.

        ``cache``: a binary table cache (``.npz``) keyed by the SHA-256 of the SKF files' bytes and the
        requested shells: a matching cache is loaded without parsing, otherwise the files are parsed
        and the cache is (re)written."""
        ns = len(species)
        paths = [[path_fmt.format(A=species[a].name, B=species[b].name) for b in range(ns)] for a in range(ns)]
        key = None
        if cache is not None:
            key = _files_key(species, [p for row in paths for p in row])
            m = cls.load(cache, key)
            if m is not None:
                return m
        skf = {}
        for a in range(ns):
            for b in range(ns):
                skf[(a, b)] = read_skf(paths[a][b], homo=(a == b))
        sp = []
        for a, s in enumerate(species):
            d = skf[(a, a)]
            sp.append(Species(s.name, list(s.shells), [float(d.onsite[l]) for l in s.shells],
                              float(d.hubbu[s.shells[0]]), [float(d.occ[l]) for l in s.shells],
                              float(d.mass)))
        model = cls.from_skf(sp, skf)
        if cache is not None:
            model.save(cache, key)
        return model

    # ------------------------------------------------------------------ binary table cache
    def save(self, path: str, key: str = "") -> None:
        """All tables, repulsives and species data in one ``.npz`` (no pickled objects)."""
        ns = self.n_species
        arrs = {"key": np.array(key), "format": np.array(CACHE_FORMAT), "n_species": np.array(ns),
                "species_json": np.array(json.dumps([dataclasses.asdict(x) for x in self.species]))}
        for (a, b), t in self.tables.items():
            arrs[f"dist_{a}_{b}"] = np.array(t.dist)
            arrs[f"ham_{a}_{b}"] = t.ham
            arrs[f"over_{a}_{b}"] = t.over
            r = self.repulsives[(a, b)]
            arrs[f"rep_{a}_{b}"] = r.pack()
            arrs[f"repn_{a}_{b}"] = np.array(len(r.x_start))
        tmp = path + ".tmp.npz"
        np.savez(tmp, **arrs)
        os.replace(tmp, path)

    @classmethod
    def load(cls, path: str, key: str | None = None) -> "Model | None":
        """The model saved at ``path``; None if it is missing, was written in another cache format,
        or its key differs from ``key``."""
        if not os.path.exists(path):
            return None
        with np.load(path, allow_pickle=False) as z:
            if "format" not in z.files or int(z["format"]) != CACHE_FORMAT:
                return None
            if key is not None and str(z["key"]) != key:
                return None
            ns = int(z["n_species"])
            species = [Species(**d) for d in json.loads(str(z["species_json"]))]
            tables, reps = {}, {}
            for a in range(ns):
                for b in range(ns):
                    tables[(a, b)] = PairTable(dist=float(z[f"dist_{a}_{b}"]), ham=np.array(z[f"ham_{a}_{b}"]),
                                               over=np.array(z[f"over_{a}_{b}"]))
                    reps[(a, b)] = SplineRepulsive.unpack(np.array(z[f"rep_{a}_{b}"]), int(z[f"repn_{a}_{b}"]))
        return cls(species, tables, reps)

    # ------------------------------------------------------------------ packing for the C-ABI
    def pack(self) -> dict:
        """Flat arrays in the layout taken by ``dftbgpu_set_model`` (see include/dftbgpu.h)."""
        ns = self.n_species
        n_shell = np.array([len(s.shells) for s in self.species], dtype=np.int32)
        ang = np.full((ns, MAX_SHELL), -1, dtype=np.int32)
        ons = np.zeros((ns, MAX_SHELL))
        occ = np.zeros((ns, MAX_SHELL))
        for i, s in enumerate(self.species):
            ang[i, :len(s.shells)] = s.shells
            ons[i, :len(s.shells)] = s.onsite
            occ[i, :len(s.shells)] = s.occ
        hub = np.array([s.hubbu for s in self.species])
        # ordered pair index p = sp1 * ns + sp2
        dist = np.zeros(ns * ns)
        n_rows = np.zeros(ns * ns, dtype=np.int32)
        n_int = np.zeros(ns * ns, dtype=np.int32)
        ham_parts, over_parts, rep_parts = [], [], []
        n_spline = np.zeros(ns * ns, dtype=np.int32)
        for a in range(ns):
            for b in range(ns):
                p = a * ns + b
                t = self.tables[(a, b)]
                dist[p] = t.dist
                n_rows[p] = t.n_rows
                n_int[p] = t.n_int
                # column-major (row fastest) per pair: table[iRow + nRows * iInt]
                ham_parts.append(np.asfortranarray(t.ham).reshape(-1, order="F"))
                over_parts.append(np.asfortranarray(t.over).reshape(-1, order="F"))
                r = self.repulsives[(a, b)]
                n_spline[p] = len(r.x_start)
                rep_parts.append(r.pack())
        return dict(n_species=ns, n_shell=n_shell, ang_shell=ang.reshape(-1), onsite=ons.reshape(-1),
                    hubbu=hub, ref_occ=occ.reshape(-1), sk_dist=dist, sk_rows=n_rows, sk_nint=n_int,
                    sk_ham=np.concatenate(ham_parts), sk_over=np.concatenate(over_parts),
                    rep_nspline=n_spline, rep_data=np.concatenate(rep_parts))

    # ------------------------------------------------------------------ orbital bookkeeping
    def orbital_offsets(self, species_idx: np.ndarray) -> np.ndarray:
        n = np.array([self.species[s].n_orb for s in species_idx], dtype=np.int64)
        off = np.zeros(len(n) + 1, dtype=np.int64)
        off[1:] = np.cumsum(n)
        return off

    def n_electrons(self, species_idx: np.ndarray, net_charge: float = 0.0) -> float:
        return float(sum(sum(self.species[s].occ) for s in species_idx)) - net_charge
