"""CPU oracle for the non-periodic Gamma-point SCC-DFTB energy + force path.

TEST INFRASTRUCTURE ONLY. This module is the checker: only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it. The product path
(``dftbplus_gb300``) never calls it.

It restates, in FP64 numpy, the reference algorithm of DFTB+ 25.1 for this path. Each function
names the reference file:line it follows. The reference itself (Fortran) cannot be compiled in this
environment (no Fortran compiler), so parity of this restatement is pinned by (1) the reference's
Broyden golden sequence (test/src/dftbp/unit/mixer/broyden.F90), (2) the reference's cluster 1/r
derivative fixture (test/src/dftbp/unit/dftb/coulomb.F90:31-101), and (3) internal identities
(rotational invariance of the SK blocks, forces vs central finite differences of E_Mermin, charge
conservation). The generalized eigensolver is LAPACK ``dsygvd`` (scipy), as in the reference's
``hegvd`` path (math/eigensolver.F90:561-660).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Tuple

import numpy as np
import scipy.linalg

EPS = np.finfo(np.float64).eps
DIST_FUDGE = 1.0            # common/accuracy.F90:44
DELTA_R = 1e-5              # slakoeqgrid.F90:90
N_INTER = 8                 # slakoeqgrid.F90:71
N_RIGHT = 4                 # slakoeqgrid.F90:84
ELEC_TOL = 1e-15            # accuracy.F90:55
ELEC_TOL_MAX = 1e-7         # accuracy.F90:61
MIN_SHORT_GAMMA = 1e-10     # accuracy.F90:86
TOL_SHORT_GAMMA = 1e-10     # accuracy.F90:94
TOL_SAME_DIST = 1e-5        # accuracy.F90:69
MIN_HUB_DIFF = 0.3125e-5    # accuracy.F90:110
MIN_NEIGH_DIST = 1e-2       # accuracy.F90:78
ARBITRARY_CONST = 0.1       # densitymatrix.F90:103
FD_DELTA = EPS ** 0.25      # nonscc.F90:43
SQ3 = math.sqrt(3.0)


# ============================================================================ SK interpolation
def neville_uniform(xp: np.ndarray, yp: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Neville interpolation on a uniform grid, vectorised over points.

    Follows ``math/interpolation.F90:182-239`` (``polyInterU2``), including its choice of the
    starting point ``iCl = ceiling((x - xp(1)) * delta(1))`` and the c/d tableau walk.
    xp: (P, n) abscissae, yp: (P, n, nInt), x: (P,) -> (P, nInt).
    """
    P, n = xp.shape
    delta = 1.0 / (xp[:, 1:] - xp[:, :1])                   # delta(ii) = 1/(xp(1+ii) - xp(1))
    c = yp.copy()
    d = yp.copy()
    icl = np.ceil((x - xp[:, 0]) * delta[:, 0]).astype(np.int64)   # 1-based
    rows = np.arange(P)
    y = yp[rows, icl - 1, :].copy()
    icl = icl - 1
    for m in range(1, n):
        for i in range(1, n - m + 1):                         # 1-based ii
            r2 = (d[:, i - 1, :] - c[:, i, :]) * delta[:, m - 1][:, None]
            c[:, i - 1, :] = (xp[:, i - 1] - x)[:, None] * r2
            d[:, i - 1, :] = (xp[:, i - 1 + m] - x)[:, None] * r2
        take_c = 2 * icl < n - m
        dy = np.where(take_c[:, None], c[rows, np.clip(icl, 0, n - 1), :],
                      d[rows, np.clip(icl - 1, 0, n - 1), :])
        icl = np.where(take_c, icl, icl - 1)
        y = y + dy
    return y


def poly5_to_zero(y0, y0p, y0pp, xx, dx, invdx):
    """5th-order polynomial to zero; ``math/interpolation.F90:31-67``."""
    dx1 = y0p * dx
    dx2 = y0pp * dx * dx
    dd = 10.0 * y0 - 4.0 * dx1 + 0.5 * dx2
    ee = -15.0 * y0 + 7.0 * dx1 - 1.0 * dx2
    ff = 6.0 * y0 - 3.0 * dx1 + 0.5 * dx2
    xr = xx * invdx
    return ((ff * xr + ee) * xr + dd) * xr * xr * xr


def sk_integrals(dist: float, table: np.ndarray, r: np.ndarray) -> np.ndarray:
    """Integrals at distances r for one pair table (nRows, nInt) -> (P, nInt).

    ``dftb/slakoeqgrid.F90:183-244`` (``SlakoEqGrid_interNew_``): 8-point Neville inside the grid,
    5th-order tail to zero over the last ``distFudge`` = 1 Bohr, zero beyond.
    """
    r = np.asarray(r, dtype=np.float64)
    leng, n_int = table.shape
    incr = dist
    rmax = leng * incr + DIST_FUDGE
    out = np.zeros((r.size, n_int))
    ind = np.floor(r / incr).astype(np.int64)
    inside = (r < rmax) & (ind < leng)
    tail = (r < rmax) & (ind >= leng)
    if inside.any():
        rr = r[inside]
        il = np.maximum(np.minimum(leng, ind[inside] + N_RIGHT), N_INTER)
        k = np.arange(1, N_INTER + 1)
        xa = (il[:, None] - N_INTER + k[None, :]) * incr
        yb = table[(il[:, None] - N_INTER + k[None, :] - 1), :]
        out[inside] = neville_uniform(xa, yb, rr)
    if tail.any():
        rr = r[tail]
        k = np.arange(1, N_INTER + 1)
        xa = ((leng - N_INTER + k) * incr)[None, :]
        yb = table[leng - N_INTER:leng, :][None, :, :]
        y0 = neville_uniform(xa, yb, np.array([xa[0, -1] - DELTA_R]))[0]
        y2 = neville_uniform(xa, yb, np.array([xa[0, -1] + DELTA_R]))[0]
        y1 = table[leng - 1, :]
        y1p = (y2 - y0) / (2.0 * DELTA_R)
        y1pp = (y2 + y0 - 2.0 * y1) / (DELTA_R * DELTA_R)
        dr = rr - rmax
        out[tail] = poly5_to_zero(y1[None, :], y1p[None, :], y1pp[None, :], dr[:, None],
                                  -DIST_FUDGE, -1.0 / DIST_FUDGE)
    return out


# ============================================================================ SK rotations
# Orbital order (type/orbitals.F90): p = (y, z, x); d = (xy, yz, z2, xz, x2-y2).
# rot_<lo><hi>(l, m, n, sk) returns (P, 2*hi+1, 2*lo+1) with element [b, a] = <lo_a at A | hi_b at B>
# for the unit vector (l, m, n) from A to B: the Slater-Koster (1954) table, in the layout of
# dftb/sk.F90:144-500 (ss, sp, sd, pp, pd, dd).

def _rot_ss(l, m, n, sk):
    return sk[:, 0][:, None, None] * np.ones((len(l), 1, 1))


def _rot_sp(l, m, n, sk):
    s = sk[:, 0]
    return np.stack([m * s, n * s, l * s], axis=1)[:, :, None]


def _d_s_coeffs(l, m, n):
    """s-d angular factors for the five d orbitals (xy, yz, z2, xz, x2-y2)."""
    return np.stack([SQ3 * l * m, SQ3 * m * n, n * n - 0.5 * (l * l + m * m), SQ3 * l * n,
                     0.5 * SQ3 * (l * l - m * m)], axis=1)


def _rot_sd(l, m, n, sk):
    return (_d_s_coeffs(l, m, n) * sk[:, 0][:, None])[:, :, None]


def _rot_pp(l, m, n, sk):
    c = np.stack([m, n, l], axis=1)                           # p order y, z, x
    sig, pi = sk[:, 0], sk[:, 1]
    out = c[:, :, None] * c[:, None, :] * (sig - pi)[:, None, None]
    out += np.eye(3)[None, :, :] * pi[:, None, None]
    return out


def _pd_factors(l, m, n):
    """(sigma, pi) factors E_{p_i, d_j}: arrays (P, 5, 3) rows d (xy,yz,z2,xz,x2-y2), cols p (y,z,x)."""
    l2, m2, n2 = l * l, m * m, n * n
    P = len(l)
    fs = np.zeros((P, 5, 3))
    fp = np.zeros((P, 5, 3))
    # p_x column (index 2)
    fs[:, 0, 2] = SQ3 * l2 * m;          fp[:, 0, 2] = m * (1 - 2 * l2)
    fs[:, 1, 2] = SQ3 * l * m * n;       fp[:, 1, 2] = -2 * l * m * n
    fs[:, 2, 2] = l * (n2 - 0.5 * (l2 + m2)); fp[:, 2, 2] = -SQ3 * l * n2
    fs[:, 3, 2] = SQ3 * l2 * n;          fp[:, 3, 2] = n * (1 - 2 * l2)
    fs[:, 4, 2] = 0.5 * SQ3 * l * (l2 - m2); fp[:, 4, 2] = l * (1 - l2 + m2)
    # p_y column (index 0)
    fs[:, 0, 0] = SQ3 * m2 * l;          fp[:, 0, 0] = l * (1 - 2 * m2)
    fs[:, 1, 0] = SQ3 * m2 * n;          fp[:, 1, 0] = n * (1 - 2 * m2)
    fs[:, 2, 0] = m * (n2 - 0.5 * (l2 + m2)); fp[:, 2, 0] = -SQ3 * m * n2
    fs[:, 3, 0] = SQ3 * l * m * n;       fp[:, 3, 0] = -2 * l * m * n
    fs[:, 4, 0] = 0.5 * SQ3 * m * (l2 - m2); fp[:, 4, 0] = -m * (1 + l2 - m2)
    # p_z column (index 1)
    fs[:, 0, 1] = SQ3 * l * m * n;       fp[:, 0, 1] = -2 * l * m * n
    fs[:, 1, 1] = SQ3 * n2 * m;          fp[:, 1, 1] = m * (1 - 2 * n2)
    fs[:, 2, 1] = n * (n2 - 0.5 * (l2 + m2)); fp[:, 2, 1] = SQ3 * n * (l2 + m2)
    fs[:, 3, 1] = SQ3 * n2 * l;          fp[:, 3, 1] = l * (1 - 2 * n2)
    fs[:, 4, 1] = 0.5 * SQ3 * n * (l2 - m2); fp[:, 4, 1] = -n * (l2 - m2)
    return fs, fp


def _rot_pd(l, m, n, sk):
    fs, fp = _pd_factors(l, m, n)
    return fs * sk[:, 0][:, None, None] + fp * sk[:, 1][:, None, None]


def _dd_factors(l, m, n):
    """(sigma, pi, delta) factors E_{d_i, d_j}, arrays (P, 5, 5), order xy, yz, z2, xz, x2-y2."""
    l2, m2, n2 = l * l, m * m, n * n
    P = len(l)
    S = np.zeros((P, 5, 5)); Pi = np.zeros((P, 5, 5)); D = np.zeros((P, 5, 5))
    XY, YZ, Z2, XZ, X2 = 0, 1, 2, 3, 4
    lm2 = l2 - m2
    q = n2 - 0.5 * (l2 + m2)

    def put(i, j, s, p, d):
        S[:, i, j] = s; Pi[:, i, j] = p; D[:, i, j] = d
        S[:, j, i] = s; Pi[:, j, i] = p; D[:, j, i] = d

    put(XY, XY, 3 * l2 * m2, l2 + m2 - 4 * l2 * m2, n2 + l2 * m2)
    put(YZ, YZ, 3 * m2 * n2, m2 + n2 - 4 * m2 * n2, l2 + m2 * n2)
    put(XZ, XZ, 3 * n2 * l2, n2 + l2 - 4 * n2 * l2, m2 + n2 * l2)
    put(XY, YZ, 3 * l * m2 * n, l * n * (1 - 4 * m2), l * n * (m2 - 1))
    put(XY, XZ, 3 * l2 * m * n, m * n * (1 - 4 * l2), m * n * (l2 - 1))
    put(YZ, XZ, 3 * l * m * n2, l * m * (1 - 4 * n2), l * m * (n2 - 1))
    put(XY, X2, 1.5 * l * m * lm2, -2 * l * m * lm2, 0.5 * l * m * lm2)
    put(YZ, X2, 1.5 * m * n * lm2, -m * n * (1 + 2 * lm2), m * n * (1 + 0.5 * lm2))
    put(XZ, X2, 1.5 * n * l * lm2, n * l * (1 - 2 * lm2), -n * l * (1 - 0.5 * lm2))
    put(XY, Z2, SQ3 * l * m * q, -2 * SQ3 * l * m * n2, 0.5 * SQ3 * l * m * (1 + n2))
    put(YZ, Z2, SQ3 * m * n * q, SQ3 * m * n * (l2 + m2 - n2), -0.5 * SQ3 * m * n * (l2 + m2))
    put(XZ, Z2, SQ3 * l * n * q, SQ3 * l * n * (l2 + m2 - n2), -0.5 * SQ3 * l * n * (l2 + m2))
    put(X2, X2, 0.75 * lm2 * lm2, l2 + m2 - lm2 * lm2, n2 + 0.25 * lm2 * lm2)
    put(X2, Z2, 0.5 * SQ3 * lm2 * q, SQ3 * n2 * (m2 - l2), 0.25 * SQ3 * (1 + n2) * lm2)
    put(Z2, Z2, q * q, 3 * n2 * (l2 + m2), 0.75 * (l2 + m2) ** 2)
    return S, Pi, D


def _rot_dd(l, m, n, sk):
    S, Pi, D = _dd_factors(l, m, n)
    return S * sk[:, 0][:, None, None] + Pi * sk[:, 1][:, None, None] + D * sk[:, 2][:, None, None]


_ROT = {(0, 0): _rot_ss, (0, 1): _rot_sp, (0, 2): _rot_sd, (1, 1): _rot_pp, (1, 2): _rot_pd,
        (2, 2): _rot_dd}


def rotate_blocks(sk: np.ndarray, l, m, n, shells1, shells2) -> np.ndarray:
    """Diatomic blocks (P, nOrb2, nOrb1): rows = orbitals of atom 2, cols = orbitals of atom 1.

    ``dftb/sk.F90:35-140`` (``rotateH0``): shell loop order (atom-1 shells outer), integral index
    advance ``min(l1,l2)+1``, and for l1 > l2 the block is ``(-1)^(l1+l2)`` times the transpose.
    """
    P = len(l)
    no1 = sum(2 * a + 1 for a in shells1)
    no2 = sum(2 * b + 1 for b in shells2)
    out = np.zeros((P, no2, no1))
    ind = 0
    col = 0
    for a1 in shells1:
        n1 = 2 * a1 + 1
        row = 0
        for a2 in shells2:
            n2 = 2 * a2 + 1
            k = min(a1, a2) + 1
            psk = sk[:, ind:ind + k]
            if a1 <= a2:
                out[:, row:row + n2, col:col + n1] = _ROT[(a1, a2)](l, m, n, psk)
            else:
                t = _ROT[(a2, a1)](l, m, n, psk)
                out[:, row:row + n2, col:col + n1] = ((-1.0) ** (a1 + a2)) * np.transpose(t, (0, 2, 1))
            ind += k
            row += n2
        col += n1
    return out


# ============================================================================ system setup
@dataclasses.dataclass
class System:
    model: object                   # dftbplus_gb300.model.Model
    coords: np.ndarray              # (3, N) Bohr
    species: np.ndarray             # (N,)

    def __post_init__(self):
        self.coords = np.asarray(self.coords, dtype=np.float64)
        self.species = np.asarray(self.species, dtype=np.int64)
        self.n_atom = self.coords.shape[1]
        self.off = self.model.orbital_offsets(self.species)
        self.n_orb = int(self.off[-1])
        self.atom_of_orb = np.repeat(np.arange(self.n_atom), np.diff(self.off))
        self.q0_atom = np.array([sum(self.model.species[s].occ) for s in self.species])
        self.hubbu = np.array([self.model.species[s].hubbu for s in self.species])


def pair_list(coords: np.ndarray, cutoff: float):
    """Half neighbour list (i < j) with r <= cutoff (dftb/periodic.F90:380-700, cluster case)."""
    N = coords.shape[1]
    ii, jj = np.triu_indices(N, k=1)
    d = coords[:, jj] - coords[:, ii]
    r = np.sqrt(np.sum(d * d, axis=0))
    keep = r * r <= cutoff * cutoff + TOL_SAME_DIST ** 2
    if np.any(r[keep] < MIN_NEIGH_DIST):
        raise ValueError("atoms too close together")
    return ii[keep], jj[keep], r[keep]


def build_h0_s(sys_: System, disp: Optional[Tuple[int, float]] = None):
    """Dense H0 and S (n x n, symmetric).

    ``dftb/nonscc.F90:66-181`` (``buildH0``/``buildS``: on-site energies on the diagonal, unit
    overlap) and ``:364-424`` (``buildDiatomicBlocks``: vector from atom 1 to its neighbour,
    ``getSKIntegrals`` for (sp1, sp2), ``rotateH0``). The half list gives each pair once; the dense
    matrix is filled symmetrically.
    """
    model = sys_.model
    n = sys_.n_orb
    H0 = np.zeros((n, n))
    S = np.eye(n)
    for a in range(sys_.n_atom):
        sp = model.species[sys_.species[a]]
        o = sys_.off[a]
        k = 0
        for l, e in zip(sp.shells, sp.onsite):
            for _ in range(2 * l + 1):
                H0[o + k, o + k] = e
                k += 1
    ii, jj, r = pair_list(sys_.coords, model.sk_cutoff())
    blocks = diatomic_blocks(sys_, ii, jj)
    for p in range(len(ii)):
        i, j = ii[p], jj[p]
        hb, sb = blocks[0][p], blocks[1][p]
        oi, oj = sys_.off[i], sys_.off[j]
        ni, nj = sys_.off[i + 1] - oi, sys_.off[j + 1] - oj
        H0[oj:oj + nj, oi:oi + ni] = hb
        H0[oi:oi + ni, oj:oj + nj] = hb.T
        S[oj:oj + nj, oi:oi + ni] = sb
        S[oi:oi + ni, oj:oj + nj] = sb.T
    return H0, S


def diatomic_blocks(sys_: System, ii, jj, vec_override=None):
    """H and S blocks for pairs (i, j): list of (nOrb_j, nOrb_i) arrays, grouped by species pair."""
    model = sys_.model
    P = len(ii)
    hb = [None] * P
    sb = [None] * P
    spi = sys_.species[ii]
    spj = sys_.species[jj]
    vec = sys_.coords[:, jj] - sys_.coords[:, ii] if vec_override is None else vec_override
    for a in range(model.n_species):
        for b in range(model.n_species):
            sel = np.nonzero((spi == a) & (spj == b))[0]
            if sel.size == 0:
                continue
            v = vec[:, sel]
            dist = np.sqrt(np.sum(v * v, axis=0))
            u = v / dist
            t = model.tables[(a, b)]
            skh = sk_integrals(t.dist, t.ham, dist)
            sks = sk_integrals(t.dist, t.over, dist)
            sh1, sh2 = model.species[a].shells, model.species[b].shells
            bh = rotate_blocks(skh, u[0], u[1], u[2], sh1, sh2)
            bs = rotate_blocks(sks, u[0], u[1], u[2], sh1, sh2)
            for k, p in enumerate(sel):
                hb[p] = bh[k]
                sb[p] = bs[k]
    return hb, sb


# ============================================================================ electrostatics
def exp_gamma(r, ua, ub):
    """Short-range gamma, ``dftb/shortgammafuncs.F90:97-150`` (``expGamma``), scalar."""
    tau_a = 3.2 * ua
    tau_b = 3.2 * ub
    if r < TOL_SAME_DIST:
        if abs(ua - ub) < MIN_HUB_DIFF:
            return -0.5 * (ua + ub)
        return -0.5 * ((tau_a * tau_b) / (tau_a + tau_b) + (tau_a * tau_b) ** 2 / (tau_a + tau_b) ** 3)
    if abs(ua - ub) < MIN_HUB_DIFF:
        tm = 0.5 * (tau_a + tau_b)
        return math.exp(-tm * r) * (1.0 / r + 0.6875 * tm + 0.1875 * r * tm ** 2
                                    + 0.02083333333333333333 * r ** 2 * tm ** 3)
    return _gsub(r, tau_a, tau_b) + _gsub(r, tau_b, tau_a)


def _gsub(r, t1, t2):
    return math.exp(-t1 * r) * ((0.5 * t2 ** 4 * t1 / (t1 ** 2 - t2 ** 2) ** 2)
                                - (t2 ** 6 - 3.0 * t2 ** 4 * t1 ** 2) / (r * (t1 ** 2 - t2 ** 2) ** 3))


def _gsub_prime(r, t1, t2):
    e = math.exp(-t1 * r)
    return (-t1 * e * ((0.5 * t2 ** 4 * t1 / (t1 ** 2 - t2 ** 2) ** 2)
                       - (t2 ** 6 - 3.0 * t2 ** 4 * t1 ** 2) / (r * (t1 ** 2 - t2 ** 2) ** 3))
            + e * (t2 ** 6 - 3.0 * t2 ** 4 * t1 ** 2) / (r ** 2 * (t1 ** 2 - t2 ** 2) ** 3))


def exp_gamma_prime(r, ua, ub):
    """d/dr of the short-range gamma, ``shortgammafuncs.F90:154-205`` (``expGammaPrime``)."""
    if r < TOL_SAME_DIST:
        return 0.0
    if abs(ua - ub) < MIN_HUB_DIFF:
        tm = 3.2 * 0.5 * (ua + ub)
        e = math.exp(-tm * r)
        return (-tm * e * (1.0 / r + 0.6875 * tm + 0.1875 * r * tm ** 2
                           + 0.02083333333333333333 * r ** 2 * tm ** 3)
                + e * (-1.0 / r ** 2 + 0.1875 * tm ** 2 + 2.0 * 0.02083333333333333333 * r * tm ** 3))
    return _gsub_prime(r, 3.2 * ua, 3.2 * ub) + _gsub_prime(r, 3.2 * ub, 3.2 * ua)


def exp_gamma_cutoff(u2, u1, cut_value=MIN_SHORT_GAMMA):
    """Distance beyond which the short gamma is below 1e-10, ``shortgammafuncs.F90:27-94``."""
    rab = 1.0
    while exp_gamma(rab, u2, u1) > cut_value:
        rab = 2.0 * rab
    min_cut = rab + 0.1
    max_cut = 0.5 * rab - 0.1
    max_g = exp_gamma(max_cut, u2, u1)
    min_g = exp_gamma(min_cut, u2, u1)
    lower_g = exp_gamma(min_cut, u2, u1)
    cut = max_cut + 0.1
    g = exp_gamma(cut, u2, u1)
    while (g - lower_g) > TOL_SHORT_GAMMA:
        max_cut = 0.5 * (cut + min_cut)
        if (max_g >= min_g) == (cut_value >= exp_gamma(max_cut, u2, u1)):
            min_cut = max_cut
            lower_g = exp_gamma(min_cut, u2, u1)
        else:
            cut = max_cut
            g = exp_gamma(cut, u2, u1)
    return min_cut


class Electrostatics:
    """Cluster 1/r (``dftb/coulomb.F90:537-585``, ``:704-733``) and short gamma
    (``dftb/shortgamma.F90:804-936``) for atom-resolved (non-orbital-resolved) Hubbard U."""

    def __init__(self, sys_: System):
        self.sys = sys_
        N = sys_.n_atom
        c = sys_.coords
        d = c[:, :, None] - c[:, None, :]
        r = np.sqrt(np.sum(d * d, axis=0))
        with np.errstate(divide="ignore"):
            inv = np.where(r > 0, 1.0 / np.where(r > 0, r, 1.0), 0.0)
        np.fill_diagonal(inv, 0.0)
        self.inv_r = inv
        self.r = r
        # short gamma matrix over pairs within the U-pair cutoff (and on-site)
        U = sys_.hubbu
        uniq = sorted(set(U.tolist()))
        cut = {}
        for a in uniq:
            for b in uniq:
                cut[(a, b)] = exp_gamma_cutoff(b, a)
        self.cutoffs = cut
        G = np.zeros((N, N))
        Gp = np.zeros((N, N))
        for i in range(N):
            G[i, i] = exp_gamma(0.0, U[i], U[i])
            for j in range(i + 1, N):
                rc = cut[(U[i], U[j])]
                if r[i, j] ** 2 <= rc * rc + TOL_SAME_DIST ** 2:
                    g = exp_gamma(r[i, j], U[j], U[i])
                    gp = exp_gamma_prime(r[i, j], U[j], U[i])
                    G[i, j] = G[j, i] = g
                    Gp[i, j] = Gp[j, i] = gp
        self.gshort = G
        self.gshort_prime = Gp

    def potential(self, dq_atom):
        """Atom potential V = (1/r) dq - gamma_short dq (shift per atom + per shell)."""
        return self.inv_r @ dq_atom - self.gshort @ dq_atom

    def energy(self, dq_atom):
        """E_SCC = 1/2 sum_A V_A dq_A (scc.F90:699-733 with coulomb.F90:376-405)."""
        return 0.5 * float(self.potential(dq_atom) @ dq_atom)

    def gradient_dc(self, dq_atom):
        """Double-counting gradient terms (scc.F90:794-843 -> shortgamma.F90:349-411,
        coulomb.F90:1140-1185): d/dR_A of 1/2 dq (1/r - gamma_short) dq at fixed dq."""
        c = self.sys.coords
        N = self.sys.n_atom
        d = c[:, :, None] - c[:, None, :]                       # R_A - R_B
        r3 = np.where(self.r > 0, self.r ** 3, 1.0)
        qq = dq_atom[:, None] * dq_atom[None, :]
        coul = -qq / r3
        np.fill_diagonal(coul, 0.0)
        rr = np.where(self.r > 0, self.r, 1.0)
        short = -qq * self.gshort_prime / rr
        np.fill_diagonal(short, 0.0)
        return np.einsum("kab,ab->ka", d, coul + short)


# ============================================================================ repulsive
def spline_rep_value(rep, r):
    """Energy and dE/dr of the spline repulsive, ``dftb/repulsive/splinerep.F90:136-266``."""
    if r < MIN_NEIGH_DIST or r >= rep.cutoff:
        return 0.0, 0.0
    c = rep.exp_coeffs
    if r < rep.x_start[0]:
        e = math.exp(-c[0] * r + c[1])
        return e + c[2], -c[0] * e
    xs = rep.x_start
    lo, hi = 0, len(xs)
    while lo < hi:                                   # search_asc_real_geq (math/binarysearch.F90:63)
        cur = lo + (hi - lo + 1) // 2
        if r - xs[cur - 1] >= -EPS:
            lo = cur
        else:
            hi = cur - 1
    im = lo                                           # 1-based
    dr = r - xs[im - 1]
    if im < len(xs):
        k = rep.sp_coeffs[im - 1]
        e = k[0]; xh = dr
        for t in range(1, 4):
            e += k[t] * xh; xh *= dr
        de = 0.0; xh = 1.0
        for t in range(1, 4):
            de += t * k[t] * xh; xh *= dr
        return e, de
    k = rep.last_coeffs
    e = k[0]; xh = dr
    for t in range(1, 6):
        e += k[t] * xh; xh *= dr
    de = 0.0; xh = 1.0
    for t in range(1, 6):
        de += t * k[t] * xh; xh *= dr
    return e, de


def repulsive(sys_: System):
    """E_rep and its gradient over pairs (dftb/repulsive/twobodyrep.F90:238-332)."""
    model = sys_.model
    ii, jj, r = pair_list(sys_.coords, model.rep_cutoff())
    e_tot = 0.0
    grad = np.zeros((3, sys_.n_atom))
    for p in range(len(ii)):
        i, j = ii[p], jj[p]
        rep = model.repulsives[(sys_.species[j], sys_.species[i])]
        e, de = spline_rep_value(rep, r[p])
        e_tot += e
        v = (sys_.coords[:, i] - sys_.coords[:, j]) / r[p]
        grad[:, i] += de * v
        grad[:, j] -= de * v
    return e_tot, grad


# ============================================================================ Fermi filling
def _neumaier(total, term, comp):
    tmp = total + term
    if abs(total) >= abs(term):
        comp += (total - tmp) + term
    else:
        comp += (term - tmp) + total
    return tmp, comp


def electron_count(ef, eig, kt):
    """``dftb/etemp.F90:196-285`` (Fermi branch): sum of 1/(1+exp((e-Ef)/kT)), Neumaier sum."""
    beta = 1.0 / kt
    tot, comp = 0.0, 0.0
    for e in eig:
        x = (e - ef) * beta
        tot, comp = _neumaier(tot, 1.0 / (1.0 + math.exp(x)) if x < 709 else 0.0, comp)
    return tot + comp


def electron_fill(eig, ef, kt):
    """``dftb/etemp.F90:294-452`` (Fermi branch): fillings, band energy, TS, E0."""
    beta = 1.0 / kt
    f = np.zeros(len(eig))
    eb, cb, ts, ct = 0.0, 0.0, 0.0, 0.0
    for j, e in enumerate(eig):
        x = (e - ef) * beta
        fj = 1.0 / (1.0 + math.exp(x)) if x < 709 else 0.0
        f[j] = fj
        if fj <= ELEC_TOL:
            break
        if EPS < fj < 1.0 - EPS:
            ts, ct = _neumaier(ts, -(fj * math.log(fj) + (1.0 - fj) * math.log(1.0 - fj)), ct)
        eb, cb = _neumaier(eb, fj * e, cb)
    eb += cb
    ts = (ts + ct) * kt
    return f, eb, ts, eb - 0.5 * ts


def middle_gap(eig, n_el):
    """``dftb/etemp.F90:481-525`` for one spin channel and one k-point."""
    order = np.argsort(eig, kind="stable")
    ind = 0
    n = 0.0
    while n < n_el:
        n += 1.0
        ind += 1
    ind = min(len(eig), ind + 1)
    return 0.5 * (eig[order[ind - 1]] + eig[order[ind - 2]])


def fermi_filling(eig, n_electrons, kt):
    """Spin-unpolarised filling: ``main.F90:4544-4649`` -> ``etemp.F90:59-191`` (``Efilling``).

    Returns (fillings x2, Ef, Eband x2, TS x2, E0 x2).
    """
    n_el = 0.5 * n_electrons
    eps2 = 2.0 * EPS
    eig = np.asarray(eig)
    if len(eig) <= n_el:
        ef = float(np.max(eig)) + 1000.0 * (kt + np.finfo(np.float32).eps)
        f, eb, ts, e0 = electron_fill(eig, ef, kt)
        return 2 * f, ef, 2 * eb, 2 * ts, 2 * e0
    if abs(n_el - round(n_el)) <= ELEC_TOL:
        ef = middle_gap(eig, n_el)
        ne = electron_count(ef, eig, kt)
        if abs(n_el - ne) <= ELEC_TOL_MAX:
            f, eb, ts, e0 = electron_fill(eig, ef, kt)
            return 2 * f, ef, 2 * eb, 2 * ts, 2 * e0
    up = float(eig[-1]) + 0.01
    lo = float(eig[0]) - 0.01
    nmax = electron_count(up, eig, kt)
    nmin = electron_count(lo, eig, kt)
    while nmin > n_el:
        lo = 2.0 * (lo - up) + lo
        nmin = electron_count(lo, eig, kt)
    while nmax < n_el:
        up = 2.0 * (up - lo) + lo
        nmax = electron_count(up, eig, kt)
    ef = 0.5 * (up + lo)
    ne = electron_count(ef, eig, kt)
    while abs(n_el - ne) > ELEC_TOL and abs(up - lo) >= max(abs(ef) * eps2, eps2):
        if (nmax >= nmin) == (n_el >= ne):
            lo = ef; nmin = ne
        else:
            up = ef; nmax = ne
        ef = 0.5 * (up + lo)
        ne = electron_count(ef, eig, kt)
    if abs(n_el - ne) > ELEC_TOL_MAX:
        raise RuntimeError("Fermi level search did not converge.")
    ne = electron_count(ef, eig, kt)
    f, eb, ts, e0 = electron_fill(eig, ef, kt)
    if n_el > eps2 and abs(n_el - ne) > eps2:
        f = f * n_el / ne
    return 2 * f, ef, 2 * eb, 2 * ts, 2 * e0


def n_levels(f):
    """Last level with |f| >= eps (densitymatrix.F90:544-550)."""
    idx = np.nonzero(np.abs(f) >= EPS)[0]
    return int(idx[-1]) + 1 if idx.size else 0


def density_matrix(C, f):
    """rho = C f C^T over the filled levels (densitymatrix.F90:530-591)."""
    k = n_levels(f)
    Ck = C[:, :k]
    return (Ck * f[:k]) @ Ck.T


def energy_density_matrix(C, f, eig):
    """W = C (f eps) C^T (densitymatrix.F90:664-733)."""
    k = n_levels(f)
    Ck = C[:, :k]
    return (Ck * (f[:k] * eig[:k])) @ Ck.T


def mulliken_orbital(rho, S):
    """q_mu = sum_nu rho_mu,nu S_mu,nu (populations.F90:120-191)."""
    return np.sum(rho * S, axis=1)


# ============================================================================ Broyden mixer
class BroydenMixer:
    """Modified Broyden mixing (Johnson 1988), ``mixer/broydenmixer.F90:180-342``."""

    def __init__(self, alpha=0.2, omega0=0.01, min_weight=1.0, max_weight=1e5, weight_fac=1e-2,
                 max_iter=100):
        self.alpha, self.omega0 = alpha, omega0
        self.min_w, self.max_w, self.wfac = min_weight, max_weight, weight_fac
        self.m_iter = max_iter
        self.reset()

    def reset(self):
        self.it = 0
        self.ww = []
        self.aa = np.zeros((self.m_iter, self.m_iter))
        self.dF = []
        self.uu = []
        self.q_last = None
        self.d_last = None

    def mix(self, q_in, q_diff):
        self.it += 1
        nn = self.it
        if nn > self.m_iter:
            raise RuntimeError("Broyden mixer: Maximal nr. of steps exceeded")
        q_in = np.array(q_in, dtype=np.float64)
        q_diff = np.asarray(q_diff, dtype=np.float64)
        if nn == 1:
            self.q_last = q_in.copy()
            self.d_last = q_diff.copy()
            return q_in + self.alpha * q_diff
        n1 = nn - 1
        w = math.sqrt(float(q_diff @ q_diff))
        w = self.wfac / w if w > self.wfac / self.max_w else self.max_w
        if w < self.min_w:
            w = self.min_w
        self.ww.append(w)
        df = q_diff - self.d_last
        inv_norm = max(math.sqrt(float(df @ df)), EPS)
        inv_norm = 1.0 / inv_norm
        df = inv_norm * df
        cc = np.zeros(n1)
        for i in range(n1 - 1):
            self.aa[i, n1 - 1] = float(self.dF[i] @ df)
            self.aa[n1 - 1, i] = self.aa[i, n1 - 1]
            cc[i] = self.ww[i] * float(self.dF[i] @ q_diff)
        self.aa[n1 - 1, n1 - 1] = 1.0
        cc[n1 - 1] = self.ww[n1 - 1] * float(df @ q_diff)
        wv = np.array(self.ww)
        beta = wv[:, None] * wv[None, :] * self.aa[:n1, :n1]
        beta[np.diag_indices(n1)] += self.omega0 ** 2
        lu, piv = scipy.linalg.lu_factor(beta)
        cc = scipy.linalg.lu_solve((lu, piv), cc, trans=1)
        self.dF.append(df)
        u = self.alpha * df + inv_norm * (q_in - self.q_last)
        self.q_last = q_in.copy()
        self.d_last = q_diff.copy()
        out = q_in + self.alpha * q_diff
        for i in range(n1 - 1):
            out = out - self.ww[i] * cc[i] * self.uu[i]
        out = out - self.ww[n1 - 1] * cc[n1 - 1] * u
        self.uu.append(u)
        return out


# ============================================================================ SCC driver
@dataclasses.dataclass
class SccResult:
    energies: dict
    ef: float
    eig: np.ndarray
    filling: np.ndarray
    q_out_atom: np.ndarray           # Mulliken populations per atom (electrons)
    q_out_orb: np.ndarray            # per orbital (n,)
    q_in_atom: np.ndarray
    n_iter: int
    converged: bool
    rho: np.ndarray
    C: np.ndarray
    potential: np.ndarray            # atom potentials from q_out
    history: list


def run_scc(sys_: System, kt=1e-3, scc_tol=1e-7, max_iter=100, mixer: Optional[BroydenMixer] = None,
            q_init_atom=None, H0S=None, net_charge=0.0):
    """SCC cycle, energies (``dftbplus/main.F90:1429-1563``; ``getenergies.F90:47-384``).

    Charges are mixed per atom (one unique U per species -> all orbitals of an atom equivalent,
    ``uniquehubbard.F90:126-160``); convergence is max|q_out - q_in| < scc_tol
    (``main.F90:4907-4908``).
    """
    model = sys_.model
    H0, S = build_h0_s(sys_) if H0S is None else H0S
    es = Electrostatics(sys_)
    e_rep, _ = repulsive(sys_)
    n_el = model.n_electrons(sys_.species, net_charge)
    mixer = mixer or BroydenMixer(max_iter=max_iter)
    mixer.reset()
    q_in = sys_.q0_atom.copy() if q_init_atom is None else np.array(q_init_atom, dtype=np.float64)
    conv = False
    hist = []
    for it in range(1, max_iter + 1):
        dq_in = q_in - sys_.q0_atom
        V = es.potential(dq_in)
        Vo = V[sys_.atom_of_orb]
        H = H0 + 0.5 * S * (Vo[:, None] + Vo[None, :])
        eig, C = scipy.linalg.eigh(H, S, driver="gvd")
        f, ef, eband, ts, e0 = fermi_filling(eig, n_el, kt)
        rho = density_matrix(C, f)
        q_orb = mulliken_orbital(rho, S)
        q_out = np.bincount(sys_.atom_of_orb, weights=q_orb, minlength=sys_.n_atom)
        dq_out = q_out - sys_.q0_atom
        V_out = es.potential(dq_out)
        e_nonscc = float(np.sum(rho * H0))
        e_scc = 0.5 * float(V_out @ dq_out)
        diff = q_out - q_in
        err = float(np.max(np.abs(diff)))
        conv = err < scc_tol
        e_total = e_nonscc + e_scc + e_rep
        hist.append(dict(iter=it, err=err, e_mermin=e_total - ts))
        if not conv and it != max_iter:
            q_in_next = mixer.mix(q_in, diff)
        else:
            q_in_next = q_in
        if conv:
            break
        q_in = q_in_next
    energies = dict(EnonSCC=e_nonscc, Escc=e_scc, Erep=e_rep, Eband=eband, TS=ts, E0=e0,
                    Etotal=e_total, EMermin=e_total - ts)
    return SccResult(energies=energies, ef=ef, eig=eig, filling=f, q_out_atom=q_out, q_out_orb=q_orb,
                     q_in_atom=q_in, n_iter=it, converged=conv, rho=rho, C=C, potential=V_out,
                     history=hist)


def fd_block_derivs(sys_: System, ii, jj):
    """Central-difference dH0/dR_i and dS/dR_i blocks, ``dftb/nonscc.F90:428-484``.

    Displaced vectors R_j - R_i -/+ delta e_k (delta = eps^(1/4)); returns lists
    dh[p] (3, nOrb_j, nOrb_i), ds[p] likewise.
    """
    base = sys_.coords[:, jj] - sys_.coords[:, ii]
    P = len(ii)
    dh = np.zeros((3,), dtype=object)
    tmp_h = {}
    tmp_s = {}
    for k in range(3):
        for sgn_idx, sgn in ((1, +1.0), (2, -1.0)):
            v = base.copy()
            v[k] = v[k] + sgn * FD_DELTA
            hb, sb = diatomic_blocks(sys_, ii, jj, vec_override=v)
            tmp_h[(k, sgn_idx)] = hb
            tmp_s[(k, sgn_idx)] = sb
    dhs, dss = [], []
    for p in range(P):
        dhs.append(np.stack([(tmp_h[(k, 2)][p] - tmp_h[(k, 1)][p]) / (2.0 * FD_DELTA) for k in range(3)]))
        dss.append(np.stack([(tmp_s[(k, 2)][p] - tmp_s[(k, 1)][p]) / (2.0 * FD_DELTA) for k in range(3)]))
    return dhs, dss


def gradients(sys_: System, res: SccResult, kt=1e-3):
    """Total energy gradient (not forces), ``main.F90:7058-7438``:
    ``derivative_blockEuclidean`` (forces.F90:548-669) + SCC double counting + repulsive."""
    model = sys_.model
    C, f, eig = res.C, res.filling, res.eig
    W = energy_density_matrix(C, f, eig)
    rho = res.rho
    V = res.potential
    ii, jj, r = pair_list(sys_.coords, model.sk_cutoff())
    dhs, dss = fd_block_derivs(sys_, ii, jj)
    g = np.zeros((3, sys_.n_atom))
    for p in range(len(ii)):
        i, j = ii[p], jj[p]
        oi, oj = sys_.off[i], sys_.off[j]
        ni, nj = sys_.off[i + 1] - oi, sys_.off[j + 1] - oj
        rb = rho[oj:oj + nj, oi:oi + ni]
        wb = W[oj:oj + nj, oi:oi + ni]
        vsum = 0.5 * (V[i] + V[j])
        dt = 2.0 * (np.einsum("kab,ab->k", dhs[p], rb) - np.einsum("kab,ab->k", dss[p], wb)) \
            + 2.0 * vsum * np.einsum("kab,ab->k", dss[p], rb)
        g[:, i] += dt
        g[:, j] -= dt
    es = Electrostatics(sys_)
    dq_out = res.q_out_atom - sys_.q0_atom
    g += es.gradient_dc(dq_out)
    _, grep = repulsive(sys_)
    g += grep
    return g


def coulomb_potential_prime(coords, dq_atom):
    """d V_B / d R_A,k of the cluster 1/r potential V = (1/r) dq at fixed charges,
    ``dftb/coulomb.F90:2691-2718`` (``invRPrimeCluster``): out[B, k, A]."""
    N = coords.shape[1]
    out = np.zeros((N, 3, N))
    for a in range(N):
        for b in range(N):
            if a == b:
                continue
            d = coords[:, b] - coords[:, a]
            f = d / np.linalg.norm(d) ** 3
            out[b, :, a] = dq_atom[a] * f
            out[a, :, a] += dq_atom[b] * f
    return out
