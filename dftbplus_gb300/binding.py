"""ctypes binding of libdftbgpu.so (C-ABI in include/dftbgpu.h) and the user-facing calculator.

``DftbGpu`` mirrors the reference's Python API (tools/pythonapi/src/dftbplus/dftbplus.py:25-399,
class ``DftbPlus``): ``set_geometry``, ``get_nr_atoms``, ``get_energy`` (Mermin free energy),
``get_gradients`` (gradients, not forces) and ``get_gross_charges`` (q0 - q per atom), with the
same units (Bohr, Hartree) and the same error behaviour (an exception on failure). There is no CPU
path: without the CUDA library or a GPU, construction fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .model import Model

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdftbgpu.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
C_float = C.c_float
C_double = C.c_double   # for methods whose argument C shadows the ctypes module

PREC_FP64 = 0
PREC_MIXED = 1
ITER_PERTURB = 2   # scc_history: perturbative update around the last FP64 iteration

ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "overlap not positive definite",
          4: "SCC not converged", 5: "Fermi level search failed", 6: "iteration cap reached",
          7: "invalid call order", 8: "no CUDA device"}


class SccOpts(C.Structure):
    _fields_ = [("kT", C.c_double), ("scc_tol", C.c_double), ("max_iter", C.c_int), ("min_iter", C.c_int),
                ("mix_alpha", C.c_double), ("mix_omega0", C.c_double), ("mix_min_weight", C.c_double),
                ("mix_max_weight", C.c_double), ("mix_weight_fac", C.c_double), ("net_charge", C.c_double),
                ("precision", C.c_int), ("convergent_only", C.c_int), ("mixed_switch_tol", C.c_double)]


class Energies(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("EnonSCC", "Escc", "Erep", "Eband", "TS", "E0", "Etotal", "EMermin")]

    def as_dict(self) -> dict:
        return {k: float(getattr(self, k)) for k, _ in self._fields_}


# name -> (restype, argtypes); every entry point declared in include/dftbgpu.h
SIGNATURES = {
    "dftbgpu_default_opts": (None, [C.POINTER(SccOpts)]),
    "dftbgpu_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "dftbgpu_destroy": (C.c_int, [C.c_void_p]),
    "dftbgpu_last_error": (C.c_char_p, [C.c_void_p]),
    "dftbgpu_set_model": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _ip, _ip, _dp, _dp, _ip, _dp]),
    "dftbgpu_set_geometry": (C.c_int, [C.c_void_p, C.c_int, _dp, _ip]),
    "dftbgpu_set_geometry_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, _ip]),
    "dftbgpu_scc": (C.c_int, [C.c_void_p, C.POINTER(SccOpts), _dp, C.POINTER(Energies), _dp, _dp, _dp, _dp, _ip, _ip]),
    "dftbgpu_scc_history": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _ip, _dp]),
    "dftbgpu_gradients": (C.c_int, [C.c_void_p, _dp]),
    "dftbgpu_batch_set_geometries": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, _ip]),
    "dftbgpu_batch_set_geometries_dev": (C.c_int, [C.c_void_p, C.c_int, _ip, C.c_void_p, _ip]),
    "dftbgpu_batch_scc": (C.c_int, [C.c_void_p, C.POINTER(SccOpts), C.c_void_p, _dp, _ip, _ip]),
    "dftbgpu_batch_gradients": (C.c_int, [C.c_void_p, _dp]),
    "dftbgpu_grad_params": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "dftbgpu_gradients_dev": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dftbgpu_n_orbitals": (C.c_int, [C.c_void_p, _ip]),
    "dftbgpu_get_orbital_populations": (C.c_int, [C.c_void_p, _dp]),
    "dftbgpu_sygvd": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp]),
    "dftbgpu_get_matrix": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "dftbgpu_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "dftbgpu_test_dgemm": (C.c_int, [C.c_void_p, C.c_char, C.c_char, C.c_int, C.c_int, C.c_int, C.c_double,
                                     _dp, _dp, C.c_double, _dp, C.c_int]),
    "dftbgpu_set_tensor_cores": (C.c_int, [C.c_int]),
    "dftbgpu_set_fp64_emulation": (C.c_int, [C.c_int]),
    "dftbgpu_set_two_stage": (C.c_int, [C.c_int]),
    "dftbgpu_test_twostage": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, _dp, _dp, _dp]),
    "dftbgpu_set_panel_mode": (C.c_int, [C.c_int]),
    "dftbgpu_set_dc_staging": (C.c_int, [C.c_int]),
    "dftbgpu_set_geometry_neighbours": (C.c_int, [C.c_void_p, C.c_int, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                  C.POINTER(C.c_int), C.c_int]),
    "dftbgpu_set_digit_gemm_kernel": (C.c_int, [C.c_int]),
    "dftbgpu_test_onestage": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, _dp, _dp, _dp]),
    "dftbgpu_test_sgemm": (C.c_int, [C.c_void_p, C.c_char, C.c_char, C.c_int, C.c_int, C.c_int, C.c_float,
                                     C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.c_int, C.c_float,
                                     C.POINTER(C.c_float), C.c_int, C.c_int]),
    "dftbgpu_test_dgemm_tc": (C.c_int, [C.c_void_p, C.c_char, C.c_char, C.c_int, C.c_int, C.c_int, C.c_double,
                                        _dp, C.c_int, _dp, C.c_int, C.c_double, _dp, C.c_int, C.c_int]),
    "dftbgpu_test_gemm_tc": (C.c_int, [C.c_void_p, C.c_char, C.c_char, C.c_int, C.c_int, C.c_int, C.c_float,
                                       C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.c_int, C.c_float,
                                       C.POINTER(C.c_float), C.c_int, C.c_int]),
    "dftbgpu_test_sgemm_digits": (C.c_int, [C.c_void_p, C.c_char, C.c_char, C.c_int, C.c_int, C.c_int, C.c_float,
                                            C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.c_int, C.c_float,
                                            C.POINTER(C.c_float), C.c_int, C.c_int]),
    "dftbgpu_set_fp32_emulation": (C.c_int, [C.c_int]),
    "dftbgpu_test_tridiag": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp]),
    "dftbgpu_test_stedc": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp]),
    "dftbgpu_profile_enable": (C.c_int, [C.c_void_p, C.c_int]),
    "dftbgpu_profile_read": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, C.POINTER(C.c_longlong)]),
    "dftbgpu_stedc_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}

PHASES = ["h0s_cholesky", "potential_h", "transform", "tridiag", "dc_tridiag", "fermi", "back_transform",
          "density", "mulliken_energy", "broyden", "gradients", "perturbation", "gemm_fp64", "gemm_fp32",
          "gemm_tc_fp64", "k_sytrd_panel", "k_panel_qr", "k_chase", "k_back_q2", "k_sytrd_panel32"]

_lib = None


def load_library(path: str = LIB_PATH):
    """Load libdftbgpu.so (raises if it is missing: there is no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} not found: build it with dftbplus_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _p(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class DftbGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dftbgpu error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Context:
    """Thin owner of a dftbgpu_ctx handle."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.dftbgpu_create(C.byref(h), device)
        if rc != 0:
            raise DftbGpuError(rc, "dftbgpu_create failed")
        self.h = h

    def check(self, rc: int):
        if rc != 0:
            msg = self.lib.dftbgpu_last_error(self.h)
            raise DftbGpuError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.dftbgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_model(self, model: Model):
        self.set_model_packed(model.pack())

    def set_model_packed(self, p: dict):
        """Upload a model in the flat layout of Model.pack() (arrays may be replaced, e.g. tables)."""
        self._model_arrays = p  # keep alive
        a = {k: np.ascontiguousarray(v) for k, v in p.items() if isinstance(v, np.ndarray)}
        self.check(self.lib.dftbgpu_set_model(
            self.h, p["n_species"], _p(a["n_shell"], C.c_int), _p(a["ang_shell"], C.c_int),
            _p(a["onsite"], C.c_double), _p(a["hubbu"], C.c_double), _p(a["ref_occ"], C.c_double),
            _p(a["sk_dist"], C.c_double), _p(a["sk_rows"], C.c_int), _p(a["sk_nint"], C.c_int),
            _p(a["sk_ham"], C.c_double), _p(a["sk_over"], C.c_double), _p(a["rep_nspline"], C.c_int),
            _p(a["rep_data"], C.c_double)))

    def set_geometry(self, coords: np.ndarray, species: np.ndarray):
        xyz = np.ascontiguousarray(np.asarray(coords, dtype=np.float64).T)  # (N, 3): x,y,z per atom
        sp = np.ascontiguousarray(species, dtype=np.int32)
        self.check(self.lib.dftbgpu_set_geometry(self.h, len(sp), _p(xyz, C.c_double), _p(sp, C.c_int)))
        self.natom = len(sp)
        n = C.c_int()
        self.check(self.lib.dftbgpu_n_orbitals(self.h, C.byref(n)))
        self.norb = n.value

    def set_geometry_neighbours(self, coords: np.ndarray, species: np.ndarray, nneigh: np.ndarray,
                                ineigh: np.ndarray):
        """Geometry with the host's neighbour list: nneigh[natom] neighbours within the SK cutoff per
        atom, ineigh (natom, maxneigh + 1) their 0-based indices, column 0 the atom itself (the
        layout of the reference's iNeighbour(0:maxNeighbour, nAtom))."""
        xyz = np.ascontiguousarray(np.asarray(coords, dtype=np.float64).T)
        sp = np.ascontiguousarray(species, dtype=np.int32)
        nn = np.ascontiguousarray(nneigh, dtype=np.int32)
        ii = np.ascontiguousarray(ineigh, dtype=np.int32)
        if ii.ndim != 2 or ii.shape[0] != len(sp) or len(nn) != len(sp):
            raise ValueError("ineigh must be (natom, maxneigh + 1) and nneigh (natom,)")
        self.check(self.lib.dftbgpu_set_geometry_neighbours(self.h, len(sp), _p(xyz, C.c_double), _p(sp, C.c_int),
                                                            _p(nn, C.c_int), _p(ii, C.c_int), ii.shape[1] - 1))
        self.natom = len(sp)
        n = C.c_int()
        self.check(self.lib.dftbgpu_n_orbitals(self.h, C.byref(n)))
        self.norb = n.value

    def scc(self, opts: SccOpts, q_init: Optional[np.ndarray] = None):
        en = Energies()
        ef = C.c_double()
        eig = np.zeros(self.norb)
        fill = np.zeros(self.norb)
        qout = np.zeros(self.natom)
        nit = C.c_int()
        conv = C.c_int()
        qi = None
        if q_init is not None:
            qi = np.ascontiguousarray(q_init, dtype=np.float64)
        self.check(self.lib.dftbgpu_scc(self.h, C.byref(opts), _p(qi, C.c_double) if qi is not None else None,
                                        C.byref(en), C.byref(ef), _p(eig, C.c_double), _p(fill, C.c_double),
                                        _p(qout, C.c_double), C.byref(nit), C.byref(conv)))
        return dict(energies=en.as_dict(), ef=ef.value, eig=eig, filling=fill, q_out=qout, n_iter=nit.value,
                    converged=bool(conv.value))

    def gradients(self) -> np.ndarray:
        g = np.zeros(3 * self.natom)
        self.check(self.lib.dftbgpu_gradients(self.h, _p(g, C.c_double)))
        return g.reshape(self.natom, 3).T.copy()

    def grad_params(self):
        """dE/d(sk_ham), dE/d(sk_over) (packed table layout) and dE/dU per species."""
        p = self._model_arrays
        gh = np.zeros(len(p["sk_ham"]))
        go = np.zeros(len(p["sk_over"]))
        gu = np.zeros(p["n_species"])
        self.check(self.lib.dftbgpu_grad_params(self.h, _p(gh, C.c_double), _p(go, C.c_double), _p(gu, C.c_double)))
        return gh, go, gu

    def orbital_populations(self) -> np.ndarray:
        q = np.zeros(self.norb)
        self.check(self.lib.dftbgpu_get_orbital_populations(self.h, _p(q, C.c_double)))
        return q

    def matrix(self, which: int) -> np.ndarray:
        out = np.zeros((self.norb, self.norb), order="F")
        self.check(self.lib.dftbgpu_get_matrix(self.h, which, _p(out, C.c_double)))
        return out

    def sygvd(self, a: np.ndarray, b: np.ndarray):
        n = a.shape[0]
        A = np.asfortranarray(a, dtype=np.float64).copy(order="F")
        B = np.asfortranarray(b, dtype=np.float64).copy(order="F")
        w = np.zeros(n)
        self.check(self.lib.dftbgpu_sygvd(self.h, n, _p(A, C.c_double), _p(B, C.c_double), _p(w, C.c_double)))
        return w, A, B

    def test_dgemm(self, ta, tb, a, b, c, alpha=1.0, beta=0.0, flags=0):
        m, n = c.shape
        k = a.shape[1] if ta == "N" else a.shape[0]
        A = np.asfortranarray(a, dtype=np.float64); B = np.asfortranarray(b, dtype=np.float64)
        Cm = np.asfortranarray(c, dtype=np.float64).copy(order="F")
        self.check(self.lib.dftbgpu_test_dgemm(self.h, ta.encode(), tb.encode(), m, n, k, alpha,
                                               _p(A, C.c_double), _p(B, C.c_double), beta, _p(Cm, C.c_double), flags))
        return Cm

    def test_tridiag(self, a):
        n = a.shape[0]
        A = np.asfortranarray(a, dtype=np.float64)
        d = np.zeros(n); e = np.zeros(max(n - 1, 1))
        self.check(self.lib.dftbgpu_test_tridiag(self.h, n, _p(A, C.c_double), _p(d, C.c_double), _p(e, C.c_double)))
        return d, e[:n - 1]

    def test_twostage(self, a, fp32=False):
        """Two-stage reduction of the symmetric a: (d, e, q) with a = q tridiag(d, e) q^T."""
        n = a.shape[0]
        A = np.asfortranarray(a, dtype=np.float64)
        d = np.zeros(n); e = np.zeros(max(n - 1, 1))
        q = np.zeros((n, n), order="F")
        self.check(self.lib.dftbgpu_test_twostage(self.h, n, _p(A, C.c_double), 1 if fp32 else 0, _p(d, C.c_double),
                                                  _p(e, C.c_double), _p(q, C.c_double)))
        return d, e[:n - 1], q

    def test_onestage(self, a, fp32=False):
        """One-stage reduction of the symmetric a: (d, e, q) with a = q tridiag(d, e) q^T."""
        n = a.shape[0]
        A = np.asfortranarray(a, dtype=np.float64)
        d = np.zeros(n); e = np.zeros(max(n - 1, 1))
        q = np.zeros((n, n), order="F")
        self.check(self.lib.dftbgpu_test_onestage(self.h, n, _p(A, C.c_double), 1 if fp32 else 0, _p(d, C.c_double),
                                                  _p(e, C.c_double), _p(q, C.c_double)))
        return d, e[:n - 1], q

    def test_stedc(self, d, e):
        n = len(d)
        dd = np.array(d, dtype=np.float64); ee = np.zeros(max(n - 1, 1)); ee[:n - 1] = e
        q = np.zeros((n, n), order="F")
        self.check(self.lib.dftbgpu_test_stedc(self.h, n, _p(dd, C.c_double), _p(ee, C.c_double), _p(q, C.c_double)))
        return dd, q

    def kernel_launches(self) -> int:
        return int(self.lib.dftbgpu_kernel_launches(self.h))

    # -------------------------------------------------------------- batched form
    def batch_set_geometries(self, coords_list, species_list):
        """Many independent molecules: coords_list[i] is (3, nat_i) in Bohr, species_list[i] (nat_i,)."""
        off = np.zeros(len(coords_list) + 1, dtype=np.int32)
        off[1:] = np.cumsum([len(sp) for sp in species_list])
        xyz = np.ascontiguousarray(np.concatenate([np.asarray(c).T for c in coords_list]), dtype=np.float64)
        sp = np.ascontiguousarray(np.concatenate(species_list), dtype=np.int32)
        self.check(self.lib.dftbgpu_batch_set_geometries(self.h, len(coords_list), _p(off, C.c_int),
                                                         _p(xyz, C.c_double), _p(sp, C.c_int)))
        self.batch_atom_off = off
        return off

    def batch_set_geometries_dev(self, atom_off: np.ndarray, coords_dev_ptr: int, species: np.ndarray):
        """Batched geometries with the (natom, 3) coordinates already on the device."""
        off = np.ascontiguousarray(atom_off, dtype=np.int32)
        sp = np.ascontiguousarray(species, dtype=np.int32)
        self.check(self.lib.dftbgpu_batch_set_geometries_dev(self.h, len(off) - 1, _p(off, C.c_int),
                                                             C.c_void_p(coords_dev_ptr), _p(sp, C.c_int)))
        self.batch_atom_off = off

    def batch_scc(self, opts: SccOpts):
        nmol = len(self.batch_atom_off) - 1
        en = (Energies * nmol)()
        qout = np.zeros(int(self.batch_atom_off[-1]))
        nit = np.zeros(nmol, dtype=np.int32)
        conv = np.zeros(nmol, dtype=np.int32)
        self.check(self.lib.dftbgpu_batch_scc(self.h, C.byref(opts), C.cast(en, C.c_void_p), _p(qout, C.c_double),
                                              _p(nit, C.c_int), _p(conv, C.c_int)))
        return dict(energies=[e.as_dict() for e in en], q_out=qout, n_iter=nit, converged=conv.astype(bool))

    def batch_gradients(self):
        """Energy gradients per molecule, list of (3, nat_i) arrays."""
        off = self.batch_atom_off
        g = np.zeros(3 * int(off[-1]))
        self.check(self.lib.dftbgpu_batch_gradients(self.h, _p(g, C.c_double)))
        g = g.reshape(-1, 3).T
        return [g[:, off[i]:off[i + 1]].copy() for i in range(len(off) - 1)]

    def test_gemm_tc(self, ta, tb, A, B, C=None, alpha=1.0, beta=0.0, flags=0):
        """C = alpha op(A) op(B) + beta C on the tensor cores (float32, column-major)."""
        A = np.asfortranarray(A, dtype=np.float32)
        B = np.asfortranarray(B, dtype=np.float32)
        m = A.shape[1] if ta == "T" else A.shape[0]
        k = A.shape[0] if ta == "T" else A.shape[1]
        n = B.shape[0] if tb == "T" else B.shape[1]
        Cm = np.zeros((m, n), dtype=np.float32, order="F") if C is None else np.array(C, dtype=np.float32, order="F")
        self.check(self.lib.dftbgpu_test_gemm_tc(self.h, ta.encode(), tb.encode(), m, n, k, alpha,
                                                 _p(A, C_float), A.shape[0], _p(B, C_float), B.shape[0], beta,
                                                 _p(Cm, C_float), m, flags))
        return Cm

    def test_sgemm_digits(self, ta, tb, A, B, C=None, alpha=1.0, beta=0.0, flags=0):
        """C = alpha op(A) op(B) + beta C as exact BF16 digit-slice products on the tensor cores
        (FP32-class; float32, column-major)."""
        A = np.asfortranarray(A, dtype=np.float32)
        B = np.asfortranarray(B, dtype=np.float32)
        m = A.shape[1] if ta == "T" else A.shape[0]
        k = A.shape[0] if ta == "T" else A.shape[1]
        n = B.shape[0] if tb == "T" else B.shape[1]
        Cm = np.zeros((m, n), dtype=np.float32, order="F") if C is None else np.array(C, dtype=np.float32, order="F")
        self.check(self.lib.dftbgpu_test_sgemm_digits(self.h, ta.encode(), tb.encode(), m, n, k, alpha,
                                                      _p(A, C_float), A.shape[0], _p(B, C_float), B.shape[0], beta,
                                                      _p(Cm, C_float), m, flags))
        return Cm

    def test_sgemm(self, ta, tb, A, B, C=None, alpha=1.0, beta=0.0, flags=0):
        """C = alpha op(A) op(B) + beta C with the library's FP32 FMA GEMM (float32, column-major)."""
        A = np.asfortranarray(A, dtype=np.float32)
        B = np.asfortranarray(B, dtype=np.float32)
        m = A.shape[1] if ta == "T" else A.shape[0]
        k = A.shape[0] if ta == "T" else A.shape[1]
        n = B.shape[0] if tb == "T" else B.shape[1]
        Cm = np.zeros((m, n), dtype=np.float32, order="F") if C is None else np.array(C, dtype=np.float32, order="F")
        self.check(self.lib.dftbgpu_test_sgemm(self.h, ta.encode(), tb.encode(), m, n, k, alpha,
                                               _p(A, C_float), A.shape[0], _p(B, C_float), B.shape[0], beta,
                                               _p(Cm, C_float), m, flags))
        return Cm

    def test_dgemm_tc(self, ta, tb, A, B, C=None, alpha=1.0, beta=0.0, flags=0):
        """C = alpha op(A) op(B) + beta C as exact BF16 digit-slice products on the tensor cores
        (float64 in and out, column-major)."""
        A = np.asfortranarray(A, dtype=np.float64)
        B = np.asfortranarray(B, dtype=np.float64)
        m = A.shape[1] if ta == "T" else A.shape[0]
        k = A.shape[0] if ta == "T" else A.shape[1]
        n = B.shape[0] if tb == "T" else B.shape[1]
        Cm = np.zeros((m, n), order="F") if C is None else np.array(C, dtype=np.float64, order="F")
        self.check(self.lib.dftbgpu_test_dgemm_tc(self.h, ta.encode(), tb.encode(), m, n, k, alpha,
                                                  _p(A, C_double), A.shape[0], _p(B, C_double), B.shape[0], beta,
                                                  _p(Cm, C_double), m, flags))
        return Cm

    def scc_history(self) -> dict:
        """Per-iteration record of the last SCC call: electronic energy, SCC error, precision form
        (PREC_FP64 / PREC_MIXED for an FP32 eigensolve) and host milliseconds."""
        n = int(self.lib.dftbgpu_scc_history(self.h, 0, None, None, None, None))
        e, err, ms = np.zeros(n), np.zeros(n), np.zeros(n)
        prec = np.zeros(n, dtype=np.int32)
        self.lib.dftbgpu_scc_history(self.h, n, _p(e, C.c_double), _p(err, C.c_double), _p(prec, C.c_int),
                                     _p(ms, C.c_double))
        return {"energy": e, "error": err, "precision": prec, "ms": ms}

    def profile(self, enable: bool):
        self.check(self.lib.dftbgpu_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        n = len(PHASES)
        ms = np.zeros(n); fl = np.zeros(n); calls = np.zeros(n, dtype=np.int64)
        self.lib.dftbgpu_profile_read(self.h, n, _p(ms, C.c_double), _p(fl, C.c_double),
                                      calls.ctypes.data_as(C.POINTER(C.c_longlong)))
        return {name: dict(ms=float(ms[i]), flops=float(fl[i]), calls=int(calls[i])) for i, name in enumerate(PHASES)}

    def set_geometry_dev(self, coords_dev_ptr: int, species: np.ndarray):
        sp = np.ascontiguousarray(species, dtype=np.int32)
        self.check(self.lib.dftbgpu_set_geometry_dev(self.h, len(sp), C.c_void_p(coords_dev_ptr), _p(sp, C.c_int)))
        self.natom = len(sp)
        n = C.c_int()
        self.check(self.lib.dftbgpu_n_orbitals(self.h, C.byref(n)))
        self.norb = n.value

    def scc_lite(self, opts: SccOpts) -> dict:
        """SCC returning only energies and iteration count (no host copies of vectors)."""
        en = Energies()
        nit = C.c_int()
        conv = C.c_int()
        self.check(self.lib.dftbgpu_scc(self.h, C.byref(opts), None, C.byref(en), None, None, None, None,
                                        C.byref(nit), C.byref(conv)))
        return dict(energies=en.as_dict(), n_iter=nit.value, converged=bool(conv.value))

    def gradients_dev(self, grad_dev_ptr: int):
        self.check(self.lib.dftbgpu_gradients_dev(self.h, C.c_void_p(grad_dev_ptr)))


def set_tensor_cores(enable: bool) -> bool:
    """Route the large FP32 products of the mixed form to the tcgen05 tensor cores (process-wide)."""
    return bool(load_library().dftbgpu_set_tensor_cores(1 if enable else 0))


def set_fp32_emulation(enable: bool) -> bool:
    """Run the FP32 products of the mixed form's FP32 eigensolves as exact BF16 digit-slice products on
    the tensor cores (process-wide, on by default); returns the previous setting."""
    return bool(load_library().dftbgpu_set_fp32_emulation(1 if enable else 0))


def set_fp64_emulation(enable: bool) -> bool:
    """Run the mixed form's FP64 products as exact BF16 digit-slice products on the tensor cores
    (process-wide, on by default); returns the previous setting."""
    return bool(load_library().dftbgpu_set_fp64_emulation(1 if enable else 0))


def set_digit_gemm_kernel(mode) -> int:
    """Kernel of the FP64-class tensor-core products (process-wide): 0 single-stage (the default),
    1 pipelined with TMA loads. Returns the previous mode."""
    m = int(mode)
    prev = load_library().dftbgpu_set_digit_gemm_kernel(m)
    if prev < 0:
        raise ValueError(f"digit GEMM kernel {mode!r}: expected 0 or 1")
    return prev


def set_panel_mode(mode) -> int:
    """Panel kernel of the one-stage tridiagonalisation (process-wide): 0 trailing matrix re-read
    per column, 1 resident tiles per panel (the default), 2 resident tiles with small limits (tests).
    Returns the previous mode."""
    m = int(mode)
    prev = load_library().dftbgpu_set_panel_mode(m)
    if prev < 0:
        raise ValueError(f"panel mode {mode!r}: expected 0, 1 or 2")
    return prev


def set_dc_staging(enable: bool) -> bool:
    """Deflation of the tridiagonal divide and conquer (process-wide): True (the default) stages each
    merge that fits in shared memory, False runs every merge in global memory. Returns the previous
    setting."""
    return bool(load_library().dftbgpu_set_dc_staging(1 if enable else 0))


def set_two_stage(mode) -> int:
    """Reduction of the FP32 eigensolves of the mixed form (process-wide): 0 / False one-stage,
    1 / True two-stage (band, then bulge chasing), 2 automatic by size (the default). Returns the
    previous mode."""
    m = int(mode)
    prev = load_library().dftbgpu_set_two_stage(m)
    if prev < 0:
        raise ValueError(f"two-stage mode {mode!r}: expected 0, 1 or 2")
    return prev


def default_opts(**kw) -> SccOpts:
    o = SccOpts()
    load_library().dftbgpu_default_opts(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class DftbGpu:
    """SCC-DFTB calculator on one GB300, API-compatible with the reference's ``DftbPlus`` for
    the non-periodic energy/gradient/charge queries."""

    # dftbgpu_scc accepts at most this many SCC iterations (the Broyden history of the device mixer
    # lives in one CTA's shared memory); geometry drivers clamp their iteration limits to it
    MAX_SCC_ITER = 150

    def __init__(self, model: Model, coords: np.ndarray, species: np.ndarray, kT: float = 1e-3,
                 scc_tol: float = 1e-7, max_iter: int = 100, mixing: float = 0.2, device: int = 0,
                 precision: int = PREC_FP64):
        self.ctx = Context(device)
        self.ctx.set_model(model)
        self.model = model
        self.species = np.asarray(species, dtype=np.int32)
        self.opts = default_opts(kT=kT, scc_tol=scc_tol, max_iter=max_iter, mix_alpha=mixing,
                                 precision=precision)
        self._q_init = None      # atomic populations to start the SCC from (None: neutral atoms)
        self.set_geometry(coords)

    def set_geometry(self, coords, latvecs=None):
        if latvecs is not None:
            raise ValueError("periodic geometries are not supported by this engine")
        self.coords = np.asarray(coords, dtype=np.float64)
        self.ctx.set_geometry(self.coords, self.species)
        self._res = None
        self._grad = None

    def _ensure(self):
        if self._res is None:
            self._res = self.ctx.scc(self.opts, q_init=self._q_init)

    def _orbitals_per_atom(self):
        return [self.model.species[s].n_orb for s in self.species]

    def read_charges(self, path: str) -> None:
        """Start the next SCC cycle from a reference charge restart file (``charges.dat`` /
        ``charges.bin``, ``ReadInitialCharges = Yes``) instead of the neutral reference charges."""
        from .restart import read_charges
        n_orb = self._orbitals_per_atom()
        q0 = sum(sum(self.model.species[s].occ) for s in self.species)
        q = read_charges(path, n_orb, n_el=q0 - self.opts.net_charge)
        offs = np.concatenate([[0], np.cumsum(n_orb)])
        self._q_init = np.add.reduceat(q, offs[:-1]) if len(q) else q
        self._res = None
        self._grad = None

    def write_charges(self, path: str) -> None:
        """Write the converged orbital populations as a reference charge restart file (format 8;
        ``.bin`` binary, otherwise ASCII), which DFTB+ reads with ``ReadInitialCharges = Yes``."""
        from .restart import write_charges
        self._ensure()
        write_charges(path, self.ctx.orbital_populations(), self._orbitals_per_atom())

    def get_nr_atoms(self) -> int:
        return int(len(self.species))

    def get_energy(self) -> float:
        self._ensure()
        return self._res["energies"]["EMermin"]

    def get_energies(self) -> dict:
        self._ensure()
        return dict(self._res["energies"])

    def get_gradients(self) -> np.ndarray:
        """(natom, 3) gradients in Hartree/Bohr (same layout as DftbPlus.get_gradients)."""
        self._ensure()
        if self._grad is None:
            self._grad = self.ctx.gradients().T.copy()
        return self._grad

    def get_gross_charges(self) -> np.ndarray:
        self._ensure()
        q0 = np.array([sum(self.model.species[s].occ) for s in self.species])
        return q0 - self._res["q_out"]

    def scc_info(self) -> dict:
        self._ensure()
        return dict(self._res)

    def close(self):
        self.ctx.close()
