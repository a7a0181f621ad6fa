"""Test infrastructure (oracle only): ctypes access to the reference's own hot-path C++
(CIStrings, CISigmaBuilder, CISpinAdapter) compiled by ``oracle/build_ref.sh`` into
``oracle/_ref/libforte2_ref.so``.

Only ``tests/`` and the golden-fixture generator use this module; the GPU product never
imports it. The library exists only where the reference sources were available to compile
(it is not part of the repository history), so callers must handle ``ReferenceUnavailable``.
"""

from __future__ import annotations

import ctypes as C
import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libforte2_ref.so")


class ReferenceUnavailable(RuntimeError):
    pass


_lib = None

_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def numpy_openblas_path():
    import numpy

    libs = glob.glob(
        os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs", "libscipy_openblas64_*.so")
    )
    return libs[0] if libs else None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ReferenceUnavailable(f"{LIB_PATH} not built (oracle/build_ref.sh)")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.ref_last_error.restype = C.c_char_p
    L.ref_strings_new.restype = vp
    L.ref_strings_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _i32p, C.c_int, _i32p,
                                  C.c_int, _i32p, C.POINTER(C.c_int)]
    L.ref_strings_free.argtypes = [vp]
    L.ref_strings_info.argtypes = [vp, _i64p]
    L.ref_strings_blocks.argtypes = [vp, _i64p]
    L.ref_strings_dump.restype = C.c_int64
    L.ref_strings_dump.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p]
    for f in ("ref_1h_dump", "ref_1h_dump_keyed", "ref_2h_dump"):
        getattr(L, f).restype = C.c_int64
        getattr(L, f).argtypes = [vp, C.c_int, C.c_void_p]
    L.ref_dets_dump.argtypes = [vp, _u64p]
    L.ref_sigma_new.restype = vp
    L.ref_sigma_new.argtypes = [vp, C.c_double, _f64p, _f64p, C.c_int, C.c_int]
    L.ref_sigma_free.argtypes = [vp]
    L.ref_sigma_set_algorithm.argtypes = [vp, C.c_char_p]
    L.ref_sigma_set_memory.argtypes = [vp, C.c_int]
    L.ref_sigma_hamiltonian.argtypes = [vp, _f64p, _f64p, C.c_int64]
    L.ref_sigma_term.argtypes = [vp, C.c_int, _f64p, _f64p, C.c_int64]
    L.ref_sigma_avg_build_time.argtypes = [vp, _f64p]
    L.ref_det_energies.argtypes = [vp, vp, _f64p]
    L.ref_spin_adapter_new.restype = vp
    L.ref_spin_adapter_new.argtypes = [C.c_int, C.c_int, C.c_int]
    L.ref_spin_adapter_free.argtypes = [vp]
    L.ref_spin_adapter_prepare.argtypes = [vp, vp]
    L.ref_spin_adapter_info.argtypes = [vp, _i64p]
    L.ref_spin_adapter_dump.argtypes = [vp, _i64p, _i64p, _f64p, _i64p]
    L.ref_csf_to_det.argtypes = [vp, _f64p, C.c_int64, _f64p, C.c_int64]
    L.ref_det_to_csf.argtypes = [vp, _f64p, C.c_int64, _f64p, C.c_int64]
    L.ref_hdiag_csf.argtypes = [vp, vp, vp, C.c_int, _f64p, C.c_int64]
    L.ref_slater_rules_csf.restype = C.c_double
    L.ref_slater_rules_csf.argtypes = [vp, vp, vp, C.c_int64, C.c_int64]
    L.ref_rdm.restype = C.c_int64
    L.ref_rdm.argtypes = [vp, C.c_int, _f64p, _f64p, C.c_int64, _f64p]
    L.oracle_blas_open.argtypes = [C.c_char_p]
    L.oracle_blas_set_threads.argtypes = [C.c_int]
    L.ref_rel_sigma_new.restype = vp
    L.ref_rel_sigma_new.argtypes = [vp, C.c_double, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    L.ref_rel_sigma_free.argtypes = [vp]
    L.ref_rel_sigma_set_algorithm.argtypes = [vp, C.c_char_p]
    L.ref_rel_sigma_hamiltonian.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_int64]
    L.ref_rel_form_hdiag.argtypes = [vp, vp, C.c_void_p]
    L.ref_rel_slater_rules.argtypes = [vp, vp, C.c_int64, C.c_int64, C.c_void_p]
    L.ref_rel_rdm.restype = C.c_int64
    L.ref_rel_rdm.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    _lib = L
    return L


def open_blas(threads=None):
    """Route the reference's dgemm_/daxpy_/ddot_ to numpy's OpenBLAS (faster, same results)."""
    L = lib()
    path = numpy_openblas_path()
    if path and L.oracle_blas_open(path.encode()) == 0:
        if threads:
            L.oracle_blas_set_threads(int(threads))
        return True
    return False


def _raise(kind):
    msg = lib().ref_last_error().decode()
    if kind == 2:
        raise ValueError(msg)
    raise RuntimeError(msg)


class RefCIStrings:
    """The reference CIStrings (ci/ci_strings.cc:26-184)."""

    def __init__(self, na, nb, symmetry, orbital_symmetry, gas_min, gas_max):
        L = lib()
        sizes = np.array([len(g) for g in orbital_symmetry], dtype=np.int32)
        flat = np.array([x for g in orbital_symmetry for x in g] or [0], dtype=np.int32)
        gmin = np.array(list(gas_min) or [0], dtype=np.int32)
        gmax = np.array(list(gas_max) or [0], dtype=np.int32)
        kind = C.c_int(0)
        h = L.ref_strings_new(na, nb, symmetry, len(orbital_symmetry), sizes if len(sizes) else
                              np.zeros(1, np.int32), flat, len(gas_min), gmin, len(gas_max), gmax,
                              C.byref(kind))
        if not h:
            _raise(kind.value)
        self.h = h
        info = np.zeros(10, np.int64)
        L.ref_strings_info(h, info)
        (self.norb, self.na, self.nb, self.nas, self.nbs, self.ndet, self.nirrep,
         self.nclass_a, self.nclass_b, self.nblocks) = [int(x) for x in info]

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_strings_free(self.h)
            self.h = None

    def blocks(self):
        out = np.zeros(4 * self.nblocks, np.int64)
        lib().ref_strings_blocks(self.h, out)
        return out.reshape(-1, 4)

    def strings(self, spin):
        L = lib()
        n = L.ref_strings_dump(self.h, spin, None, None)
        masks = np.zeros(n, np.uint64)
        classes = np.zeros(n, np.int32)
        L.ref_strings_dump(self.h, spin, masks.ctypes.data, classes.ctypes.data)
        return masks, classes

    def list_1h(self, spin, keyed=False):
        L = lib()
        f = L.ref_1h_dump_keyed if keyed else L.ref_1h_dump
        n = f(self.h, spin, None)
        out = np.zeros((n, 6), np.int32)
        f(self.h, spin, out.ctypes.data)
        return out

    def list_2h(self, spin):
        L = lib()
        n = L.ref_2h_dump(self.h, spin, None)
        out = np.zeros((n, 7), np.int32)
        L.ref_2h_dump(self.h, spin, out.ctypes.data)
        return out

    def determinants(self):
        out = np.zeros(2 * self.ndet, np.uint64)
        lib().ref_dets_dump(self.h, out)
        return out.reshape(-1, 2)


class RefSigmaBuilder:
    """The reference CISigmaBuilder (ci/ci_sigma_builder.cc)."""

    TERMS = {"h0": 0, "h1_a": 1, "h1_b": 2, "aabb": 3, "aaaa": 4, "bbbb": 5}

    def __init__(self, strings: RefCIStrings, E, H, V, log_level=0):
        self.strings = strings
        H = np.ascontiguousarray(H, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        self.h = lib().ref_sigma_new(strings.h, float(E), H, V, H.shape[0], log_level)
        if not self.h:
            raise RuntimeError(lib().ref_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_sigma_free(self.h)
            self.h = None

    def set_algorithm(self, name):
        rc = lib().ref_sigma_set_algorithm(self.h, name.encode())
        if rc:
            _raise(rc)

    def set_memory(self, mb):
        rc = lib().ref_sigma_set_memory(self.h, int(mb))
        if rc:
            _raise(rc)

    def Hamiltonian(self, basis, sigma):
        rc = lib().ref_sigma_hamiltonian(self.h, basis, sigma, basis.shape[0])
        if rc:
            _raise(rc)

    def term(self, name, basis):
        sigma = np.zeros_like(basis)
        rc = lib().ref_sigma_term(self.h, self.TERMS[name], basis, sigma, basis.shape[0])
        if rc:
            _raise(rc)
        return sigma

    def avg_build_time(self):
        out = np.zeros(4)
        lib().ref_sigma_avg_build_time(self.h, out)
        return out

    def det_energies(self):
        out = np.zeros(self.strings.ndet)
        lib().ref_det_energies(self.h, self.strings.h, out)
        return out

    RDM_KINDS = {"a_1rdm": 0, "b_1rdm": 1, "sf_1rdm": 2, "aa_2rdm": 3, "bb_2rdm": 4, "ab_2rdm": 5,
                 "sf_2rdm": 6, "sf_2cumulant": 7, "aaa_3rdm": 8, "bbb_3rdm": 9, "aab_3rdm": 10, "abb_3rdm": 11,
                 "sf_3rdm": 12, "sf_3cumulant": 13}

    def rdm(self, kind, CL, CR):
        """The reference's compute_<kind> (ci_sigma_builder_1rdm.cc, _2rdm.cc, _3rdm.cc) as a flat array."""
        n = self.strings.norb
        P, T = n * (n - 1) // 2, n * (n - 1) * (n - 2) // 6
        size = {0: n * n, 1: n * n, 2: n * n, 3: P * P, 4: P * P, 5: n ** 4, 6: n ** 4, 7: n ** 4, 8: T * T,
                9: T * T, 10: (P * n) ** 2, 11: (P * n) ** 2}.get(self.RDM_KINDS[kind], n ** 6)
        out = np.zeros(max(size, 1))
        got = lib().ref_rdm(self.h, self.RDM_KINDS[kind], np.ascontiguousarray(CL, dtype=np.float64),
                            np.ascontiguousarray(CR, dtype=np.float64), CL.shape[0], out)
        if got < 0:
            _raise(1)
        return out[:got]

    def form_Hdiag_csf(self, spin_adapter, full=False):
        out = np.zeros(spin_adapter.ncsf)
        lib().ref_hdiag_csf(self.h, spin_adapter.h, self.strings.h, int(full), out, out.shape[0])
        return out

    def slater_rules_csf(self, spin_adapter, I, J):
        return lib().ref_slater_rules_csf(self.h, spin_adapter.h, self.strings.h, int(I), int(J))


class RefRelSigmaBuilder:
    """The reference's two-component RelCISigmaBuilder (ci/rel_ci_sigma_builder*.cc) on strings
    with nb == 0: complex H (n, n) and physicist V (n, n, n, n)."""

    RDM_KINDS = ("so_1rdm", "so_2rdm", "so_2cumulant", "so_3rdm", "so_3cumulant")

    def __init__(self, strings: RefCIStrings, E, H, V, log_level=0):
        self.strings = strings
        self.norb = strings.norb
        self._H = np.ascontiguousarray(H, dtype=np.complex128)
        self._V = np.ascontiguousarray(V, dtype=np.complex128)
        h = lib().ref_rel_sigma_new(strings.h, float(E), self._H.ctypes.data, self._V.ctypes.data, self.norb,
                                    log_level)
        if not h:
            raise RuntimeError(lib().ref_last_error().decode())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_rel_sigma_free(self.h)
            self.h = None

    def set_algorithm(self, name):
        if lib().ref_rel_sigma_set_algorithm(self.h, name.encode()):
            raise RuntimeError(lib().ref_last_error().decode())

    def Hamiltonian(self, basis, sigma):
        b = np.ascontiguousarray(basis, dtype=np.complex128)
        out = np.zeros(self.strings.ndet, dtype=np.complex128)
        if lib().ref_rel_sigma_hamiltonian(self.h, b.ctypes.data, out.ctypes.data, self.strings.ndet):
            raise RuntimeError(lib().ref_last_error().decode())
        sigma[:] = out
        return sigma

    def form_Hdiag(self):
        out = np.zeros(self.strings.ndet, dtype=np.complex128)
        lib().ref_rel_form_hdiag(self.h, self.strings.h, out.ctypes.data)
        return out

    def slater_rules(self, I, J):
        out = np.zeros(2)
        lib().ref_rel_slater_rules(self.h, self.strings.h, int(I), int(J), out.ctypes.data)
        return complex(out[0], out[1])

    def rdm(self, kind, CL, CR):
        n = self.norb
        size = {0: n ** 2, 1: n ** 4, 2: n ** 4, 3: n ** 6, 4: n ** 6}[self.RDM_KINDS.index(kind)]
        out = np.zeros(max(size, 1), dtype=np.complex128)
        cl = np.ascontiguousarray(CL, dtype=np.complex128)
        cr = np.ascontiguousarray(CR, dtype=np.complex128)
        got = lib().ref_rel_rdm(self.h, self.RDM_KINDS.index(kind), cl.ctypes.data, cr.ctypes.data,
                                self.strings.ndet, out.ctypes.data)
        if got < 0:
            raise RuntimeError(lib().ref_last_error().decode())
        return out[:got]


class RefSpinAdapter:
    """The reference CISpinAdapter (determinant/ci_spin_adapter.cc)."""

    def __init__(self, twoS, twoMs, norb):
        self.h = lib().ref_spin_adapter_new(twoS, twoMs, norb)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_spin_adapter_free(self.h)
            self.h = None

    def prepare_couplings(self, strings: RefCIStrings):
        self.ndet = strings.ndet
        lib().ref_spin_adapter_prepare(self.h, strings.h)
        info = np.zeros(3, np.int64)
        lib().ref_spin_adapter_info(self.h, info)
        self.nconf, self.ncsf, self.ncoupling = [int(x) for x in info]

    def couplings(self):
        bounds = np.zeros(self.ncsf + 1, np.int64)
        det_idx = np.zeros(max(self.ncoupling, 1), np.int64)
        coeff = np.zeros(max(self.ncoupling, 1))
        ranges = np.zeros(2 * max(self.nconf, 1), np.int64)
        lib().ref_spin_adapter_dump(self.h, bounds, det_idx, coeff, ranges)
        return bounds, det_idx[: self.ncoupling], coeff[: self.ncoupling], ranges[: 2 * self.nconf].reshape(-1, 2)

    def csf_C_to_det_C(self, csf):
        det = np.zeros(self.ndet)
        lib().ref_csf_to_det(self.h, np.ascontiguousarray(csf), csf.shape[0], det, self.ndet)
        return det

    def det_C_to_csf_C(self, det):
        csf = np.zeros(self.ncsf)
        lib().ref_det_to_csf(self.h, np.ascontiguousarray(det), det.shape[0], csf, self.ncsf)
        return csf
