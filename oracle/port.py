"""Oracle (test infrastructure only): ctypes access to the CPU restatement in
``oracle/port/ci_port.cc``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
module, always as the parity reference or the timed CPU baseline, never as a product path. The library
is compiled by ``build_port()`` (called from ``__graft_entry__.build()``) on the machine that
runs it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libci_port.so")
SOURCES = [os.path.join(HERE, "port", "ci_port.cc"), os.path.join(HERE, "blas_bridge.cc")]

_lib = None
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


def build_port(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", *SOURCES, "-o", LIB_PATH, "-ldl", "-lpthread"]
    subprocess.run(cmd, check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build_port()
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.port_last_error.restype = C.c_char_p
    L.port_new.restype = vp
    L.port_new.argtypes = [C.c_int, C.c_int, C.c_int]
    L.port_free.argtypes = [vp]
    L.port_info.argtypes = [vp, _i64p]
    L.port_strings.argtypes = [vp, C.c_int, _u64p]
    L.port_1h.restype = C.c_int64
    L.port_1h.argtypes = [vp, C.c_int, C.c_void_p]
    L.port_2h.restype = C.c_int64
    L.port_2h.argtypes = [vp, C.c_int, C.c_void_p]
    L.port_set_hamiltonian.argtypes = [vp, C.c_double, _f64p, _f64p]
    L.port_set_memory.argtypes = [vp, C.c_int]
    L.port_set_fraction.argtypes = [vp, C.c_double]
    L.port_sigma.argtypes = [vp, _f64p, _f64p, C.c_int]
    L.port_det_energies.argtypes = [vp, _f64p]
    L.port_spin_adapter_new.restype = vp
    L.port_spin_adapter_new.argtypes = [vp, C.c_int, C.c_int]
    L.port_spin_adapter_free.argtypes = [vp]
    L.port_spin_adapter_info.argtypes = [vp, _i64p]
    L.port_spin_adapter_dump.argtypes = [vp, _i64p, _i64p, _f64p, _i64p]
    L.port_csf_to_det.argtypes = [vp, _f64p, _f64p, C.c_int64]
    L.port_det_to_csf.argtypes = [vp, _f64p, _f64p]
    L.port_hdiag_csf.argtypes = [vp, vp, _f64p]
    L.port_rdm.restype = C.c_int64
    L.port_rdm.argtypes = [vp, C.c_int, _f64p, _f64p, _f64p]
    L.oracle_blas_open.argtypes = [C.c_char_p]
    L.oracle_blas_set_threads.argtypes = [C.c_int]
    _lib = L
    return L


def open_blas(threads: int | None = None) -> bool:
    """Route dgemm_ to numpy's bundled OpenBLAS when present (as the reference links a BLAS)."""
    import glob
    import numpy

    libs = glob.glob(os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs", "libscipy_openblas64_*.so"))
    if not libs:
        return False
    L = lib()
    if L.oracle_blas_open(libs[0].encode()) != 0:
        return False
    if threads:
        L.oracle_blas_set_threads(int(threads))
    return True


TERM_BITS = {"h0": 1, "h1_a": 2, "h1_b": 4, "aabb": 8, "aaaa": 16, "bbbb": 32}
ALL_TERMS = 63


class PortCI:
    """CAS (C1) strings, lists and HZ sigma of the oracle port."""

    def __init__(self, norb: int, na: int, nb: int):
        L = lib()
        self.h = L.port_new(norb, na, nb)
        if not self.h:
            raise RuntimeError(L.port_last_error().decode())
        self.norb, self.na, self.nb = norb, na, nb
        info = np.zeros(7, np.int64)
        L.port_info(self.h, info)
        self.nas, self.nbs, self.ndet, self.n1a, self.n1b, self.n2a, self.n2b = [int(x) for x in info]

    def __del__(self):
        if getattr(self, "h", None):
            lib().port_free(self.h)
            self.h = None

    def strings(self, spin):
        out = np.zeros(self.nas if spin == 0 else self.nbs, np.uint64)
        lib().port_strings(self.h, spin, out)
        return out

    def list_1h(self, spin):
        L = lib()
        n = L.port_1h(self.h, spin, None)
        out = np.zeros((n, 6), np.int32)
        L.port_1h(self.h, spin, out.ctypes.data)
        return out

    def list_2h(self, spin):
        L = lib()
        n = L.port_2h(self.h, spin, None)
        out = np.zeros((n, 7), np.int32)
        L.port_2h(self.h, spin, out.ctypes.data)
        return out

    def set_hamiltonian(self, E, H, V):
        lib().port_set_hamiltonian(self.h, float(E), np.ascontiguousarray(H, np.float64),
                                   np.ascontiguousarray(V, np.float64))

    def set_memory(self, mb):
        rc = lib().port_set_memory(self.h, int(mb))
        if rc == 2:
            raise ValueError(lib().port_last_error().decode())

    def set_fraction(self, frac):
        lib().port_set_fraction(self.h, float(frac))

    def sigma(self, c, terms=ALL_TERMS):
        c = np.ascontiguousarray(c, np.float64)
        out = np.zeros(self.ndet)
        if lib().port_sigma(self.h, c, out, int(terms)) != 0:
            raise RuntimeError(lib().port_last_error().decode())
        return out

    def det_energies(self):
        out = np.zeros(self.ndet)
        lib().port_det_energies(self.h, out)
        return out

    RDM_KINDS = {"a_1rdm": 0, "b_1rdm": 1, "sf_1rdm": 2, "aa_2rdm": 3, "bb_2rdm": 4, "ab_2rdm": 5,
                 "sf_2rdm": 6, "sf_2cumulant": 7, "aaa_3rdm": 8, "bbb_3rdm": 9, "aab_3rdm": 10, "abb_3rdm": 11,
                 "sf_3rdm": 12, "sf_3cumulant": 13}

    def rdm(self, kind, CL, CR):
        """Reduced density matrix `kind` between determinant vectors CL (bra) and CR (ket), flat."""
        n = self.norb
        npair, ntrip = n * (n - 1) // 2, n * (n - 1) * (n - 2) // 6
        size = {0: n * n, 1: n * n, 2: n * n, 3: npair * npair, 4: npair * npair, 5: n ** 4, 6: n ** 4, 7: n ** 4,
                8: ntrip ** 2, 9: ntrip ** 2, 10: (npair * n) ** 2, 11: (npair * n) ** 2}.get(self.RDM_KINDS[kind], n ** 6)
        out = np.zeros(max(size, 1))
        got = lib().port_rdm(self.h, self.RDM_KINDS[kind], np.ascontiguousarray(CL, np.float64),
                             np.ascontiguousarray(CR, np.float64), out)
        if got < 0:
            raise ValueError(f"unknown RDM kind {kind}")
        return out[:got]


class PortSpinAdapter:
    def __init__(self, ci: PortCI, twoS: int, twoMs: int):
        L = lib()
        self.ci = ci
        self.h = L.port_spin_adapter_new(ci.h, twoS, twoMs)
        if not self.h:
            raise RuntimeError(L.port_last_error().decode())
        info = np.zeros(3, np.int64)
        L.port_spin_adapter_info(self.h, info)
        self.nconf, self.ncsf, self.ncoupling = [int(x) for x in info]

    def __del__(self):
        if getattr(self, "h", None):
            lib().port_spin_adapter_free(self.h)
            self.h = None

    def couplings(self):
        b = np.zeros(self.ncsf + 1, np.int64)
        d = np.zeros(max(1, self.ncoupling), np.int64)
        c = np.zeros(max(1, self.ncoupling))
        r = np.zeros(max(2, 2 * self.nconf), np.int64)
        lib().port_spin_adapter_dump(self.h, b, d, c, r)
        return b, d[: self.ncoupling], c[: self.ncoupling], r[: 2 * self.nconf].reshape(-1, 2)

    def csf_to_det(self, csf):
        out = np.zeros(self.ci.ndet)
        lib().port_csf_to_det(self.h, np.ascontiguousarray(csf, np.float64), out, self.ci.ndet)
        return out

    def det_to_csf(self, det):
        out = np.zeros(self.ncsf)
        lib().port_det_to_csf(self.h, np.ascontiguousarray(det, np.float64), out)
        return out

    def hdiag(self):
        out = np.zeros(self.ncsf)
        lib().port_hdiag_csf(self.ci.h, self.h, out)
        return out
