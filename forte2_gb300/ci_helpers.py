"""Drop-in mirror of the reference's ``forte2.lib.ci_helpers`` module (CIStrings, CISigmaBuilder,
CISpinAdapter; bound in forte2/api/ci_helpers_api.cc:35-200) backed by the GB300 CUDA library.

Method names, argument meaning and error types/messages follow the reference. Vectors may be
numpy arrays (host; copied to and from the device around the call, the reference's own calling
convention) or torch CUDA float64 tensors (device-resident; no copies). Everything runs on the
GPU through ``include/forte2_gb300.h``; there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib, stream_handle


def _torch():
    import torch

    return torch


def _is_cuda_tensor(x):
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, torch.Tensor) and x.is_cuda


def _host_vec(x, what="np_vector"):
    if not isinstance(x, np.ndarray) or x.dtype != np.float64:
        raise TypeError(f"{what} must be a float64 numpy array or a CUDA float64 tensor")
    if x.ndim != 1:
        raise RuntimeError("np_vector must be 1-dimensional to convert to std::span.")
    if x.strides[0] != 8:
        raise RuntimeError("np_vector must have stride 1 to convert to std::span.")
    return x


def _dev_vec(x):
    if x.dtype != _torch().float64:
        raise TypeError("device vectors must be float64")
    if not x.is_contiguous():
        raise RuntimeError("device vectors must be contiguous")
    return x


class Determinants:
    """The determinant list of a CIStrings object (CIStrings::make_determinants,
    ci/ci_strings.cc:186-194): address order, each entry an (alpha mask, beta mask) pair."""

    def __init__(self, strings: "CIStrings"):
        self.strings = strings

    def __len__(self):
        return self.strings.ndet

    def masks(self) -> np.ndarray:
        return self.strings.determinant_masks()

    def __getitem__(self, i):
        return self.strings.determinant(i)


def enumerate_blocks(na, nb, symmetry, orbital_symmetry, gas_min, gas_max):
    """The determinant blocks of a space on the host alone (no device call): a dict with the
    class strings and classes of both spins ('alpha', 'alpha_class', 'beta', 'beta_class'), the
    block table ('blocks': alpha class, beta class, size, offset, alpha strings, beta strings),
    'ndet', 'nirrep' and 'trivial'."""
    sizes = np.array([len(g) for g in orbital_symmetry] or [0], dtype=np.int32)
    flat = np.array([int(x) for g in orbital_symmetry for x in g] or [0], dtype=np.int32)
    gmin = np.array(list(gas_min) or [0], dtype=np.int32)
    gmax = np.array(list(gas_max) or [0], dtype=np.int32)
    args = (int(na), int(nb), int(symmetry), len(orbital_symmetry), sizes.ctypes.data, flat.ctypes.data,
            len(gas_min), gmin.ctypes.data, len(gas_max), gmax.ctypes.data)
    info = np.zeros(16, dtype=np.int64)
    check(lib().f2g_blocks_enumerate(*args, info.ctypes.data, None, None, None, None, None))
    out = {"alpha": np.zeros(info[6], np.uint64), "alpha_class": np.zeros(info[6], np.int32),
           "beta": np.zeros(info[7], np.uint64), "beta_class": np.zeros(info[7], np.int32),
           "blocks": np.zeros((info[5], 6), np.int64)}
    check(lib().f2g_blocks_enumerate(*args, info.ctypes.data, out["alpha"].ctypes.data,
                                     out["alpha_class"].ctypes.data, out["beta"].ctypes.data,
                                     out["beta_class"].ctypes.data, out["blocks"].ctypes.data))
    out.update(ndet=int(info[13]), nirrep=int(info[1]), trivial=bool(info[0]))
    return out


class CIStrings:
    """CI strings of an active space (forte2/ci/ci_strings.cc:26-184), built on the device.

    Any number (up to six) of GAS spaces with their electron bounds, orbital irreps 0..7 and a
    state irrep: the determinants are the reference's blocks in its order
    (ci_occupation.cc:35-142, ci_string_class.cc:7-66, ci_strings_makers.cc:13-73). The sigma,
    RDM and CSF kernels run on the C1 CAS space of all orbitals; a blocked space's vectors are
    embedded into it (zero elsewhere) and read back, which is P H P, the reference's blocked
    operator, at the cost of the C1 space.
    """

    def __init__(self, na, nb, symmetry, orbital_symmetry, gas_min, gas_max):
        if not isinstance(orbital_symmetry, (list, tuple)) or not all(
                isinstance(g, (list, tuple)) for g in orbital_symmetry):
            raise TypeError("orbital_symmetry must be a list of lists of orbital irreps")
        if int(na) < 0 or int(nb) < 0:
            raise ValueError("CIStrings: the number of electrons must be non-negative")
        if len(gas_min) > len(orbital_symmetry) or len(gas_max) > len(orbital_symmetry):
            raise ValueError(
                f"CIStrings: The number of GAS spaces specified by gas_min ({len(gas_min)}) and gas_max "
                f"({len(gas_max)}) must be less than or equal to the number of orbital symmetries "
                f"({len(orbital_symmetry)})")
        norb = sum(len(g) for g in orbital_symmetry)
        self._na, self._nb, self._norb = int(na), int(nb), int(norb)
        self.symmetry = int(symmetry)
        self.orbital_symmetry = [[int(x) for x in g] for g in orbital_symmetry]
        self.gas_min, self.gas_max = [int(x) for x in gas_min], [int(x) for x in gas_max]
        nonempty = [g for g in self.orbital_symmetry if len(g) > 0]
        plain = (len(nonempty) <= 1 and all(x == 0 for g in nonempty for x in g) and self.symmetry == 0
                 and not self.gas_min and not self.gas_max)
        if self._na > norb or self._nb > norb:
            # the reference produces an empty determinant space
            self._empty = True
            self.h = None
            self._info = [norb, self._na, self._nb, 0, 0, 0, 0, 0, 0, 0]
            self._binfo = [1, 1, len(self.orbital_symmetry), 1, 1, 1, 0, 0, 0, 1, 1, 1, self.symmetry, 0, 0, 0]
            self._det_cache = np.zeros((0, 2), dtype=np.uint64)
            return
        self._empty = False
        h = C.c_void_p()
        if plain:
            check(lib().f2g_strings_create(self._na, self._nb, self._norb, C.byref(h)))
        else:
            sizes = np.array([len(g) for g in self.orbital_symmetry] or [0], dtype=np.int32)
            flat = np.array([x for g in self.orbital_symmetry for x in g] or [0], dtype=np.int32)
            gmin = np.array(self.gas_min or [0], dtype=np.int32)
            gmax = np.array(self.gas_max or [0], dtype=np.int32)
            check(lib().f2g_strings_create_general(self._na, self._nb, self.symmetry, len(self.orbital_symmetry),
                                                   sizes.ctypes.data, flat.ctypes.data, len(self.gas_min),
                                                   gmin.ctypes.data, len(self.gas_max), gmax.ctypes.data,
                                                   C.byref(h)))
        self.h = h
        info = np.zeros(10, dtype=np.int64)
        check(lib().f2g_strings_info(self.h, info.ctypes.data))
        self._info = [int(x) for x in info]
        binfo = np.zeros(16, dtype=np.int64)
        check(lib().f2g_strings_blocks_info(self.h, binfo.ctypes.data))
        self._binfo = [int(x) for x in binfo]
        self._det_cache = None

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().f2g_strings_destroy(h)
            self.h = None

    # properties of the reference binding (api/ci_helpers_api.cc:55-86)
    na = property(lambda self: self._na)
    nb = property(lambda self: self._nb)
    norb = property(lambda self: self._norb)
    nas = property(lambda self: self._binfo[6])
    nbs = property(lambda self: self._binfo[7])
    ndet = property(lambda self: self._info[5])
    ngas_spaces = property(lambda self: len(self.orbital_symmetry))
    gas_size = property(lambda self: [len(g) for g in self.orbital_symmetry])
    nirrep = property(lambda self: self._binfo[1])
    # True when the space is a set of blocks of the C1 CAS space (irreps or GAS restrictions)
    blocked = property(lambda self: not self._empty and self._binfo[0] == 0)
    # determinants of the C1 CAS space the kernels run on
    nfull = property(lambda self: self._info[3] * self._info[4])

    def _occupations(self):
        if self._empty:
            return np.zeros((0, 6), np.int32), np.zeros((0, 6), np.int32), np.zeros((0, 2), np.int32)
        na_, nb_, npair = self._binfo[9], self._binfo[10], self._binfo[11]
        a = np.zeros((na_, 6), np.int32)
        b = np.zeros((nb_, 6), np.int32)
        pr = np.zeros((npair, 2), np.int32)
        check(lib().f2g_strings_occupations(self.h, a.ctypes.data, b.ctypes.data, pr.ctypes.data))
        return a, b, pr

    @property
    def gas_alpha_occupations(self):
        return [list(map(int, r)) for r in self._occupations()[0]]

    @property
    def gas_beta_occupations(self):
        return [list(map(int, r)) for r in self._occupations()[1]]

    @property
    def gas_occupations(self):
        return [tuple(map(int, r)) for r in self._occupations()[2]]

    def class_strings(self, spin):
        """Strings of one spin in (class, address) order and their class indices."""
        n = self._binfo[6 + spin]
        masks = np.zeros(n, dtype=np.uint64)
        classes = np.zeros(n, dtype=np.int32)
        if n:
            check(lib().f2g_strings_class_strings(self.h, spin, masks.ctypes.data, classes.ctypes.data))
        return masks, classes

    def block_table(self):
        """Per block: alpha class, beta class, size, offset, alpha strings, beta strings."""
        nblk = 0 if self._empty else self._binfo[5]
        out = np.zeros((nblk, 6), dtype=np.int64)
        if nblk:
            check(lib().f2g_strings_block_table(self.h, out.ctypes.data))
        return out

    def _masks(self, spin):
        n = self.nas if spin == 0 else self.nbs
        out = np.zeros(n, dtype=np.uint64)
        if n and not self._empty:
            if self.blocked:
                out = self.class_strings(spin)[0]
            else:
                check(lib().f2g_strings_masks(self.h, spin, out.ctypes.data))
        return out

    def alpha_masks(self):
        return self._masks(0)

    def beta_masks(self):
        return self._masks(1)

    def determinant_masks(self):
        """(ndet, 2) alpha and beta masks of every determinant in address order."""
        if self._det_cache is None:
            a, b = self.alpha_masks(), self.beta_masks()
            if not self.blocked:
                out = np.empty((len(a) * len(b), 2), dtype=np.uint64)
                out[:, 0] = np.repeat(a, len(b))
                out[:, 1] = np.tile(b, len(a))
            else:
                aoff = np.zeros(self._binfo[3] + 1, np.int64)
                boff = np.zeros(self._binfo[4] + 1, np.int64)
                _, ac = self.class_strings(0)
                _, bc = self.class_strings(1)
                aoff[1:] = np.cumsum(np.bincount(ac, minlength=self._binfo[3]))
                boff[1:] = np.cumsum(np.bincount(bc, minlength=self._binfo[4]))
                out = np.empty((self.ndet, 2), dtype=np.uint64)
                for ca, cb, size, off, nia, nib in self.block_table():
                    if size == 0:
                        continue
                    out[off:off + size, 0] = np.repeat(a[aoff[ca]:aoff[ca] + nia], nib)
                    out[off:off + size, 1] = np.tile(b[boff[cb]:boff[cb] + nib], nia)
            self._det_cache = out
        return self._det_cache

    def determinant(self, address):
        if not self.blocked:
            a = self.alpha_masks()
            b = self.beta_masks()
            return int(a[address // len(b)]), int(b[address % len(b)])
        m = self.determinant_masks()[address]
        return int(m[0]), int(m[1])

    def determinant_index(self, det):
        a, b = det
        if not self.blocked:
            am, bm = self.alpha_masks(), self.beta_masks()
            ia = int(np.nonzero(am == np.uint64(a))[0][0])
            ib = int(np.nonzero(bm == np.uint64(b))[0][0])
            return ia * len(bm) + ib
        m = self.determinant_masks()
        hit = np.nonzero((m[:, 0] == np.uint64(a)) & (m[:, 1] == np.uint64(b)))[0]
        if len(hit) == 0:
            raise KeyError("determinant not in this space")
        return int(hit[0])

    def make_determinants(self):
        return Determinants(self)

    def _c1_only(self):
        if self.blocked:
            raise NotImplementedError("CIStrings: the coupling lists are those of the C1 CAS space; a blocked "
                                      "space keeps no lists of its own")

    def list_1h(self, spin):
        """1-hole list rows (class_K, K, class_I, sign, p, I) in the reference's order."""
        self._c1_only()
        cnt = C.c_int64(0)
        check(lib().f2g_strings_list1h(self.h, spin, None, C.byref(cnt)))
        out = np.zeros((cnt.value, 6), dtype=np.int32)
        if cnt.value:
            check(lib().f2g_strings_list1h(self.h, spin, out.ctypes.data, C.byref(cnt)))
        return out

    def list_2h(self, spin):
        """2-hole list rows (class_K, K, class_I, sign, p, q, I) in the reference's order."""
        self._c1_only()
        cnt = C.c_int64(0)
        check(lib().f2g_strings_list2h(self.h, spin, None, C.byref(cnt)))
        out = np.zeros((cnt.value, 7), dtype=np.int32)
        if cnt.value:
            check(lib().f2g_strings_list2h(self.h, spin, out.ctypes.data, C.byref(cnt)))
        return out


class RelCISigmaBuilder:
    """Two-component sigma builder (forte2/ci/rel_ci_sigma_builder.cc:15-238,
    rel_ci_sigma_builder_harrison_zarrabian.cc) on the device: strings with nb == 0, complex H
    and V. As in the reference the default algorithm is "kh", for which Hamiltonian applies only E;
    "hz" applies the full operator."""

    def __init__(self, lists: CIStrings, E, H, V, log_level=3):
        if lists.nb != 0:
            raise RuntimeError("RelCISigmaBuilder requires nb == 0 (two-component CI treats all electrons as "
                               "alpha spinors).")
        n = lists.norb
        H = np.ascontiguousarray(H, dtype=np.complex128)
        V = np.ascontiguousarray(V, dtype=np.complex128)
        if H.ndim != 2:
            raise RuntimeError("H must be a 2D matrix.")
        if H.shape != (n, n):
            raise RuntimeError("H shape does not match the number of orbitals.")
        if V.ndim != 4:
            raise RuntimeError("V must be a 4D tensor.")
        if V.shape != (n, n, n, n):
            raise RuntimeError("V shape does not match the number of orbitals.")
        self.lists = lists
        self.log_level = int(log_level)
        self.h = None
        if getattr(lists, "_empty", False):
            self._E = float(E)
            return
        h = C.c_void_p()
        check(lib().f2g_rel_sigma_create(lists.h, float(E), H.ctypes.data, V.ctypes.data, C.byref(h)))
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().f2g_rel_sigma_destroy(h)
            self.h = None

    def set_algorithm(self, algorithm):
        check(lib().f2g_rel_sigma_set_algorithm(self.h, str(algorithm).encode()))

    def get_algorithm(self):
        buf = C.create_string_buffer(64)
        check(lib().f2g_rel_sigma_get_algorithm(self.h, buf, 64))
        return buf.value.decode()

    def set_memory(self, mb):
        check(lib().f2g_rel_sigma_set_memory(self.h, int(mb)))

    def Hamiltonian(self, basis, sigma):
        """sigma <- H basis (overwritten). numpy complex128 vectors, or CUDA complex128 tensors
        ((ndet,) or (nvec, ndet), contiguous) that stay on the device."""
        torch = _torch()
        nd = self.lists.ndet
        if _is_cuda_tensor(basis) and _is_cuda_tensor(sigma):
            if basis.dtype != torch.complex128 or sigma.dtype != torch.complex128:
                raise TypeError("device vectors must be complex128")
            if not basis.is_contiguous() or not sigma.is_contiguous():
                raise RuntimeError("device vectors must be contiguous")
            nvec = 1 if basis.dim() == 1 else basis.shape[0]
            if basis.numel() != nvec * nd or sigma.numel() != basis.numel():
                raise RuntimeError("vector length does not match the number of determinants")
            check(lib().f2g_rel_sigma_apply(self.h, basis.data_ptr(), sigma.data_ptr(), nvec, stream_handle()))
            return sigma
        b = np.ascontiguousarray(basis, dtype=np.complex128)
        if b.shape[0] != nd or np.shape(sigma)[0] != nd:
            raise RuntimeError("vector length does not match the number of determinants")
        db = torch.from_numpy(b).cuda()
        ds = torch.empty_like(db)
        check(lib().f2g_rel_sigma_apply(self.h, db.data_ptr(), ds.data_ptr(), 1, stream_handle()))
        sigma[:] = ds.cpu().numpy()
        return sigma

    def form_Hdiag(self, dets=None):
        torch = _torch()
        out = torch.empty(max(1, self.lists.ndet), dtype=torch.complex128, device="cuda")
        check(lib().f2g_rel_sigma_hdiag(self.h, out.data_ptr(), stream_handle()))
        return out[: self.lists.ndet].cpu().numpy()

    def slater_rules(self, dets, I, J):
        out = np.zeros(2)
        check(lib().f2g_rel_sigma_element(self.h, int(I), int(J), out.ctypes.data))
        return complex(out[0], out[1])

    _SO_KINDS = {"so_1rdm": 0, "so_2rdm": 1, "so_2cumulant": 2, "so_3rdm": 3, "so_3cumulant": 4}

    def _so_rdm(self, kind, C_left, C_right):
        """Spin-orbital RDM `kind` between the bra C_left (conjugated) and the ket C_right, complex
        (rel_ci_sigma_builder_rdm.cc). numpy vectors give a numpy array; CUDA complex128 tensors
        give a CUDA tensor."""
        torch = _torch()
        n = self.lists.norb
        k = self._SO_KINDS[kind]
        shape = (n,) * (2, 4, 4, 6, 6)[k]
        size = int(lib().f2g_rel_rdm_size(n, k))
        if size < 0:
            check(-1)
        device = _is_cuda_tensor(C_left)
        if device:
            if not _is_cuda_tensor(C_right):
                raise TypeError("C_left and C_right must both be CUDA tensors or both numpy arrays")
            if C_left.dtype != torch.complex128 or C_right.dtype != torch.complex128:
                raise TypeError("device vectors must be complex128")
            L, R = C_left.contiguous().view(-1), C_right.contiguous().view(-1)
        else:
            L = torch.from_numpy(np.ascontiguousarray(C_left, dtype=np.complex128).reshape(-1)).cuda()
            R = torch.from_numpy(np.ascontiguousarray(C_right, dtype=np.complex128).reshape(-1)).cuda()
        if L.numel() != self.lists.ndet or R.numel() != self.lists.ndet:
            raise RuntimeError("vector length does not match the number of determinants")
        out = torch.zeros(max(size, 1), dtype=torch.complex128, device="cuda")
        if self.h is not None:
            check(lib().f2g_rel_sigma_rdm(self.h, k, L.data_ptr(), R.data_ptr(), out.data_ptr(), stream_handle()))
        res = out[:size].view(shape)
        return res if device else res.cpu().numpy()

    def so_1rdm(self, C_left, C_right):
        """gamma[p][q] = <L| a+_p a_q |R> over spinors (rel_ci_sigma_builder_rdm.cc:14-71)."""
        return self._so_rdm("so_1rdm", C_left, C_right)

    def so_2rdm(self, C_left, C_right):
        """gamma[p][q][r][s] = <L| a+_p a+_q a_s a_r |R> (rel_ci_sigma_builder_rdm.cc:73-183)."""
        return self._so_rdm("so_2rdm", C_left, C_right)

    def so_2cumulant(self, C_left, C_right):
        """lambda2 = gamma2 - g1[p][r] g1[q][s] + g1[p][s] g1[q][r] (rel_ci_sigma_builder_rdm.cc:185-207)."""
        return self._so_rdm("so_2cumulant", C_left, C_right)

    def so_3rdm(self, C_left, C_right):
        """The spin-orbital 3-RDM (n^6) (rel_ci_sigma_builder_rdm.cc:209-365)."""
        return self._so_rdm("so_3rdm", C_left, C_right)

    def so_3cumulant(self, C_left, C_right):
        """The spin-orbital 3-cumulant (rel_ci_sigma_builder_rdm.cc:367-404)."""
        return self._so_rdm("so_3cumulant", C_left, C_right)


class CISpinAdapter:
    """CSF <-> determinant transforms (forte2/determinant/ci_spin_adapter.cc:55-288) on the device."""

    def __init__(self, twoS, twoMs, norb):
        self.twoS, self.twoMs, self.norb = int(twoS), int(twoMs), int(norb)
        self.h = None
        self.log_level = 3
        self._info = [0, 0, 0]

    def set_log_level(self, level):
        self.log_level = int(level)

    def prepare_couplings(self, dets):
        strings = dets.strings if isinstance(dets, Determinants) else dets
        if self.h:
            lib().f2g_spin_adapter_destroy(self.h)
            self.h = None
        self.strings = strings
        h = C.c_void_p()
        check(lib().f2g_spin_adapter_create(strings.h, self.twoS, self.twoMs, C.byref(h)))
        self.h = h
        info = np.zeros(3, dtype=np.int64)
        check(lib().f2g_spin_adapter_info(self.h, info.ctypes.data))
        self._info = [int(x) for x in info]

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().f2g_spin_adapter_destroy(h)
            self.h = None

    nconf = property(lambda self: self._info[0])
    ncsf = property(lambda self: self._info[1])
    ncoupling = property(lambda self: self._info[2])
    ndet = property(lambda self: self.strings.ndet)

    def _transform(self, fn, src, dst, nsrc, ndst):
        torch = _torch()
        if _is_cuda_tensor(src) and _is_cuda_tensor(dst):
            _dev_vec(src)
            _dev_vec(dst)
            nvec = 1 if src.dim() == 1 else src.shape[0]
            check(fn(self.h, src.data_ptr(), dst.data_ptr(), nvec, stream_handle()))
            return dst
        s = torch.from_numpy(np.ascontiguousarray(_host_vec(src) if src.ndim == 1 else src)).cuda()
        d = torch.empty(ndst, dtype=torch.float64, device="cuda")
        check(fn(self.h, s.data_ptr(), d.data_ptr(), 1, stream_handle()))
        dst[:] = d.cpu().numpy()
        return dst

    def csf_C_to_det_C(self, csf_C, det_C):
        return self._transform(lib().f2g_csf_to_det, csf_C, det_C, self.ncsf, self.ndet)

    def det_C_to_csf_C(self, det_C, csf_C):
        return self._transform(lib().f2g_det_to_csf, det_C, csf_C, self.ndet, self.ncsf)

    def couplings(self):
        """(bounds[ncsf+1], det_idx, coeff, conf_ranges[nconf, 2]) in the reference's order."""
        b = np.zeros(self.ncsf + 1, dtype=np.int64)
        d = np.zeros(max(1, self.ncoupling), dtype=np.int64)
        c = np.zeros(max(1, self.ncoupling))
        r = np.zeros(max(2, 2 * self.nconf), dtype=np.int64)
        check(lib().f2g_spin_adapter_dump(self.h, b.ctypes.data, d.ctypes.data, c.ctypes.data, r.ctypes.data))
        return b, d[: self.ncoupling], c[: self.ncoupling], r[: 2 * self.nconf].reshape(-1, 2)


class CISigmaBuilder:
    """sigma = H C for determinant vectors (forte2/ci/ci_sigma_builder.h:26-117), on the GPU.

    ``set_algorithm`` accepts the reference's four names; both algorithms return the same
    sigma (to rounding) and run the same device kernels. ``set_precision("fp32")`` selects
    FP32 arithmetic for every term (the mixed-precision mode; FP64 is the default and matches
    the reference's arithmetic).
    """

    def __init__(self, lists: CIStrings, E, H, V, log_level=3):
        self.lists = lists
        self.log_level = int(log_level)
        H, V = self._validate(H, V)
        self._E = float(E)
        self.h = C.c_void_p()
        self._H, self._V = H, V
        check(lib().f2g_sigma_create(lists.h, self._E, H.ctypes.data, V.ctypes.data, self.log_level,
                                     C.byref(self.h)))
        self._algorithm = "Knowles-Handy"
        self._precision = 0

    def _validate(self, H, V):
        H = np.asarray(H, dtype=np.float64)
        V = np.asarray(V, dtype=np.float64)
        n = self.lists.norb
        if H.ndim != 2:
            raise RuntimeError("H must be a 2D matrix.")
        if H.shape != (n, n):
            raise RuntimeError("H shape does not match the number of orbitals.")
        if V.ndim != 4:
            raise RuntimeError("V must be a 4D tensor.")
        if V.shape != (n, n, n, n):
            raise RuntimeError("V shape does not match the number of orbitals.")
        return np.ascontiguousarray(H), np.ascontiguousarray(V)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().f2g_sigma_destroy(h)
            self.h = None

    def set_log_level(self, level):
        self.log_level = int(level)

    def update_integrals(self, E, H, V):
        """Replace the integrals, ordered on the current CUDA stream (no counterpart in the reference,
        whose builder takes its integrals once, ci_sigma_builder.cc:102-185). Nothing waits for the
        rest of the device and the device buffers keep their addresses, so a pool of builders can
        serve new requests of the same active space without new allocations or graph captures."""
        H, V = self._validate(H, V)
        self._E, self._H, self._V = float(E), H, V
        check(lib().f2g_sigma_set_hamiltonian_async(self.h, self._E, H.ctypes.data, V.ctypes.data, stream_handle()))

    def set_memory(self, mb):
        check(lib().f2g_sigma_set_memory(self.h, int(mb)))

    def set_tensor_cores(self, on=True):
        """FP32 precision: opposite-spin term on the tensor cores (split-FP16 products, FP32
        accumulation, exact fixed-point row sums). Returns whether this space supports it (else the
        CUDA-core kernel runs). No counterpart in the reference."""
        avail = np.zeros(1, dtype=np.int32)
        check(lib().f2g_sigma_set_tensor_cores(self.h, int(bool(on)), avail.ctypes.data))
        return bool(avail[0])

    _VARIANTS = {"tensor_cores": 0, "narrow_same_spin": 1, "persistent_opposite": 2, "tc_wait_limit": 3,
                 "irrep_blocks": 4, "tma_b": 5, "dense_same_spin": 6}

    def set_variant(self, name, value):
        """Select a kernel variant with identical results (see forte2_gb300.autotune)."""
        check(lib().f2g_sigma_set_variant(self.h, self._VARIANTS[name], int(value)))

    def tensor_core_error(self):
        out = np.zeros(1, dtype=np.int32)
        check(lib().f2g_sigma_tc_error(self.h, out.ctypes.data))
        return int(out[0])

    def set_max_blocks(self, n):
        """Cap the opposite-spin kernel at n thread blocks (one per SM; 0 = no cap), leaving the
        other SMs to concurrent solves. Same sigma. No counterpart in the reference."""
        check(lib().f2g_sigma_set_max_blocks(self.h, int(n)))

    def set_algorithm(self, algorithm):
        check(lib().f2g_sigma_set_algorithm(self.h, algorithm.encode()))

    def get_algorithm(self):
        buf = C.create_string_buffer(64)
        check(lib().f2g_sigma_get_algorithm(self.h, buf, 64))
        return buf.value.decode()

    def set_precision(self, precision):
        p = {"fp64": 0, "fp32": 1, 0: 0, 1: 1}[precision]
        check(lib().f2g_sigma_set_precision(self.h, p))
        self._precision = p
        # kernel variants chosen by the autotuner for this precision (forte2_gb300.autotune)
        for name, value in getattr(self, "_tuned", {}).get(self.get_precision(), {}).items():
            self.set_variant(name, value)

    def get_precision(self):
        return "fp64" if self._precision == 0 else "fp32"

    def set_Hamiltonian(self, E, H, V):
        H, V = self._validate(H, V)
        self._E, self._H, self._V = float(E), H, V
        check(lib().f2g_sigma_set_hamiltonian(self.h, self._E, H.ctypes.data, V.ctypes.data))

    def Hamiltonian(self, basis, sigma):
        """sigma <- H basis. numpy (host) or CUDA float64 tensors; a (nvec, ndet) CUDA tensor
        applies H to every row."""
        if _is_cuda_tensor(basis) and _is_cuda_tensor(sigma):
            _dev_vec(basis)
            _dev_vec(sigma)
            nvec = 1 if basis.dim() == 1 else basis.shape[0]
            if basis.numel() != nvec * self.lists.ndet or sigma.numel() != basis.numel():
                raise RuntimeError("vector length does not match the number of determinants")
            check(lib().f2g_sigma_apply(self.h, basis.data_ptr(), sigma.data_ptr(), nvec, stream_handle()))
            return
        b = _host_vec(basis)
        s = _host_vec(sigma, "sigma")
        if b.shape[0] != self.lists.ndet or s.shape[0] != self.lists.ndet:
            raise RuntimeError("vector length does not match the number of determinants")
        check(lib().f2g_sigma_apply_host(self.h, b.ctypes.data, s.ctypes.data, 1))

    # ---- reduced density matrices (ci_sigma_builder_1rdm.cc:9-84, ci_sigma_builder_2rdm.cc:46-282)

    _RDM_KINDS = {"a_1rdm": 0, "b_1rdm": 1, "sf_1rdm": 2, "aa_2rdm": 3, "bb_2rdm": 4, "ab_2rdm": 5,
                  "sf_2rdm": 6, "sf_2cumulant": 7, "aaa_3rdm": 8, "bbb_3rdm": 9, "aab_3rdm": 10, "abb_3rdm": 11,
                  "sf_3rdm": 12, "sf_3cumulant": 13}

    @staticmethod
    def _rdm_shape(k, n):
        npair = n * (n - 1) // 2
        ntrip = n * (n - 1) * (n - 2) // 6
        return {0: (n, n), 1: (n, n), 2: (n, n), 3: (npair, npair), 4: (npair, npair), 8: (ntrip, ntrip),
                9: (ntrip, ntrip), 10: (npair, n, npair, n), 11: (n, npair, n, npair), 12: (n,) * 6,
                13: (n,) * 6}.get(k, (n, n, n, n))

    def _rdm(self, kind, C_left, C_right):
        """RDM `kind` between the bra C_left and the ket C_right. numpy vectors give a numpy array
        (the reference's return type); CUDA float64 tensors give a CUDA tensor and stay on the
        device. Passing the same vector twice selects the symmetric kernels."""
        torch = _torch()
        n = self.lists.norb
        k = self._RDM_KINDS[kind]
        shape = self._rdm_shape(k, n)
        size = int(lib().f2g_rdm_size(n, k))
        device = _is_cuda_tensor(C_left)
        if device:
            if not _is_cuda_tensor(C_right):
                raise TypeError("C_left and C_right must both be CUDA tensors or both numpy arrays")
            L, R = _dev_vec(C_left), _dev_vec(C_right)
        else:
            hl = _host_vec(C_left, "C_left")
            L = torch.from_numpy(np.ascontiguousarray(hl)).cuda()
            R = L if C_right is C_left else torch.from_numpy(np.ascontiguousarray(_host_vec(C_right, "C_right"))).cuda()
        if L.numel() != self.lists.ndet or R.numel() != self.lists.ndet:
            raise RuntimeError("vector length does not match the number of determinants")
        out = torch.empty(max(size, 1), dtype=torch.float64, device="cuda")
        check(lib().f2g_sigma_rdm(self.h, k, L.data_ptr(), R.data_ptr(), out.data_ptr(), stream_handle()))
        res = out[:size].view(shape)
        return res if device else res.cpu().numpy()

    def a_1rdm(self, C_left, C_right):
        """gamma[p][q] = <L| a+_p a_q |R>, alpha (ci_sigma_builder_1rdm.cc:9-65)."""
        return self._rdm("a_1rdm", C_left, C_right)

    def b_1rdm(self, C_left, C_right):
        return self._rdm("b_1rdm", C_left, C_right)

    def sf_1rdm(self, C_left, C_right):
        return self._rdm("sf_1rdm", C_left, C_right)

    def aa_2rdm(self, C_left, C_right):
        """Packed alpha-alpha 2-RDM [pq][rs], p > q, r > s (ci_sigma_builder_2rdm.cc:46-117)."""
        return self._rdm("aa_2rdm", C_left, C_right)

    def bb_2rdm(self, C_left, C_right):
        return self._rdm("bb_2rdm", C_left, C_right)

    def ab_2rdm(self, C_left, C_right):
        """Alpha-beta 2-RDM [u][v][x][y] (ci_sigma_builder_2rdm.cc:119-201)."""
        return self._rdm("ab_2rdm", C_left, C_right)

    def sf_2rdm(self, C_left, C_right):
        return self._rdm("sf_2rdm", C_left, C_right)

    def sf_2cumulant(self, C_left, C_right):
        return self._rdm("sf_2cumulant", C_left, C_right)

    # three-body RDMs (ci_sigma_builder_3rdm.cc:84-541)
    def aaa_3rdm(self, C_left, C_right):
        """Packed alpha 3-RDM [pqr][stu], p > q > r, s > t > u (triplet index
        p(p-1)(p-2)/6 + q(q-1)/2 + r)."""
        return self._rdm("aaa_3rdm", C_left, C_right)

    def bbb_3rdm(self, C_left, C_right):
        return self._rdm("bbb_3rdm", C_left, C_right)

    def aab_3rdm(self, C_left, C_right):
        """[pq][r][st][u]: alpha pairs pq, st (p > q, s > t), beta r, u."""
        return self._rdm("aab_3rdm", C_left, C_right)

    def abb_3rdm(self, C_left, C_right):
        """[p][qr][s][tu]: alpha p, s; beta pairs qr, tu (q > r, t > u)."""
        return self._rdm("abb_3rdm", C_left, C_right)

    def sf_3rdm(self, C_left, C_right):
        return self._rdm("sf_3rdm", C_left, C_right)

    def sf_3cumulant(self, C_left, C_right):
        return self._rdm("sf_3cumulant", C_left, C_right)

    # transition 1-RDMs between two wave functions (ci_sigma_builder_1trdm.cc:10-131): both must
    # have the same orbitals and electron counts; in a CAS space they then share one determinant
    # list, so the transition RDM is the RDM between the two vectors
    def _check_trdm_partner(self, sigmabuilder_right):
        left, right = self.lists, sigmabuilder_right.lists
        if left.norb != right.norb:
            raise RuntimeError("FCI transition RDMs: The number of MOs must be the same in the two wave functions.")
        if left.na != right.na or left.nb != right.nb:
            raise RuntimeError("FCI transition RDMs: The number of alpha and beta electrons must be the same in the "
                               "two wave functions.")

    def a_1trdm(self, sigmabuilder_right, C_left, C_right):
        self._check_trdm_partner(sigmabuilder_right)
        return self._rdm("a_1rdm", C_left, C_right)

    def b_1trdm(self, sigmabuilder_right, C_left, C_right):
        self._check_trdm_partner(sigmabuilder_right)
        return self._rdm("b_1rdm", C_left, C_right)

    def sf_1trdm(self, sigmabuilder_right, C_left, C_right):
        self._check_trdm_partner(sigmabuilder_right)
        return self._rdm("sf_1rdm", C_left, C_right)

    def term(self, which, basis):
        """One HZ term alone (device tensors): "h0", "h1_a", "h1_b", "aabb", "aaaa", "bbbb"."""
        torch = _torch()
        idx = {"h0": 0, "h1_a": 1, "h1_b": 2, "aabb": 3, "aaaa": 4, "bbbb": 5}[which]
        out = torch.empty_like(basis)
        check(lib().f2g_sigma_term(self.h, idx, basis.data_ptr(), out.data_ptr(), stream_handle()))
        return out

    def apply_csf(self, spin_adapter, basis, sigma):
        """sigma = P^T H P basis for CSF vectors (device tensors, rows or one vector): the CI
        driver's sigma closure (ci.py:221-235) in one call; FP32 transforms in FP32 precision."""
        nvec = 1 if basis.dim() == 1 else basis.shape[0]
        if basis.shape != sigma.shape or basis.shape[-1] != spin_adapter.ncsf:
            raise RuntimeError("CSF vectors must be (nvec, ncsf) with matching shapes")
        if not (basis.is_contiguous() and sigma.is_contiguous()):
            raise RuntimeError("CSF vectors must be contiguous")
        check(lib().f2g_sigma_apply_csf(self.h, spin_adapter.h, basis.data_ptr(), sigma.data_ptr(), nvec,
                                        stream_handle()))

    def reset_build_times(self):
        check(lib().f2g_sigma_reset_build_times(self.h))

    def avg_build_time(self):
        out = np.zeros(4)
        check(lib().f2g_sigma_avg_build_time(self.h, out.ctypes.data))
        return [float(x) for x in out]

    def det_energies(self):
        torch = _torch()
        out = torch.empty(self.lists.ndet, dtype=torch.float64, device="cuda")
        check(lib().f2g_sigma_det_energies(self.h, out.data_ptr(), stream_handle()))
        return out

    def hdiag_csf_device(self, spin_adapter: CISpinAdapter):
        torch = _torch()
        out = torch.empty(spin_adapter.ncsf, dtype=torch.float64, device="cuda")
        check(lib().f2g_hdiag_csf(self.h, spin_adapter.h, out.data_ptr(), stream_handle()))
        return out

    def form_Hdiag_csf(self, dets, spin_adapter: CISpinAdapter, spin_adapt_full_preconditioner=False):
        """Approximate CSF diagonal sum_i c_i^2 E(det_i) (ci_sigma_builder.cc:317-370). With
        spin_adapt_full_preconditioner the exact <I|H|I> is used (ci_sigma_builder.cc:323-330)."""
        if spin_adapt_full_preconditioner:
            return np.array([self.energy_csf(dets, spin_adapter, i) for i in range(spin_adapter.ncsf)])
        return self.hdiag_csf_device(spin_adapter).cpu().numpy()

    def csf_matrix(self, spin_adapter: CISpinAdapter, indices):
        idx = np.ascontiguousarray(indices, dtype=np.int64)
        m = len(idx)
        out = np.zeros((m, m))
        if m:
            check(lib().f2g_csf_matrix(self.h, spin_adapter.h, idx.ctypes.data, m, out.ctypes.data))
        return out

    def slater_rules_csf(self, dets, spin_adapter, I, J):
        return float(self.csf_matrix(spin_adapter, [I, J])[0, 1]) if I != J else self.energy_csf(
            dets, spin_adapter, I)

    def energy_csf(self, dets, spin_adapter, I):
        return float(self.csf_matrix(spin_adapter, [I])[0, 0])

    def form_H_csf(self, dets, spin_adapter, memory_mb=1024):
        ncsf = spin_adapter.ncsf
        if ncsf * ncsf * 8 > memory_mb * 1024 * 1024:
            raise RuntimeError(
                "Not enough memory to form the full Hamiltonian matrix in the CSF basis. Increase the "
                "memory limit or use a different algorithm.")
        return self.csf_matrix(spin_adapter, np.arange(ncsf))
