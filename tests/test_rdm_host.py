"""CPU checks of the reduced-density-matrix boundary: the orbital-pair lists the mixed-spin 2-RDM
kernel runs over are built by host code in the CUDA library (no GPU call). Their layout is
decoded here and the kernel's contraction is replayed in numpy, sentinel padding included, and
compared with the oracle's mixed-spin 2-RDM; the list invariants are checked directly."""

import ctypes as C
import os
import shutil
from math import comb

import numpy as np
import pytest

from forte2_gb300.synthetic import random_ci_vector
from oracle.port import PortCI, build_port

SEG = 64


@pytest.fixture(scope="module")
def lib():
    from forte2_gb300.build import LIB_PATH, build

    if not os.path.exists(LIB_PATH):
        if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("nvcc not available")
        build()
    from forte2_gb300._lib import lib as L

    build_port()
    return L()


def pair_list(L, n, k, wide=False):
    counts = np.zeros(4, np.int64)
    assert L.f2g_rdm_pair_list(n, k, int(wide), None, None, counts.ctypes.data) == 0
    nseg, nentry, is_wide, N0 = (int(x) for x in counts)
    ent = np.zeros(max(1, nseg * SEG), np.uint64 if is_wide else np.uint32)
    pair = np.zeros(max(1, nseg), np.uint16)
    if nseg:
        assert L.f2g_rdm_pair_list(n, k, int(wide), ent.ctypes.data, pair.ctypes.data, counts.ctypes.data) == 0
    return dict(nseg=nseg, nentry=nentry, wide=bool(is_wide), N0=N0, ent=ent[: nseg * SEG], pair=pair[:nseg])


def decode(pl):
    """(segment, left, right, negative) per stored slot, in segment-major order."""
    nseg = pl["nseg"]
    g = np.arange(nseg)[:, None]
    j = np.arange(SEG)[None, :]
    at = ((g // 32) * SEG + j) * 32 + g % 32
    e = pl["ent"][at].astype(np.uint64)
    if pl["wide"]:
        left, right, neg = e & 0xFFFFFF, (e >> 24) & 0xFFFFFF, (e >> 48) & 1
    else:
        left, right, neg = e & 0x7FFF, (e >> 15) & 0x7FFF, (e >> 30) & 1
    seg = np.broadcast_to(g, left.shape)
    return seg.astype(np.int64), left.astype(np.int64), right.astype(np.int64), neg.astype(np.int64)


def replay_ab(n, pa, pb, CL, CR, NA, NB):
    """The mixed-spin kernel's contraction in numpy: per alpha entry, sum every beta segment with
    the zero sentinel at index NB, add into the (u, x) slab by segment pair."""
    ga = np.zeros((n, n, n, n))
    sa, la, ra, na_ = (x.ravel() for x in decode(pa))
    sb, lb, rb, nb_ = (x.ravel() for x in decode(pb))
    ZL = np.zeros((NA, NB + 1))
    ZR = np.zeros((NA, NB + 1))
    ZL[:, :NB] = CL.reshape(NA, NB)
    ZR[:, :NB] = CR.reshape(NA, NB)
    wb = 1.0 - 2.0 * nb_
    for s, il, ir, ng in zip(sa, la, ra, na_):
        if il >= NA:  # padding entry of the alpha list
            continue
        u, x = divmod(int(pa["pair"][s]), n)
        terms = wb * ZL[il, lb] * ZR[ir, rb]
        seg_sum = np.bincount(sb, weights=terms, minlength=pb["nseg"])
        slab = np.bincount(pb["pair"].astype(np.int64), weights=seg_sum, minlength=n * n).reshape(n, n)
        ga[u, :, x, :] += (-1.0 if ng else 1.0) * slab
    return ga


@pytest.mark.parametrize("n,na,nb", [(4, 2, 2), (6, 3, 3), (6, 2, 3), (5, 1, 4), (6, 3, 1), (7, 3, 2)])
def test_pair_lists_replay_matches_oracle(lib, n, na, nb):
    pa = pair_list(lib, n, na, wide=True)
    pb = pair_list(lib, n, nb)
    port = PortCI(n, na, nb)
    CL = random_ci_vector(port.ndet, 300 + n)
    CR = random_ci_vector(port.ndet, 400 + n)
    NA, NB = comb(n, na), comb(n, nb)
    ref = port.rdm("ab_2rdm", CL, CR).reshape(n, n, n, n)
    got = replay_ab(n, pa, pb, CL, CR, NA, NB)
    assert np.abs(got - ref).max() < 1e-13 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("n,k", [(1, 1), (3, 1), (4, 2), (6, 3), (8, 4), (9, 2), (16, 8)])
@pytest.mark.parametrize("wide", [False, True])
def test_pair_list_invariants(lib, n, k, wide):
    pl = pair_list(lib, n, k, wide)
    N0 = comb(n, k)
    assert pl["N0"] == N0
    assert pl["nseg"] % 32 == 0
    # every ordered pair (p, q): C(n-2, k-1) strings K without p and q, C(n-1, k-1) when p == q
    per_pair = {p * n + q: comb(n - 1, k - 1) if p == q else comb(n - 2, k - 1) for p in range(n) for q in range(n)}
    assert pl["nentry"] == sum(per_pair.values()) == comb(n, k - 1) * (n - k + 1) ** 2
    seg, left, right, neg = decode(pl)
    real = left < N0
    assert np.all((left == N0) == (right == N0))  # padding has both sides at the sentinel
    assert int(real.sum()) == pl["nentry"]
    pairs = pl["pair"][seg[real]].astype(np.int64)
    counts = np.bincount(pairs, minlength=n * n)
    assert all(counts[pq] == c for pq, c in per_pair.items())
    # entries are (K+p, K+q) for one K: the two strings differ by moving one electron q -> p
    port = PortCI(n, k, 0)
    strings = port.strings(0)
    ml, mr = strings[left[real]], strings[right[real]]
    p, q = pairs // n, pairs % n
    one = np.uint64(1)
    has_p = (ml >> p.astype(np.uint64)) & one
    has_q = (mr >> q.astype(np.uint64)) & one
    assert np.all(has_p == 1) and np.all(has_q == 1)
    K_l = ml & ~(one << p.astype(np.uint64))
    K_r = mr & ~(one << q.astype(np.uint64))
    assert np.array_equal(K_l, K_r)
    # sign = (-1)^{#occupied below p in K} (-1)^{#occupied below q in K}
    below = lambda m, o: np.array([bin(int(a) & ((1 << int(b)) - 1)).count("1") & 1 for a, b in zip(m, o)])
    assert np.array_equal(neg[real], below(K_l, p) ^ below(K_l, q))
    if not wide:
        assert pl["wide"] == (N0 > 32766)


def test_pair_list_validation(lib):
    counts = np.zeros(4, np.int64)
    assert lib.f2g_rdm_pair_list(4, 5, 0, None, None, counts.ctypes.data) == 2
    assert lib.f2g_rdm_pair_list(-1, 0, 0, None, None, counts.ctypes.data) == 2
    assert lib.f2g_rdm_pair_list(4, 2, 0, None, None, None) == 2
    assert lib.f2g_rdm_size(6, 0) == 36 and lib.f2g_rdm_size(6, 3) == 225 and lib.f2g_rdm_size(6, 7) == 6 ** 4
    assert lib.f2g_rdm_size(1, 3) == 0 and lib.f2g_rdm_size(6, 14) == -1
    # three-body kinds: (T, T), (P, n, P, n), n^6
    assert lib.f2g_rdm_size(6, 8) == 20 * 20 and lib.f2g_rdm_size(6, 10) == (15 * 6) ** 2
    assert lib.f2g_rdm_size(6, 12) == 6 ** 6 and lib.f2g_rdm_size(2, 9) == 0
    # spin-orbital (two-component) kinds: full complex tensors n^2, n^4, n^4, n^6, n^6
    assert [lib.f2g_rel_rdm_size(5, k) for k in range(5)] == [25, 625, 625, 5 ** 6, 5 ** 6]
    assert lib.f2g_rel_rdm_size(5, 5) == -1 and lib.f2g_rel_rdm_size(-1, 0) == -1


def replay_hole_gram(rows_of_K, ncol, CL, CR, d):
    """The hole-list Gram kernel's contraction: per hole string K with entries (I, o, sign),
    out[o_i][o_j] += s_i s_j <CL row I_i | CR row I_j>."""
    out = np.zeros((d, d))
    L = CL.reshape(-1, ncol)
    R = CR.reshape(-1, ncol)
    for ent in rows_of_K:
        I = np.array([e[0] for e in ent])
        o = np.array([e[1] for e in ent])
        s = np.array([e[2] for e in ent], dtype=float)
        G = (s[:, None] * L[I]) @ (s[:, None] * R[I]).T
        np.add.at(out, (o[:, None], o[None, :]), G)
    return out


@pytest.mark.parametrize("n,na,nb", [(6, 3, 3), (6, 2, 4), (7, 3, 2), (5, 4, 1)])
def test_hole_gram_replay_matches_oracle(n, na, nb):
    """The 1-RDM / same-spin 2-RDM kernels' formula over the 1-hole and 2-hole lists (the device
    builds these lists bit for bit as the oracle does) reproduces the oracle's RDMs; beta rows are
    the rows of the transposed vectors, as on the device."""
    build_port()
    port = PortCI(n, na, nb)
    CL = random_ci_vector(port.ndet, 500 + n)
    CR = random_ci_vector(port.ndet, 600 + n)
    NA, NB = comb(n, na), comb(n, nb)
    npair = n * (n - 1) // 2
    for spin, kind1, kind2 in ((0, "a_1rdm", "aa_2rdm"), (1, "b_1rdm", "bb_2rdm")):
        L, R, ncol = (CL, CR, NB) if spin == 0 else (CL.reshape(NA, NB).T.ravel(), CR.reshape(NA, NB).T.ravel(), NA)
        l1 = port.list_1h(spin)  # rows (class_K, K, class_I, sign, p, I)
        byK = {}
        for r in l1:
            byK.setdefault(int(r[1]), []).append((int(r[5]), int(r[4]), int(r[3])))
        got1 = replay_hole_gram(byK.values(), ncol, L, R, n)
        ref1 = port.rdm(kind1, CL, CR).reshape(n, n)
        assert np.abs(got1 - ref1).max(initial=0) < 1e-13
        l2 = port.list_2h(spin)  # rows (class_K, K, class_I, sign, p, q, I)
        byK = {}
        for r in l2:
            p, q = int(r[4]), int(r[5])
            byK.setdefault(int(r[1]), []).append((int(r[6]), p * (p - 1) // 2 + q, int(r[3])))
        got2 = replay_hole_gram(byK.values(), ncol, L, R, npair)
        ref2 = port.rdm(kind2, CL, CR).reshape(npair, npair)
        assert np.abs(got2 - ref2).max(initial=0) < 1e-13


def test_packed_expansion_and_top_determinants():
    """Host helpers of the CI driver: the packed same-spin 2-RDM expansion used by the RDM energy
    check (ci.py:337-341) reproduces the oracle's energy through the antisymmetrised integrals, and
    the top-determinant selection of ci.py:823-830."""
    from forte2_gb300.ci import packed_tensor4_to_tensor4, top_determinants
    from forte2_gb300.synthetic import make_integrals

    build_port()
    n, na, nb = 6, 3, 3
    ints = make_integrals(n, 41)
    port = PortCI(n, na, nb)
    port.set_hamiltonian(ints.E, ints.H, ints.V)
    c = random_ci_vector(port.ndet, 42)
    npair = n * (n - 1) // 2
    aa = port.rdm("aa_2rdm", c, c).reshape(npair, npair)
    full = packed_tensor4_to_tensor4(aa, n)
    assert np.allclose(full, -full.transpose(1, 0, 2, 3)) and np.allclose(full, -full.transpose(0, 1, 3, 2))
    assert full[3, 1, 2, 0] == aa[3 * 2 // 2 + 1, 1]
    V = ints.V
    A = V - V.transpose(0, 1, 3, 2)
    i, j = np.tril_indices(n, k=-1)
    M = A[i[:, None], j[:, None], i[None, :], j[None, :]]
    assert abs(np.einsum("ij,ij", aa, M) - 0.25 * np.einsum("ijkl,ijkl", full, A)) < 1e-12
    assert packed_tensor4_to_tensor4(np.zeros((0, 0)), 1).shape == (1, 1, 1, 1)
    top = top_determinants(np.array([0.1, -0.9, 0.3, 0.0]), ["a", "b", "c", "d"], 3)
    assert top == [("b", -0.9), ("c", 0.3), ("a", 0.1)]
    assert top_determinants(np.array([0.5]), ["a"], 5) == [("a", 0.5)]
