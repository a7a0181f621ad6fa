"""Seeded synthetic active-space integrals and CASCI workload definitions.

The recipe stands in for the molecular integrals the reference obtains from
``RestrictedMOIntegrals`` (forte2/jkbuilder/mointegrals.py:15-86); no public dataset is involved.

Per instance ``rng = np.random.default_rng(seed)``, draws in this order:

1. orbital energies ``eps = sort(rng.uniform(-2, 1, n))`` on the diagonal of h;
2. the strict upper triangle of h (``np.triu_indices(n, 1)`` order) from ``N(0, 0.05)``,
   mirrored to keep h symmetric;
3. ``B = rng.normal(0, 0.1, (naux, n, n))`` with ``naux = 4 n``, made symmetric in (p, q) by
   keeping the upper triangle (diagonal included) and mirroring it;

then the chemist integrals ``(pq|rs) = sum_Q B[Q,p,q] B[Q,r,s]`` are handed to the sigma
builder in the reference's physicist layout ``V[p,q,r,s] = <pq|rs> = (pr|qs)``
(forte2/ci/ci_sigma_builder.h:293-296). The scalar (core) energy is 0.
"""

from __future__ import annotations

from dataclasses import dataclass
from math import comb

import numpy as np


@dataclass
class ActiveSpaceIntegrals:
    E: float
    H: np.ndarray  # (n, n)
    V: np.ndarray  # (n, n, n, n) physicist <pq|rs>
    eri: np.ndarray  # (n, n, n, n) chemist (pq|rs)

    @property
    def norb(self):
        return self.H.shape[0]


def make_integrals(norb: int, seed: int, naux: int | None = None) -> ActiveSpaceIntegrals:
    n = int(norb)
    naux = 4 * n if naux is None else int(naux)
    rng = np.random.default_rng(seed)
    eps = np.sort(rng.uniform(-2.0, 1.0, n))
    h = np.diag(eps)
    iu = np.triu_indices(n, 1)
    off = rng.normal(0.0, 0.05, len(iu[0]))
    h[iu] = off
    h[(iu[1], iu[0])] = off
    B = rng.normal(0.0, 0.1, (naux, n, n))
    B = np.triu(B) + np.transpose(np.triu(B, 1), (0, 2, 1))
    eri = np.einsum("Qpq,Qrs->pqrs", B, B, optimize=True)
    V = np.ascontiguousarray(eri.transpose(0, 2, 1, 3))
    return ActiveSpaceIntegrals(0.0, np.ascontiguousarray(h), V, eri)


def rotate_integrals(ints: ActiveSpaceIntegrals, seed: int, theta: float = 0.05) -> ActiveSpaceIntegrals:
    """The active-space integrals of the next macro-iteration of an orbital optimiser
    (forte2/mcopt/mc_optimizer.py:297-328), from ``default_rng(seed)``:

    1. an active-active rotation U = exp(K), K antisymmetric with strict-upper entries N(0, theta)
       (``np.triu_indices(n, 1)`` order): h -> U^T h U, (pq|rs) -> sum U_ap U_bq U_cr U_ds (ab|cd);
       alone it leaves the CASCI energies unchanged but changes every determinant matrix element;
    2. the change an inactive-active rotation makes, modelled as a mix with a fresh draw of the
       integral recipe: x -> (1 - theta) x + theta x', x' = make_integrals(n, seed + 1) (the energies
       move by O(theta); the 8-fold symmetry of (pq|rs) is kept).
    """
    from scipy.linalg import expm

    n = ints.norb
    rng = np.random.default_rng(seed)
    iu = np.triu_indices(n, 1)
    K = np.zeros((n, n))
    K[iu] = rng.normal(0.0, theta, len(iu[0]))
    K = K - K.T
    U = expm(K)
    fresh = make_integrals(n, seed + 1)
    h = (1.0 - theta) * (U.T @ ints.H @ U) + theta * fresh.H
    h = 0.5 * (h + h.T)
    eri = np.einsum("ap,bq,cr,ds,abcd->pqrs", U, U, U, U, ints.eri, optimize=True)
    eri = (1.0 - theta) * eri + theta * fresh.eri
    V = np.ascontiguousarray(eri.transpose(0, 2, 1, 3))
    return ActiveSpaceIntegrals(ints.E, np.ascontiguousarray(h), V, eri)


def make_spinor_integrals(nspinor: int, seed: int, naux: int | None = None):
    """Seeded complex integrals of a two-component (spinor) active space: E, a Hermitian h
    (nspinor x nspinor) and physicist V[p][q][r][s] = (pr|qs) with (pr|qs) = sum_Q L_Q[p][r]
    L_Q[q][s] over Hermitian L_Q, so that V[p][q][r][s] = V[q][p][s][r] and
    conj(V[p][q][r][s]) = V[r][s][p][q] (a Hermitian two-body operator)."""
    n = int(nspinor)
    naux = 3 * n if naux is None else int(naux)
    rng = np.random.default_rng(seed)
    eps = np.sort(rng.uniform(-2.0, 1.0, n))
    A = rng.normal(0.0, 0.05, (n, n)) + 1j * rng.normal(0.0, 0.05, (n, n))
    h = np.diag(eps).astype(np.complex128) + np.triu(A, 1) + np.triu(A, 1).conj().T
    L = rng.normal(0.0, 0.1, (naux, n, n)) + 1j * rng.normal(0.0, 0.1, (naux, n, n))
    L = 0.5 * (L + np.conj(np.transpose(L, (0, 2, 1))))
    eri = np.einsum("Qpr,Qqs->prqs", L, L, optimize=True)
    V = np.ascontiguousarray(eri.transpose(0, 2, 1, 3))
    return 0.25, np.ascontiguousarray(h), V


def random_complex_vector(ndet: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.normal(size=ndet) + 1j * rng.normal(size=ndet)
    return c / np.linalg.norm(c)


def symmetrize_integrals(ints: ActiveSpaceIntegrals, orbsym) -> ActiveSpaceIntegrals:
    """The integrals of a molecule with an abelian point group: with irreps ``orbsym[p]`` (0..7,
    the product of two irreps their XOR), h[p][q] = 0 unless p and q share an irrep and
    (pq|rs) = 0 unless the product of the four irreps is the totally symmetric one."""
    g = np.asarray(orbsym, dtype=np.int64)
    h = np.where(g[:, None] == g[None, :], ints.H, 0.0)
    allowed = (g[:, None, None, None] ^ g[None, :, None, None] ^ g[None, None, :, None] ^ g[None, None, None, :]) == 0
    eri = np.where(allowed, ints.eri, 0.0)
    V = np.ascontiguousarray(eri.transpose(0, 2, 1, 3))
    return ActiveSpaceIntegrals(ints.E, np.ascontiguousarray(h), V, eri)


def random_ci_vector(ndet: int, seed: int) -> np.ndarray:
    """Normalised N(0,1) determinant vector (as in the reference's tests/ci/test_ci_rdms.py:387)."""
    rng = np.random.default_rng(seed)
    c = rng.normal(size=ndet)
    return c / np.linalg.norm(c)


def cas_dims(nel: int, norb: int, twice_ms: int = 0):
    """(na, nb, N0a, N0b, ndet) for a CAS(nel e, norb o) space with 2*Ms = twice_ms."""
    na = (nel + twice_ms) // 2
    nb = nel - na
    n0a = comb(norb, na)
    n0b = comb(norb, nb)
    return na, nb, n0a, n0b, n0a * n0b


def hz_flops(norb: int, na: int, nb: int):
    """The reference's Harrison-Zarrabian GEMM FLOP counts per sigma build (dense form).

    F_ab = 2 n^4 N1a N1b, F_ss = 2 P^2 (N2a N0b + N2b N0a), F_1e = 2 n^2 (N1a N0b + N1b N0a).
    """
    n = norb
    P = n * (n - 1) // 2

    def c(k, m):
        return comb(n, m) if 0 <= m <= n else 0

    n0a, n0b = c(n, na), c(n, nb)
    n1a, n1b = c(n, na - 1), c(n, nb - 1)
    n2a, n2b = c(n, na - 2), c(n, nb - 2)
    f_ab = 2 * n**4 * n1a * n1b
    f_ss = 2 * P * P * (n2a * n0b + n2b * n0a)
    f_1e = 2 * n * n * (n1a * n0b + n1b * n0a)
    return {"ab": f_ab, "ss": f_ss, "1e": f_1e}


def sparse_flops(norb: int, na: int, nb: int):
    """Useful (non-zero) multiply-add FLOPs of one sigma build in the forms this package runs.

    Opposite spin: every (Ka, Kb) 1-hole pair contracts its (n-na+1)(n-nb+1) gathered values
    against as many outputs: 2 * N1a N1b [(n-na+1)(n-nb+1)]^2.
    Same spin (per spin, string-Hamiltonian form): every determinant takes 1 + singles + doubles
    contributions, 2 * Ndet * (1 + na(n-na) + C(na,2) C(n-na,2)).
    """
    n = norb

    def c(m):
        return comb(n, m) if 0 <= m <= n else 0

    n0a, n0b = c(na), c(nb)
    n1a, n1b = c(na - 1), c(nb - 1)
    ua, ub = n - na + 1, n - nb + 1
    f_ab = 2 * n1a * n1b * (ua * ub) ** 2 if na > 0 and nb > 0 else 0
    ndet = n0a * n0b

    def ss(k):
        return 1 + k * (n - k) + comb(k, 2) * comb(n - k, 2)

    f_ss = 2 * ndet * (ss(na) - 1) + 2 * ndet * (ss(nb) - 1)
    return {"ab": f_ab, "ss": f_ss}
