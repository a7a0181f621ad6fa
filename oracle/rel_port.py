"""Oracle (test infrastructure only): a NumPy restatement, for small spaces, of the two-component
(relativistic) CI sigma and spin-orbital RDMs of forte2/ci/rel_ci_sigma_builder.cc,
rel_ci_sigma_builder_harrison_zarrabian.cc and rel_ci_sigma_builder_rdm.cc.

Determinants are strings of k electrons in n spinors (nb = 0), in the reference's string order
(the oracle port's strings, pinned bit for bit to the reference's own lists). Operators act on
them by explicit second quantisation: a+_p / a_p on a string give the string with bit p set /
cleared and the sign (-1)^(number of occupied spinors below p). The Hamiltonian is

    H = E + sum_pq h_pq a+_p a_q + 1/2 sum_pqrs V[p][q][r][s] a+_p a+_q a_s a_r

with V the physicist integrals <pq|rs>, and the RDMs are expectation values with the bra
conjugated: G1[p][q] = <L|a+_p a_q|R>, G2[p][q][r][s] = <L|a+_p a+_q a_s a_r|R>,
G3[p][q][r][s][t][u] = <L|a+_p a+_q a+_r a_u a_t a_s|R>. The cumulants follow the reference's
formulas (rel_ci_sigma_builder_rdm.cc, compute_2cumulant and compute_3cumulant).

Only tests/ use this module, as the parity reference; it runs on the CPU in pure Python loops and
is meant for spaces of a few hundred determinants at most.
"""

from __future__ import annotations

import itertools

import numpy as np


def apply_ops(mask: int, ops):
    """Apply (p, create) operators in order (first element first) to a string; returns
    (string, sign) or None when the result vanishes."""
    sign = 1
    for p, create in ops:
        bit = 1 << p
        if create == bool(mask & bit):
            return None
        if bin(mask & (bit - 1)).count("1") & 1:
            sign = -sign
        mask ^= bit
    return mask, sign


class RelPort:
    """Two-component determinant space of k electrons in n spinors (C1)."""

    def __init__(self, n: int, k: int):
        from .port import PortCI

        self.n, self.k = n, k
        self.strings = [int(x) for x in PortCI(n, k, 0).strings(0)]
        self.index = {m: i for i, m in enumerate(self.strings)}
        self.ndet = len(self.strings)

    def _occ(self, m):
        return [p for p in range(self.n) if m >> p & 1]

    def hamiltonian(self, E, H, V):
        """The dense Hamiltonian matrix (ndet x ndet, complex)."""
        n, nd = self.n, self.ndet
        M = np.zeros((nd, nd), dtype=np.complex128)
        for j, J in enumerate(self.strings):
            M[j, j] += E
            occ = self._occ(J)
            for q in occ:
                for p in range(n):
                    res = apply_ops(J, [(q, False), (p, True)])
                    if res:
                        M[self.index[res[0]], j] += res[1] * H[p, q]
            for r, s in itertools.permutations(occ, 2):
                for q in range(n):
                    for p in range(n):
                        res = apply_ops(J, [(r, False), (s, False), (q, True), (p, True)])
                        if res:
                            M[self.index[res[0]], j] += 0.5 * res[1] * V[p, q, r, s]
        return M

    def sigma(self, E, H, V, c):
        return self.hamiltonian(E, H, V) @ np.asarray(c, dtype=np.complex128)

    def _rdm(self, CL, CR, order):
        """<L| a+_{p1} .. a+_{pk} a_{sk} .. a_{s1} |R> as an n^(2k) tensor, indices (p1..pk, s1..sk)."""
        n = self.n
        out = np.zeros((n,) * (2 * order), dtype=np.complex128)
        L = np.conj(np.asarray(CL, dtype=np.complex128))
        R = np.asarray(CR, dtype=np.complex128)
        for j, J in enumerate(self.strings):
            if R[j] == 0:
                continue
            occ = self._occ(J)
            for ann in itertools.permutations(occ, order):
                # a_{s1} acts first: annihilate s1, s2, ..., then create pk, ..., p1
                for cre in itertools.product(range(n), repeat=order):
                    ops = [(s, False) for s in ann] + [(p, True) for p in reversed(cre)]
                    res = apply_ops(J, ops)
                    if res:
                        out[tuple(cre) + tuple(ann)] += L[self.index[res[0]]] * res[1] * R[j]
        return out

    def so_1rdm(self, CL, CR):
        return self._rdm(CL, CR, 1)

    def so_2rdm(self, CL, CR):
        return self._rdm(CL, CR, 2)

    def so_3rdm(self, CL, CR):
        return self._rdm(CL, CR, 3)

    def so_2cumulant(self, CL, CR):
        g1 = self.so_1rdm(CL, CR)
        return self.so_2rdm(CL, CR) - np.einsum("pr,qs->pqrs", g1, g1) + np.einsum("ps,qr->pqrs", g1, g1)

    def so_3cumulant(self, CL, CR):
        g1 = self.so_1rdm(CL, CR)
        g2 = self.so_2rdm(CL, CR)
        e = np.einsum
        out = self.so_3rdm(CL, CR)
        out -= e("ps,qrtu->pqrstu", g1, g2) + e("qt,prsu->pqrstu", g1, g2) + e("ru,pqst->pqrstu", g1, g2)
        out += e("pt,qrsu->pqrstu", g1, g2) + e("pu,qrts->pqrstu", g1, g2) + e("qs,prtu->pqrstu", g1, g2)
        out += e("qu,prst->pqrstu", g1, g2) + e("rs,pqut->pqrstu", g1, g2) + e("rt,pqsu->pqrstu", g1, g2)
        out += 2.0 * (e("ps,qt,ru->pqrstu", g1, g1, g1) - e("ps,qu,rt->pqrstu", g1, g1, g1)
                      - e("pu,qt,rs->pqrstu", g1, g1, g1) - e("pt,qs,ru->pqrstu", g1, g1, g1)
                      + e("pt,qu,rs->pqrstu", g1, g1, g1) + e("pu,qs,rt->pqrstu", g1, g1, g1))
        return out
