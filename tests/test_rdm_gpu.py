"""Reduced density matrices on the GPU against the reference's (golden fixtures from
ci_sigma_builder_1rdm.cc / ci_sigma_builder_2rdm.cc compiled unmodified) and the oracle, plus the
size-independent energy identity <C|H|C> = E + sum h G1 + 1/2 sum V G2 at CAS(14,14).

Tolerance: 1e-12 of the largest element (FP64 sums in a different order than the reference's)."""

from math import comb

import numpy as np
import pytest

from conftest import list_cases
from forte2_gb300.synthetic import make_integrals, random_ci_vector

pytestmark = pytest.mark.gpu

KINDS = ("a_1rdm", "b_1rdm", "sf_1rdm", "aa_2rdm", "bb_2rdm", "ab_2rdm", "sf_2rdm", "sf_2cumulant")


def builder(n, na, nb, seed):
    from forte2_gb300.ci_helpers import CISigmaBuilder, CIStrings

    ints = make_integrals(n, seed)
    s = CIStrings(na, nb, 0, [[0] * n], [], [])
    return s, CISigmaBuilder(s, ints.E, ints.H, ints.V, 0), ints


def close(got, ref, tol=1e-12):
    got = np.asarray(got).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    assert got.shape == ref.shape
    scale = max(1.0, float(np.abs(ref).max(initial=0.0)))
    return float(np.abs(got - ref).max(initial=0.0)) <= tol * scale


def test_rdms_match_reference_golden(cuda, golden_rdm):
    for na, nb, n in list_cases(golden_rdm):
        key = f"{na}_{nb}_{n}"
        sl, sr = (int(x) for x in golden_rdm[f"{key}_seeds"])
        s, sb, _ = builder(n, na, nb, sl)
        cl = random_ci_vector(s.ndet, sl)
        cr = random_ci_vector(s.ndet, sr)
        for kind in KINDS:
            got = getattr(sb, kind)(cl, cr)  # two vectors: general kernels
            assert close(got, golden_rdm[f"{key}_{kind}_LR"]), (key, kind, "LR")
            got = getattr(sb, kind)(cl, cl)  # one vector: symmetric kernels
            assert close(got, golden_rdm[f"{key}_{kind}_LL"]), (key, kind, "LL")


def test_rdm_device_tensors_and_shapes(cuda):
    torch = cuda
    n, na, nb = 6, 3, 2
    s, sb, _ = builder(n, na, nb, 7)
    cl = random_ci_vector(s.ndet, 1)
    cr = random_ci_vector(s.ndet, 2)
    dl, dr = torch.from_numpy(cl).cuda(), torch.from_numpy(cr).cuda()
    shapes = {"a_1rdm": (n, n), "aa_2rdm": (15, 15), "ab_2rdm": (n, n, n, n), "sf_2cumulant": (n, n, n, n)}
    for kind, shape in shapes.items():
        d = getattr(sb, kind)(dl, dr)
        h = getattr(sb, kind)(cl, cr)
        assert d.is_cuda and tuple(d.shape) == shape and h.shape == shape
        assert close(d.cpu().numpy(), h, 1e-14)
    # transition RDMs: gamma(L, R)^T = gamma(R, L)
    assert close(sb.a_1rdm(cl, cr).T, sb.a_1rdm(cr, cl), 1e-14)
    assert close(sb.ab_2rdm(cl, cr).transpose(2, 3, 0, 1), sb.ab_2rdm(cr, cl), 1e-13)
    with pytest.raises(RuntimeError):
        sb.a_1rdm(cl[:-1], cr[:-1])
    with pytest.raises(TypeError):
        sb.a_1rdm(dl, cr)
    s1, sb1, _ = builder(1, 1, 1, 3)
    assert sb1.aa_2rdm(np.ones(1), np.ones(1)).shape == (0, 0)
    # transition 1-RDMs between two wave functions of the same space (ci_sigma_builder_1trdm.cc)
    _, sb2, _ = builder(n, na, nb, 8)
    assert close(sb.a_1trdm(sb2, cl, cr), sb.a_1rdm(cl, cr), 1e-14)
    assert close(sb.sf_1trdm(sb2, cl, cr), sb.sf_1rdm(cl, cr), 1e-14)
    _, sb3, _ = builder(n, nb, na, 8)
    with pytest.raises(RuntimeError, match="alpha and beta electrons"):
        sb.b_1trdm(sb3, cl, cr)
    _, sb4, _ = builder(n - 1, na, nb, 8)
    with pytest.raises(RuntimeError, match="number of MOs"):
        sb.a_1trdm(sb4, cl, cr)


def test_rdms_wide_lists_global_rows_vs_oracle(cuda):
    """18 orbitals, 1 alpha and 9 beta electrons: 48,620 beta strings, so the beta pair list uses
    64-bit entries and the mixed-spin kernel reads its rows from global memory."""
    from oracle.port import PortCI, build_port

    build_port()
    n, na, nb = 18, 1, 9
    s, sb, _ = builder(n, na, nb, 9)
    assert s.ndet == comb(18, 1) * comb(18, 9)
    port = PortCI(n, na, nb)
    cl = random_ci_vector(s.ndet, 11)
    cr = random_ci_vector(s.ndet, 12)
    assert close(sb.ab_2rdm(cl, cr), port.rdm("ab_2rdm", cl, cr))
    assert close(sb.ab_2rdm(cl, cl), port.rdm("ab_2rdm", cl, cl))
    assert close(sb.b_1rdm(cl, cr), port.rdm("b_1rdm", cl, cr))
    assert close(sb.bb_2rdm(cl, cl), port.rdm("bb_2rdm", cl, cl))


def test_rdm_energy_identity_cas14(cuda):
    """<C|H|C> from the FP64 sigma build equals the energy from the RDMs, in the reference's three
    forms (ci.py:323-403), for a random normalised C of CAS(14,14) (11.8 M determinants)."""
    torch = cuda
    from forte2_gb300.ci import packed_tensor4_to_tensor4

    n = 14
    s, sb, ints = builder(n, 7, 7, 4000)
    c = torch.from_numpy(random_ci_vector(s.ndet, 4001)).cuda()
    sig = torch.empty_like(c)
    sb.Hamiltonian(c, sig)
    e_sigma = float(torch.dot(c, sig))
    g1 = sb.sf_1rdm(c, c).cpu().numpy()
    aa, ab, bb = (getattr(sb, k)(c, c).cpu().numpy() for k in ("aa_2rdm", "ab_2rdm", "bb_2rdm"))
    g2 = sb.sf_2rdm(c, c).cpu().numpy()
    H, V = ints.H, ints.V
    A = V - np.einsum("ijkl->ijlk", V)
    i, j = np.tril_indices(n, k=-1)
    M = A[i[:, None], j[:, None], i[None, :], j[None, :]]
    e1 = ints.E + np.einsum("ij,ij", g1, H)
    packed = e1 + np.einsum("ij,ij", aa, M) + np.einsum("ijkl,ijkl", ab, V) + np.einsum("ij,ij", bb, M)
    expanded = e1 + 0.25 * np.einsum("ijkl,ijkl", packed_tensor4_to_tensor4(aa, n), A) + np.einsum(
        "ijkl,ijkl", ab, V) + 0.25 * np.einsum("ijkl,ijkl", packed_tensor4_to_tensor4(bb, n), A)
    spin_free = e1 + 0.5 * np.einsum("ijkl,ijkl", g2, V)
    for e in (packed, expanded, spin_free):
        assert abs(e - e_sigma) < 1e-10 * abs(e_sigma), (e, e_sigma)
    # trace conditions: tr G1 = N, sum G2[p][q][p][q] = N (N - 1)
    assert abs(np.trace(g1) - 14.0) < 1e-10
    assert abs(np.einsum("pqpq", g2) - 14.0 * 13.0) < 1e-9
    # cumulant = G2 - G1 G1 + G1 G1 / 2 (exchange), from the same pieces
    L2 = sb.sf_2cumulant(c, c).cpu().numpy()
    want = g2 - np.einsum("pr,qs->pqrs", g1, g1) + 0.5 * np.einsum("ps,qr->pqrs", g1, g1)
    assert close(L2, want, 1e-12)


@pytest.mark.parametrize("mult", [1, 3])
def test_casci_rdm_self_check(cuda, mult):
    """The CI driver's RDM self-check (ci.py:203-204, 323-403) on converged roots."""
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import DavidsonLiuParams

    # the CAS(8,8) cases of the reference Davidson fixtures (singlet 4 roots, triplet 3 roots)
    n = 8
    seed, nroot = (35, 4) if mult == 1 else (36, 3)
    ints = make_integrals(n, seed)
    solver = CASCISolver(norb=n, na=4, nb=4, multiplicity=mult, nroot=nroot, E=ints.E, H=ints.H, V=ints.V,
                         davidson_liu_params=DavidsonLiuParams(e_tol=1e-12, maxiter=1000), do_test_rdms=True).run()
    assert solver.converged
    for root in range(nroot):
        for e in solver.rdm_energies(root):
            assert abs(e - solver.evals[root]) < 1e-9
    a, b = solver.make_sd_1rdm(0)
    assert abs(np.trace(a) - 4) < 1e-10 and abs(np.trace(b) - 4) < 1e-10
    # transition 1-RDM between orthogonal roots is traceless
    assert abs(np.trace(solver.make_1rdm(0, 1))) < 1e-10
    # natural occupations (ci.py:770-785): 8 electrons, each in [0, 2], descending per root
    no = solver.compute_natural_occupation_numbers()
    assert no.shape == (n, nroot)
    assert np.allclose(no.sum(axis=0), 8.0, atol=1e-10)
    assert np.all(no > -1e-10) and np.all(no < 2.0 + 1e-10)
    assert np.all(np.diff(no, axis=0) <= 1e-12)
    # leading determinants (ci.py:804-832)
    c0 = solver._root_vector_det(0)
    assert abs(np.linalg.norm(c0) - 1.0) < 1e-10
    top = solver.get_top_determinants(3)
    assert len(top) == nroot and all(len(t) == 3 for t in top)
    (alpha, beta), coef = top[0][0]
    assert abs(abs(coef) - np.abs(c0).max()) < 1e-12
    assert bin(alpha).count("1") == 4 and bin(beta).count("1") == 4
