"""GPU parity of spaces with point-group irreps and GAS restrictions (the reference's determinant
blocks) against the reference's own blocked code (tests/golden/blocks.npz / blocks.json, made by
make_golden.py --only blocks): determinant order, sigma, determinant energies, CSF couplings and
diagonal, CASCI energies; and the property that a symmetric Hamiltonian's blocked spectrum is part
of its C1 spectrum."""

import json
import os

import numpy as np
import pytest

from forte2_gb300.synthetic import make_integrals, random_ci_vector, symmetrize_integrals

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

with open(os.path.join(GOLD, "blocks.json")) as _f:
    META = json.load(_f)
CASES = [c for c in META["cases"] if c["ndet"] > 0]


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLD, "blocks.npz"))


def _ints(case, iseed_key="iseed"):
    n = sum(len(g) for g in case["orbital_symmetry"])
    ints = make_integrals(n, case[iseed_key])
    if case["symmetric"]:
        ints = symmetrize_integrals(ints, [x for g in case["orbital_symmetry"] for x in g])
    return ints


def _strings(case):
    from forte2_gb300.ci_helpers import CIStrings

    return CIStrings(case["na"], case["nb"], case["symmetry"], case["orbital_symmetry"], case["gas_min"],
                     case["gas_max"])


@pytest.mark.parametrize("case", META["cases"], ids=lambda c: c["key"])
def test_blocked_strings_and_determinants(cuda, gold, case):
    s = _strings(case)
    k = case["key"]
    assert (s.ndet, s.nas, s.nbs, s.nirrep) == (case["ndet"], case["nas"], case["nbs"], case["nirrep"])
    assert np.array_equal(s.alpha_masks(), gold[f"{k}_a_strings"])
    assert np.array_equal(s.beta_masks(), gold[f"{k}_b_strings"])
    dets = gold[f"{k}_dets"].reshape(-1, 2)
    assert np.array_equal(s.make_determinants().masks(), dets)
    if s.ndet:
        i = s.ndet // 2
        assert s.determinant(i) == (int(dets[i, 0]), int(dets[i, 1]))
        assert s.determinant_index(s.determinant(i)) == i


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["key"])
def test_blocked_sigma_matches_reference(cuda, gold, case):
    """sigma = P H P C of the reference's block loops, FP64 to 1e-12; FP32 to FP32 accuracy;
    bitwise reproducible; determinant energies to 1e-12."""
    torch = cuda
    from forte2_gb300.ci_helpers import CISigmaBuilder

    s = _strings(case)
    assert s.blocked
    ints = _ints(case)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    sb.set_algorithm("hz")
    k = case["key"]
    c = random_ci_vector(s.ndet, case["cseed"])
    sig = np.zeros(s.ndet)
    sb.Hamiltonian(c, sig)
    ref = gold[f"{k}_sigma"]
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(sig - ref).max() < 1e-12 * scale
    # several vectors at once, on the device, twice: the same bits
    X = torch.as_tensor(np.stack([c, 0.5 * c, np.roll(c, 3)]), device="cuda")
    S1 = torch.empty_like(X)
    S2 = torch.empty_like(X)
    sb.Hamiltonian(X, S1)
    sb.Hamiltonian(X, S2)
    assert torch.equal(S1, S2)
    assert np.array_equal(S1[0].cpu().numpy(), sig)
    assert np.abs(S1[1].cpu().numpy() - 0.5 * sig).max() < 1e-12 * scale
    # FP32 operator
    sb.set_precision("fp32")
    s32 = np.zeros(s.ndet)
    sb.Hamiltonian(c, s32)
    assert np.linalg.norm(s32 - ref) / np.linalg.norm(ref) < 2e-6
    sb.set_precision("fp64")
    e = sb.det_energies().cpu().numpy()
    assert np.abs(e - gold[f"{k}_det_energies"]).max() < 1e-12 * max(1.0, np.abs(e).max())


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["key"])
def test_blocked_csf_couplings_and_diagonal(cuda, gold, case):
    from forte2_gb300.ci_helpers import CISigmaBuilder, CISpinAdapter

    s = _strings(case)
    ints = _ints(case)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    n = sum(len(g) for g in case["orbital_symmetry"])
    k = case["key"]
    tms = case["na"] - case["nb"]
    checked = 0
    for twoS in (abs(tms), abs(tms) + 2):
        tag = f"{k}_S{twoS}"
        if f"{tag}_bounds" not in gold.files:
            continue
        sa = CISpinAdapter(twoS, tms, n)
        sa.prepare_couplings(s.make_determinants())
        b, d, cf, r = sa.couplings()
        assert np.array_equal(b, gold[f"{tag}_bounds"]), tag
        assert np.array_equal(d, gold[f"{tag}_det_idx"]), tag
        assert np.array_equal(r, gold[f"{tag}_ranges"]), tag
        assert np.abs(cf - gold[f"{tag}_coeff"]).max() < 1e-14, tag
        hd = sb.form_Hdiag_csf(s.make_determinants(), sa)
        assert np.abs(hd - gold[f"{tag}_hdiag"]).max() < 1e-12 * max(1.0, np.abs(hd).max()), tag
        checked += 1
    assert checked >= 1


@pytest.mark.parametrize("name", sorted(META["casci"]))
@pytest.mark.parametrize("precision,graph", [("fp64", False), ("fp64", True), ("mixed", None)])
def test_blocked_casci_energies(cuda, name, precision, graph):
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import CIParams, DavidsonLiuParams

    c = META["casci"][name]
    n = sum(len(g) for g in c["orbital_symmetry"])
    ints = _ints(c)
    sol = CASCISolver(norb=n, na=c["na"], nb=c["nb"], multiplicity=c["multiplicity"], nroot=c["nroot"], E=ints.E,
                      H=ints.H, V=ints.V, symmetry=c["symmetry"], orbital_symmetry=c["orbital_symmetry"],
                      gas_min=c["gas_min"], gas_max=c["gas_max"], use_graph=graph,
                      ci_params=CIParams(precision=precision),
                      davidson_liu_params=DavidsonLiuParams(e_tol=1e-12, maxiter=400)).run()
    assert sol.converged
    assert sol.basis_size == c["ncsf"] and sol.ndet == c["ndet"]
    tol = 1e-10 if precision == "fp64" else 1e-8
    np.testing.assert_allclose(sol.evals, c["evals"], rtol=0, atol=tol)


def test_symmetric_hamiltonian_blocks_are_c1_sectors(cuda):
    """With point-group-symmetric integrals, every irrep's CASCI roots are roots of the C1 CASCI of
    the same orbitals: the blocked solves over all eight irreps give the C1 spectrum's lowest roots."""
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import DavidsonLiuParams

    orbsym = [[0, 1, 2, 3, 4, 5, 6, 7]]
    n, na, nb = 8, 3, 3
    ints = symmetrize_integrals(make_integrals(n, 91), orbsym[0])
    dl = DavidsonLiuParams(e_tol=1e-12, maxiter=400)
    c1 = CASCISolver(norb=n, na=na, nb=nb, multiplicity=1, nroot=6, E=ints.E, H=ints.H, V=ints.V,
                     davidson_liu_params=dl).run()
    sector = []
    for h in range(8):
        sol = CASCISolver(norb=n, na=na, nb=nb, multiplicity=1, nroot=1, E=ints.E, H=ints.H, V=ints.V, symmetry=h,
                          orbital_symmetry=orbsym, davidson_liu_params=dl).run()
        sector.append(float(sol.evals[0]))
    lowest = sorted(sector)
    # the C1 ground state is the lowest sector ground state; every sector ground state is a C1 root
    assert abs(lowest[0] - c1.evals[0]) < 1e-10
    for e in sector:
        assert np.min(np.abs(np.asarray(c1.evals) - e)) < 1e-9 or e > max(c1.evals)


def test_blocked_rdm_energy_identity(cuda):
    """RDMs of a blocked root (embedded into the C1 space) reproduce its energy."""
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import DavidsonLiuParams

    c = META["casci"]["c3"]
    n = sum(len(g) for g in c["orbital_symmetry"])
    ints = _ints(c)
    sol = CASCISolver(norb=n, na=c["na"], nb=c["nb"], multiplicity=c["multiplicity"], nroot=1, E=ints.E, H=ints.H,
                      V=ints.V, symmetry=c["symmetry"], orbital_symmetry=c["orbital_symmetry"], gas_min=c["gas_min"],
                      gas_max=c["gas_max"], davidson_liu_params=DavidsonLiuParams(e_tol=1e-12, maxiter=400)).run()
    g1 = np.asarray(sol.make_sf_1rdm(0))
    g2 = np.asarray(sol.make_sf_2rdm(0))
    e = ints.E + np.einsum("pq,pq->", ints.H, g1) + 0.5 * np.einsum("pqrs,pqrs->", ints.V, g2)
    assert abs(e - sol.evals[0]) < 1e-10


@pytest.mark.parametrize("na,nb,sym,orbsym,symmetric", [
    (5, 5, 0, [[0, 1, 2, 3, 4, 5, 6, 7, 0, 3]], True),
    (5, 4, 2, [[0, 0, 1, 1, 2, 3, 0, 1, 2, 3, 1]], False),
    (6, 6, 3, [[0, 1, 2, 3] * 3], True),
    (4, 4, 1, [[0, 1] * 4], False),
])
def test_irrep_aware_opposite_spin_kernel(cuda, na, nb, sym, orbsym, symmetric):
    """Spaces blocked by irreps alone: the FP64 opposite-spin term runs on the irrep-aware kernel
    (only the couplings inside the space); it equals the C1 kernel on the embedding to rounding,
    for symmetric and non-symmetric integrals, and is bitwise repeatable."""
    torch = cuda
    from forte2_gb300.ci_helpers import CISigmaBuilder, CIStrings

    n = sum(len(g) for g in orbsym)
    s = CIStrings(na, nb, sym, orbsym, [], [])
    assert s.blocked
    ints = make_integrals(n, 500 + n)
    if symmetric:
        ints = symmetrize_integrals(ints, orbsym[0])
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    X = torch.as_tensor(np.stack([random_ci_vector(s.ndet, 71), random_ci_vector(s.ndet, 72)]), device="cuda")
    S1, S2, S3 = (torch.empty_like(X) for _ in range(3))
    sb.Hamiltonian(X, S1)
    sb.Hamiltonian(X, S2)
    assert torch.equal(S1, S2)
    sb.set_variant("irrep_blocks", 0)
    sb.Hamiltonian(X, S3)
    sb.set_variant("irrep_blocks", 1)
    rel = (torch.linalg.norm(S1 - S3) / torch.linalg.norm(S3)).item()
    assert rel < 1e-13
