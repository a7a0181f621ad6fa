"""The oracle itself, pinned against the golden fixtures generated from the reference (CPU only).

The CPU restatement (oracle/port) must reproduce the reference's integer content bit for bit
(strings, 1-hole and 2-hole lists, CSF couplings) and its floating-point results to rounding
(sigma per term, KH = HZ, Slater diagonal, CSF diagonal and transforms).
"""

import hashlib
import os

import numpy as np
import pytest

from forte2_gb300.synthetic import cas_dims, hz_flops, make_integrals, random_ci_vector
from oracle.port import PortCI, PortSpinAdapter, build_port, TERM_BITS

from conftest import list_cases, sigma_cases

build_port()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_port_lists_match_reference(golden_lists):
    for na, nb, n in list_cases(golden_lists):
        p = PortCI(n, na, nb)
        key = f"{na}_{nb}_{n}"
        for spin, tag in ((0, "a"), (1, "b")):
            assert np.array_equal(p.strings(spin), golden_lists[f"{key}_{tag}_strings"]), key
            assert np.array_equal(p.list_1h(spin), golden_lists[f"{key}_{tag}_1h"]), key
            assert np.array_equal(p.list_2h(spin), golden_lists[f"{key}_{tag}_2h"]), key


def test_port_lists_cas16_hash(golden_lists_meta):
    p = PortCI(16, 8, 8)
    m = golden_lists_meta["8_8_16_a"]
    assert sha(p.strings(0)) == m["strings_sha"]
    assert sha(p.list_1h(0)) == m["l1_sha"]
    assert sha(p.list_2h(0)) == m["l2_sha"]


def test_integral_recipe_is_pinned(golden_sigma):
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        iseed, cseed = golden_sigma[f"{key}_seeds"]
        ints = make_integrals(n, int(iseed))
        assert sha(ints.V) == bytes(golden_sigma[f"{key}_V_sha"]).decode()
        c = random_ci_vector(cas_dims(na + nb, n, na - nb)[4], int(cseed))
        assert sha(c) == bytes(golden_sigma[f"{key}_C_sha"]).decode()


def test_port_sigma_matches_reference(golden_sigma):
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        iseed, cseed = golden_sigma[f"{key}_seeds"]
        ints = make_integrals(n, int(iseed))
        p = PortCI(n, na, nb)
        p.set_hamiltonian(ints.E, ints.H, ints.V)
        c = random_ci_vector(p.ndet, int(cseed))
        ref = golden_sigma[f"{key}_sigma"]
        got = p.sigma(c)
        assert np.linalg.norm(got - ref) <= 1e-12 * max(np.linalg.norm(ref), 1e-300), key
        for t, bit in TERM_BITS.items():
            if f"{key}_term_{t}" in golden_sigma.files:
                r = golden_sigma[f"{key}_term_{t}"]
                assert np.abs(p.sigma(c, bit) - r).max() <= 1e-12 * max(np.abs(ref).max(), 1.0), (key, t)
        if f"{key}_sigma_kh" in golden_sigma.files:
            kh = golden_sigma[f"{key}_sigma_kh"]
            if na > 0 and nb > 0:
                assert np.abs(kh - ref).max() < 1e-12, key
            else:
                # With one spin empty the reference's Knowles-Handy path has no 1h1p strings for
                # that spin and skips H2_kh entirely: its sigma is H0 + H1 with the KH-modified
                # one-electron integrals h - 1/2 sum_r <pr|rq> only. Pin that behaviour.
                p2 = PortCI(n, na, nb)
                p2.set_hamiltonian(ints.E, ints.H - 0.5 * np.einsum("prrq->pq", ints.V), np.zeros_like(ints.V))
                assert np.abs(p2.sigma(c) - kh).max() < 1e-12, key


def test_port_csf_matches_reference(golden_sigma):
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        iseed, cseed = golden_sigma[f"{key}_seeds"]
        ints = make_integrals(n, int(iseed))
        p = PortCI(n, na, nb)
        p.set_hamiltonian(ints.E, ints.H, ints.V)
        sig = golden_sigma[f"{key}_sigma"]
        for twoS in (abs(na - nb), abs(na - nb) + 2):
            tag = f"{key}_S{twoS}"
            if f"{tag}_hdiag" not in golden_sigma.files:
                continue
            sa = PortSpinAdapter(p, twoS, na - nb)
            if f"{tag}_bounds" in golden_sigma.files:
                b, d, cf, r = sa.couplings()
                assert np.array_equal(b, golden_sigma[f"{tag}_bounds"]), tag
                assert np.array_equal(d, golden_sigma[f"{tag}_det_idx"]), tag
                assert np.array_equal(r, golden_sigma[f"{tag}_conf_ranges"]), tag
                assert np.array_equal(cf, golden_sigma[f"{tag}_coeff"]), tag
            else:
                assert [sa.nconf, sa.ncsf, sa.ncoupling] == list(golden_sigma[f"{tag}_info"]), tag
            assert np.abs(sa.hdiag() - golden_sigma[f"{tag}_hdiag"]).max() < 1e-12, tag
            csf = random_ci_vector(sa.ncsf, int(cseed) + 7)
            assert np.abs(sa.csf_to_det(csf) - golden_sigma[f"{tag}_csf_to_det"]).max() < 1e-14, tag
            assert np.abs(sa.det_to_csf(sig) - golden_sigma[f"{tag}_det_to_csf"]).max() < 1e-12, tag


def test_port_sigma_checksums_cas12(golden_checksums):
    meta = golden_checksums["6_6_12"]
    ints = make_integrals(12, meta["iseed"])
    assert sha(ints.V) == meta["V_sha"]
    p = PortCI(12, 6, 6)
    p.set_hamiltonian(ints.E, ints.H, ints.V)
    sig = p.sigma(random_ci_vector(p.ndet, meta["cseed"]))
    assert abs(np.linalg.norm(sig) - meta["norm"]) < 1e-12 * meta["norm"]
    idx = np.array(meta["idx"])
    assert np.abs(sig[idx] - np.array(meta["vals"])).max() < 1e-12 * meta["norm"]


def test_port_memory_contract():
    p = PortCI(6, 2, 2)
    ints = make_integrals(6, 5)
    p.set_hamiltonian(0.25, ints.H, ints.V)
    with pytest.raises(ValueError, match="memory must be non-negative"):
        p.set_memory(-1)
    c = random_ci_vector(p.ndet, 205)
    p.set_memory(1)
    expected = p.sigma(c)
    p.set_memory(0)
    with pytest.raises(RuntimeError, match="too small for one K-block column"):
        p.sigma(c)
    p.set_memory(1)
    np.testing.assert_allclose(p.sigma(c), expected, rtol=1e-12, atol=1e-12)


def test_flop_formulas():
    f = hz_flops(16, 8, 8)
    assert abs(f["ab"] - 1.715e13) / 1.715e13 < 1e-3
    assert abs(f["ss"] - 5.94e12) / 5.94e12 < 1e-2


def test_reference_oracle_matches_port_when_built(golden_sigma):
    """The compiled reference exists only where its sources were available; check it there."""
    from oracle import reference as ref

    if not os.path.exists(ref.LIB_PATH):
        pytest.skip("compiled reference not built here")
    s = ref.RefCIStrings(3, 3, 0, [[0] * 6], [], [])
    ints = make_integrals(6, 13)
    sb = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
    sb.set_algorithm("hz")
    c = random_ci_vector(s.ndet, 103)
    out = np.zeros(s.ndet)
    sb.Hamiltonian(c, out)
    np.testing.assert_allclose(out, golden_sigma["3_3_6_sigma"], rtol=0, atol=1e-13)


RDM_KINDS = ("a_1rdm", "b_1rdm", "sf_1rdm", "aa_2rdm", "bb_2rdm", "ab_2rdm", "sf_2rdm", "sf_2cumulant")


def test_port_rdms_match_reference(golden_rdm):
    """Every RDM kind of the restatement equals the reference's (ci_sigma_builder_1rdm.cc,
    ci_sigma_builder_2rdm.cc) for a transition pair and for one vector with itself."""
    for na, nb, n in list_cases(golden_rdm):
        key = f"{na}_{nb}_{n}"
        sl, sr = golden_rdm[f"{key}_seeds"]
        p = PortCI(n, na, nb)
        cl = random_ci_vector(p.ndet, int(sl))
        cr = random_ci_vector(p.ndet, int(sr))
        assert sha(cl) == bytes(golden_rdm[f"{key}_CL_sha"]).decode()
        assert sha(cr) == bytes(golden_rdm[f"{key}_CR_sha"]).decode()
        for kind in RDM_KINDS:
            for tag, b in (("LR", cr), ("LL", cl)):
                ref = golden_rdm[f"{key}_{kind}_{tag}"]
                got = p.rdm(kind, cl, b)
                assert got.shape == ref.shape, (key, kind)
                scale = max(1.0, float(np.abs(ref).max())) if ref.size else 1.0
                assert np.abs(got - ref).max(initial=0.0) <= 1e-13 * scale, (key, kind, tag)


def test_port_rdm_energy_identity():
    """<C|H|C> from the oracle's sigma equals the energy from its spin-free RDMs."""
    for na, nb, n, seed in ((3, 3, 6, 5), (4, 3, 8, 6), (5, 5, 10, 7)):
        ints = make_integrals(n, seed)
        p = PortCI(n, na, nb)
        p.set_hamiltonian(ints.E, ints.H, ints.V)
        c = random_ci_vector(p.ndet, seed + 100)
        e_sigma = float(c @ p.sigma(c))
        g1 = p.rdm("sf_1rdm", c, c).reshape(n, n)
        g2 = p.rdm("sf_2rdm", c, c).reshape(n, n, n, n)
        e_rdm = ints.E + np.einsum("ij,ij", g1, ints.H) + 0.5 * np.einsum("ijkl,ijkl", g2, ints.V)
        assert abs(e_sigma - e_rdm) < 1e-11 * max(1.0, abs(e_sigma)), (n, e_sigma, e_rdm)


RDM3_KINDS = ("aaa_3rdm", "bbb_3rdm", "aab_3rdm", "abb_3rdm", "sf_3rdm", "sf_3cumulant")


def test_port_3rdms_match_reference(golden_rdm, golden_rdm3):
    """The restatement's 3-RDMs and 3-cumulant equal the reference's (ci_sigma_builder_3rdm.cc):
    full arrays for up to 4 orbitals, checksums (norm, seeded dot product, 64 sampled entries)
    for all spaces of the RDM fixtures."""
    from conftest import rdm_checksum_matches

    meta, full = golden_rdm3
    for na, nb, n in list_cases(golden_rdm):
        key = f"{na}_{nb}_{n}"
        sl, sr = golden_rdm[f"{key}_seeds"]
        p = PortCI(n, na, nb)
        cl = random_ci_vector(p.ndet, int(sl))
        cr = random_ci_vector(p.ndet, int(sr))
        for j, kind in enumerate(RDM3_KINDS):
            for tag, b in (("LR", cr), ("LL", cl)):
                got = p.rdm(kind, cl, b)
                name = f"{key}_{kind}_{tag}"
                assert rdm_checksum_matches(got, meta[name], 7000 + 10 * j + (tag == "LL")), name
                if name in full.files:
                    ref = full[name]
                    assert got.shape == ref.shape
                    assert np.abs(got - ref).max(initial=0.0) <= 1e-13 * max(1.0, np.abs(ref).max(initial=0.0))


def test_port_3rdm_partial_trace():
    """sum_r G3[p,q,r,s,t,r] = (N - 2) G2[p,q,s,t] for the spin-free RDMs of one vector."""
    for na, nb, n in ((3, 3, 6), (4, 2, 7)):
        p = PortCI(n, na, nb)
        c = random_ci_vector(p.ndet, 77)
        g3 = p.rdm("sf_3rdm", c, c).reshape((n,) * 6)
        g2 = p.rdm("sf_2rdm", c, c).reshape((n,) * 4)
        assert np.abs(np.einsum("pqrstr->pqst", g3) - (na + nb - 2) * g2).max() < 1e-12
