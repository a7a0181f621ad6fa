"""Determinant blocks of spaces with point-group irreps and GAS restrictions, enumerated on the
host (f2g_blocks_enumerate, no device call) against the reference's own CIStrings
(tests/golden/blocks.npz, made by make_golden.py --only blocks from ci/ci_strings.cc)."""

import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _cases():
    with open(os.path.join(GOLD, "blocks.json")) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLD, "blocks.npz"))


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["key"])
def test_block_enumeration_matches_reference(gold, case):
    from forte2_gb300.ci_helpers import enumerate_blocks

    k = case["key"]
    e = enumerate_blocks(case["na"], case["nb"], case["symmetry"], case["orbital_symmetry"], case["gas_min"],
                         case["gas_max"])
    assert e["ndet"] == case["ndet"] and e["nirrep"] == case["nirrep"]
    # class strings and classes of both spins: bit-exact, same order
    assert np.array_equal(e["alpha"], gold[f"{k}_a_strings"])
    assert np.array_equal(e["alpha_class"], gold[f"{k}_a_classes"])
    assert np.array_equal(e["beta"], gold[f"{k}_b_strings"])
    assert np.array_equal(e["beta_class"], gold[f"{k}_b_classes"])
    # blocks: (alpha class, beta class, size, offset)
    assert np.array_equal(e["blocks"][:, :4], gold[f"{k}_blocks"])
    # the determinant list rebuilt from the blocks is the reference's make_determinants()
    a, b = e["alpha"], e["beta"]
    aoff = np.concatenate([[0], np.cumsum(np.bincount(e["alpha_class"], minlength=1))])
    boff = np.concatenate([[0], np.cumsum(np.bincount(e["beta_class"], minlength=1))])
    dets = np.zeros((e["ndet"], 2), np.uint64)
    for ca, cb, size, off, nia, nib in e["blocks"]:
        if size:
            dets[off:off + size, 0] = np.repeat(a[aoff[ca]:aoff[ca] + nia], nib)
            dets[off:off + size, 1] = np.tile(b[boff[cb]:boff[cb] + nib], nia)
    assert np.array_equal(dets, gold[f"{k}_dets"].reshape(-1, 2))


def test_plain_cas_is_trivial():
    from forte2_gb300.ci_helpers import enumerate_blocks

    e = enumerate_blocks(3, 3, 0, [[0] * 6], [], [])
    assert e["trivial"] and e["ndet"] == 400
    # irreps present, or a GAS bound that removes determinants: blocked
    assert not enumerate_blocks(3, 3, 0, [[0, 1, 0, 1, 0, 1]], [], [])["trivial"]
    assert not enumerate_blocks(3, 3, 0, [[0, 0, 0], [0, 0, 0]], [4], [6])["trivial"]
    # a GAS split without bounds keeps every determinant but reorders them: blocked
    e = enumerate_blocks(3, 3, 0, [[0, 0, 0], [0, 0, 0]], [], [])
    assert e["ndet"] == 400 and not e["trivial"]


def test_block_enumeration_errors():
    from forte2_gb300.ci_helpers import enumerate_blocks

    with pytest.raises((ValueError, RuntimeError)):
        enumerate_blocks(2, 2, 4, [[0, 1, 0, 1]], [], [])  # state irrep outside the orbitals' group
    with pytest.raises((ValueError, RuntimeError)):
        enumerate_blocks(2, 2, 0, [[0]] * 7, [], [])  # more than six GAS spaces


@pytest.mark.parametrize("case", [c for c in _cases() if c["ndet"] > 0], ids=lambda c: c["key"])
def test_port_sigma_on_the_embedding_is_the_reference_blocked_sigma(gold, case):
    """The design's premise, on the CPU: the reference's sigma of a blocked space (irreps and/or
    GAS bounds, its own block loops) equals the oracle port's C1 sigma of the vector embedded in
    the C1 CAS space of the same orbitals, read back on the space's determinants (P H P)."""
    from forte2_gb300.synthetic import make_integrals, random_ci_vector, symmetrize_integrals
    from oracle.port import PortCI

    k = case["key"]
    orbsym = [x for g in case["orbital_symmetry"] for x in g]
    n, na, nb = len(orbsym), case["na"], case["nb"]
    ints = make_integrals(n, case["iseed"])
    if case["symmetric"]:
        ints = symmetrize_integrals(ints, orbsym)
    port = PortCI(n, na, nb)
    port.set_hamiltonian(ints.E, ints.H, ints.V)
    ia = {int(m): i for i, m in enumerate(port.strings(0))}
    ib = {int(m): i for i, m in enumerate(port.strings(1))}
    dets = gold[f"{k}_dets"].reshape(-1, 2)
    pos = np.array([ia[int(a)] * port.nbs + ib[int(b)] for a, b in dets])
    c = random_ci_vector(case["ndet"], case["cseed"])
    full = np.zeros(port.ndet)
    full[pos] = c
    got = port.sigma(full)[pos]
    ref = gold[f"{k}_sigma"]
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
