"""The oracle's NumPy restatement of the two-component sigma and spin-orbital RDMs
(oracle/rel_port.py) against the reference's own outputs (tests/golden/rel.npz and rel_rdm.npz,
made by make_golden.py from the reference's RelCISigmaBuilder compiled into the oracle). CPU only."""

import json
import os

import numpy as np
import pytest

from forte2_gb300.synthetic import make_spinor_integrals, random_complex_vector

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _cases(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("case", [c for c in _cases("rel.json") if not c["orbital_symmetry"] and c["nspinor"] <= 10],
                         ids=lambda c: c["key"])
def test_rel_sigma_restatement_matches_reference(case):
    from oracle.rel_port import RelPort

    gold = np.load(os.path.join(GOLD, "rel.npz"))
    n, k = case["nspinor"], case["nel"]
    port = RelPort(n, k)
    assert port.ndet == case["ndet"]
    E, H, V = make_spinor_integrals(n, case["iseed"])
    c = random_complex_vector(port.ndet, case["cseed"])
    M = port.hamiltonian(E, H, V)
    ref = gold[f"{case['key']}_sigma"]
    assert np.abs(M @ c - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    assert np.abs(np.diag(M) - gold[f"{case['key']}_hdiag"]).max() < 1e-12 * max(1.0, np.abs(M).max())
    for (i, j), x in zip(gold[f"{case['key']}_pairs"], gold[f"{case['key']}_elements"]):
        assert abs(M[i, j] - x) < 1e-12 * max(1.0, np.abs(M).max())
    assert np.abs(M - M.conj().T).max() < 1e-12  # Hermitian


@pytest.mark.parametrize("case", [c for c in _cases("rel_rdm.json") if not c["orbital_symmetry"] and c["nspinor"] <= 6],
                         ids=lambda c: c["key"])
def test_rel_rdm_restatement_matches_reference(case):
    from oracle.rel_port import RelPort

    gold = np.load(os.path.join(GOLD, "rel_rdm.npz"))
    n, k, key = case["nspinor"], case["nel"], case["key"]
    port = RelPort(n, k)
    cl = random_complex_vector(port.ndet, case["cseed"])
    cr = random_complex_vector(port.ndet, case["cseed"] + 1)
    for kind in ("so_1rdm", "so_2rdm", "so_2cumulant", "so_3rdm", "so_3cumulant"):
        got = getattr(port, kind)(cl, cr).reshape(-1)
        ref = gold[f"{key}_{kind}"].reshape(-1)
        assert np.abs(got - ref).max() < 1e-12 * max(1.0, np.abs(ref).max()), kind
    for kind in ("so_1rdm", "so_2rdm"):
        got = getattr(port, kind)(cl, cl).reshape(-1)
        ref = gold[f"{key}_{kind}_diag"].reshape(-1)
        assert np.abs(got - ref).max() < 1e-12 * max(1.0, np.abs(ref).max()), kind
