"""GPU parity of the CSF machinery (couplings bit-exact, transforms, diagonal, guess matrix) and
of the Davidson-Liu solver / CASCI energies against the reference."""

import numpy as np
import pytest

from conftest import sigma_cases
from forte2_gb300.synthetic import make_integrals, random_ci_vector

pytestmark = pytest.mark.gpu


def setup(na, nb, n, iseed, twoS):
    from forte2_gb300.ci_helpers import CISigmaBuilder, CISpinAdapter, CIStrings

    s = CIStrings(na, nb, 0, [[0] * n], [], [])
    ints = make_integrals(n, iseed)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    sa = CISpinAdapter(twoS, na - nb, n)
    sa.prepare_couplings(s.make_determinants())
    return s, sb, sa


def test_csf_couplings_transforms_and_diagonal(cuda, golden_sigma):
    torch = cuda
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        iseed, cseed = golden_sigma[f"{key}_seeds"]
        for twoS in (abs(na - nb), abs(na - nb) + 2):
            tag = f"{key}_S{twoS}"
            if f"{tag}_hdiag" not in golden_sigma.files:
                continue
            s, sb, sa = setup(na, nb, n, int(iseed), twoS)
            if f"{tag}_bounds" in golden_sigma.files:
                b, d, cf, r = sa.couplings()
                assert np.array_equal(b, golden_sigma[f"{tag}_bounds"]), tag
                assert np.array_equal(d, golden_sigma[f"{tag}_det_idx"]), tag
                assert np.array_equal(r, golden_sigma[f"{tag}_conf_ranges"]), tag
                assert np.array_equal(cf, golden_sigma[f"{tag}_coeff"]), tag
            else:
                assert [sa.nconf, sa.ncsf, sa.ncoupling] == [int(x) for x in golden_sigma[f"{tag}_info"]], tag
            hd = sb.form_Hdiag_csf(s.make_determinants(), sa)
            assert np.abs(hd - golden_sigma[f"{tag}_hdiag"]).max() < 1e-12, tag
            csf = random_ci_vector(sa.ncsf, int(cseed) + 7)
            det = np.zeros(s.ndet)
            sa.csf_C_to_det_C(csf, det)
            assert np.abs(det - golden_sigma[f"{tag}_csf_to_det"]).max() < 1e-14, tag
            out = np.zeros(sa.ncsf)
            sa.det_C_to_csf_C(np.ascontiguousarray(golden_sigma[f"{key}_sigma"]), out)
            assert np.abs(out - golden_sigma[f"{tag}_det_to_csf"]).max() < 1e-12, tag
            # device-resident path gives the same numbers
            dcsf = torch.as_tensor(csf, device="cuda")
            ddet = torch.empty(s.ndet, dtype=torch.float64, device="cuda")
            sa.csf_C_to_det_C(dcsf, ddet)
            assert np.array_equal(ddet.cpu().numpy(), det)
            m = golden_sigma[f"{tag}_slater_csf"].shape[0]
            Hm = sb.csf_matrix(sa, np.arange(m))
            assert np.abs(Hm - golden_sigma[f"{tag}_slater_csf"]).max() < 1e-12, tag


def test_csf_counts_cas16_singlet(cuda):
    """CAS(16,16) singlet: 34,763,300 CSFs (Weyl dimension), every determinant covered."""
    from forte2_gb300.ci_helpers import CISpinAdapter, CIStrings

    s = CIStrings(8, 8, 0, [[0] * 16], [], [])
    sa = CISpinAdapter(0, 0, 16)
    sa.prepare_couplings(s.make_determinants())
    assert sa.ncsf == 34763300


def test_davidson_vs_numpy_reference_cases(cuda):
    """The reference's own Davidson tests (tests/helpers/test_davidsonliu.py:8-46, 91-120):
    seeded random symmetric matrices with a numpy sigma callable."""
    from forte2_gb300.davidson import DavidsonLiuSolver
    from forte2_gb300.params import DavidsonLiuParams

    np.random.seed(0)
    size, nroot = 100, 3
    H = np.random.randn(size, size)
    H = 0.5 * (H + H.T)

    def sigma_builder(basis_block, sigma_block):
        sigma_block[:] = H @ basis_block

    solver = DavidsonLiuSolver(size=size, nroot=nroot,
                               davidson_liu_params=DavidsonLiuParams(collapse_per_root=3, basis_per_root=6))
    solver.add_h_diag(np.diag(H))
    solver.add_sigma_builder(sigma_builder)
    evals, evecs = solver.solve()
    ref_vals, ref_vecs = np.linalg.eigh(H)
    assert np.allclose(np.sort(evals), ref_vals[:nroot], atol=1e-12)
    E = evecs.cpu().numpy()
    assert np.linalg.norm(E @ E.T - ref_vecs[:, :3] @ ref_vecs[:, :3].T) < 1e-5

    matrix = np.array([[-1, 1, 1, 1], [1, 0, 1, 1], [1, 1, 0, 1], [1, 1, 1, 0]], dtype=float)
    s2 = DavidsonLiuSolver(size=4, nroot=1, davidson_liu_params=DavidsonLiuParams(collapse_per_root=1, basis_per_root=5))
    s2.add_h_diag(np.diag(matrix))
    s2.add_guesses(np.eye(4))
    s2.add_sigma_builder(lambda B, S: S.__setitem__(slice(None), matrix @ B))
    ev, _ = s2.solve()
    assert abs(ev[0] - np.linalg.eigvalsh(matrix)[0]) < 1e-12


M4 = np.array([[-1, 1, 1, 1], [1, 0, 1, 1], [1, 1, 0, 1], [1, 1, 1, 0]], dtype=float)


def _solver(size, nroot, matrix, collapse=1, basis=5, maxiter=100, **kw):
    from forte2_gb300.davidson import DavidsonLiuSolver
    from forte2_gb300.params import DavidsonLiuParams

    s = DavidsonLiuSolver(size=size, nroot=nroot,
                          davidson_liu_params=DavidsonLiuParams(collapse_per_root=collapse, basis_per_root=basis,
                                                                maxiter=maxiter), **kw)
    s.add_h_diag(np.diag(matrix))
    s.add_sigma_builder(lambda B, S: S.__setitem__(slice(None), matrix @ B))
    return s


def test_dl_unnormalized_guess_and_no_guess(cuda):
    """tests/helpers/test_davidsonliu.py:126-155 and :213-235 of the reference."""
    ref = np.linalg.eigh(M4)[0]
    s = _solver(4, 1, M4)
    s.add_guesses(np.array([[1.0], [0.0], [0.0], [0.0]]))
    assert abs(s.solve()[0][0] - ref[0]) < 5e-8
    s = _solver(4, 1, M4)
    assert abs(s.solve()[0][0] - ref[0]) < 5e-8


def test_dl_sizes_and_roots(cuda):
    """solve_dl of the reference (test_davidsonliu.py:158-210), a representative subset."""
    for size, nroot in [(10, 1), (10, 5), (10, 10), (100, 3), (100, 10), (1000, 4), (7, 7), (25, 13)]:
        m = np.zeros((size, size))
        for i in range(size):
            m[i, i] = -1.0 + i * 0.1
            for j in range(i):
                m[i, j] = m[j, i] = 0.05 / (1.0 + abs(i - j))
        ref = np.linalg.eigh(m)[0][:nroot]
        s = _solver(size, nroot, m)
        s.add_guesses(np.eye(size)[:, :nroot])
        ev, _ = s.solve()
        assert np.allclose(np.sort(ev), np.sort(ref), atol=1e-6), (size, nroot)


def test_dl_project_out(cuda):
    """test_davidsonliu.py:238-265: projecting out the lowest eigenvector exposes the next one."""
    w, v = np.linalg.eigh(M4)
    s = _solver(4, 1, M4)
    s.add_project_out([v[:, 0]])
    assert abs(s.solve()[0][0] - w[1]) < 5e-8


def test_dl_restarts(cuda):
    """test_davidsonliu.py:269-360: restart with the same matrix, a changed matrix, and from an
    unconverged solution."""
    ref = np.linalg.eigh(M4)[0]
    s = _solver(4, 1, M4)
    s.add_guesses(np.eye(4)[:, :1])
    s.solve()
    assert abs(s.solve()[0][0] - ref[0]) < 5e-8
    m2 = M4.copy()
    m2[0, 0] = -2
    s.add_h_diag(np.diag(m2))
    s.add_sigma_builder(lambda B, S: S.__setitem__(slice(None), m2 @ B))
    assert abs(s.solve()[0][0] - np.linalg.eigh(m2)[0][0]) < 5e-8
    rng = np.random.default_rng(42)
    A = rng.random((500, 500))
    A = 0.05 * (A + A.T) + np.diag(rng.uniform(2, 4, 500))
    s = _solver(500, 10, A, collapse=2, basis=5, maxiter=10)
    s.add_guesses(np.eye(500)[:, :10])
    ev, _ = s.solve()
    n = 0
    while not s.converged and n < 50:
        ev, _ = s.solve()
        n += 1
    assert s.converged
    np.testing.assert_allclose(ev, np.linalg.eigh(A)[0][:10], atol=5e-8)


def test_dl_shift(cuda):
    """test_davidsonliu.py:364-410: five roots closest to a shift, from random initial vectors."""
    np.random.seed(0)
    H = np.random.randn(100, 100)
    H = 0.5 * (H + H.T)
    w, v = np.linalg.eigh(H)
    eta = w[20] + np.random.uniform(-1, 1)
    idx = np.argsort(np.abs(w - eta))
    s = _solver(100, 5, H, collapse=5, basis=10, energy_shift=eta)
    ev, evecs = s.solve()
    assert np.allclose(ev, w[idx][:5], atol=1e-12)
    E = evecs.cpu().numpy()
    assert np.linalg.norm(E @ E.T - v[:, idx[:5]] @ v[:, idx[:5]].T) < 1e-5


@pytest.mark.parametrize("key", ["2_2_4_m1_r2_it100", "3_3_6_m1_r3_it100", "3_3_6_m3_r2_it100",
                                 "4_3_7_m2_r2_it100", "4_4_8_m1_r4_it100", "4_4_8_m3_r3_it100",
                                 "5_5_10_m1_r4_it1000"])
@pytest.mark.parametrize("graph", [False, True])
def test_casci_energies_match_reference(cuda, golden_davidson, key, graph):
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import DavidsonLiuParams

    g = golden_davidson[key]
    ints = make_integrals(g["norb"], g["iseed"])
    sol = CASCISolver(norb=g["norb"], na=g["na"], nb=g["nb"], multiplicity=g["multiplicity"], nroot=g["nroot"],
                      E=ints.E, H=ints.H, V=ints.V, use_graph=graph,
                      davidson_liu_params=DavidsonLiuParams(e_tol=g["e_tol"], maxiter=1000)).run()
    assert sol.converged
    assert sol.eigensolver.used_graph == graph
    assert sol.spin_adapter.ncsf == g["ncsf"]
    np.testing.assert_allclose(np.sort(sol.evals), np.sort(g["evals"]), rtol=0, atol=1e-10)


@pytest.mark.parametrize("graph", [False, True])
def test_casci_mixed_precision_within_1e8(cuda, golden_davidson, graph):
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import CIParams, DavidsonLiuParams

    g = golden_davidson["5_5_10_m1_r4_it1000"]
    ints = make_integrals(g["norb"], g["iseed"])
    sol = CASCISolver(norb=10, na=5, nb=5, multiplicity=1, nroot=4, E=ints.E, H=ints.H, V=ints.V,
                      ci_params=CIParams(precision="mixed"), use_graph=graph,
                      davidson_liu_params=DavidsonLiuParams(e_tol=1e-10, maxiter=1000)).run()
    assert sol.converged
    assert sol.phases[0][0] == "fp32"
    np.testing.assert_allclose(np.sort(sol.evals), np.sort(g["evals"]), rtol=0, atol=1e-8)


def test_casci_energy_shift_and_warm_start(cuda, golden_davidson):
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import CIParams, DavidsonLiuParams

    g = golden_davidson["4_4_8_m1_r4_it100"]
    ints = make_integrals(8, g["iseed"])
    target = g["evals"][2]
    sol = CASCISolver(norb=8, na=4, nb=4, multiplicity=1, nroot=1, E=ints.E, H=ints.H, V=ints.V,
                      ci_params=CIParams(energy_shift=target + 1e-4),
                      davidson_liu_params=DavidsonLiuParams(maxiter=500)).run()
    # Shift targeting sorts Ritz values by |lambda - shift| (davidsonliu.py:262-265); the root it
    # converges to is an eigenvalue near the shift, not necessarily the closest one.
    assert min(abs(sol.evals[0] - e) for e in g["evals"]) < 1e-9
    assert sol.converged
    sol2 = CASCISolver(norb=8, na=4, nb=4, multiplicity=1, nroot=2, E=ints.E, H=ints.H, V=ints.V).run()
    it_first = sol2.eigensolver.iter
    sol2.run()  # MCSCF-style second run with the same integrals: warm start from the last vectors
    assert sol2.eigensolver.iter <= min(3, it_first)
    np.testing.assert_allclose(sol2.evals, g["evals"][:2], atol=1e-10)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("key", ["4_4_8_m1_r2", "5_5_10_m1_r1", "4_4_8_m3_r1"])
def test_mcscf_loop_with_new_integrals(cuda, key, graph):
    """The orbital optimiser's use of the CI solver (mcopt/mc_optimizer.py:297-328): set_ints with
    the next macro-iteration's integrals, then run(), warm-started from the last vectors. Each
    solve matches the energies of the reference's own Davidson, driven the same way on the
    reference's compiled sigma (tests/golden/mcscf.json), to 1e-10 Eh; warm starts take fewer
    iterations than the cold first solve."""
    import json
    import os

    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import DavidsonLiuParams
    from forte2_gb300.synthetic import rotate_integrals

    with open(os.path.join(os.path.dirname(__file__), "golden", "mcscf.json")) as f:
        g = json.load(f)[key]
    ints = make_integrals(g["norb"], g["iseed"])
    sol = CASCISolver(norb=g["norb"], na=g["na"], nb=g["nb"], multiplicity=g["multiplicity"], nroot=g["nroot"],
                      E=ints.E, H=ints.H, V=ints.V, use_graph=graph,
                      davidson_liu_params=DavidsonLiuParams(e_tol=g["e_tol"], maxiter=400))
    iters = []
    for k, step in enumerate(g["steps"]):
        if k > 0:
            ints = rotate_integrals(ints, g["rotation_seeds"][k - 1], g["theta"])
            sol.set_ints(ints.E, ints.H, ints.V)
        sol.run()
        assert sol.converged, (key, k)
        np.testing.assert_allclose(np.sort(sol.evals), np.sort(step["evals"]), rtol=0, atol=1e-10)
        iters.append(sol.eigensolver.iter)
    assert max(iters[1:]) < iters[0], iters
