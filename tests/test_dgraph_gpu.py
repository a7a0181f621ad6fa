"""Graph-captured Davidson-Liu iterations (f2g_dgraph_*) against the host-driven iterations."""

import numpy as np
import pytest

from forte2_gb300.synthetic import make_integrals

pytestmark = pytest.mark.gpu


def _solver(norb, mult, nroot, iseed, graph, **kw):
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import CIParams, DavidsonLiuParams

    ints = make_integrals(norb, iseed)
    dl = DavidsonLiuParams(e_tol=kw.pop("e_tol", 1e-10), maxiter=kw.pop("maxiter", 1000))
    return CASCISolver(norb=norb, na=norb // 2, nb=norb // 2, multiplicity=mult, nroot=nroot, E=ints.E, H=ints.H,
                       V=ints.V, use_graph=graph, davidson_liu_params=dl,
                       ci_params=CIParams(precision=kw.pop("precision", "fp64")), **kw)


@pytest.mark.parametrize("norb,mult,nroot", [(6, 1, 1), (6, 3, 3), (8, 1, 4), (8, 3, 2)])
def test_graph_matches_host_iterations(cuda, norb, mult, nroot):
    host = _solver(norb, mult, nroot, 900 + norb, False).run()
    gr = _solver(norb, mult, nroot, 900 + norb, True).run()
    assert gr.eigensolver.used_graph and not host.eigensolver.used_graph
    assert gr.converged and host.converged
    np.testing.assert_allclose(gr.evals, host.evals, rtol=0, atol=1e-10)
    # same algorithm and decisions, different summation order in the reductions
    assert abs(gr.eigensolver.iter - host.eigensolver.iter) <= 3
    # Ritz vectors: same subspace (sign-insensitive overlap)
    ov = (gr.evecs.T @ host.evecs).abs().diagonal().cpu().numpy()
    np.testing.assert_allclose(ov, 1.0, atol=1e-6)


def test_graph_launch_length_does_not_change_results(cuda):
    a = _solver(8, 1, 3, 77, True)
    b = _solver(8, 1, 3, 77, True)
    a.run()  # creates the eigensolver
    a.eigensolver.iters_per_launch = 1
    a.eigensolver._graphs.clear()
    a.new_problem(a.E, a.H, a.V)
    a.run()
    b.run()
    # the same kernels in the same order, and every kernel sums in a fixed order: the same bits
    assert a.eigensolver.iter == b.eigensolver.iter
    assert np.array_equal(a.evals, b.evals)


def test_graph_iteration_limit(cuda):
    host = _solver(8, 1, 2, 31, False, maxiter=3).run()
    gr = _solver(8, 1, 2, 31, True, maxiter=3).run()
    assert not host.converged and not gr.converged
    assert host.eigensolver.iter == gr.eigensolver.iter == 2
    assert gr.eigensolver.graph_status == 2
    hist = gr.eigensolver.graph_history()
    assert len(hist) == 3 and all(h[3] > 0 for h in hist)


@pytest.mark.parametrize("mult,nroot,precision", [(1, 2, "fp64"), (3, 1, "mixed")])
def test_graph_iterations_on_long_vectors(cuda, mult, nroot, precision):
    """CAS(12,12) (226,512 singlet / 382,239 triplet CSFs): graph-captured iterations with the
    multi-block dot products and Gram-Schmidt give the host-driven energies."""
    host = _solver(12, mult, nroot, 1212, False, precision=precision).run()
    gr = _solver(12, mult, nroot, 1212, True, precision=precision).run()
    assert gr.eigensolver.used_graph and not host.eigensolver.used_graph
    assert gr.eigensolver.size > 1 << 15
    assert gr.converged and host.converged
    np.testing.assert_allclose(gr.evals, host.evals, rtol=0, atol=1e-10 if precision == "fp64" else 1e-8)
    if precision == "fp64":
        assert abs(gr.eigensolver.iter - host.eigensolver.iter) <= 3


def test_pooled_solver_reuses_graphs(cuda):
    s = _solver(8, 3, 2, 41, True).run()
    graphs = dict(s.eigensolver._graphs)
    ints = make_integrals(8, 42)
    s.new_problem(ints.E, ints.H, ints.V)
    s.run()
    fresh = _solver(8, 3, 2, 42, True).run()
    np.testing.assert_allclose(s.evals, fresh.evals, rtol=0, atol=1e-10)
    assert dict(s.eigensolver._graphs) == graphs  # nothing captured again


def test_graph_mixed_precision(cuda):
    ref = _solver(8, 1, 3, 55, False).run()
    mx = _solver(8, 1, 3, 55, True, precision="mixed").run()
    assert mx.converged and mx.eigensolver.used_graph
    np.testing.assert_allclose(mx.evals, ref.evals, rtol=0, atol=1e-8)


def test_gs_append_kernel(cuda):
    import torch

    from forte2_gb300._lib import check, lib, stream_handle

    n, cap = 3000, 12
    g = torch.Generator(device="cuda").manual_seed(3)
    R = torch.rand((8, n), generator=g, dtype=torch.float64, device="cuda") - 0.5
    R[3] = 2.0 * R[1] - R[0]  # dependent: rejected
    R[6] = 0.0  # zero: rejected
    B = torch.zeros((cap, n), dtype=torch.float64, device="cuda")
    added = torch.zeros(1, dtype=torch.int32, device="cuda")
    check(lib().f2g_dav_gs_append(B.data_ptr(), n, cap, 0, R.data_ptr(), n, 8, n, 1e-8, 1e-12, 9, 5,
                                  added.data_ptr(), stream_handle()))
    k = int(added.item())
    assert k == 9  # 6 independent candidates + 3 random rows to reach min_total
    S = (B[:k] @ B[:k].T).cpu().numpy()
    np.testing.assert_allclose(S, np.eye(k), atol=1e-12)
    with pytest.raises(ValueError):
        check(lib().f2g_dav_gs_append(B.data_ptr(), n, cap, 10, R.data_ptr(), n, 8, n, 1e-8, 1e-12, 0, 5,
                                      added.data_ptr(), stream_handle()))


@pytest.mark.parametrize("m", [1, 2, 3, 7, 16, 33, 64])
def test_dav_eigh_matches_numpy(cuda, m):
    import torch

    from forte2_gb300._lib import check, lib, stream_handle

    rng = np.random.default_rng(m)
    A = rng.normal(size=(m, m))
    A = A + A.T
    if m >= 7:
        A[:3, :] = 0.0  # a threefold-degenerate zero eigenvalue
        A[:, :3] = 0.0
    G = torch.as_tensor(A, device="cuda")
    ev = torch.empty(m, dtype=torch.float64, device="cuda")
    V = torch.empty((m, m), dtype=torch.float64, device="cuda")
    check(lib().f2g_dav_eigh(m, G.data_ptr(), ev.data_ptr(), V.data_ptr(), stream_handle()))
    w = ev.cpu().numpy()
    Q = V.cpu().numpy()
    scale = max(1.0, np.abs(A).max())
    np.testing.assert_allclose(w, np.linalg.eigvalsh(A), rtol=0, atol=1e-12 * scale * m)
    assert np.all(np.diff(w) >= 0)
    np.testing.assert_allclose(Q.T @ Q, np.eye(m), atol=1e-12 * m)
    np.testing.assert_allclose(A @ Q, Q * w, atol=1e-11 * scale * m)


@pytest.mark.parametrize("norb,mult", [(6, 1), (8, 3), (10, 1)])
def test_csf_space_sigma_call(cuda, norb, mult):
    """apply_csf = csf -> det -> H -> det -> csf in one call: FP64 equals the three-call path to
    rounding,
    FP32 (transforms in FP32 too) agrees to FP32 accuracy."""
    import torch

    from forte2_gb300.ci_helpers import CISigmaBuilder, CISpinAdapter, CIStrings

    s = CIStrings(norb // 2, norb // 2, 0, [[0] * norb], [], [])
    sa = CISpinAdapter(mult - 1, 0, norb)
    sa.prepare_couplings(s.make_determinants())
    ints = make_integrals(norb, 50 + norb)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    sb.set_algorithm("hz")
    g = torch.Generator(device="cuda").manual_seed(norb)
    X = torch.rand((3, sa.ncsf), generator=g, dtype=torch.float64, device="cuda") - 0.5
    det = torch.empty((3, s.ndet), dtype=torch.float64, device="cuda")
    sdet = torch.empty_like(det)
    ref = torch.empty_like(X)
    sa.csf_C_to_det_C(X, det)
    sb.Hamiltonian(det, sdet)
    sa.det_C_to_csf_C(sdet, ref)
    out = torch.empty_like(X)
    sb.apply_csf(sa, X, out)
    # the one-call closure against the three separate calls
    assert (torch.linalg.norm(out - ref) / torch.linalg.norm(ref)).item() < 1e-14
    sb.set_precision("fp32")
    out32 = torch.empty_like(X)
    sb.apply_csf(sa, X, out32)
    rel = (torch.linalg.norm(out32 - ref) / torch.linalg.norm(ref)).item()
    assert 0 < rel < 2e-6
