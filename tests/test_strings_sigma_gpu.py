"""GPU parity: device-built strings and coupling lists (bit-exact) and sigma = H C (1e-12
relative in FP64) against the golden fixtures from the reference, through the C ABI."""

import hashlib

import numpy as np
import pytest

from conftest import list_cases, sigma_cases
from forte2_gb300.synthetic import make_integrals, random_ci_vector

pytestmark = pytest.mark.gpu


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make(na, nb, n):
    from forte2_gb300.ci_helpers import CIStrings

    return CIStrings(na, nb, 0, [[0] * n], [], [])


def test_strings_and_lists_bit_exact(cuda, golden_lists):
    for na, nb, n in list_cases(golden_lists):
        s = make(na, nb, n)
        key = f"{na}_{nb}_{n}"
        assert np.array_equal(s.alpha_masks(), golden_lists[f"{key}_a_strings"]), key
        assert np.array_equal(s.beta_masks(), golden_lists[f"{key}_b_strings"]), key
        for spin, tag in ((0, "a"), (1, "b")):
            assert np.array_equal(s.list_1h(spin), golden_lists[f"{key}_{tag}_1h"]), (key, tag)
            assert np.array_equal(s.list_2h(spin), golden_lists[f"{key}_{tag}_2h"]), (key, tag)


def test_lists_cas16_bit_exact_hash(cuda, golden_lists_meta):
    s = make(8, 8, 16)
    for spin, tag in ((0, "a"), (1, "b")):
        m = golden_lists_meta[f"8_8_16_{tag}"]
        masks = s.alpha_masks() if spin == 0 else s.beta_masks()
        assert sha(masks) == m["strings_sha"]
        assert sha(s.list_1h(spin)) == m["l1_sha"]
        assert sha(s.list_2h(spin)) == m["l2_sha"]
    assert s.ndet == 12870 * 12870


def builder(na, nb, n, iseed):
    from forte2_gb300.ci_helpers import CISigmaBuilder

    s = make(na, nb, n)
    ints = make_integrals(n, iseed)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    sb.set_algorithm("hz")
    return s, sb, ints


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_sigma_matches_reference_fp64(cuda, golden_sigma):
    torch = cuda
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        iseed, cseed = golden_sigma[f"{key}_seeds"]
        s, sb, _ = builder(na, nb, n, int(iseed))
        c = random_ci_vector(s.ndet, int(cseed))
        ref = golden_sigma[f"{key}_sigma"]
        dc = torch.as_tensor(c, device="cuda")
        out = torch.empty_like(dc)
        sb.Hamiltonian(dc, out)
        got = out.cpu().numpy()
        assert rel(got, ref) <= 1e-12, (key, rel(got, ref))
        assert np.abs(got - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.0), key
        # host (numpy) path: the reference's own calling convention
        host = np.zeros(s.ndet)
        sb.Hamiltonian(c, host)
        assert rel(host, ref) <= 1e-12, key


def test_sigma_terms_match_reference(cuda, golden_sigma):
    torch = cuda
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        iseed, cseed = golden_sigma[f"{key}_seeds"]
        s, sb, _ = builder(na, nb, n, int(iseed))
        dc = torch.as_tensor(random_ci_vector(s.ndet, int(cseed)), device="cuda")
        scale = max(np.abs(golden_sigma[f"{key}_sigma"]).max(), 1.0)
        for t in ("h0", "h1_a", "h1_b", "aabb", "aaaa", "bbbb"):
            if f"{key}_term_{t}" not in golden_sigma.files:
                continue
            got = sb.term(t, dc).cpu().numpy()
            assert np.abs(got - golden_sigma[f"{key}_term_{t}"]).max() <= 1e-12 * scale, (key, t)


def test_kh_returns_the_same_sigma(cuda, golden_sigma):
    """"kh" runs the same device operator; it equals the reference's KH wherever both spins are
    occupied (the reference's KH drops the two-electron term when one spin is empty)."""
    torch = cuda
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        if f"{key}_sigma_kh" not in golden_sigma.files:
            continue
        iseed, cseed = golden_sigma[f"{key}_seeds"]
        s, sb, _ = builder(na, nb, n, int(iseed))
        sb.set_algorithm("knowles-handy")
        assert sb.get_algorithm() == "Knowles-Handy"
        dc = torch.as_tensor(random_ci_vector(s.ndet, int(cseed)), device="cuda")
        out = torch.empty_like(dc)
        sb.Hamiltonian(dc, out)
        ref = golden_sigma[f"{key}_sigma_kh"] if (na and nb) else golden_sigma[f"{key}_sigma"]
        assert rel(out.cpu().numpy(), ref) <= 1e-12, key


def test_sigma_checksums_cas12_cas14(cuda, golden_checksums):
    torch = cuda
    for key in ("6_6_12", "7_7_14"):
        meta = golden_checksums[key]
        na, nb, n = map(int, key.split("_"))
        # The integral recipe's bits can differ between machines (BLAS rounding in the einsum);
        # the sigma tolerances below are far above that level, so only x86 pins the hash.
        s, sb, ints = builder(na, nb, n, meta["iseed"])
        dc = torch.as_tensor(random_ci_vector(s.ndet, meta["cseed"]), device="cuda")
        out = torch.empty_like(dc)
        sb.Hamiltonian(dc, out)
        sig = out.cpu().numpy()
        rng = np.random.default_rng(meta["cseed"] + 1)
        w = rng.normal(size=s.ndet)
        assert abs(np.linalg.norm(sig) - meta["norm"]) <= 1e-12 * meta["norm"], key
        assert abs(sig @ w - meta["dot_w"]) <= 1e-11 * meta["norm"] * np.sqrt(s.ndet), key
        idx = np.array(meta["idx"])
        assert np.abs(sig[idx] - np.array(meta["vals"])).max() <= 1e-12 * meta["norm"], key


def test_sigma_linearity_and_symmetry_large(cuda):
    """Size-independent properties at CAS(14,14): H is linear and symmetric (<x|Hy> = <y|Hx>)."""
    torch = cuda
    s, sb, _ = builder(7, 7, 14, 2000)
    x = torch.as_tensor(random_ci_vector(s.ndet, 1), device="cuda")
    y = torch.as_tensor(random_ci_vector(s.ndet, 2), device="cuda")
    hx, hy, hz = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    sb.Hamiltonian(x, hx)
    sb.Hamiltonian(y, hy)
    sb.Hamiltonian(0.5 * x - 2.0 * y, hz)
    assert torch.linalg.norm(hz - (0.5 * hx - 2.0 * hy)) <= 1e-12 * torch.linalg.norm(hz)
    assert abs(float(x @ hy) - float(y @ hx)) <= 1e-12 * float(torch.linalg.norm(hx))


def test_multivector_apply(cuda, golden_sigma):
    torch = cuda
    s, sb, _ = builder(4, 4, 8, 19)
    c1 = random_ci_vector(s.ndet, 109)
    c2 = random_ci_vector(s.ndet, 5)
    X = torch.as_tensor(np.stack([c1, c2]), device="cuda")
    Y = torch.empty_like(X)
    sb.Hamiltonian(X, Y)
    assert rel(Y[0].cpu().numpy(), golden_sigma["4_4_8_sigma"]) <= 1e-12
    y2 = torch.empty_like(X[1])
    sb.Hamiltonian(X[1].contiguous(), y2)
    assert torch.equal(Y[1], y2)


def test_memory_contract(cuda):
    """tests/ci/test_ci_rdms.py:412-436 of the reference: set_memory(-1) -> ValueError,
    set_memory(0) -> RuntimeError on Hamiltonian, and a failed call does not corrupt later builds."""
    from forte2_gb300.ci_helpers import CISigmaBuilder

    norb = 6
    lists = make(2, 2, norb)
    H = np.diag(np.linspace(-1.0, 1.0, norb))
    V = np.zeros((norb,) * 4)
    b = CISigmaBuilder(lists, 0.25, H, V, 0)
    b.set_algorithm("hz")
    rng = np.random.default_rng(205)
    basis = rng.normal(size=lists.ndet)
    basis /= np.linalg.norm(basis)
    with pytest.raises(ValueError, match="memory must be non-negative"):
        b.set_memory(-1)
    b.set_memory(1)
    expected = np.zeros(lists.ndet)
    b.Hamiltonian(basis, expected)
    b.set_memory(0)
    with pytest.raises(RuntimeError, match="too small for one K-block column"):
        b.Hamiltonian(basis, np.zeros(lists.ndet))
    b.set_memory(1)
    actual = np.zeros(lists.ndet)
    b.Hamiltonian(basis, actual)
    np.testing.assert_allclose(actual, expected, rtol=1e-12, atol=1e-12)
    b.set_memory(64)
    again = np.zeros(lists.ndet)
    b.Hamiltonian(basis, again)
    np.testing.assert_allclose(again, expected, rtol=1e-12, atol=1e-12)


def test_shape_errors(cuda):
    from forte2_gb300.ci_helpers import CISigmaBuilder

    s = make(2, 2, 4)
    with pytest.raises(RuntimeError, match="H shape does not match"):
        CISigmaBuilder(s, 0.0, np.zeros((3, 3)), np.zeros((4,) * 4))
    with pytest.raises(RuntimeError, match="V must be a 4D tensor"):
        CISigmaBuilder(s, 0.0, np.zeros((4, 4)), np.zeros((4, 4)))
    with pytest.raises(RuntimeError, match="V shape does not match"):
        CISigmaBuilder(s, 0.0, np.zeros((4, 4)), np.zeros((4, 4, 4, 3)))
    sb = CISigmaBuilder(s, 0.0, np.zeros((4, 4)), np.zeros((4,) * 4))
    with pytest.raises(RuntimeError, match="CI algorithm foo not valid"):
        sb.set_algorithm("foo")
    with pytest.raises(RuntimeError, match="stride 1"):
        sb.Hamiltonian(np.zeros(2 * s.ndet)[::2], np.zeros(s.ndet))


def test_fp32_mode_error_bound(cuda, golden_sigma):
    torch = cuda
    s, sb, _ = builder(5, 5, 10, 1000)
    sb.set_precision("fp32")
    dc = torch.as_tensor(random_ci_vector(s.ndet, 110), device="cuda")
    out = torch.empty_like(dc)
    sb.Hamiltonian(dc, out)
    err = rel(out.cpu().numpy(), golden_sigma["5_5_10_sigma"])
    assert err < 1e-5, err
    sb.set_precision("fp64")
    sb.Hamiltonian(dc, out)
    assert rel(out.cpu().numpy(), golden_sigma["5_5_10_sigma"]) <= 1e-12


def test_avg_build_time(cuda):
    torch = cuda
    s, sb, _ = builder(4, 4, 8, 19)
    assert sb.avg_build_time() == [0.0, 0.0, 0.0, 0.0]
    dc = torch.as_tensor(random_ci_vector(s.ndet, 1), device="cuda")
    out = torch.empty_like(dc)
    for _ in range(3):
        sb.Hamiltonian(dc, out)
    t = sb.avg_build_time()
    assert t[0] > 0 and abs(t[0] - (t[1] + t[2] + t[3])) < 1e-9


def test_det_energies_match_reference(cuda, golden_sigma):
    for na, nb, n in sigma_cases(golden_sigma):
        key = f"{na}_{nb}_{n}"
        if f"{key}_det_energies" not in golden_sigma.files:
            continue
        iseed, _ = golden_sigma[f"{key}_seeds"]
        s, sb, _ = builder(na, nb, n, int(iseed))
        got = sb.det_energies().cpu().numpy()
        assert np.abs(got - golden_sigma[f"{key}_det_energies"]).max() < 1e-12, key


def test_capped_opposite_grid_same_sigma(cuda, golden_sigma):
    """A capped opposite-spin grid (blocks loop over the alpha strings) gives the same sigma."""
    torch = cuda
    s, sb, _ = builder(4, 4, 8, 19)
    X = torch.as_tensor(np.stack([random_ci_vector(s.ndet, 109), random_ci_vector(s.ndet, 5)]), device="cuda")
    Y = torch.empty_like(X)
    sb.Hamiltonian(X, Y)
    sb.set_max_blocks(5)  # 70 alpha strings over 5 blocks
    Y5 = torch.empty_like(X)
    sb.Hamiltonian(X, Y5)
    sb.set_max_blocks(0)
    assert rel(Y5[0].cpu().numpy(), golden_sigma["4_4_8_sigma"]) <= 1e-12
    np.testing.assert_allclose(Y5.cpu().numpy(), Y.cpu().numpy(), rtol=0, atol=1e-13)
    with pytest.raises(ValueError):
        sb.set_max_blocks(-1)


@pytest.mark.parametrize("na,nb,n", [(3, 3, 6), (4, 3, 7), (2, 5, 8), (5, 5, 10), (7, 7, 14)])
def test_fp32_tensor_core_opposite_spin(cuda, na, nb, n):
    """FP32 sigma with the opposite-spin term on the tensor cores (split-FP16 products) agrees with
    the FP64 sigma to FP32 accuracy, and with the CUDA-core FP32 kernel."""
    torch = cuda
    from forte2_gb300.ci_helpers import CISigmaBuilder

    s = make(na, nb, n)
    ints = make_integrals(n, 600 + n)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    c = torch.as_tensor(np.stack([random_ci_vector(s.ndet, 3 + n), random_ci_vector(s.ndet, 4 + n)]), device="cuda")
    ref = torch.empty_like(c)
    sb.Hamiltonian(c, ref)
    sb.set_precision("fp32")
    assert sb.set_tensor_cores(False) is True  # available for these spaces
    cc = torch.empty_like(c)
    sb.Hamiltonian(c, cc)
    sb.set_tensor_cores(True)
    tc = torch.empty_like(c)
    sb.Hamiltonian(c, tc)
    assert sb.tensor_core_error() == 0
    for i in range(2):
        e_tc = rel(tc[i].cpu().numpy(), ref[i].cpu().numpy())
        e_cc = rel(cc[i].cpu().numpy(), ref[i].cpu().numpy())
        assert e_tc < 2e-6 and e_tc < 3 * e_cc + 1e-7
    # the B tiles fed by TMA from the prebuilt operands (default) and built by each CTA give the
    # same bits, also after new integrals (the operands are rebuilt in place, in stream order)
    sb.set_variant("tma_b", False)
    own = torch.empty_like(c)
    sb.Hamiltonian(c, own)
    assert torch.equal(own, tc)
    sb.set_variant("tma_b", True)
    ints2 = make_integrals(n, 700 + n)
    for update in (sb.update_integrals, sb.set_Hamiltonian):
        update(ints2.E, ints2.H, ints2.V)
        t1, t2 = torch.empty_like(c), torch.empty_like(c)
        sb.Hamiltonian(c, t1)
        sb.set_variant("tma_b", False)
        sb.Hamiltonian(c, t2)
        sb.set_variant("tma_b", True)
        assert sb.tensor_core_error() == 0
        assert torch.equal(t1, t2) and not torch.equal(t1, tc)


@pytest.mark.parametrize("precision,n", [("fp64", 12), ("fp32", 12), ("fp32", 14)])
def test_sigma_is_bitwise_reproducible(cuda, precision, n):
    """The same vectors give bitwise-identical sigma across repeated calls, capped grids and batch
    shapes: every kernel sums each element in a fixed order (FP64 opposite spin: one write phase
    per created orbital; FP32 tensor cores: exact fixed-point row sums; CAS(14,14) FP32 also runs
    the grouped same-spin kernel, input rows in ascending order)."""
    torch = cuda
    s, sb, _ = builder(n // 2, n // 2, n, 77)
    sb.set_precision(precision)
    if precision == "fp32":
        assert sb.set_tensor_cores(True) is True
    X = torch.as_tensor(np.stack([random_ci_vector(s.ndet, 31), random_ci_vector(s.ndet, 32)]), device="cuda")
    first = torch.empty_like(X)
    sb.Hamiltonian(X, first)
    for _ in range(4):
        again = torch.empty_like(X)
        sb.Hamiltonian(X, again)
        assert torch.equal(again, first)
    for cap in ((5, 37, 152, 0) if n <= 12 else (37, 0)):
        sb.set_max_blocks(cap)
        capped = torch.empty_like(X)
        sb.Hamiltonian(X, capped)
        assert torch.equal(capped, first), cap
    for i in range(2):
        single = torch.empty_like(X[i])
        sb.Hamiltonian(X[i].contiguous(), single)
        assert torch.equal(single, first[i])
    if precision == "fp32":
        assert sb.tensor_core_error() == 0


def test_tensor_core_wait_limit_reports_error_and_recovers(cuda):
    """A bounded wait that gives up sets the tensor-core error flag (the kernel then drains its
    committed MMAs and releases tensor memory); the context stays usable and the next build with
    the default limit is correct."""
    torch = cuda
    s, sb, _ = builder(5, 5, 10, 1000)
    dc = torch.as_tensor(random_ci_vector(s.ndet, 110), device="cuda")
    ref = torch.empty_like(dc)
    sb.Hamiltonian(dc, ref)
    sb.set_precision("fp32")
    assert sb.set_tensor_cores(True) is True
    sb.set_variant("tc_wait_limit", 1)  # one poll: the first wait gives up
    out = torch.empty_like(dc)
    sb.Hamiltonian(dc, out)
    torch.cuda.synchronize()
    assert sb.tensor_core_error() == 1
    sb.set_variant("tc_wait_limit", 0)  # default limit; clears the flag
    assert sb.tensor_core_error() == 0
    sb.Hamiltonian(dc, out)
    assert sb.tensor_core_error() == 0
    assert rel(out.cpu().numpy(), ref.cpu().numpy()) < 2e-6


@pytest.mark.parametrize("na,nb,n", [(3, 3, 6), (4, 3, 7), (5, 5, 10), (6, 6, 12), (7, 7, 14)])
def test_fp32_dense_same_spin(cuda, na, nb, n):
    """FP32 sigma with the same-spin terms as dense tensor-core GEMMs (split FP16, three cuBLAS
    products): FP32 accuracy against the FP64 sigma, the same bits call after call and for a vector
    alone or in a batch, and new integrals (in place, in stream order) give the sigma of a fresh
    builder with those integrals."""
    torch = cuda
    from forte2_gb300.ci_helpers import CISigmaBuilder

    s = make(na, nb, n)
    ints = make_integrals(n, 800 + n)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    c = torch.as_tensor(np.stack([random_ci_vector(s.ndet, 5 + n), random_ci_vector(s.ndet, 6 + n)]), device="cuda")
    ref = torch.empty_like(c)
    sb.Hamiltonian(c, ref)
    sb.set_precision("fp32")
    sb.set_variant("dense_same_spin", 0)  # (the default from 512 strings per spin)
    sparse = torch.empty_like(c)
    sb.Hamiltonian(c, sparse)
    sb.set_variant("dense_same_spin", 1)
    dense = torch.empty_like(c)
    sb.Hamiltonian(c, dense)
    again = torch.empty_like(c)
    sb.Hamiltonian(c, again)
    assert torch.equal(dense, again)
    one = torch.empty_like(c[1])
    sb.Hamiltonian(c[1].contiguous(), one)
    assert torch.equal(one, dense[1])
    for i in range(2):
        e_d = rel(dense[i].cpu().numpy(), ref[i].cpu().numpy())
        e_s = rel(sparse[i].cpu().numpy(), ref[i].cpu().numpy())
        assert e_d < 2e-6 and e_d < 4 * e_s + 1e-7
    ints2 = make_integrals(n, 900 + n)
    fresh = CISigmaBuilder(s, ints2.E, ints2.H, ints2.V, 0)
    fresh.set_precision("fp32")
    fresh.set_variant("dense_same_spin", 1)
    want = torch.empty_like(c)
    fresh.Hamiltonian(c, want)
    for update in (sb.update_integrals, sb.set_Hamiltonian):
        update(ints2.E, ints2.H, ints2.V)
        got = torch.empty_like(c)
        sb.Hamiltonian(c, got)
        assert torch.equal(got, want)
    big = make_integrals(15, 1)  # C(15, 7) = 6,435 strings per spin: above the dense limit
    with pytest.raises(ValueError):
        CISigmaBuilder(make(7, 7, 15), big.E, big.H, big.V, 0).set_variant("dense_same_spin", 1)
