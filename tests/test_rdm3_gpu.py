"""Three-body RDMs and the 3-cumulant on the GPU against the reference's own
ci_sigma_builder_3rdm.cc (tests/golden/rdm3_checksums.json: norm, seeded dot product and 64
sampled entries of every kind for the 11 RDM spaces; full arrays up to 4 orbitals), and the
partial-trace identity sum_r G3[p,q,r,s,t,r] = (N - 2) G2[p,q,s,t] at sizes beyond the fixtures,
blocked spaces included.

Tolerance: 1e-12 relative to the largest element (FP64 sums in another order)."""

import numpy as np
import pytest

from conftest import list_cases, rdm_checksum_matches
from forte2_gb300.synthetic import make_integrals, random_ci_vector

pytestmark = pytest.mark.gpu

RDM3_KINDS = ("aaa_3rdm", "bbb_3rdm", "aab_3rdm", "abb_3rdm", "sf_3rdm", "sf_3cumulant")


def builder(n, na, nb, seed, space=None):
    from forte2_gb300.ci_helpers import CISigmaBuilder, CIStrings

    ints = make_integrals(n, seed)
    s = CIStrings(na, nb, *space) if space else CIStrings(na, nb, 0, [[0] * n], [], [])
    return s, CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)


def test_3rdms_match_reference(cuda, golden_rdm, golden_rdm3):
    meta, full = golden_rdm3
    for na, nb, n in list_cases(golden_rdm):
        key = f"{na}_{nb}_{n}"
        sl, sr = (int(x) for x in golden_rdm[f"{key}_seeds"])
        s, sb = builder(n, na, nb, sl)
        cl = random_ci_vector(s.ndet, sl)
        cr = random_ci_vector(s.ndet, sr)
        for j, kind in enumerate(RDM3_KINDS):
            for tag, b in (("LR", cr), ("LL", cl)):
                got = np.asarray(getattr(sb, kind)(cl, b))
                name = f"{key}_{kind}_{tag}"
                assert rdm_checksum_matches(got, meta[name], 7000 + 10 * j + (tag == "LL")), name
                if name in full.files:
                    ref = full[name]
                    assert got.reshape(-1).shape == ref.reshape(-1).shape, name
                    scale = max(1.0, np.abs(ref).max(initial=0.0))
                    assert np.abs(got.reshape(-1) - ref.reshape(-1)).max(initial=0.0) <= 1e-12 * scale, name


@pytest.mark.parametrize("n,na,nb,space", [
    (10, 5, 5, None),
    (9, 5, 3, None),
    (12, 6, 6, None),
    (8, 4, 4, (2, [[0, 1, 2, 3, 0, 1, 2, 3]], [], [])),
    (8, 4, 3, (0, [[0, 0, 0, 0], [0, 0, 0, 0]], [5], [7])),
])
def test_3rdm_partial_trace_and_device_tensors(cuda, n, na, nb, space):
    """sum_r G3[p,q,r,s,t,r] = (N - 2) G2[p,q,s,t]; the spin blocks obey their own traces; CUDA
    tensors in give CUDA tensors out with the same numbers."""
    torch = cuda
    s, sb = builder(n, na, nb, 300 + n, space)
    c = random_ci_vector(s.ndet, 40 + n)
    g3 = np.asarray(sb.sf_3rdm(c, c))
    g2 = np.asarray(sb.sf_2rdm(c, c))
    assert g3.shape == (n,) * 6
    scale = max(1.0, np.abs(g2).max())
    assert np.abs(np.einsum("pqrstr->pqst", g3) - (na + nb - 2) * g2).max() < 1e-11 * scale
    # aab summed over its beta index pair (r = u) gives (nb) x the packed aa 2-RDM
    aab = np.asarray(sb.aab_3rdm(c, c))
    aa = np.asarray(sb.aa_2rdm(c, c))
    if aab.size and aa.size:
        assert np.abs(np.einsum("prqr->pq", aab) - nb * aa).max() < 1e-11 * scale
    dc = torch.from_numpy(c).cuda()
    d = sb.sf_3rdm(dc, dc)
    assert d.is_cuda and np.abs(d.cpu().numpy() - g3).max() < 1e-13 * max(1.0, np.abs(g3).max())


def test_3cumulant_vanishes_for_a_closed_shell_determinant(cuda):
    """A closed-shell determinant has no connected three-body part: its 3-cumulant is zero."""
    n, na, nb = 7, 3, 3
    s, sb = builder(n, na, nb, 5)
    c = np.zeros(s.ndet)
    N0 = 35
    c[5 * N0 + 5] = 1.0  # the same alpha and beta string
    l3 = np.asarray(sb.sf_3cumulant(c, c))
    assert np.abs(l3).max() < 1e-13


def test_ci_driver_3rdms(cuda):
    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import DavidsonLiuParams

    n = 8
    ints = make_integrals(n, 77)
    sol = CASCISolver(norb=n, na=4, nb=4, multiplicity=1, nroot=2, E=ints.E, H=ints.H, V=ints.V,
                      davidson_liu_params=DavidsonLiuParams(e_tol=1e-12)).run()
    aaa, aab, abb, bbb = sol.make_sd_3rdm(0)
    assert aaa.shape == bbb.shape == (56, 56) and aab.shape == (28, 8, 28, 8) and abb.shape == (8, 28, 8, 28)
    # a singlet: alpha and beta blocks are mirror images
    assert np.abs(aaa - bbb).max() < 1e-10
    assert np.abs(aab - abb.transpose(1, 0, 3, 2)).max() < 1e-10
    g3 = sol.make_sf_3rdm(0, 1)  # a transition 3-RDM
    assert g3.shape == (n,) * 6
    l3 = sol.make_3cumulant(0)
    assert l3.shape == (n,) * 6
