"""Sigma autotuner: every kernel variant gives the same sigma; the choice is cached per shape."""

import numpy as np
import pytest

from forte2_gb300.synthetic import make_integrals, random_ci_vector

pytestmark = pytest.mark.gpu


def _builder(na, nb, n, seed):
    from forte2_gb300.ci_helpers import CISigmaBuilder, CIStrings

    s = CIStrings(na, nb, 0, [[0] * n], [], [])
    ints = make_integrals(n, seed)
    sb = CISigmaBuilder(s, ints.E, ints.H, ints.V, 0)
    sb.set_algorithm("hz")
    return s, sb


@pytest.mark.parametrize("na,nb,n", [(3, 3, 6), (4, 3, 8), (5, 5, 10)])
def test_all_variants_same_sigma(cuda, na, nb, n):
    torch = cuda
    from forte2_gb300.autotune import _apply, candidates

    s, sb = _builder(na, nb, n, 700 + n)
    c = torch.as_tensor(random_ci_vector(s.ndet, 9), device="cuda")
    ref = torch.empty_like(c)
    sb.Hamiltonian(c, ref)
    nref = torch.linalg.norm(ref).item()
    for prec, tol in (("fp64", 1e-13), ("fp32", 2e-6)):
        sb.set_precision(prec)
        for choice in candidates(sb, prec):
            _apply(sb, choice)
            out = torch.empty_like(c)
            sb.Hamiltonian(c, out)
            assert torch.linalg.norm(out - ref).item() / nref < tol, (prec, choice)
    assert sb.tensor_core_error() == 0


def test_autotune_picks_and_caches(cuda):
    torch = cuda
    from forte2_gb300.autotune import autotune_sigma, cached_choice, clear_cache

    clear_cache()
    s, sb = _builder(4, 4, 8, 31)
    r64 = autotune_sigma(sb, 8, 4, 4, "fp64")
    r32 = autotune_sigma(sb, 8, 4, 4, "fp32")
    assert r64["ms"] <= r64["default_ms"] + 1e-9 and len(r64["timings"]) == 4
    assert len(r32["timings"]) == 16  # tensor cores and the dense same-spin GEMMs available for this space
    assert cached_choice(8, 4, 4, "fp64") == r64["choice"]
    # a second builder of the same shape takes the cached choice without timing
    s2, sb2 = _builder(4, 4, 8, 32)
    assert autotune_sigma(sb2, 8, 4, 4, "fp64") is r64
    assert sb2._tuned["fp64"] == r64["choice"]
    c = torch.as_tensor(random_ci_vector(s2.ndet, 3), device="cuda")
    a, b = torch.empty_like(c), torch.empty_like(c)
    sb2.Hamiltonian(c, a)
    sb2.set_precision("fp32")  # applies the tuned FP32 variants
    sb2.Hamiltonian(c, b)
    assert torch.linalg.norm(a - b).item() / torch.linalg.norm(a).item() < 2e-6
    clear_cache()
