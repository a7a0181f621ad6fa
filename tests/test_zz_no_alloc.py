"""The allocation-free dot-product entry point, f2g_dav_dots_noalloc.

It serves callers that cannot allocate device memory at the point where they need the Davidson
dot products: a host program whose device memory comes from its own pool (a cudaMalloc would
bypass the pool and fails once the pool has reserved the GPU), or one that must not add the
device-wide synchronisation a cudaMalloc/cudaFree can cause inside its iteration loop. Its
partial sums live in a static device array, so it takes no scratch argument.

The test calls it through the C ABI and compares it with f2g_dav_dots (which takes a
caller-provided scratch buffer) on two calls in a row, then checks the size limit. This file is
collected last so that a run stopping at the first failure has already run every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call_both(torch, L, A, B):
    na, nb, n = A.shape[0], B.shape[0], A.shape[1]
    ref = torch.empty(na * nb, dtype=torch.float64, device="cuda")
    got = torch.empty(na * nb, dtype=torch.float64, device="cuda")
    scratch = torch.empty(int(L.f2g_dav_scratch_size(n)), dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.f2g_dav_dots(A.data_ptr(), na, A.stride(0), B.data_ptr(), nb, B.stride(0), n, ref.data_ptr(),
                          scratch.data_ptr(), stream) == 0, L.f2g_last_error()
    assert L.f2g_dav_dots_noalloc(A.data_ptr(), na, A.stride(0), B.data_ptr(), nb, B.stride(0), n,
                                  got.data_ptr(), stream) == 0, L.f2g_last_error()
    torch.cuda.synchronize()
    return ref.cpu().numpy().reshape(na, nb), got.cpu().numpy().reshape(na, nb)


def test_dots_noalloc_matches_dots_twice(cuda):
    torch = cuda
    from forte2_gb300._lib import lib

    L = lib()
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    # two calls in a row with different shapes and data: the shared static array must not carry
    # anything from the first call into the second
    for na, nb, n in [(16, 16, 3_000_001), (5, 3, 777)]:
        A = torch.randn((na, n), generator=g, dtype=torch.float64, device="cuda")
        B = torch.randn((nb, n), generator=g, dtype=torch.float64, device="cuda")
        ref, got = _call_both(torch, L, A, B)
        exact = (A @ B.T).cpu().numpy()
        scale = np.abs(exact).max()
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * scale)
        np.testing.assert_allclose(got, exact, rtol=1e-10, atol=1e-12 * scale * np.sqrt(n))


def test_dots_noalloc_rejects_sizes_beyond_the_static_limit(cuda):
    torch = cuda
    from forte2_gb300._lib import lib

    L = lib()
    A = torch.zeros((32, 10), dtype=torch.float64, device="cuda")
    out = torch.zeros(32 * 32, dtype=torch.float64, device="cuda")
    rc = L.f2g_dav_dots_noalloc(A.data_ptr(), 32, 10, A.data_ptr(), 32, 10, 10, out.data_ptr(), None)
    assert rc == 2
    assert b"static scratch limit of 256" in L.f2g_last_error()
    assert float(out.abs().sum()) == 0.0
