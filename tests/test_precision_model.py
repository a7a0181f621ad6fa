"""CPU models of the mixed mode's arithmetic (no GPU): the exact fixed-point split of the
tensor-core kernel's scatter and the accuracy of split-FP16 products with FP32 accumulation.

The device code does the same operations with fmaf (one rounding); here a fused multiply-add of
FP32 values is modelled as the FP64 result rounded once to FP32, which is exact for these
operands (their FP64 product and sum carry no rounding)."""

import numpy as np

C = np.float32(12582912.0)  # 1.5 * 2^23


def fmaf(a, b, c):
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(np.float32)


def split_fixed(x):
    """hi = round(x / 2^15), lo = round((x - hi 2^15) 2^7) as in the scatter (both exact)."""
    x = np.asarray(x, dtype=np.float32)
    t = fmaf(x, np.float32(2.0 ** -15), C)
    rem = fmaf(-(t - C), np.float32(32768.0), x)
    u = fmaf(rem, np.float32(128.0), C)
    hi = t.view(np.int32).astype(np.int64) - np.array(C).view(np.int32).astype(np.int64)
    lo = u.view(np.int32).astype(np.int64) - np.array(C).view(np.int32).astype(np.int64)
    return hi, lo


def test_fixed_point_split_is_exact_round_half_even():
    rng = np.random.default_rng(0)
    # magnitudes spread over [2^-10, 2^37) scaled units, both signs, plus exact halves
    x = (rng.uniform(-1, 1, 200_000) * 2.0 ** rng.uniform(-10, 37, 200_000)).astype(np.float32)
    x = np.concatenate([x, np.float32([0.5 / 128, 1.5 / 128, -2.5 / 128, 2.0 ** 36 + 0.5 / 128])])
    hi, lo = split_fixed(x)
    want = np.round(x.astype(np.float64) * 128.0)  # numpy rounds half to even, as the FP32 offset does
    assert np.array_equal(hi * 2 ** 22 + lo, want.astype(np.int64))
    assert np.abs(lo).max() <= 2 ** 21
    # a tile's products are bounded: |A|, |B| <= 2^15 (hi parts; the lo parts add under 2^-10 of
    # that) and K <= 72, so |x| < 72 * 2^30 * (1 + 2^-9) < 2^36.2 and |hi| < 2^21.2
    bound = 72 * 2.0 ** 30 * (1 + 2.0 ** -9)
    inside = np.abs(x.astype(np.float64)) < bound
    assert np.abs(hi[inside]).max() < 2 ** 21.2
    # at most 72 contributions per element: both sums stay exact in 32-bit integers
    assert 72 * 2 ** 21.2 < 2 ** 31


def split16(x, e):
    s = (np.asarray(x, dtype=np.float32) * np.float32(2.0 ** e)).astype(np.float32)
    hi = s.astype(np.float16)
    lo = (s - hi.astype(np.float32)).astype(np.float16)
    return hi, lo


def scale_exponent(m):
    return 15 - int(np.frexp(np.float32(m))[1])


def model_product(A, B, chunk):
    """sum_k A[i,k] B[k,j] as the kernels form it: both operands scaled into [2^14, 2^15) and split
    into FP16 hi + lo, three products hi.hi + lo.hi + hi.lo, FP32 sums over K chunks."""
    ea, eb = scale_exponent(np.abs(A).max()), scale_exponent(np.abs(B).max())
    ah, al = split16(A, ea)
    bh, bl = split16(B, eb)
    out = np.zeros((A.shape[0], B.shape[1]), dtype=np.float32)
    for k0 in range(0, A.shape[1], chunk):
        sl = slice(k0, k0 + chunk)
        for a, b in ((ah, bh), (al, bh), (ah, bl)):
            out += (a[:, sl].astype(np.float64) @ b[sl].astype(np.float64)).astype(np.float32)
    return out.astype(np.float64) * 2.0 ** (-ea - eb)


def test_split_fp16_products_reach_fp32_accuracy():
    rng = np.random.default_rng(1)
    # opposite-spin tile: K = 72 alpha excitations; same-spin dense GEMM: K = 3432 in chunks of 1024
    for K, chunk in ((72, 72), (3432, 1024)):
        A = rng.normal(size=(64, K))
        B = rng.normal(size=(K, 48)) * (rng.uniform(size=(K, 48)) < 0.1)  # sparse like the string Hamiltonian
        ref = A @ B
        got = model_product(A, B, chunk)
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert rel < 5e-7, (K, rel)
