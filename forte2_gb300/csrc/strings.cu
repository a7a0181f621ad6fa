// Device string graph and coupling lists for a CAS active space (C1 symmetry, one GAS space).
//
// The content is the reference's (forte2/ci/ci_strings.cc:34-184, ci_strings_makers.cc:13-274):
//   strings   in std::next_permutation order of (b0..b_{n-1}) (ci_strings_makers.cc:39-52);
//   up1[K]    1-hole list of each (k-1)-electron string K: entries (sign, p, I) with I = K + p,
//             sign = <K|a_p|I> = (-1)^{#occupied below p in I}, in ascending address of I
//             (ci_strings_makers.cc:163-241);
//   up2[K]    2-hole list of each (k-2)-electron string K: entries (sign, p, q, I), p > q,
//             I = K + p + q, sign = <K|a_p a_q|I> (ci_strings_makers.cc:243-274), ascending I;
//   down1[I]  the inverse of up1: for each string I the k entries (K = I - p, p, sign), p ascending.
//
// Every list is built by one thread per hole string: the entries of K are produced directly in
// the reference's order (ascending address of I = descending p for one hole; descending q, then
// descending p, for two holes), so no sort or hash map is needed.
#include "strings.cuh"

namespace f2g {

__global__ void k_unrank(int n, int k, int64_t N, const uint64_t* binom, uint64_t* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N)
        out[i] = string_unrank((uint64_t)i, n, k, binom);
}

__global__ void k_up1(int n, int k, int64_t N1, int m1, const uint64_t* binom, uint32_t* out) {
    const int64_t K = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (K >= N1)
        return;
    const uint64_t mK = string_unrank((uint64_t)K, n, k - 1, binom);
    int j = 0;
    for (int p = n - 1; p >= 0; --p) {
        if (mK >> p & 1)
            continue;
        const uint64_t mI = mK | (uint64_t(1) << p);
        const uint64_t I = string_rank(mI, n, k, binom);
        if (j < m1)
            out[K * m1 + j] = pack1((uint32_t)I, p, parity_below(mI, p));
        ++j;
    }
}

__global__ void k_down1(int n, int k, int64_t N0, const uint64_t* binom, uint32_t* out) {
    const int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= N0)
        return;
    const uint64_t mI = string_unrank((uint64_t)I, n, k, binom);
    int j = 0;
    for (int p = 0; p < n; ++p) {
        if (!(mI >> p & 1))
            continue;
        const uint64_t mK = mI & ~(uint64_t(1) << p);
        const uint64_t K = string_rank(mK, n, k - 1, binom);
        if (j < k)
            out[I * k + j] = pack1((uint32_t)K, p, parity_below(mI, p));
        ++j;
    }
}

__global__ void k_up2(int n, int k, int64_t N2, int m2, const uint64_t* binom, uint64_t* out) {
    const int64_t K = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (K >= N2)
        return;
    const uint64_t mK = string_unrank((uint64_t)K, n, k - 2, binom);
    int j = 0;
    for (int q = n - 1; q >= 0; --q) {
        if (mK >> q & 1)
            continue;
        for (int p = n - 1; p > q; --p) {
            if (mK >> p & 1)
                continue;
            const uint64_t mI = mK | (uint64_t(1) << p) | (uint64_t(1) << q);
            const uint64_t I = string_rank(mI, n, k, binom);
            const int neg = parity_below(mI, q) ^ parity_below(mI & ~(uint64_t(1) << q), p);
            if (j < m2)
                out[K * m2 + j] = I | (uint64_t(p) << 32) | (uint64_t(q) << 40) | (uint64_t(neg) << 48);
            ++j;
        }
    }
}

// 3-hole list of each (k-3)-electron string K: entries (sign, p, q, r, I), p > q > r,
// I = K + p + q + r, sign = <K|a_p a_q a_r|I> (r removed first, then q, then p;
// ci_strings_makers.cc:276-321); ascending r, then q, then p.
__global__ void k_up3(int n, int k, int64_t N3, int m3, const uint64_t* binom, uint64_t* out) {
    const int64_t K = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (K >= N3)
        return;
    const uint64_t mK = string_unrank((uint64_t)K, n, k - 3, binom);
    int j = 0;
    for (int r = 0; r < n; ++r) {
        if (mK >> r & 1)
            continue;
        for (int q = r + 1; q < n; ++q) {
            if (mK >> q & 1)
                continue;
            for (int p = q + 1; p < n; ++p) {
                if (mK >> p & 1)
                    continue;
                const uint64_t mI = mK | (uint64_t(1) << p) | (uint64_t(1) << q) | (uint64_t(1) << r);
                const uint64_t I = string_rank(mI, n, k, binom);
                const uint64_t mr = mI & ~(uint64_t(1) << r), mq = mr & ~(uint64_t(1) << q);
                const int neg = parity_below(mI, r) ^ parity_below(mr, q) ^ parity_below(mq, p);
                if (j < m3)
                    out[K * m3 + j] = I | (uint64_t(p) << 32) | (uint64_t(q) << 40) | (uint64_t(r) << 48) |
                                      (uint64_t(neg) << 56);
                ++j;
            }
        }
    }
}

void SpinStrings::build(int norb, int nel, const uint64_t* d_binom, cudaStream_t st) {
    n = norb;
    k = nel;
    N0 = (int64_t)host_binom(n, k);
    N1 = k >= 1 ? (int64_t)host_binom(n, k - 1) : 0;
    N2 = k >= 2 ? (int64_t)host_binom(n, k - 2) : 0;
    N3 = k >= 3 ? (int64_t)host_binom(n, k - 3) : 0;
    m1 = n - k + 1;
    m2 = (int)host_binom(n - k + 2, 2);
    m3 = (int)host_binom(n - k + 3, 3);
    if (N0 > (int64_t)kAddrMask)
        throw Error(1, "CIStrings: too many strings for 24-bit string addresses");
    const int T = 256;
    str.reserve(N0);
    if (N0)
        k_unrank<<<ceil_div(N0, T), T, 0, st>>>(n, k, N0, d_binom, str.get());
    F2G_LAUNCH("k_unrank");
    if (N1) {
        up1.reserve(N1 * m1);
        k_up1<<<ceil_div(N1, T), T, 0, st>>>(n, k, N1, m1, d_binom, up1.get());
        F2G_LAUNCH("k_up1");
        down1.reserve(N0 * k);
        k_down1<<<ceil_div(N0, T), T, 0, st>>>(n, k, N0, d_binom, down1.get());
        F2G_LAUNCH("k_down1");
    }
}

void SpinStrings::build_up3(const uint64_t* d_binom, cudaStream_t st) {
    if (!N3 || up3.get())
        return;
    up3.reserve(N3 * m3);
    k_up3<<<ceil_div(N3, 256), 256, 0, st>>>(n, k, N3, m3, d_binom, up3.get());
    F2G_LAUNCH("k_up3");
}

void SpinStrings::build_up2(const uint64_t* d_binom, cudaStream_t st) {
    if (!N2 || up2.get())
        return;
    up2.reserve(N2 * m2);
    k_up2<<<ceil_div(N2, 256), 256, 0, st>>>(n, k, N2, m2, d_binom, up2.get());
    F2G_LAUNCH("k_up2");
}

CIStrings::CIStrings(int na_, int nb_, int norb_) : norb(norb_), na(na_), nb(nb_) {
    build_c1();
    blocks.set_c1(na, nb, a.N0, b.N0);
    ndet = nfull;
}

CIStrings::CIStrings(int na_, int nb_, int symmetry, const std::vector<std::vector<int>>& orbital_symmetry,
                     const std::vector<int>& gas_min, const std::vector<int>& gas_max)
    : na(na_), nb(nb_) {
    norb = 0;
    for (const auto& sp : orbital_symmetry)
        norb += (int)sp.size();
    build_c1();
    blocks.build(na, nb, symmetry, orbital_symmetry, gas_min, gas_max);
    ndet = blocks.ndet;
    if (blocks.trivial)
        blocks.set_c1(na, nb, a.N0, b.N0); // the C1 strings themselves, one block
    else
        blocks.build_filter(a.N0, b.N0);
}

void CIStrings::build_c1() {
    if (norb < 0 || norb > kMaxOrb)
        throw Error(2, "CIStrings: the number of active orbitals must be between 0 and 62");
    std::vector<uint64_t> h(kBinomLd * kBinomLd, 0);
    for (int x = 0; x < kBinomLd; ++x)
        for (int y = 0; y < kBinomLd; ++y)
            h[x * kBinomLd + y] = host_binom(x, y);
    binom.reserve(h.size());
    F2G_CUDA(cudaMemcpy(binom.get(), h.data(), h.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
    a.build(norb, na, binom.get(), 0);
    b.build(norb, nb, binom.get(), 0);
    F2G_CUDA(cudaStreamSynchronize(0)); // set-up ran on the legacy stream: wait for it alone
    nfull = a.N0 * b.N0;
}

DetEnum CIStrings::dets() const {
    if (blocked())
        return blocks.view(b.N0);
    DetEnum d;
    d.ndet = nfull;
    d.nblk = nfull > 0 ? 1 : 0;
    d.blk = blocks.dblk.get();
    d.amask = a.str.get();
    d.bmask = b.str.get();
    d.N0b = b.N0;
    return d;
}

} // namespace f2g
