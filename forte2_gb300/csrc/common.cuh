// Shared device helpers for the GB300 determinant-CI library.
//
// Strings are 64-bit occupation masks (bit p = orbital p occupied). A string's address is its
// rank among all strings with the same electron count in std::next_permutation order of the
// boolean sequence (b0, b1, ..., b_{n-1}), i.e. lexicographic with false < true
// (forte2/ci/ci_strings_makers.cc:39-52). Address 0 therefore has the highest orbitals occupied.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>

namespace f2g {

constexpr int kMaxOrb = 62;       // string masks and binomial table limit
constexpr int kBinomLd = 64;      // leading dimension of the binomial table

// Error carried to the C-ABI: code 1 -> RuntimeError, 2 -> ValueError, 3 -> CUDA error,
// 4 -> out of device memory.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation)
            throw Error(4, std::string(what) + ": out of device memory");
        throw Error(3, std::string(what) + ": " + cudaGetErrorString(e));
    }
}
#define F2G_CUDA(x) ::f2g::cuda_check((x), #x)
#define F2G_LAUNCH(what) ::f2g::cuda_check(cudaGetLastError(), what)

// ---- packed coupling-list entries ------------------------------------------------------------
// One 32-bit word per 1-hole entry: bits 0-23 string address, bits 24-29 orbital, bit 31 sign.
constexpr uint32_t kAddrMask = (1u << 24) - 1;
__host__ __device__ inline uint32_t pack1(uint32_t addr, int orb, int negative) {
    return addr | (uint32_t(orb) << 24) | (negative ? 0x80000000u : 0u);
}
__host__ __device__ inline uint32_t e_addr(uint32_t e) { return e & kAddrMask; }
__host__ __device__ inline int e_orb(uint32_t e) { return int((e >> 24) & 63u); }
__host__ __device__ inline int e_neg(uint32_t e) { return int(e >> 31); }

// ---- bit helpers ---------------------------------------------------------------------------
__host__ __device__ inline int popc64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}
// parity of the occupied orbitals strictly below p (the fermionic sign of a_p / a^+_p)
__host__ __device__ inline int parity_below(uint64_t m, int p) {
    return popc64(m & ((uint64_t(1) << p) - 1)) & 1;
}
// parity of the occupied orbitals strictly between n and m
__host__ __device__ inline int parity_between(uint64_t x, int n, int m) {
    if (n > m) {
        int t = n;
        n = m;
        m = t;
    }
    if (m - n <= 1)
        return 0;
    const uint64_t mask = ((uint64_t(1) << m) - 1) & ~((uint64_t(1) << (n + 1)) - 1);
    return popc64(x & mask) & 1;
}

// Lexicographic rank of a k-electron string among the C(n,k) strings of n orbitals.
// binom is the (kBinomLd x kBinomLd) table binom[a*kBinomLd+b] = C(a,b).
__host__ __device__ inline uint64_t string_rank(uint64_t m, int n, int k, const uint64_t* binom) {
    uint64_t r = 0;
    int left = k;
    while (m && left > 0) {
#ifdef __CUDA_ARCH__
        const int i = __ffsll((long long)m) - 1;
#else
        const int i = __builtin_ctzll(m);
#endif
        r += binom[(n - i - 1) * kBinomLd + left];
        --left;
        m &= m - 1;
    }
    return r;
}

__host__ __device__ inline uint64_t string_unrank(uint64_t r, int n, int k, const uint64_t* binom) {
    uint64_t m = 0;
    int left = k;
    for (int i = 0; i < n && left > 0; ++i) {
        const uint64_t c = binom[(n - i - 1) * kBinomLd + left]; // sequences with a 0 at i
        if (r >= c) {
            m |= uint64_t(1) << i;
            r -= c;
            --left;
        }
    }
    return m;
}

// C(n, k) for 0 <= n < kBinomLd by Pascal's rule (no intermediate overflow).
inline uint64_t host_binom(int n, int k) {
    if (k < 0 || n < 0 || k > n || n >= kBinomLd)
        return 0;
    static uint64_t table[kBinomLd][kBinomLd] = {};
    static bool ready = false;
    if (!ready) {
        for (int a = 0; a < kBinomLd; ++a) {
            table[a][0] = 1;
            for (int b = 1; b <= a; ++b)
                table[a][b] = table[a - 1][b - 1] + (b <= a - 1 ? table[a - 1][b] : 0);
        }
        ready = true;
    }
    return table[n][k];
}

inline int ceil_div(long long a, long long b) { return int((a + b - 1) / b); }

} // namespace f2g

namespace f2g {

// Owning device allocation (cudaMalloc / cudaFree), grown on demand.
template <typename T> struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // (re)allocate to at least count elements; contents are not preserved
    T* reserve(size_t count) {
        if (count <= n && p)
            return p;
        release();
        if (count == 0)
            return nullptr;
        F2G_CUDA(cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T)));
        n = count;
        return p;
    }
    T* get() const { return p; }
};

// Scratch of one set-up step: allocated and released in stream order on `st` (cudaMallocAsync /
// cudaFreeAsync), so that releasing it does not wait for work on other streams.
template <typename T> struct TmpBuf {
    T* p = nullptr;
    cudaStream_t st = nullptr;
    TmpBuf(size_t count, cudaStream_t s) : st(s) {
        F2G_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), std::max<size_t>(count, 1) * sizeof(T), st));
    }
    TmpBuf(const TmpBuf&) = delete;
    TmpBuf& operator=(const TmpBuf&) = delete;
    ~TmpBuf() {
        if (p)
            cudaFreeAsync(p, st);
    }
    T* get() const { return p; }
};

} // namespace f2g
