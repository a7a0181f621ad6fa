// Device-resident CI strings and coupling lists (see strings.cu).
#pragma once

#include <vector>

#include "blocks.cuh"
#include "common.cuh"

namespace f2g {

struct SpinStrings {
    int n = 0, k = 0;            // orbitals, electrons of this spin
    int64_t N0 = 0, N1 = 0, N2 = 0, N3 = 0; // strings with k, k-1, k-2, k-3 electrons
    int m1 = 0;                  // entries per 1-hole string: n - k + 1
    int m2 = 0;                  // entries per 2-hole string: C(n - k + 2, 2)
    int m3 = 0;                  // entries per 3-hole string: C(n - k + 3, 3)
    DevBuf<uint64_t> str;        // [N0] occupation masks in address order
    DevBuf<uint32_t> up1;        // [N1][m1] packed (I, p, sign)
    DevBuf<uint32_t> down1;      // [N0][k]  packed (K, p, sign)
    DevBuf<uint64_t> up2;        // [N2][m2] I | p<<32 | q<<40 | negative<<48 (built on demand)
    DevBuf<uint64_t> up3;        // [N3][m3] I | p<<32 | q<<40 | r<<48 | negative<<56, p > q > r (on demand)

    void build(int norb, int nel, const uint64_t* d_binom, cudaStream_t st);
    void build_up2(const uint64_t* d_binom, cudaStream_t st);
    void build_up3(const uint64_t* d_binom, cudaStream_t st);
};

// The strings of an active space. The coupling lists and the sigma kernels always cover the C1
// CAS space of all orbitals (a, b: every string of na / nb electrons, nfull determinants). A
// space with point-group irreps or GAS restrictions is a set of determinant blocks of it
// (`blocks`, ndet determinants in the reference's order); its vectors are embedded into C1
// vectors for the sigma and RDM kernels. A C1 CAS space is one trivial block.
struct CIStrings {
    int norb, na, nb;
    int64_t ndet = 0;  // determinants of the space
    int64_t nfull = 0; // determinants of the C1 CAS space (the sigma kernels' vectors)
    DevBuf<uint64_t> binom; // C(a, b) at [a * kBinomLd + b]
    SpinStrings a, b;
    DetBlocks blocks;
    CIStrings(int na, int nb, int norb);
    // the reference's CIStrings(na, nb, symmetry, orbital_symmetry, gas_min, gas_max)
    CIStrings(int na, int nb, int symmetry, const std::vector<std::vector<int>>& orbital_symmetry,
              const std::vector<int>& gas_min, const std::vector<int>& gas_max);
    bool blocked() const { return !blocks.trivial; }
    DetEnum dets() const; // determinant i of the space -> its strings
    const SpinStrings& spin(int s) const { return s == 0 ? a : b; }
    SpinStrings& spin(int s) { return s == 0 ? a : b; }

  private:
    void build_c1();
};

} // namespace f2g
