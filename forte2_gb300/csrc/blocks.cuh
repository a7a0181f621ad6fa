// Determinant blocks of a general CI space: point-group irreps and GAS occupations (see blocks.cu).
#pragma once

#include <array>
#include <utility>
#include <vector>

#include "common.cuh"

namespace f2g {

constexpr int kMaxGasSpaces = 6; // the reference's occupation patterns hold six spaces

// Device view of the determinants of a blocked space: determinant i of the space (the
// reference's address, blocks back to back, alpha-major inside a block) -> its alpha and beta
// strings. A C1 CAS space is one block over all strings.
struct DetEnum {
    int64_t ndet = 0;
    int nblk = 0;
    const int64_t* blk = nullptr;    // [nblk][kBlkCols]: offset, nIb, alpha start, beta start
    const uint64_t* amask = nullptr; // class strings of each spin in (class, address) order
    const uint64_t* bmask = nullptr;
    const uint32_t* arank = nullptr; // their C1 addresses (for the embedding)
    const uint32_t* brank = nullptr;
    int64_t N0b = 0;                 // C1 beta strings

    static constexpr int kBlkCols = 4;
    __device__ __forceinline__ int block_of(int64_t i) const {
        // largest block with offset <= i (empty blocks share their successor's offset)
        int lo = 0, hi = nblk;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (blk[mid * kBlkCols] <= i)
                lo = mid;
            else
                hi = mid;
        }
        return lo;
    }
    // alpha and beta positions (indices into amask/bmask) of determinant i
    __device__ __forceinline__ void pos(int64_t i, int64_t& ja, int64_t& jb) const {
        const int64_t* b = blk + block_of(i) * kBlkCols;
        const int64_t r = i - b[0], nIb = b[1];
        ja = b[2] + r / nIb;
        jb = b[3] + r % nIb;
    }
    __device__ __forceinline__ void at(int64_t i, uint64_t& a, uint64_t& b) const {
        int64_t ja, jb;
        pos(i, ja, jb);
        a = amask[ja];
        b = bmask[jb];
    }
    // C1 address (alpha-major over all strings of the active space) of determinant i
    __device__ __forceinline__ int64_t c1(int64_t i) const {
        int64_t ja, jb;
        pos(i, ja, jb);
        return (int64_t)arank[ja] * N0b + brank[jb];
    }
};

// Host description and device tables of the blocks. Built by build(); `trivial` when the space is
// the C1 CAS space in its own order (one block, identity embedding).
struct DetBlocks {
    using Occ = std::array<int, kMaxGasSpaces>;
    bool trivial = true;
    int symmetry = 0, nirrep = 1, nspace = 1;
    std::vector<int> orbsym;                     // irrep of every active orbital
    std::vector<int> gas_size;                   // orbitals per GAS space (as given)
    std::vector<Occ> aocc, bocc;                 // allowed alpha / beta occupation patterns
    std::vector<std::pair<int, int>> occ_pairs;  // allowed (alpha pattern, beta pattern) pairs
    std::vector<uint64_t> str[2];                // class strings per spin, (class, address) order
    std::vector<int64_t> cls_off[2];             // class offsets into str (nclass + 1)
    std::vector<int64_t> hblk;                   // [nblk][6]: alpha class, beta class, size, offset, nIa, nIb
    int64_t ndet = 0;
    DevBuf<int64_t> dblk;                        // [nblk][DetEnum::kBlkCols]
    DevBuf<uint64_t> dstr[2];
    DevBuf<uint32_t> drank[2];

    int nblk() const { return (int)(hblk.size() / 6); }
    int nclass(int spin) const { return (int)cls_off[spin].size() - 1; }
    std::vector<uint32_t> rank[2];               // C1 addresses of the class strings
    // Enumerates the space on the host (ci_strings.cc:34-184 with ci_occupation.cc:35-142,
    // ci_string_class.cc:7-66, ci_strings_makers.cc:13-73); no device call.
    void enumerate(int na, int nb, int symmetry, const std::vector<std::vector<int>>& orbital_symmetry,
                   const std::vector<int>& gas_min, const std::vector<int>& gas_max);
    // enumerate() and the device tables
    void build(int na, int nb, int symmetry, const std::vector<std::vector<int>>& orbital_symmetry,
               const std::vector<int>& gas_min, const std::vector<int>& gas_max);
    DetEnum view(int64_t N0b_c1) const;
    // the C1 CAS space as one trivial block over the C1 strings (host metadata filled in when
    // build() did not run)
    void set_c1(int na, int nb, int64_t N0a, int64_t N0b);

    // Same-spin filter of a blocked space, per spin: the class of every C1 string (-1: in no
    // class) and compat[c][c'] = 1 when some class of the other spin pairs with both c and c' in a
    // non-empty block. A same-spin coupling <J|H|I> can reach the space only if compat[cls J][cls I].
    DevBuf<int16_t> dcls[2];
    DevBuf<int32_t> dpos[2]; // position of every C1 string inside its class (-1: in no class)
    DevBuf<uint8_t> dcompat[2];
    void build_filter(int64_t N0a, int64_t N0b);
};

// vectors of the space <-> C1-sized vectors (zero outside the space); nvec vectors back to back
template <typename T>
void blocks_embed(const DetEnum& de, int64_t nfull, const T* sub, T* full, int nvec, cudaStream_t st);
template <typename T>
void blocks_extract(const DetEnum& de, int64_t nfull, const T* full, T* sub, int nvec, cudaStream_t st,
                    bool add = false);

} // namespace f2g
