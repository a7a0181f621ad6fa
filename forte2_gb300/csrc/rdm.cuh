// Reduced density matrices between two determinant vectors, on the device (see rdm.cu).
#pragma once

#include <cstdint>
#include <vector>

#include "sigma.cuh"

namespace f2g {

// Kinds, in the order of the C-ABI (f2g_sigma_rdm): the reference's compute_<kind> methods.
enum RdmKind : int {
    kRdmA1 = 0,   // a_1rdm  (n, n)
    kRdmB1 = 1,   // b_1rdm  (n, n)
    kRdmSf1 = 2,  // sf_1rdm (n, n)
    kRdmAA = 3,   // aa_2rdm (P, P), P = n(n-1)/2, pair index p(p-1)/2 + q for p > q
    kRdmBB = 4,   // bb_2rdm (P, P)
    kRdmAB = 5,   // ab_2rdm (n, n, n, n) as [u][v][x][y]: u, x alpha; v, y beta
    kRdmSf2 = 6,  // sf_2rdm (n, n, n, n)
    kRdmCum2 = 7, // sf_2cumulant (n, n, n, n)
    kRdmAAA = 8,  // aaa_3rdm (T, T), T = n(n-1)(n-2)/6, triplet index p(p-1)(p-2)/6 + q(q-1)/2 + r, p > q > r
    kRdmBBB = 9,  // bbb_3rdm (T, T)
    kRdmAAB = 10, // aab_3rdm (P, n, P, n) as [pq][r][st][u]: pq, st alpha pairs; r, u beta
    kRdmABB = 11, // abb_3rdm (n, P, n, P) as [p][qr][s][tu]: p, s alpha; qr, tu beta pairs
    kRdmSf3 = 12, // sf_3rdm (n, n, n, n, n, n)
    kRdmCum3 = 13, // sf_3cumulant (n, n, n, n, n, n)
};

int64_t rdm_size(int norb, int kind);

// Orbital-pair lists of one spin (k electrons in n orbitals), the work lists of the mixed-spin
// 2-RDM: for every ordered orbital pair (p, q) the (k-1)-electron strings K that contain
// neither p nor q, each as an entry (K+p, K+q, s(K,p) s(K,q)) with s(K,p) = (-1)^{#occupied
// below p in K}. A list is cut into segments of `seg` entries (the last one padded with
// entries that point at index N0, a zero sentinel) and the segment count is padded to a
// multiple of 32. Segments are stored interleaved by 32 so that the 32 lanes of a warp, each
// reading its own segment, read 32 consecutive entries:
//   entry j of segment g is at ((g / 32) * seg + j) * 32 + g % 32.
// The beta lists (summed per thread) use kRdmSeg entries per segment; the alpha lists (the
// blocks' work units) use kRdmSegA, small enough to balance the blocks.
// Narrow entries (N0 <= 32766): left | right << 15 | negative << 30 (32 bit);
// wide entries: left | right << 24 | negative << 48 (64 bit).
constexpr int kRdmSeg = 64;
constexpr int kRdmSegA = 16;

// Hole-set pair lists generalise them: with h = 2 the groups are ordered pairs (P, Q) of orbital
// pairs (p > q, pair index p(p-1)/2 + q) and the entries run over the (k-2)-electron strings K
// that contain none of the orbitals of P and Q, sign s(K;P) s(K;Q) with s(K;pq) the 2-hole list
// sign. Group (P, Q) is P * D + Q with D = n (h = 1) or n(n-1)/2 (h = 2).
struct PairListHost {
    int n = 0, k = 0, h = 1, D = 0, seg = kRdmSeg;
    int64_t N0 = 0;      // strings with k electrons (also the padding index)
    int64_t nseg = 0;    // segments, a multiple of 32
    int64_t nentry = 0;  // real (unpadded) entries
    bool wide = false;
    std::vector<uint32_t> e32;
    std::vector<uint64_t> e64;
    std::vector<uint16_t> pair; // per segment: P * D + Q
};
void build_pair_list(int n, int k, bool force_wide, int seg, PairListHost& out);
void build_pair_list(int n, int k, int h, bool force_wide, int seg, PairListHost& out);

// Device pair lists of one mixed-spin contraction: alpha lists with h_a holes, beta lists with
// h_b holes (ab 2-RDM: 1, 1; aab 3-RDM: 2, 1; abb 3-RDM: 1, 2).
struct MixedLists {
    bool ready = false;
    int DA = 0, DB = 0;
    int64_t nsega = 0, nsegb = 0;
    bool wideb = false;
    // alpha segments that hold entries: all of them, and those with P <= Q (bra = ket)
    int64_t nwork_all = 0, nwork_sym = 0;
    DevBuf<int32_t> work_all, work_sym;
    DevBuf<uint64_t> ea;       // alpha pair list, always wide (read once per row pair)
    DevBuf<uint32_t> eb32;     // beta pair list, narrow or wide
    DevBuf<uint64_t> eb64;
    DevBuf<uint16_t> pa, pb;   // segment groups
};

// Device scratch of the RDM builder, owned by a SigmaBuilder (created on first use).
struct RdmScratch {
    MixedLists mixed[3];       // ab (2-RDM), aab, abb (3-RDMs)
    DevBuf<double> tl, tr;     // transposed bra / ket (beta-string rows)
    DevBuf<double> t_ab, t_ss, t_g1; // spin-free assembly temporaries
    DevBuf<double> t_aaa, t_bbb, t_aab, t_abb, t_g2; // spin-free 3-RDM / 3-cumulant temporaries
};

// out (device, rdm_size(n, kind) doubles) <- RDM `kind` between the bra CL and the ket CR
// (device FP64 determinant vectors), ordered on st.
void compute_rdm(SigmaBuilder& sb, int kind, const double* CL, const double* CR, double* out, cudaStream_t st);

} // namespace f2g
