// Reduced density matrices between two determinant vectors (bra CL, ket CR) for a CAS space,
// the reference's CISigmaBuilder::compute_{a,b,sf}_1rdm (forte2/ci/ci_sigma_builder_1rdm.cc:9-84),
// compute_{aa,bb,ab,sf}_2rdm and compute_sf_2cumulant (ci_sigma_builder_2rdm.cc:46-282).
//
// Hole-list Gram kernel (1-RDMs, same-spin 2-RDMs). With K a string with one (two) fewer
// electrons and its hole-list entries (I = K + p (+ q), sign), every element is a sum over K of
// sign * sign' * <bra row I | ket row I'> over pairs of entries of the same K:
//   gamma[p][q]    = sum_K s(K,p) s(K,q) <CL(K+p) | CR(K+q)>            (1-hole list up1)
//   gamma[pq][rs]  = sum_K s(K;p,q) s(K;r,s) <CL(K+p+q) | CR(K+r+s)>    (2-hole list up2)
// which is the reference's vo-list / 2h-list contraction written per hole string. A block takes
// one K at a time, stages the m bra rows and m ket rows of K chunk by chunk in shared memory and
// accumulates the m x m Gram matrix there (half of it when bra = ket), then adds it into the
// output with global atomics. Rows are C rows for alpha and rows of the transposed vectors for
// beta. The FP64 pipe bounds it: 2 m^2 FLOP per hole string and column.
//
// Mixed-spin 2-RDM. gamma[u][v][x][y] = sum_{Ka,Kb} s(Ka,u) s(Kb,v) CL(Ka+u, Kb+v)
// s(Ka,x) s(Kb,y) CR(Ka+x, Kb+y) (the reference's composite-hole GEMM,
// ci_sigma_builder_2rdm.cc:119-201, whose n^2 x n^2 operands are (n-k+1)^2 / n^2 non-zero).
// Grouping the alpha part by the orbital pair (u, x) and the beta part by (v, y) turns it into
//   gamma[u][v][x][y] = sum_{(IaL, IaR, sa) in A(u,x)} sa sum_{(JbL, JbR, sb) in B(v,y)}
//                       sb CL(IaL, JbL) CR(IaR, JbR)
// with the orbital-pair lists A and B (PairListHost). A block takes a segment of A(u,x) (one
// output slab gamma[u][:][x][:]), stages the bra row IaL and the ket row IaR in shared memory,
// and its threads run over the segments of B: each thread sums one segment (one (v, y)) in a
// register and adds it to the slab in shared memory. Every multiply-add of the sparse
// contraction is done once, on the FP64 pipe; no scatter into global memory except one slab per
// segment of A. When bra = ket only u <= x is computed and gamma[x][y][u][v] = gamma[u][v][x][y]
// fills the rest.
#include <algorithm>

#include "rdm.cuh"

namespace f2g {

void transpose_f64(int64_t rows, int64_t cols, const double* in, double* out, cudaStream_t st);

int64_t rdm_size(int n, int kind) {
    const int64_t n2 = (int64_t)n * n, np = n >= 2 ? (int64_t)n * (n - 1) / 2 : 0;
    switch (kind) {
    case kRdmA1:
    case kRdmB1:
    case kRdmSf1:
        return n2;
    case kRdmAA:
    case kRdmBB:
        return np * np;
    case kRdmAB:
    case kRdmSf2:
    case kRdmCum2:
        return n2 * n2;
    case kRdmAAA:
    case kRdmBBB: {
        const int64_t nt = n >= 3 ? (int64_t)n * (n - 1) * (n - 2) / 6 : 0;
        return nt * nt;
    }
    case kRdmAAB:
    case kRdmABB:
        return np * n * np * n;
    case kRdmSf3:
    case kRdmCum3:
        return n2 * n2 * n2;
    default:
        throw Error(2, "RDM kind must be between 0 and 13");
    }
}

// ---- orbital-pair lists (host) ---------------------------------------------------------------

void build_pair_list(int n, int k, bool force_wide, int seg, PairListHost& L) {
    build_pair_list(n, k, 1, force_wide, seg, L);
}

void build_pair_list(int n, int k, int h, bool force_wide, int seg, PairListHost& L) {
    L = PairListHost{};
    L.n = n;
    L.k = k;
    L.h = h;
    L.seg = seg;
    L.N0 = (int64_t)host_binom(n, k);
    if (h != 1 && h != 2)
        throw Error(2, "RDM pair list: 1 or 2 holes");
    L.D = h == 1 ? n : n * (n - 1) / 2;
    if (k < h || n < h)
        return;
    if ((int64_t)L.D * L.D > 65536)
        throw Error(1, "RDM pair list: more than 256 hole sets (at most 23 orbitals for two holes)");
    L.wide = force_wide || L.N0 > 32766;
    const int D = L.D;
    const int64_t NK = (int64_t)host_binom(n, k - h);
    std::vector<uint64_t> bt(kBinomLd * kBinomLd);
    for (int a = 0; a < kBinomLd; ++a)
        for (int b = 0; b < kBinomLd; ++b)
            bt[a * kBinomLd + b] = host_binom(a, b);
    // the orbitals of every hole set
    std::vector<uint64_t> setmask(D);
    for (int P = 0; P < D; ++P) {
        if (h == 1) {
            setmask[P] = uint64_t(1) << P;
        } else {
            int p = 1;
            while ((p + 1) * p / 2 <= P)
                ++p;
            const int q = P - p * (p - 1) / 2;
            setmask[P] = (uint64_t(1) << p) | (uint64_t(1) << q);
        }
    }
    // list lengths (strings of k - h electrons outside both sets), segment starts
    std::vector<int64_t> len((size_t)D * D), start((size_t)D * D), cur((size_t)D * D, 0);
    int64_t nseg = 0;
    for (int P = 0; P < D; ++P)
        for (int Q = 0; Q < D; ++Q) {
            const int used = popc64(setmask[P] | setmask[Q]);
            const size_t g = (size_t)P * D + Q;
            len[g] = (int64_t)host_binom(n - used, k - h);
            start[g] = nseg;
            nseg += (len[g] + seg - 1) / seg;
        }
    nseg = (nseg + 31) / 32 * 32;
    L.nseg = nseg;
    L.pair.assign(nseg, 0);
    for (size_t g = 0; g < (size_t)D * D; ++g) {
        const int64_t ns = (len[g] + seg - 1) / seg;
        for (int64_t j = 0; j < ns; ++j)
            L.pair[start[g] + j] = (uint16_t)g;
    }
    const uint64_t pad = (uint64_t)L.N0;
    const size_t total = (size_t)nseg * seg;
    if (L.wide)
        L.e64.assign(total, pad | (pad << 24));
    else
        L.e32.assign(total, (uint32_t)(pad | (pad << 15)));
    std::vector<int> sets;
    std::vector<int64_t> addr(D);
    std::vector<int> sgn(D);
    for (int64_t K = 0; K < NK; ++K) {
        const uint64_t mK = string_unrank((uint64_t)K, n, k - h, bt.data());
        sets.clear();
        for (int P = 0; P < D; ++P) {
            if (mK & setmask[P])
                continue;
            sets.push_back(P);
            addr[P] = (int64_t)string_rank(mK | setmask[P], n, k, bt.data());
            // <K|a_p|K+p> = parity below p in K; two holes: <K|a_p a_q|K+p+q>, q removed first
            int neg = 0;
            for (uint64_t t = setmask[P]; t; t &= t - 1)
                neg ^= parity_below(mK, __builtin_ctzll(t));
            sgn[P] = neg;
        }
        for (int P : sets)
            for (int Q : sets) {
                const size_t gq = (size_t)P * D + Q;
                const int64_t idx = cur[gq]++;
                if (idx >= len[gq])
                    throw Error(1, "RDM pair list: list longer than its binomial count");
                const int64_t g = start[gq] + idx / seg, j = idx % seg;
                const size_t at = (size_t)(((g / 32) * seg + j) * 32 + g % 32);
                const uint64_t neg = (uint64_t)(sgn[P] ^ sgn[Q]);
                if (L.wide)
                    L.e64[at] = (uint64_t)addr[P] | ((uint64_t)addr[Q] << 24) | (neg << 48);
                else
                    L.e32[at] = (uint32_t)((uint64_t)addr[P] | ((uint64_t)addr[Q] << 15) | (neg << 30));
                ++L.nentry;
            }
    }
    for (size_t g = 0; g < (size_t)D * D; ++g)
        if (cur[g] != len[g])
            throw Error(1, "RDM pair list: list shorter than its binomial count");
}

// ---- entry decoding ----------------------------------------------------------------------------

__device__ __forceinline__ void pair_entry(uint32_t e, int64_t& l, int64_t& r, uint32_t& neg) {
    l = e & 0x7fffu;
    r = (e >> 15) & 0x7fffu;
    neg = (e >> 30) & 1u;
}
__device__ __forceinline__ void pair_entry(uint64_t e, int64_t& l, int64_t& r, uint32_t& neg) {
    l = (int64_t)(e & 0xffffffull);
    r = (int64_t)((e >> 24) & 0xffffffull);
    neg = (uint32_t)((e >> 48) & 1ull);
}
// x with its sign flipped when neg is 1 (an integer operation: the FP64 pipe only does the FMA)
__device__ __forceinline__ double flip(double x, uint32_t neg) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x) ^ ((unsigned long long)neg << 63);
    return __longlong_as_double((long long)bits);
}

// ---- hole-list Gram kernel (1-RDMs, same-spin 2-RDMs) ------------------------------------------

// LIST 1: 1-hole lists up1[K][m] (packed 32-bit: address, orbital, sign); output index = orbital.
// LIST 2: 2-hole lists up2[K][m] (I | p << 32 | q << 40 | negative << 48, p > q); output index
// p(p-1)/2 + q.
// LIST 3: 3-hole lists up3[K][m] (I | p << 32 | q << 40 | r << 48 | negative << 56, p > q > r);
// output index p(p-1)(p-2)/6 + q(q-1)/2 + r.
template <int LIST>
__device__ __forceinline__ void hole_entry(const void* list, int64_t at, int64_t& I, int& o, int& neg) {
    if (LIST == 1) {
        const uint32_t e = static_cast<const uint32_t*>(list)[at];
        I = e_addr(e);
        o = e_orb(e);
        neg = e_neg(e);
    } else if (LIST == 2) {
        const uint64_t e = static_cast<const uint64_t*>(list)[at];
        I = (int64_t)(e & 0xffffffffull);
        const int p = (int)((e >> 32) & 0xff), q = (int)((e >> 40) & 0xff);
        o = p * (p - 1) / 2 + q;
        neg = (int)((e >> 48) & 1);
    } else {
        const uint64_t e = static_cast<const uint64_t*>(list)[at];
        I = (int64_t)(e & 0xffffffffull);
        const int p = (int)((e >> 32) & 0xff), q = (int)((e >> 40) & 0xff), r = (int)((e >> 48) & 0xff);
        o = p * (p - 1) * (p - 2) / 6 + q * (q - 1) / 2 + r;
        neg = (int)((e >> 56) & 1);
    }
}

// Long hole lists are cut into tiles of mt entries; a block takes one (K, tile a, tile b) and
// forms the mt x mt Gram block of those rows (bra = ket: tile a <= tile b, the upper triangle on
// the diagonal tiles).
struct HoleGramShape {
    int m, mt, ntile, TL;
    size_t smem;
};

static size_t hole_gram_smem(int mt, int TL, bool sym) {
    const size_t full = (size_t)mt * mt, diag = sym ? (size_t)mt * (mt + 1) / 2 : 0;
    return (size_t)(2 * mt * (TL + 1) + full + 2 * mt) * sizeof(double) + (size_t)2 * mt * sizeof(int64_t) +
           (size_t)2 * mt * sizeof(int) + (full + diag) * sizeof(uint16_t);
}

static HoleGramShape hole_gram_shape(int m, bool sym, size_t limit) {
    HoleGramShape s{};
    s.m = m;
    for (int mt = std::min(m, 255); mt >= 1; mt = mt > 64 ? mt * 3 / 4 : mt / 2) {
        const int tl_max = mt <= 16 ? 256 : mt <= 32 ? 128 : mt <= 64 ? 64 : 32;
        for (int TL = tl_max; TL >= 16; TL /= 2) {
            const size_t sm = hole_gram_smem(mt, TL, sym);
            if (sm <= limit) {
                s.mt = mt;
                s.ntile = (m + mt - 1) / mt;
                s.TL = TL;
                s.smem = sm;
                return s;
            }
        }
    }
    throw Error(1, "RDM: hole lists of " + std::to_string(m) + " entries do not fit the shared-memory kernel");
}

template <int LIST>
__global__ void __launch_bounds__(256) k_rdm_hole(int64_t nK, int m, int mt, int ntile, const void* __restrict__ list,
                                                  int64_t d, int64_t ncol, const double* __restrict__ CL,
                                                  const double* __restrict__ CR, int sym, int TL,
                                                  double* __restrict__ out) {
    extern __shared__ double sm[];
    const int ld = TL + 1; // odd stride: the rows of one warp's pairs fall in different banks
    const int nfull = mt * mt, ndiag = sym ? mt * (mt + 1) / 2 : 0;
    double* sA = sm;
    double* sB = sA + (size_t)mt * ld;
    double* acc = sB + (size_t)mt * ld;
    double* sg = acc + nfull;                              // [2][mt]: signs of the a and b rows (0: none)
    int64_t* rows = reinterpret_cast<int64_t*>(sg + 2 * mt); // [2][mt]
    int* outo = reinterpret_cast<int*>(rows + 2 * mt);      // [2][mt]
    uint16_t* pfull = reinterpret_cast<uint16_t*>(outo + 2 * mt);
    uint16_t* pdiag = pfull + nfull;
    // pair tables: i << 8 | j over all (i, j), and over i <= j (diagonal tiles when bra = ket)
    for (int P = threadIdx.x; P < nfull; P += blockDim.x)
        pfull[P] = (uint16_t)(((P / mt) << 8) | (P % mt));
    for (int P = threadIdx.x; P < ndiag; P += blockDim.x) {
        int i = 0, r = P;
        while (r >= mt - i) {
            r -= mt - i;
            ++i;
        }
        pdiag[P] = (uint16_t)((i << 8) | (i + r));
    }
    const int ntp = sym ? ntile * (ntile + 1) / 2 : ntile * ntile;
    for (int64_t w = blockIdx.x; w < nK * ntp; w += gridDim.x) {
        const int64_t K = w / ntp;
        int tp = (int)(w - K * ntp), ta = 0, tb = 0;
        if (sym) {
            while (tp >= ntile - ta) {
                tp -= ntile - ta;
                ++ta;
            }
            tb = ta + tp;
        } else {
            ta = tp / ntile;
            tb = tp % ntile;
        }
        const bool diag = sym && ta == tb;
        __syncthreads(); // the previous work item is finished with rows, signs and sums
        for (int e = threadIdx.x; e < 2 * mt; e += blockDim.x) {
            const int side = e / mt, i = (side ? tb : ta) * mt + e % mt;
            int64_t I = -1;
            int o = 0, neg = 0;
            if (i < m)
                hole_entry<LIST>(list, K * m + i, I, o, neg);
            rows[e] = I;
            outo[e] = o;
            sg[e] = I < 0 ? 0.0 : neg ? -1.0 : 1.0;
        }
        const int np = diag ? ndiag : nfull;
        const uint16_t* pij = diag ? pdiag : pfull;
        for (int P = threadIdx.x; P < np; P += blockDim.x)
            acc[P] = 0.0;
        __syncthreads();
        for (int64_t c0 = 0; c0 < ncol; c0 += TL) {
            const int64_t wd = min((int64_t)TL, ncol - c0);
            for (int idx = threadIdx.x; idx < mt * TL; idx += blockDim.x) {
                const int i = idx / TL, t = idx - i * TL;
                double va = 0.0, vb = 0.0;
                if (t < wd) {
                    if (rows[i] >= 0)
                        va = CL[rows[i] * ncol + c0 + t];
                    if (rows[mt + i] >= 0)
                        vb = CR[rows[mt + i] * ncol + c0 + t];
                }
                sA[i * ld + t] = va;
                sB[i * ld + t] = vb;
            }
            __syncthreads();
            for (int P = threadIdx.x; P < np; P += blockDim.x) {
                const int i = pij[P] >> 8, j = pij[P] & 255;
                const double* a = sA + i * ld;
                const double* b = sB + j * ld;
                double t0 = 0.0, t1 = 0.0;
                int t = 0;
                for (; t + 1 < TL; t += 2) {
                    t0 = fma(a[t], b[t], t0);
                    t1 = fma(a[t + 1], b[t + 1], t1);
                }
                for (; t < TL; ++t)
                    t0 = fma(a[t], b[t], t0);
                acc[P] += t0 + t1;
            }
            __syncthreads();
        }
        for (int P = threadIdx.x; P < np; P += blockDim.x) {
            const int i = pij[P] >> 8, j = pij[P] & 255;
            const double sgn = sg[i] * sg[mt + j];
            if (sgn == 0.0)
                continue; // a padding row of a partial tile
            const double v = sgn * acc[P];
            atomicAdd(out + outo[i] * d + outo[mt + j], v);
            if (sym && !(diag && i == j))
                atomicAdd(out + outo[mt + j] * d + outo[i], v);
        }
    }
}

static int device_sms() {
    int dev = 0, sms = 0;
    F2G_CUDA(cudaGetDevice(&dev));
    F2G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return sms;
}

static size_t smem_optin() {
    int dev = 0, v = 0;
    F2G_CUDA(cudaGetDevice(&dev));
    F2G_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    return (size_t)v;
}

// out[o_i * d + o_j] += hole-list Gram contributions of one spin's list (rows of ncol columns)
template <int LIST>
static void launch_hole_gram(int64_t nK, int m, const void* list, int64_t d, int64_t ncol, const double* CL,
                             const double* CR, bool sym, double* out, cudaStream_t st) {
    if (nK == 0 || m == 0 || ncol == 0)
        return;
    const size_t limit = std::min<size_t>(smem_optin(), 200 * 1024);
    const HoleGramShape s = hole_gram_shape(m, sym, limit);
    F2G_CUDA(cudaFuncSetAttribute(k_rdm_hole<LIST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem));
    const int per_sm = std::max(1, (int)std::min<size_t>(4, limit / std::max<size_t>(s.smem, 1)));
    const int64_t ntp = sym ? (int64_t)s.ntile * (s.ntile + 1) / 2 : (int64_t)s.ntile * s.ntile;
    const int grid = (int)std::min<int64_t>(nK * ntp, (int64_t)device_sms() * per_sm);
    k_rdm_hole<LIST><<<grid, 256, s.smem, st>>>(nK, m, s.mt, s.ntile, list, d, ncol, CL, CR, sym ? 1 : 0, s.TL, out);
    F2G_LAUNCH("k_rdm_hole");
}

// ---- mixed-spin 2-RDM kernel ---------------------------------------------------------------------

// Beta-row value at index i of a staged row: in shared memory the row has a zero at index NB
// (the padding index); read from global memory the padding index is tested instead.
template <bool SM>
__device__ __forceinline__ double row_at(const double* r, int64_t i, int64_t NB) {
    if (SM)
        return r[i];
    return i < NB ? __ldg(r + i) : 0.0;
}

// gamma[u][v][x][y] += sum over the alpha segments of the work list given to this block (all
// segments, or those with u <= x when bra = ket; see the file comment). Shared memory: bra row,
// ket row (NB + 1 each when SM) and the n x n slab of the current alpha pair.
// Generalised to hole sets (aab / abb 3-RDMs): alpha groups (A1, A2) of DA x DA, beta groups
// (v, y) of DB x DB, output [A1][v][A2][y] of (DA, DB, DA, DB).
template <typename EB, bool SM>
__global__ void __launch_bounds__(1024, 1)
    k_rdm_ab(int DA, int DB, int64_t nwork, const int32_t* __restrict__ work, const uint64_t* __restrict__ ea,
             const uint16_t* __restrict__ pa, int64_t nsegb, const EB* __restrict__ eb, const uint16_t* __restrict__ pb,
             int64_t NA, int64_t NB, const double* __restrict__ CL, const double* __restrict__ CR,
             double* __restrict__ out) {
    extern __shared__ double sm[];
    const int64_t n2 = (int64_t)DB * DB;
    double* g = sm;                           // DB x DB slab
    double* a = g + n2;                       // bra row (SM)
    double* b = a + (SM ? NB + 1 : 0);        // ket row (SM)
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31;
    for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        const int64_t sa = work[w];
        const int pair_a = pa[sa];
        const int u = pair_a / DA, x = pair_a - u * DA;
        __syncthreads(); // the previous segment's slab has been flushed
        for (int i = tid; i < n2; i += T)
            g[i] = 0.0;
        for (int e = 0; e < kRdmSegA; ++e) {
            int64_t IL, IR;
            uint32_t nega;
            pair_entry(ea[((sa >> 5) * kRdmSegA + e) * 32 + (sa & 31)], IL, IR, nega);
            if (IL >= NA)
                continue; // padding (same entry in every thread)
            const double* rl = CL + IL * NB;
            const double* rr = CR + IR * NB;
            __syncthreads(); // readers of the previous rows are done; slab zeroing is visible
            if (SM) {
                for (int64_t t = tid; t < NB; t += T) {
                    a[t] = rl[t];
                    b[t] = rr[t];
                }
                if (tid == 0) {
                    a[NB] = 0.0;
                    b[NB] = 0.0;
                }
                __syncthreads();
            }
            const double* ra = SM ? a : rl;
            const double* rb = SM ? b : rr;
            const double sgn_a = nega ? -1.0 : 1.0;
            for (int64_t sb = tid; sb < nsegb; sb += T) {
                const EB* pe = eb + (sb >> 5) * (kRdmSeg * 32) + lane;
                double acc0 = 0.0, acc1 = 0.0;
#pragma unroll 8
                for (int j = 0; j < kRdmSeg; j += 2) {
                    int64_t l0, r0, l1, r1;
                    uint32_t n0, n1;
                    pair_entry(pe[j * 32], l0, r0, n0);
                    pair_entry(pe[(j + 1) * 32], l1, r1, n1);
                    acc0 = fma(flip(row_at<SM>(ra, l0, NB), n0), row_at<SM>(rb, r0, NB), acc0);
                    acc1 = fma(flip(row_at<SM>(ra, l1, NB), n1), row_at<SM>(rb, r1, NB), acc1);
                }
                atomicAdd(g + pb[sb], sgn_a * (acc0 + acc1));
            }
        }
        __syncthreads();
        for (int64_t i = tid; i < n2; i += T) {
            const double v = g[i];
            if (v != 0.0) {
                const int vv = (int)(i / DB), y = (int)(i - (int64_t)vv * DB);
                atomicAdd(out + (((int64_t)u * DB + vv) * DA + x) * DB + y, v);
            }
        }
    }
}

// gamma[u][v][x][y] = gamma[x][y][u][v] for u > x (bra = ket: only u <= x was accumulated);
// (DA, DB, DA, DB) layout
__global__ void k_rdm_ab_mirror(int DA, int DB, double* g) {
    const int64_t half = (int64_t)DA * DB, total = half * half;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t uv = i / half, xy = i - uv * half;
        const int64_t u = uv / DB, x = xy / DB;
        if (u > x)
            g[i] = g[xy * half + uv];
    }
}

// sf[p][q][r][s] = ab[p][q][r][s] + ab[q][p][s][r] + the antisymmetric expansion of the packed
// same-spin sum ss = aa + bb (ci_sigma_builder_2rdm.cc:203-250)
__global__ void k_rdm_sf2(int n, const double* __restrict__ ab, const double* __restrict__ ss, double* __restrict__ sf) {
    const int64_t n2 = (int64_t)n * n, total = n2 * n2, np = (int64_t)n * (n - 1) / 2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / (n2 * n)), q = (int)(i / n2 % n), r = (int)(i / n % n), s = (int)(i % n);
        double v = ab[i] + ab[(((int64_t)q * n + p) * n + s) * n + r];
        if (ss && p != q && r != s) {
            const int hi1 = max(p, q), lo1 = min(p, q), hi2 = max(r, s), lo2 = min(r, s);
            const double e = ss[((int64_t)hi1 * (hi1 - 1) / 2 + lo1) * np + (int64_t)hi2 * (hi2 - 1) / 2 + lo2];
            v += ((p > q) == (r > s)) ? e : -e;
        }
        sf[i] = v;
    }
}

// L2[p][q][r][s] = G2[p][q][r][s] - G1[p][r] G1[q][s] + G1[p][s] G1[q][r] / 2 (in place;
// ci_sigma_builder_2rdm.cc:252-278)
__global__ void k_rdm_cumulant(int n, const double* __restrict__ g1, double* __restrict__ l2) {
    const int64_t n2 = (int64_t)n * n, total = n2 * n2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / (n2 * n)), q = (int)(i / n2 % n), r = (int)(i / n % n), s = (int)(i % n);
        l2[i] += -g1[p * n + r] * g1[q * n + s] + 0.5 * g1[p * n + s] * g1[q * n + r];
    }
}

static int elementwise_grid(int64_t total) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 4096));
}

// ---- orchestration ---------------------------------------------------------------------------------

// which: 0 the mixed-spin 2-RDM (alpha and beta 1-hole sets), 1 aab (alpha 2-hole sets, beta
// 1-hole), 2 abb (alpha 1-hole, beta 2-hole)
static MixedLists& ensure_pair_lists(SigmaBuilder& sb, RdmScratch& R, int which, cudaStream_t st) {
    MixedLists& M = R.mixed[which];
    if (M.ready)
        return M;
    const CIStrings& s = *sb.s;
    const int ha = which == 1 ? 2 : 1, hb = which == 2 ? 2 : 1;
    PairListHost A, B;
    build_pair_list(s.norb, s.na, ha, true, kRdmSegA, A);
    build_pair_list(s.norb, s.nb, hb, false, kRdmSeg, B);
    M.DA = A.D;
    M.DB = B.D;
    M.nsega = A.nseg;
    M.nsegb = B.nseg;
    M.wideb = B.wide;
    std::vector<int32_t> all, sym;
    if (A.nseg) {
        M.ea.reserve(A.e64.size());
        M.pa.reserve(A.pair.size());
        F2G_CUDA(cudaMemcpyAsync(M.ea.get(), A.e64.data(), A.e64.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        F2G_CUDA(cudaMemcpyAsync(M.pa.get(), A.pair.data(), A.pair.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
        // work lists: segments whose first entry is real (padding segments hold none)
        const uint64_t pad = (uint64_t)A.N0;
        for (int64_t g = 0; g < A.nseg; ++g) {
            const uint64_t first = A.e64[(size_t)(((g / 32) * A.seg) * 32 + g % 32)] & 0xffffffull;
            if (first == pad)
                continue;
            all.push_back((int32_t)g);
            const int u = A.pair[g] / A.D, x = A.pair[g] % A.D;
            if (u <= x)
                sym.push_back((int32_t)g);
        }
        M.nwork_all = (int64_t)all.size();
        M.nwork_sym = (int64_t)sym.size();
        M.work_all.reserve(all.size());
        M.work_sym.reserve(sym.size());
        if (!all.empty())
            F2G_CUDA(cudaMemcpyAsync(M.work_all.get(), all.data(), all.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        if (!sym.empty())
            F2G_CUDA(cudaMemcpyAsync(M.work_sym.get(), sym.data(), sym.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    if (B.nseg) {
        if (B.wide) {
            M.eb64.reserve(B.e64.size());
            F2G_CUDA(cudaMemcpyAsync(M.eb64.get(), B.e64.data(), B.e64.size() * sizeof(uint64_t),
                                     cudaMemcpyHostToDevice, st));
        } else {
            M.eb32.reserve(B.e32.size());
            F2G_CUDA(cudaMemcpyAsync(M.eb32.get(), B.e32.data(), B.e32.size() * sizeof(uint32_t),
                                     cudaMemcpyHostToDevice, st));
        }
        M.pb.reserve(B.pair.size());
        F2G_CUDA(cudaMemcpyAsync(M.pb.get(), B.pair.data(), B.pair.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
    }
    F2G_CUDA(cudaStreamSynchronize(st)); // the host lists go out of scope
    M.ready = true;
    return M;
}

template <typename EB, bool SM>
static void launch_ab(MixedLists& M, const EB* eb, int64_t NA, int64_t NB, const double* CL, const double* CR,
                      bool sym, double* out, cudaStream_t st, size_t smem) {
    const int64_t nwork = sym ? M.nwork_sym : M.nwork_all;
    if (nwork == 0)
        return;
    const int32_t* work = sym ? M.work_sym.get() : M.work_all.get();
    F2G_CUDA(cudaFuncSetAttribute(k_rdm_ab<EB, SM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nwork, device_sms()));
    k_rdm_ab<EB, SM><<<grid, 1024, smem, st>>>(M.DA, M.DB, nwork, work, M.ea.get(), M.pa.get(), M.nsegb, eb,
                                                M.pb.get(), NA, NB, CL, CR, out);
    F2G_LAUNCH("k_rdm_ab");
}

// out (zeroed by the caller) += mixed-spin 2-RDM (which 0), aab (1) or abb (2) 3-RDM
static void rdm_ab(SigmaBuilder& sb, RdmScratch& R, int which, const double* CL, const double* CR, double* out,
                   cudaStream_t st) {
    const CIStrings& s = *sb.s;
    const int n = s.norb;
    const int ha = which == 1 ? 2 : 1, hb = which == 2 ? 2 : 1;
    if (s.na < ha || s.nb < hb || n < std::max(ha, hb))
        return;
    MixedLists& M = ensure_pair_lists(sb, R, which, st);
    const bool sym = CL == CR;
    const int64_t NA = s.a.N0, NB = s.b.N0;
    const size_t slab = (size_t)M.DB * M.DB * sizeof(double);
    const size_t smem_sm = slab + 2 * (size_t)(NB + 1) * sizeof(double);
    const bool use_sm = smem_sm <= smem_optin();
    const size_t smem = use_sm ? smem_sm : slab;
    if (smem > smem_optin())
        throw Error(1, "RDM: the mixed-spin slab does not fit in shared memory");
    if (M.wideb) {
        if (use_sm)
            launch_ab<uint64_t, true>(M, M.eb64.get(), NA, NB, CL, CR, sym, out, st, smem);
        else
            launch_ab<uint64_t, false>(M, M.eb64.get(), NA, NB, CL, CR, sym, out, st, smem);
    } else {
        if (use_sm)
            launch_ab<uint32_t, true>(M, M.eb32.get(), NA, NB, CL, CR, sym, out, st, smem);
        else
            launch_ab<uint32_t, false>(M, M.eb32.get(), NA, NB, CL, CR, sym, out, st, smem);
    }
    if (sym) {
        const int64_t total = (int64_t)M.DA * M.DB * M.DA * M.DB;
        k_rdm_ab_mirror<<<elementwise_grid(total), 256, 0, st>>>(M.DA, M.DB, out);
        F2G_LAUNCH("k_rdm_ab_mirror");
    }
}

// rows of one spin: the vectors themselves (alpha) or their transposes (beta)
static void spin_rows(SigmaBuilder& sb, RdmScratch& R, int spin, const double* CL, const double* CR, cudaStream_t st,
                      const double*& L, const double*& Rr, int64_t& ncol) {
    const CIStrings& s = *sb.s;
    const int64_t NA = s.a.N0, NB = s.b.N0;
    if (spin == 0) {
        L = CL;
        Rr = CR;
        ncol = NB;
        return;
    }
    R.tl.reserve((size_t)(NA * NB));
    transpose_f64(NA, NB, CL, R.tl.get(), st);
    L = R.tl.get();
    if (CR == CL) {
        Rr = L;
    } else {
        R.tr.reserve((size_t)(NA * NB));
        transpose_f64(NA, NB, CR, R.tr.get(), st);
        Rr = R.tr.get();
    }
    ncol = NA;
}

// out (zeroed) += 1-RDM of one spin
static void rdm_one(SigmaBuilder& sb, RdmScratch& R, int spin, const double* CL, const double* CR, double* out,
                    cudaStream_t st) {
    const SpinStrings& ss = sb.s->spin(spin);
    if (ss.k < 1 || ss.N1 == 0 || sb.n < 1)
        return;
    const double *L, *Rr;
    int64_t ncol;
    spin_rows(sb, R, spin, CL, CR, st, L, Rr, ncol);
    launch_hole_gram<1>(ss.N1, ss.m1, ss.up1.get(), sb.n, ncol, L, Rr, L == Rr, out, st);
}

// out (zeroed) += packed same-spin 2-RDM of one spin
static void rdm_same(SigmaBuilder& sb, RdmScratch& R, int spin, const double* CL, const double* CR, double* out,
                     cudaStream_t st) {
    SpinStrings& ss = sb.s->spin(spin);
    if (ss.k < 2 || ss.N2 == 0 || sb.n < 2)
        return;
    ss.build_up2(sb.s->binom.get(), st);
    const double *L, *Rr;
    int64_t ncol;
    spin_rows(sb, R, spin, CL, CR, st, L, Rr, ncol);
    launch_hole_gram<2>(ss.N2, ss.m2, ss.up2.get(), (int64_t)sb.n * (sb.n - 1) / 2, ncol, L, Rr, L == Rr, out, st);
}

// out (zeroed) += packed same-spin 3-RDM of one spin, [pqr][stu] (ci_sigma_builder_3rdm.cc:84-162)
static void rdm_same3(SigmaBuilder& sb, RdmScratch& R, int spin, const double* CL, const double* CR, double* out,
                      cudaStream_t st) {
    SpinStrings& ss = sb.s->spin(spin);
    if (ss.k < 3 || ss.N3 == 0 || sb.n < 3)
        return;
    ss.build_up3(sb.s->binom.get(), st);
    const double *L, *Rr;
    int64_t ncol;
    spin_rows(sb, R, spin, CL, CR, st, L, Rr, ncol);
    launch_hole_gram<3>(ss.N3, ss.m3, ss.up3.get(), (int64_t)sb.n * (sb.n - 1) * (sb.n - 2) / 6, ncol, L, Rr,
                        L == Rr, out, st);
}

__device__ __forceinline__ int pidx(int a, int b) { return a > b ? a * (a - 1) / 2 + b : b * (b - 1) / 2 + a; }
__device__ __forceinline__ double sgn2(int a, int b) { return a > b ? 1.0 : -1.0; }
// sign of the permutation that sorts (a, b, c) into descending order, and the triplet index
__device__ __forceinline__ double sgn3(int a, int b, int c) {
    const int inv = (a < b) + (a < c) + (b < c);
    return (inv & 1) ? -1.0 : 1.0;
}
__device__ __forceinline__ int tidx(int a, int b, int c) {
    int x = max(a, max(b, c)), z = min(a, min(b, c)), y = a + b + c - x - z;
    return x * (x - 1) * (x - 2) / 6 + y * (y - 1) / 2 + z;
}

// Spin-free 3-RDM, one output element per thread (owner computes, no atomics): the aab, abb and
// aaa + bbb elements that the reference's scatter (ci_sigma_builder_3rdm.cc:320-497) adds into
// element (o1..o6), gathered with the same signs:
//   aab[(o1o2)][o3][(o4o5)][o6], aab[(o1o3)][o2][(o4o6)][o5], aab[(o2o3)][o1][(o5o6)][o4],
//   abb[o1][(o2o3)][o4][(o5o6)], abb[o2][(o1o3)][o5][(o4o6)], abb[o3][(o1o2)][o6][(o4o5)],
// each times the signs of the two pairs (+ when the first index is the larger), and
// sss[(o1o2o3)][(o4o5o6)] times the signs of the two permutations into descending order.
__global__ void k_rdm_sf3(int n, const double* __restrict__ aab, const double* __restrict__ abb,
                          const double* __restrict__ sss, double* __restrict__ out) {
    const int64_t n2 = (int64_t)n * n, n3 = n2 * n, total = n3 * n3;
    const int64_t np = (int64_t)n * (n - 1) / 2, nt = n >= 3 ? (int64_t)n * (n - 1) * (n - 2) / 6 : 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int o1 = (int)(i / (n3 * n2)), o2 = (int)(i / (n3 * n) % n), o3 = (int)(i / n3 % n);
        const int o4 = (int)(i / n2 % n), o5 = (int)(i / n % n), o6 = (int)(i % n);
        auto ab = [&](int P, int r, int S, int u) { return aab[(((int64_t)P * n + r) * np + S) * n + u]; };
        auto bb = [&](int p, int Q, int s2, int T) { return abb[(((int64_t)p * np + Q) * n + s2) * np + T]; };
        double v = 0.0;
        if (aab) {
            if (o1 != o2 && o4 != o5)
                v += sgn2(o1, o2) * sgn2(o4, o5) * ab(pidx(o1, o2), o3, pidx(o4, o5), o6);
            if (o1 != o3 && o4 != o6)
                v += sgn2(o1, o3) * sgn2(o4, o6) * ab(pidx(o1, o3), o2, pidx(o4, o6), o5);
            if (o2 != o3 && o5 != o6)
                v += sgn2(o2, o3) * sgn2(o5, o6) * ab(pidx(o2, o3), o1, pidx(o5, o6), o4);
        }
        if (abb) {
            if (o2 != o3 && o5 != o6)
                v += sgn2(o2, o3) * sgn2(o5, o6) * bb(o1, pidx(o2, o3), o4, pidx(o5, o6));
            if (o1 != o3 && o4 != o6)
                v += sgn2(o1, o3) * sgn2(o4, o6) * bb(o2, pidx(o1, o3), o5, pidx(o4, o6));
            if (o1 != o2 && o4 != o5)
                v += sgn2(o1, o2) * sgn2(o4, o5) * bb(o3, pidx(o1, o2), o6, pidx(o4, o5));
        }
        if (sss && o1 != o2 && o1 != o3 && o2 != o3 && o4 != o5 && o4 != o6 && o5 != o6)
            v += sgn3(o1, o2, o3) * sgn3(o4, o5, o6) * sss[(int64_t)tidx(o1, o2, o3) * nt + tidx(o4, o5, o6)];
        out[i] = v;
    }
}

// 3-cumulant in place over the spin-free 3-RDM (ci_sigma_builder_3rdm.cc:499-541)
__global__ void k_rdm_cum3(int n, const double* __restrict__ g1, const double* __restrict__ g2,
                           double* __restrict__ l3) {
    const int64_t n2 = (int64_t)n * n, n3 = n2 * n, total = n3 * n3;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / (n3 * n2)), q = (int)(i / (n3 * n) % n), r = (int)(i / n3 % n);
        const int s = (int)(i / n2 % n), t = (int)(i / n % n), u = (int)(i % n);
        auto G1 = [&](int a, int b) { return g1[a * n + b]; };
        auto G2 = [&](int a, int b, int c, int d) { return g2[(((int64_t)a * n + b) * n + c) * n + d]; };
        l3[i] += -G1(p, s) * G2(q, r, t, u) - G1(q, t) * G2(p, r, s, u) - G1(r, u) * G2(p, q, s, t) +
                 0.5 * G1(p, t) * G2(q, r, s, u) + 0.5 * G1(p, u) * G2(q, r, t, s) + 0.5 * G1(q, s) * G2(p, r, t, u) +
                 0.5 * G1(q, u) * G2(p, r, s, t) + 0.5 * G1(r, s) * G2(p, q, u, t) + 0.5 * G1(r, t) * G2(p, q, s, u) +
                 2.0 * G1(p, s) * G1(q, t) * G1(r, u) - G1(p, s) * G1(q, u) * G1(r, t) -
                 G1(p, u) * G1(q, t) * G1(r, s) - G1(p, t) * G1(q, s) * G1(r, u) +
                 0.5 * G1(p, t) * G1(q, u) * G1(r, s) + 0.5 * G1(p, u) * G1(q, s) * G1(r, t);
    }
}

// spin-free 2-RDM into out (n^4, overwritten)
static void rdm_sf2(SigmaBuilder& sb, RdmScratch& R, const double* CL, const double* CR, double* out,
                    cudaStream_t st) {
    const int n = sb.n;
    const int64_t n4 = rdm_size(n, kRdmSf2), np2 = rdm_size(n, kRdmAA);
    R.t_ab.reserve((size_t)n4);
    F2G_CUDA(cudaMemsetAsync(R.t_ab.get(), 0, (size_t)n4 * sizeof(double), st));
    rdm_ab(sb, R, 0, CL, CR, R.t_ab.get(), st);
    const double* ss = nullptr;
    if (np2 > 0) {
        R.t_ss.reserve((size_t)np2);
        F2G_CUDA(cudaMemsetAsync(R.t_ss.get(), 0, (size_t)np2 * sizeof(double), st));
        rdm_same(sb, R, 0, CL, CR, R.t_ss.get(), st);
        rdm_same(sb, R, 1, CL, CR, R.t_ss.get(), st);
        ss = R.t_ss.get();
    }
    k_rdm_sf2<<<elementwise_grid(n4), 256, 0, st>>>(n, R.t_ab.get(), ss, out);
    F2G_LAUNCH("k_rdm_sf2");
}

// spin-free 1-RDM into out (n^2, overwritten)
static void rdm_sf1(SigmaBuilder& sb, RdmScratch& R, const double* CL, const double* CR, double* out,
                    cudaStream_t st) {
    F2G_CUDA(cudaMemsetAsync(out, 0, (size_t)sb.n * sb.n * sizeof(double), st));
    rdm_one(sb, R, 0, CL, CR, out, st);
    rdm_one(sb, R, 1, CL, CR, out, st);
}

void compute_rdm(SigmaBuilder& sb, int kind, const double* CL, const double* CR, double* out, cudaStream_t st) {
    const int n = sb.n;
    const int64_t size = rdm_size(n, kind);
    if (!sb.rdm)
        sb.rdm = std::make_shared<RdmScratch>();
    RdmScratch& R = *sb.rdm;
    if (size == 0)
        return;
    if (!CL || !CR || !out)
        throw Error(2, "RDM: NULL vector or output");
    if (sb.s->blocked()) {
        // a blocked space's vectors embedded into C1 vectors: the RDMs are those of the embedding
        const DetEnum de = sb.s->dets();
        const int64_t nf = sb.s->nfull;
        double* xl = sb.xC.reserve(nf);
        blocks_embed<double>(de, nf, CL, xl, 1, st);
        const double* xr = xl;
        if (CR != CL) {
            double* t = sb.xS.reserve(nf);
            blocks_embed<double>(de, nf, CR, t, 1, st);
            xr = t;
        }
        CL = xl;
        CR = xr;
    }
    F2G_CUDA(cudaMemsetAsync(out, 0, (size_t)size * sizeof(double), st));
    switch (kind) {
    case kRdmA1:
        rdm_one(sb, R, 0, CL, CR, out, st);
        break;
    case kRdmB1:
        rdm_one(sb, R, 1, CL, CR, out, st);
        break;
    case kRdmSf1:
        rdm_one(sb, R, 0, CL, CR, out, st);
        rdm_one(sb, R, 1, CL, CR, out, st);
        break;
    case kRdmAA:
        rdm_same(sb, R, 0, CL, CR, out, st);
        break;
    case kRdmBB:
        rdm_same(sb, R, 1, CL, CR, out, st);
        break;
    case kRdmAB:
        rdm_ab(sb, R, 0, CL, CR, out, st);
        break;
    case kRdmSf2:
    case kRdmCum2: {
        rdm_sf2(sb, R, CL, CR, out, st);
        if (kind == kRdmCum2) {
            R.t_g1.reserve((size_t)n * n);
            rdm_sf1(sb, R, CL, CR, R.t_g1.get(), st);
            k_rdm_cumulant<<<elementwise_grid(size), 256, 0, st>>>(n, R.t_g1.get(), out);
            F2G_LAUNCH("k_rdm_cumulant");
        }
        break;
    }
    case kRdmAAA:
        rdm_same3(sb, R, 0, CL, CR, out, st);
        break;
    case kRdmBBB:
        rdm_same3(sb, R, 1, CL, CR, out, st);
        break;
    case kRdmAAB:
        rdm_ab(sb, R, 1, CL, CR, out, st);
        break;
    case kRdmABB:
        rdm_ab(sb, R, 2, CL, CR, out, st);
        break;
    case kRdmSf3:
    case kRdmCum3: {
        // spin-resolved parts, then the owner-computes assembly
        const int64_t n3p = rdm_size(n, kRdmAAB), nss = rdm_size(n, kRdmAAA);
        const double *aab = nullptr, *abb = nullptr, *sss = nullptr;
        if (n3p > 0) {
            R.t_aab.reserve((size_t)n3p);
            R.t_abb.reserve((size_t)n3p);
            F2G_CUDA(cudaMemsetAsync(R.t_aab.get(), 0, (size_t)n3p * sizeof(double), st));
            F2G_CUDA(cudaMemsetAsync(R.t_abb.get(), 0, (size_t)n3p * sizeof(double), st));
            rdm_ab(sb, R, 1, CL, CR, R.t_aab.get(), st);
            rdm_ab(sb, R, 2, CL, CR, R.t_abb.get(), st);
            aab = R.t_aab.get();
            abb = R.t_abb.get();
        }
        if (nss > 0) {
            R.t_aaa.reserve((size_t)nss);
            F2G_CUDA(cudaMemsetAsync(R.t_aaa.get(), 0, (size_t)nss * sizeof(double), st));
            rdm_same3(sb, R, 0, CL, CR, R.t_aaa.get(), st);
            rdm_same3(sb, R, 1, CL, CR, R.t_aaa.get(), st);
            sss = R.t_aaa.get();
        }
        k_rdm_sf3<<<elementwise_grid(size), 256, 0, st>>>(n, aab, abb, sss, out);
        F2G_LAUNCH("k_rdm_sf3");
        if (kind == kRdmCum3) {
            R.t_g1.reserve((size_t)n * n);
            R.t_g2.reserve((size_t)rdm_size(n, kRdmSf2));
            rdm_sf1(sb, R, CL, CR, R.t_g1.get(), st);
            rdm_sf2(sb, R, CL, CR, R.t_g2.get(), st);
            k_rdm_cum3<<<elementwise_grid(size), 256, 0, st>>>(n, R.t_g1.get(), R.t_g2.get(), out);
            F2G_LAUNCH("k_rdm_cum3");
        }
        break;
    }
    default:
        throw Error(2, "RDM kind must be between 0 and 13");
    }
}

} // namespace f2g
