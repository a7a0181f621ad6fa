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
    default:
        throw Error(2, "RDM kind must be between 0 and 7");
    }
}

// ---- orbital-pair lists (host) ---------------------------------------------------------------

void build_pair_list(int n, int k, bool force_wide, int seg, PairListHost& L) {
    L = PairListHost{};
    L.n = n;
    L.k = k;
    L.seg = seg;
    L.N0 = (int64_t)host_binom(n, k);
    if (k < 1 || n < 1)
        return;
    L.wide = force_wide || L.N0 > 32766;
    const int64_t N1 = (int64_t)host_binom(n, k - 1);
    std::vector<uint64_t> bt(kBinomLd * kBinomLd);
    for (int a = 0; a < kBinomLd; ++a)
        for (int b = 0; b < kBinomLd; ++b)
            bt[a * kBinomLd + b] = host_binom(a, b);
    // list lengths, segment starts
    std::vector<int64_t> len(n * n), start(n * n), cur(n * n, 0);
    int64_t nseg = 0;
    for (int p = 0; p < n; ++p)
        for (int q = 0; q < n; ++q) {
            len[p * n + q] = (int64_t)(p == q ? host_binom(n - 1, k - 1) : host_binom(n - 2, k - 1));
            start[p * n + q] = nseg;
            nseg += (len[p * n + q] + seg - 1) / seg;
        }
    nseg = (nseg + 31) / 32 * 32;
    L.nseg = nseg;
    L.pair.assign(nseg, 0);
    for (int pq = 0; pq < n * n; ++pq) {
        const int64_t ns = (len[pq] + seg - 1) / seg;
        for (int64_t g = 0; g < ns; ++g)
            L.pair[start[pq] + g] = (uint16_t)pq;
    }
    const uint64_t pad = (uint64_t)L.N0;
    const size_t total = (size_t)nseg * seg;
    if (L.wide)
        L.e64.assign(total, pad | (pad << 24));
    else
        L.e32.assign(total, (uint32_t)(pad | (pad << 15)));
    std::vector<int64_t> addr(n);
    std::vector<int> sgn(n);
    for (int64_t K = 0; K < N1; ++K) {
        const uint64_t mK = string_unrank((uint64_t)K, n, k - 1, bt.data());
        for (int p = 0; p < n; ++p) {
            if (mK >> p & 1)
                continue;
            addr[p] = (int64_t)string_rank(mK | (uint64_t(1) << p), n, k, bt.data());
            sgn[p] = parity_below(mK, p);
        }
        for (int p = 0; p < n; ++p) {
            if (mK >> p & 1)
                continue;
            for (int q = 0; q < n; ++q) {
                if (mK >> q & 1)
                    continue;
                const int pq = p * n + q;
                const int64_t idx = cur[pq]++;
                if (idx >= len[pq])
                    throw Error(1, "RDM pair list: list longer than its binomial count");
                const int64_t g = start[pq] + idx / seg, j = idx % seg;
                const size_t at = (size_t)(((g / 32) * seg + j) * 32 + g % 32);
                const uint64_t neg = (uint64_t)(sgn[p] ^ sgn[q]);
                if (L.wide)
                    L.e64[at] = (uint64_t)addr[p] | ((uint64_t)addr[q] << 24) | (neg << 48);
                else
                    L.e32[at] = (uint32_t)((uint64_t)addr[p] | ((uint64_t)addr[q] << 15) | (neg << 30));
                ++L.nentry;
            }
        }
    }
    for (int pq = 0; pq < n * n; ++pq)
        if (cur[pq] != len[pq])
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
template <int LIST>
__device__ __forceinline__ void hole_entry(const void* list, int64_t at, int64_t& I, int& o, int& neg) {
    if (LIST == 1) {
        const uint32_t e = static_cast<const uint32_t*>(list)[at];
        I = e_addr(e);
        o = e_orb(e);
        neg = e_neg(e);
    } else {
        const uint64_t e = static_cast<const uint64_t*>(list)[at];
        I = (int64_t)(e & 0xffffffffull);
        const int p = (int)((e >> 32) & 0xff), q = (int)((e >> 40) & 0xff);
        o = p * (p - 1) / 2 + q;
        neg = (int)((e >> 48) & 1);
    }
}

struct HoleGramShape {
    int m, npair, TL;
    size_t smem;
};

static HoleGramShape hole_gram_shape(int m, bool sym, size_t limit) {
    HoleGramShape s{};
    s.m = m;
    s.npair = sym ? m * (m + 1) / 2 : m * m;
    int TL = m <= 16 ? 256 : m <= 32 ? 128 : m <= 64 ? 64 : 32;
    for (; TL >= 8; TL /= 2) {
        s.TL = TL;
        s.smem = (size_t)(2 * m * (TL + 1) + s.npair + m) * sizeof(double) + (size_t)m * sizeof(int64_t) +
                 (size_t)m * sizeof(int) + (size_t)s.npair * sizeof(uint16_t);
        if (s.smem <= limit)
            return s;
    }
    throw Error(1, "RDM: hole lists of " + std::to_string(m) + " entries do not fit the shared-memory kernel");
}

template <int LIST>
__global__ void __launch_bounds__(256) k_rdm_hole(int64_t nK, int m, const void* __restrict__ list, int64_t d,
                                                  int64_t ncol, const double* __restrict__ CL,
                                                  const double* __restrict__ CR, int sym, int TL,
                                                  double* __restrict__ out) {
    extern __shared__ double sm[];
    const int ld = TL + 1; // odd stride: the rows of one warp's pairs fall in different banks
    const int npair = sym ? m * (m + 1) / 2 : m * m;
    double* sA = sm;
    double* sB = sA + (size_t)m * ld;
    double* acc = sB + (size_t)m * ld;
    double* sg = acc + npair;
    int64_t* rows = reinterpret_cast<int64_t*>(sg + m);
    int* outo = reinterpret_cast<int*>(rows + m);
    uint16_t* pij = reinterpret_cast<uint16_t*>(outo + m);
    // pair table: i << 8 | j over all (i, j), or over i <= j when bra = ket
    for (int P = threadIdx.x; P < npair; P += blockDim.x) {
        int i = 0, j = 0;
        if (sym) {
            int r = P;
            while (r >= m - i) {
                r -= m - i;
                ++i;
            }
            j = i + r;
        } else {
            i = P / m;
            j = P - i * m;
        }
        pij[P] = (uint16_t)((i << 8) | j);
    }
    for (int64_t K = blockIdx.x; K < nK; K += gridDim.x) {
        __syncthreads(); // the previous hole string is finished with rows, signs and sums
        for (int e = threadIdx.x; e < m; e += blockDim.x) {
            int64_t I;
            int o, neg;
            hole_entry<LIST>(list, K * m + e, I, o, neg);
            rows[e] = I;
            outo[e] = o;
            sg[e] = neg ? -1.0 : 1.0;
        }
        for (int P = threadIdx.x; P < npair; P += blockDim.x)
            acc[P] = 0.0;
        __syncthreads();
        for (int64_t c0 = 0; c0 < ncol; c0 += TL) {
            const int64_t w = min((int64_t)TL, ncol - c0);
            for (int idx = threadIdx.x; idx < m * TL; idx += blockDim.x) {
                const int i = idx / TL, t = idx - i * TL;
                double va = 0.0, vb = 0.0;
                if (t < w) {
                    const int64_t at = rows[i] * ncol + c0 + t;
                    va = CL[at];
                    vb = CR[at];
                }
                sA[i * ld + t] = va;
                sB[i * ld + t] = vb;
            }
            __syncthreads();
            for (int P = threadIdx.x; P < npair; P += blockDim.x) {
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
        for (int P = threadIdx.x; P < npair; P += blockDim.x) {
            const int i = pij[P] >> 8, j = pij[P] & 255;
            const double v = sg[i] * sg[j] * acc[P];
            atomicAdd(out + outo[i] * d + outo[j], v);
            if (sym && i != j)
                atomicAdd(out + outo[j] * d + outo[i], v);
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
    if (m > 255)
        throw Error(1, "RDM: hole lists longer than 255 entries are not supported");
    const size_t limit = std::min<size_t>(smem_optin(), 200 * 1024);
    const HoleGramShape s = hole_gram_shape(m, sym, limit);
    F2G_CUDA(cudaFuncSetAttribute(k_rdm_hole<LIST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem));
    const int per_sm = std::max(1, (int)std::min<size_t>(4, limit / std::max<size_t>(s.smem, 1)));
    const int grid = (int)std::min<int64_t>(nK, (int64_t)device_sms() * per_sm);
    k_rdm_hole<LIST><<<grid, 256, s.smem, st>>>(nK, m, list, d, ncol, CL, CR, sym ? 1 : 0, s.TL, out);
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
template <typename EB, bool SM>
__global__ void __launch_bounds__(1024, 1)
    k_rdm_ab(int n, int64_t nwork, const int32_t* __restrict__ work, const uint64_t* __restrict__ ea,
             const uint16_t* __restrict__ pa, int64_t nsegb, const EB* __restrict__ eb, const uint16_t* __restrict__ pb,
             int64_t NA, int64_t NB, const double* __restrict__ CL, const double* __restrict__ CR,
             double* __restrict__ out) {
    extern __shared__ double sm[];
    double* g = sm;                           // n * n slab
    double* a = g + n * n;                    // bra row (SM)
    double* b = a + (SM ? NB + 1 : 0);        // ket row (SM)
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31;
    const int64_t n2 = (int64_t)n * n;
    for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        const int64_t sa = work[w];
        const int pair_a = pa[sa];
        const int u = pair_a / n, x = pair_a - u * n;
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
                const int vv = (int)(i / n), y = (int)(i - (int64_t)vv * n);
                atomicAdd(out + (((int64_t)u * n + vv) * n + x) * n + y, v);
            }
        }
    }
}

// gamma[u][v][x][y] = gamma[x][y][u][v] for u > x (bra = ket: only u <= x was accumulated)
__global__ void k_rdm_ab_mirror(int n, double* g) {
    const int64_t n2 = (int64_t)n * n, total = n2 * n2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t uv = i / n2, xy = i - uv * n2;
        const int64_t u = uv / n, x = xy / n;
        if (u > x)
            g[i] = g[xy * n2 + uv];
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

static void ensure_pair_lists(SigmaBuilder& sb, RdmScratch& R, cudaStream_t st) {
    if (R.lists_ready)
        return;
    const CIStrings& s = *sb.s;
    PairListHost A, B;
    build_pair_list(s.norb, s.na, true, kRdmSegA, A);
    build_pair_list(s.norb, s.nb, false, kRdmSeg, B);
    R.nsega = A.nseg;
    R.nsegb = B.nseg;
    R.wideb = B.wide;
    std::vector<int32_t> all, sym;
    if (A.nseg) {
        R.ea.reserve(A.e64.size());
        R.pa.reserve(A.pair.size());
        F2G_CUDA(cudaMemcpyAsync(R.ea.get(), A.e64.data(), A.e64.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        F2G_CUDA(cudaMemcpyAsync(R.pa.get(), A.pair.data(), A.pair.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
        // work lists: segments whose first entry is real (padding segments hold none)
        const uint64_t pad = (uint64_t)A.N0;
        for (int64_t g = 0; g < A.nseg; ++g) {
            const uint64_t first = A.e64[(size_t)(((g / 32) * A.seg) * 32 + g % 32)] & 0xffffffull;
            if (first == pad)
                continue;
            all.push_back((int32_t)g);
            const int u = A.pair[g] / s.norb, x = A.pair[g] % s.norb;
            if (u <= x)
                sym.push_back((int32_t)g);
        }
        R.nwork_all = (int64_t)all.size();
        R.nwork_sym = (int64_t)sym.size();
        R.work_all.reserve(all.size());
        R.work_sym.reserve(sym.size());
        if (!all.empty())
            F2G_CUDA(cudaMemcpyAsync(R.work_all.get(), all.data(), all.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        if (!sym.empty())
            F2G_CUDA(cudaMemcpyAsync(R.work_sym.get(), sym.data(), sym.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    if (B.nseg) {
        if (B.wide) {
            R.eb64.reserve(B.e64.size());
            F2G_CUDA(cudaMemcpyAsync(R.eb64.get(), B.e64.data(), B.e64.size() * sizeof(uint64_t),
                                     cudaMemcpyHostToDevice, st));
        } else {
            R.eb32.reserve(B.e32.size());
            F2G_CUDA(cudaMemcpyAsync(R.eb32.get(), B.e32.data(), B.e32.size() * sizeof(uint32_t),
                                     cudaMemcpyHostToDevice, st));
        }
        R.pb.reserve(B.pair.size());
        F2G_CUDA(cudaMemcpyAsync(R.pb.get(), B.pair.data(), B.pair.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
    }
    F2G_CUDA(cudaStreamSynchronize(st)); // the host lists go out of scope
    R.lists_ready = true;
}

template <typename EB, bool SM>
static void launch_ab(int n, RdmScratch& R, const EB* eb, int64_t NA, int64_t NB, const double* CL, const double* CR,
                      bool sym, double* out, cudaStream_t st, size_t smem) {
    const int64_t nwork = sym ? R.nwork_sym : R.nwork_all;
    if (nwork == 0)
        return;
    const int32_t* work = sym ? R.work_sym.get() : R.work_all.get();
    F2G_CUDA(cudaFuncSetAttribute(k_rdm_ab<EB, SM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nwork, device_sms()));
    k_rdm_ab<EB, SM><<<grid, 1024, smem, st>>>(n, nwork, work, R.ea.get(), R.pa.get(), R.nsegb, eb, R.pb.get(), NA,
                                                NB, CL, CR, out);
    F2G_LAUNCH("k_rdm_ab");
}

// out (zeroed by the caller) += mixed-spin 2-RDM
static void rdm_ab(SigmaBuilder& sb, RdmScratch& R, const double* CL, const double* CR, double* out, cudaStream_t st) {
    const CIStrings& s = *sb.s;
    const int n = s.norb;
    if (s.na < 1 || s.nb < 1 || n < 1)
        return;
    ensure_pair_lists(sb, R, st);
    const bool sym = CL == CR;
    const int64_t NA = s.a.N0, NB = s.b.N0;
    const size_t slab = (size_t)n * n * sizeof(double);
    const size_t smem_sm = slab + 2 * (size_t)(NB + 1) * sizeof(double);
    const bool use_sm = smem_sm <= smem_optin();
    const size_t smem = use_sm ? smem_sm : slab;
    if (R.wideb) {
        if (use_sm)
            launch_ab<uint64_t, true>(n, R, R.eb64.get(), NA, NB, CL, CR, sym, out, st, smem);
        else
            launch_ab<uint64_t, false>(n, R, R.eb64.get(), NA, NB, CL, CR, sym, out, st, smem);
    } else {
        if (use_sm)
            launch_ab<uint32_t, true>(n, R, R.eb32.get(), NA, NB, CL, CR, sym, out, st, smem);
        else
            launch_ab<uint32_t, false>(n, R, R.eb32.get(), NA, NB, CL, CR, sym, out, st, smem);
    }
    if (sym) {
        const int64_t total = (int64_t)n * n * n * n;
        k_rdm_ab_mirror<<<elementwise_grid(total), 256, 0, st>>>(n, out);
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
        rdm_ab(sb, R, CL, CR, out, st);
        break;
    case kRdmSf2:
    case kRdmCum2: {
        const int64_t n4 = size, np2 = rdm_size(n, kRdmAA);
        R.t_ab.reserve((size_t)n4);
        F2G_CUDA(cudaMemsetAsync(R.t_ab.get(), 0, (size_t)n4 * sizeof(double), st));
        rdm_ab(sb, R, CL, CR, R.t_ab.get(), st);
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
        if (kind == kRdmCum2) {
            R.t_g1.reserve((size_t)n * n);
            F2G_CUDA(cudaMemsetAsync(R.t_g1.get(), 0, (size_t)n * n * sizeof(double), st));
            rdm_one(sb, R, 0, CL, CR, R.t_g1.get(), st);
            rdm_one(sb, R, 1, CL, CR, R.t_g1.get(), st);
            k_rdm_cumulant<<<elementwise_grid(n4), 256, 0, st>>>(n, R.t_g1.get(), out);
            F2G_LAUNCH("k_rdm_cumulant");
        }
        break;
    }
    default:
        throw Error(2, "RDM kind must be between 0 and 7");
    }
}

} // namespace f2g
