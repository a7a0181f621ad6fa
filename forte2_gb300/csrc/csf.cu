// Configuration-state-function (CSF) spin adaptation on the device.
//
// Content follows the reference's CISpinAdapter (forte2/determinant/ci_spin_adapter.cc):
//   * configurations (doubly / singly occupied orbital sets) with at least 2S open shells, in the
//     order in which they first appear over the determinants in address order (the insertion
//     order of its ankerl::unordered_dense set, :151-160);
//   * for N open shells, the genealogical spin couplings (make_spin_couplings, :237-266), the
//     determinant spin patterns (make_determinant_occupations, :268-288) and their
//     Clebsch-Gordan overlaps (:23-51);
//   * each determinant's coefficient is overlap x the sign of creating its open shells from
//     the highest orbital down on top of the closed shells (conf_to_csfs, :200-235).
//
// GPU layout. Instead of the reference's (det index, coefficient) list per CSF (billions of
// entries at CAS(16,16)), every determinant of a configuration is stored once in a permutation
// `perm` grouped by configuration and ordered by spin pattern, with its sign in bit 31, and the
// overlaps live in one small dense table per open-shell count N. Both transforms are owner-
// computes: csf -> det writes each determinant once, det -> csf writes each CSF once.
//
// Configuration order is found without a hash map: every determinant computes the canonical
// rank of its configuration, an atomicMin keeps the first determinant address per
// configuration, and an exclusive scan over "is first" flags in address order numbers the
// configurations in insertion order.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>

#include "csf.cuh"

namespace f2g {

namespace {

// ---- host tables -----------------------------------------------------------------------------
double cg(double twoS, double twoM, int dtwoS, double dtwoM) {
    if (dtwoS == 1)
        return std::sqrt(0.5 * (twoS + dtwoM * twoM) / twoS);
    if (dtwoS == -1)
        return -dtwoM * std::sqrt(0.5 * (twoS + 2. - dtwoM * twoM) / (twoS + 2.));
    return 0.0;
}

double overlap(int N, const std::vector<int>& coupling, const std::vector<int>& occ) {
    double o = 1.0;
    int pi = 0, qi = 0;
    for (int i = 0; i < N; ++i) {
        const int dS = 1 - 2 * coupling[i];
        const int dM = 1 - 2 * occ[i];
        pi += dS;
        qi += dM;
        if (std::abs(qi) > pi)
            return 0.0;
        o *= cg(pi, qi, dS, dM);
    }
    return o;
}

std::vector<std::vector<int>> couplings(int N, int twoS) {
    if (N == 0)
        return {std::vector<int>()};
    std::vector<std::vector<int>> out;
    const int nup = (N + twoS) / 2;
    std::vector<int> c(N, 1);
    for (int i = 0; i < nup && i < N; ++i)
        c[i] = 0;
    do {
        bool valid = true;
        for (int i = 0, p = 0; i < N; ++i) {
            p += 1 - 2 * c[i];
            if (p < 0)
                valid = false;
        }
        if (valid)
            out.push_back(c);
    } while (std::next_permutation(c.begin() + 1, c.end()));
    return out;
}

std::vector<std::vector<int>> patterns(int N, int twoMs) {
    if (N == 0)
        return {std::vector<int>()};
    std::vector<std::vector<int>> out;
    const int nup = (N + twoMs) / 2;
    std::vector<int> o(N, 1);
    for (int i = 0; i < nup && i < N; ++i)
        o[i] = 0;
    do {
        out.push_back(o);
    } while (std::next_permutation(o.begin(), o.end()));
    return out;
}

} // namespace

// ---- device helpers --------------------------------------------------------------------------

struct ConfSpace {
    int n, nel;
    const int64_t* base; // [n+1] canonical offset per number of doubly occupied orbitals
    const uint64_t* binom;
};

__device__ inline uint64_t conf_rank(uint64_t d, uint64_t s, const ConfSpace& cs) {
    const int nd = popc64(d), ns = popc64(s);
    const uint64_t rd = string_rank(d, cs.n, nd, cs.binom);
    uint64_t comp = 0;
    int pos = 0;
    for (int p = 0; p < cs.n; ++p) {
        if (d >> p & 1)
            continue;
        if (s >> p & 1)
            comp |= uint64_t(1) << pos;
        ++pos;
    }
    const uint64_t rs = string_rank(comp, cs.n - nd, ns, cs.binom);
    return (uint64_t)cs.base[nd] + rd * cs.binom[(cs.n - nd) * kBinomLd + ns] + rs;
}

// spin pattern index (beta open shells among the open shells, lexicographic) and creation sign
__device__ inline void pattern_and_sign(uint64_t a, uint64_t b, int twoMs, const uint64_t* binom, uint64_t& j,
                                        int& neg) {
    const uint64_t d = a & b, s = a ^ b;
    const int N = popc64(s);
    uint64_t occ = 0;
    int k = 0;
    uint64_t t = s;
    while (t) {
        const int p = __ffsll((long long)t) - 1;
        if (b >> p & 1)
            occ |= uint64_t(1) << k;
        ++k;
        t &= t - 1;
    }
    j = string_rank(occ, N, (N - twoMs) / 2, binom);
    // create open shells from the highest orbital down on top of the closed shells
    uint64_t acur = d;
    int ng = 0;
    t = s;
    while (t) {
        const int p = 63 - __clzll((long long)t);
        const int below = parity_below(d, p);
        if (b >> p & 1) {
            ng ^= (popc64(acur) & 1) ^ below;
        } else {
            ng ^= below;
            acur |= uint64_t(1) << p;
        }
        t &= ~(uint64_t(1) << p);
    }
    neg = ng;
}

// Determinant i of the space comes from the enumerator (blocks of a point-group / GAS space, or
// the C1 strings); configurations are ranked over all configurations of the active orbitals.
__global__ void k_conf_first(DetEnum de, int twoS, ConfSpace cs, uint32_t* first) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= de.ndet)
        return;
    uint64_t a, b;
    de.at(i, a, b);
    const uint64_t d = a & b, s = a ^ b;
    if (popc64(s) < twoS)
        return;
    atomicMin(first + conf_rank(d, s, cs), (uint32_t)i);
}

__global__ void k_conf_flag(DetEnum de, int twoS, ConfSpace cs, const uint32_t* first, uint32_t* flag) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= de.ndet)
        return;
    uint64_t a, b;
    de.at(i, a, b);
    const uint64_t d = a & b, s = a ^ b;
    uint32_t f = 0;
    if (popc64(s) >= twoS)
        f = first[conf_rank(d, s, cs)] == (uint32_t)i ? 1u : 0u;
    flag[i] = f;
}

__global__ void k_conf_fill(DetEnum de, const uint32_t* flag, const uint32_t* cidx, const int* ncsfN,
                            const int* ndetN, uint64_t* conf_d, uint64_t* conf_s, int64_t* conf_ncsf,
                            int64_t* conf_nslot) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= de.ndet || !flag[i])
        return;
    uint64_t a, b;
    de.at(i, a, b);
    const uint32_t c = cidx[i];
    const uint64_t s = a ^ b;
    conf_d[c] = a & b;
    conf_s[c] = s;
    conf_ncsf[c] = ncsfN[popc64(s)];
    conf_nslot[c] = ndetN[popc64(s)];
}

__global__ void k_conf_perm(DetEnum de, int twoS, int twoMs, ConfSpace cs, const uint32_t* first,
                            const uint32_t* cidx, const int64_t* conf_slot, uint32_t* perm) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= de.ndet)
        return;
    uint64_t a, b;
    de.at(i, a, b);
    const uint64_t d = a & b, s = a ^ b;
    if (popc64(s) < twoS)
        return;
    const uint32_t c = cidx[first[conf_rank(d, s, cs)]];
    uint64_t j;
    int neg;
    pattern_and_sign(a, b, twoMs, cs.binom, j, neg);
    perm[conf_slot[c] + (int64_t)j] = (uint32_t)i | (neg ? 0x80000000u : 0u);
}

__global__ void k_hist(int64_t nconf, const uint64_t* conf_s, unsigned long long* hist) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c < nconf)
        atomicAdd(hist + popc64(conf_s[c]), 1ull);
}

__device__ inline int64_t find_bucket(const int64_t* off, int64_t n, int64_t x) {
    // largest c with off[c] <= x, off has n+1 non-decreasing entries
    int64_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (off[mid] <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// largest c in [lo, hi] with off[c] <= x, given off[lo] <= x (a search inside one thread block's
// bracket of configurations: a few steps on one or two cache lines)
__device__ inline int64_t find_in(const int64_t* off, int64_t lo, int64_t hi, int64_t x) {
    ++hi;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (off[mid] <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// bracket[b] = the configuration holding element b * kBracket of the offsets `off` (nconf + 1
// entries, total = off[nconf]); bracket[nb] = the configuration of the last element
constexpr int kBracket = 256;
__global__ void k_brackets(const int64_t* off, int64_t nconf, int64_t total, int64_t nb, int64_t* bracket) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b > nb)
        return;
    const int64_t x = b < nb ? b * kBracket : total - 1;
    bracket[b] = find_bucket(off, nconf, x);
}

struct CsfView {
    int64_t nconf;
    const uint64_t* conf_s;
    const int64_t* conf_csf;
    const int64_t* conf_slot;
    const uint32_t* perm;
    const double* O;
    const int64_t* offN;
    const int* ncsfN;
    const int* ndetN;
    const float* Of;  // FP32 copy of the overlap tables (the FP32 transforms of the mixed mode)
    const double* OT; // the tables transposed, [ndetN][ncsfN] (det -> CSF reads them along the CSFs)
    const float* OTf;
    const int64_t* slot_brk; // configuration brackets of the slot blocks (k_brackets)
    const int64_t* csf_brk;  // and of the CSF blocks
};

template <typename T> __device__ __forceinline__ const T* overlaps(const CsfView& v);
template <> __device__ __forceinline__ const double* overlaps<double>(const CsfView& v) { return v.O; }
template <> __device__ __forceinline__ const float* overlaps<float>(const CsfView& v) { return v.Of; }
template <typename T> __device__ __forceinline__ const T* overlaps_t(const CsfView& v);
template <> __device__ __forceinline__ const double* overlaps_t<double>(const CsfView& v) { return v.OT; }
template <> __device__ __forceinline__ const float* overlaps_t<float>(const CsfView& v) { return v.OTf; }

// Vector blockIdx.y of a batch: csf + y * ncsf_stride, det + y * ndet_stride. T = double, or float
// for the FP32 sigma of the mixed mode.
template <typename T>
__global__ void k_csf_to_det(int64_t nslot, CsfView v, const T* __restrict__ csf, T* __restrict__ det,
                             int64_t ncsf_stride, int64_t ndet_stride) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nslot)
        return;
    csf += blockIdx.y * ncsf_stride;
    det += blockIdx.y * ndet_stride;
    const int64_t c = find_in(v.conf_slot, v.slot_brk[blockIdx.x], v.slot_brk[blockIdx.x + 1], t);
    const int N = popc64(v.conf_s[c]);
    const int nd = v.ndetN[N], nc = v.ncsfN[N];
    const int64_t j = t - v.conf_slot[c];
    const T* O = overlaps<T>(v) + v.offN[N] + j;
    const T* x = csf + v.conf_csf[c];
    T acc = 0;
    for (int i = 0; i < nc; ++i)
        acc += O[(int64_t)i * nd] * x[i];
    const uint32_t e = v.perm[t];
    det[e & 0x7fffffffu] = (e >> 31) ? -acc : acc;
}

template <bool SQUARE, typename T = double>
__global__ void k_det_to_csf(int64_t ncsf, CsfView v, const T* __restrict__ det, T* __restrict__ csf,
                             int64_t ndet_stride, int64_t ncsf_stride) {
    const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (u >= ncsf)
        return;
    det += blockIdx.y * ndet_stride;
    csf += blockIdx.y * ncsf_stride;
    const int64_t c = find_in(v.conf_csf, v.csf_brk[blockIdx.x], v.csf_brk[blockIdx.x + 1], u);
    const int N = popc64(v.conf_s[c]);
    const int nd = v.ndetN[N], nc = v.ncsfN[N];
    const int64_t i = u - v.conf_csf[c];
    // transposed table: the threads of a configuration (consecutive i) read consecutive entries
    const T* O = overlaps_t<T>(v) + v.offN[N] + i;
    const uint32_t* pm = v.perm + v.conf_slot[c];
    // eight determinants per step: their table entries and addresses, then their values, are
    // requested together (the value loads depend on the addresses); zero entries skip the load.
    // The sum runs over j in order, as one determinant per step would.
    constexpr int U = 8;
    T acc = 0;
    int j = 0;
    for (; j + U <= nd; j += U) {
        T o[U], x[U];
        uint32_t e[U];
#pragma unroll
        for (int k = 0; k < U; ++k) {
            o[k] = O[(int64_t)(j + k) * nc];
            e[k] = pm[j + k];
        }
#pragma unroll
        for (int k = 0; k < U; ++k)
            x[k] = o[k] != T(0) ? det[e[k] & 0x7fffffffu] : T(0);
#pragma unroll
        for (int k = 0; k < U; ++k) {
            if (o[k] == T(0))
                continue;
            if (SQUARE)
                acc += o[k] * o[k] * x[k];
            else
                acc += ((e[k] >> 31) ? -o[k] : o[k]) * x[k];
        }
    }
    for (; j < nd; ++j) {
        const T o = O[(int64_t)j * nc];
        if (o == T(0))
            continue;
        const uint32_t e = pm[j];
        const T x = det[e & 0x7fffffffu];
        if (SQUARE)
            acc += o * o * x;
        else
            acc += ((e >> 31) ? -o : o) * x;
    }
    csf[u] = acc;
}

// ---- Slater rules between two determinants (slater_rules.cc:86-201) ---------------------------
__device__ inline double vv(const double* V, int n, int p, int q, int r, int s) {
    return V[(((size_t)p * n + q) * n + r) * n + s];
}

__device__ double det_energy(uint64_t a, uint64_t b, int n, double E0, const double* h, const double* V) {
    double e = E0;
    for (int p = 0; p < n; ++p) {
        if (!(a >> p & 1))
            continue;
        e += h[p * n + p];
        for (int q = 0; q < p; ++q)
            if (a >> q & 1)
                e += vv(V, n, q, p, q, p) - vv(V, n, q, p, p, q);
        for (int q = 0; q < n; ++q)
            if (b >> q & 1)
                e += vv(V, n, p, q, p, q);
    }
    for (int p = 0; p < n; ++p) {
        if (!(b >> p & 1))
            continue;
        e += h[p * n + p];
        for (int q = 0; q < p; ++q)
            if (b >> q & 1)
                e += vv(V, n, q, p, q, p) - vv(V, n, q, p, p, q);
    }
    return e;
}

__device__ inline int sign_aaaa_neg(uint64_t w, int i, int j, int a, int b) {
    const bool all_below = (i < a) && (j < a) && (i < b) && (j < b);
    const bool none_below = !((i < a) || (j < a) || (i < b) || (j < b));
    const int flip = ((i < j) ^ (a < b)) ? 1 : 0;
    if (all_below || none_below)
        return flip ^ parity_between(w, i, j) ^ parity_between(w, a, b);
    if (flip)
        return 1 ^ parity_between(w, i, b) ^ parity_between(w, j, a);
    return parity_between(w, i, a) ^ parity_between(w, j, b);
}

__device__ double slater_rules(uint64_t la, uint64_t lb, uint64_t ra, uint64_t rb, int n, double E0, const double* h,
                               const double* V) {
    const int da = popc64(la ^ ra), db = popc64(lb ^ rb);
    if (popc64(la) != popc64(ra) || popc64(lb) != popc64(rb))
        return 0.0;
    if (da > 4 || db > 4 || da + db > 4)
        return 0.0;
    auto lowest = [](uint64_t x) { return __ffsll((long long)x) - 1; };
    if (da == 2 && db == 2) {
        const int i = lowest(la & ~ra), a = lowest(ra & ~la), j = lowest(lb & ~rb), b = lowest(rb & ~lb);
        const int neg = parity_between(la, i, a) ^ parity_between(lb, j, b);
        const double x = vv(V, n, i, j, a, b);
        return neg ? -x : x;
    }
    if ((da == 4 && db == 0) || (da == 0 && db == 4)) {
        const uint64_t l = da ? la : lb, r = da ? ra : rb;
        uint64_t lo = l & ~r, ro = r & ~l;
        const int i = lowest(lo);
        lo &= lo - 1;
        const int j = lowest(lo);
        const int a = lowest(ro);
        ro &= ro - 1;
        const int b = lowest(ro);
        const int neg = sign_aaaa_neg(l, i, j, a, b);
        const double x = vv(V, n, i, j, a, b) - vv(V, n, i, j, b, a);
        return neg ? -x : x;
    }
    if ((da == 2 && db == 0) || (da == 0 && db == 2)) {
        const bool alpha = da == 2;
        const uint64_t l = alpha ? la : lb, r = alpha ? ra : rb;
        const int i = lowest(l & ~r), a = lowest(r & ~l);
        double x = h[i * n + a];
        for (int j = 0; j < n; ++j) {
            const bool same = alpha ? (ra >> j & 1) : (rb >> j & 1);
            const bool other = alpha ? (rb >> j & 1) : (ra >> j & 1);
            if (same)
                x += vv(V, n, i, j, a, j) - vv(V, n, i, j, j, a);
            if (other)
                x += vv(V, n, i, j, a, j);
        }
        return parity_between(l, i, a) ? -x : x;
    }
    return det_energy(la, lb, n, E0, h, V);
}

__global__ void k_csf_matrix(int m, const int64_t* idx, CsfView v, DetEnum de, int n, double E0, const double* h,
                             const double* V, double* out) {
    const int A = blockIdx.x, B = blockIdx.y;
    if (B > A)
        return;
    __shared__ double red[256];
    const int64_t ua = idx[A], ub = idx[B];
    const int64_t ca = find_bucket(v.conf_csf, v.nconf, ua), cb = find_bucket(v.conf_csf, v.nconf, ub);
    const int Na = popc64(v.conf_s[ca]), Nb = popc64(v.conf_s[cb]);
    const int nda = v.ndetN[Na], ndb = v.ndetN[Nb];
    const double* Oa = v.O + v.offN[Na] + (ua - v.conf_csf[ca]) * nda;
    const double* Ob = v.O + v.offN[Nb] + (ub - v.conf_csf[cb]) * ndb;
    const uint32_t* pa = v.perm + v.conf_slot[ca];
    const uint32_t* pb = v.perm + v.conf_slot[cb];
    double acc = 0.0;
    for (int64_t t = threadIdx.x; t < (int64_t)nda * ndb; t += blockDim.x) {
        const int ja = (int)(t / ndb), jb = (int)(t % ndb);
        const double oa = Oa[ja], ob = Ob[jb];
        if (oa == 0.0 || ob == 0.0)
            continue;
        const uint32_t ea = pa[ja], eb = pb[jb];
        const int64_t da = ea & 0x7fffffffu, db = eb & 0x7fffffffu;
        const double c = ((ea >> 31) ? -oa : oa) * ((eb >> 31) ? -ob : ob);
        uint64_t la, lb, ra, rb;
        de.at(da, la, lb);
        de.at(db, ra, rb);
        acc += c * slater_rules(la, lb, ra, rb, n, E0, h, V);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[(int64_t)A * m + B] = red[0];
        out[(int64_t)B * m + A] = red[0];
    }
}

// ---- host ----------------------------------------------------------------------------------

__global__ void k_convert_d2f(int64_t n, const double* __restrict__ in, float* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = (float)in[i];
}

template <typename T> static void exclusive_scan(const T* in, T* out, int64_t n, cudaStream_t st) {
    size_t bytes = 0;
    F2G_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, st));
    TmpBuf<unsigned char> tmp(bytes, st);
    F2G_CUDA(cub::DeviceScan::ExclusiveSum(tmp.get(), bytes, in, out, n, st));
    F2G_CUDA(cudaStreamSynchronize(st));
}

SpinAdapter::SpinAdapter(const CIStrings* s_, int twoS_, int twoMs_)
    : s(s_), twoS(twoS_), twoMs(twoMs_), norb(s_->norb) {
    const int n = norb, nel = s->na + s->nb;
    if (twoS < 0)
        throw Error(2, "CISpinAdapter: twoS must be non-negative");
    if (twoMs != s->na - s->nb)
        throw Error(2, "CISpinAdapter: twoMs does not match the determinant space (na - nb)");
    cudaStream_t st = 0;
    // per-N tables
    ncsfN.assign(n + 1, 0);
    ndetN.assign(n + 1, 0);
    offN.assign(n + 2, 0);
    std::vector<double> Ohost;
    std::vector<int64_t> nnzN(n + 1, 0);
    for (int N = 0; N <= n; ++N) {
        offN[N] = (int64_t)Ohost.size();
        if (N < twoS || ((N - twoMs) % 2) != 0 || N < std::abs(twoMs) || (N - twoMs) / 2 > N)
            continue;
        const auto cp = couplings(N, twoS);
        const auto pt = patterns(N, twoMs);
        ncsfN[N] = (int)cp.size();
        ndetN[N] = (int)pt.size();
        const size_t base = Ohost.size();
        Ohost.resize(base + cp.size() * pt.size());
        for (size_t i = 0; i < cp.size(); ++i)
            for (size_t j = 0; j < pt.size(); ++j) {
                const double o = overlap(N, cp[i], pt[j]);
                Ohost[base + i * pt.size() + j] = o;
                if (std::fabs(o) > 0.0)
                    nnzN[N]++;
            }
    }
    offN[n + 1] = (int64_t)Ohost.size();
    O.reserve(std::max<size_t>(1, Ohost.size()));
    if (!Ohost.empty())
        F2G_CUDA(cudaMemcpy(O.get(), Ohost.data(), Ohost.size() * sizeof(double), cudaMemcpyHostToDevice));
    {
        std::vector<double> T_(Ohost.size());
        for (int N = 0; N <= n; ++N) {
            const int64_t nc = ncsfN[N], nd = ndetN[N], b = offN[N];
            for (int64_t i = 0; i < nc; ++i)
                for (int64_t j = 0; j < nd; ++j)
                    T_[b + j * nc + i] = Ohost[b + i * nd + j];
        }
        OT.reserve(std::max<size_t>(1, T_.size()));
        if (!T_.empty())
            F2G_CUDA(cudaMemcpy(OT.get(), T_.data(), T_.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    dOff.reserve(n + 2);
    dNcsf.reserve(n + 1);
    dNdet.reserve(n + 1);
    F2G_CUDA(cudaMemcpy(dOff.get(), offN.data(), (n + 2) * sizeof(int64_t), cudaMemcpyHostToDevice));
    F2G_CUDA(cudaMemcpy(dNcsf.get(), ncsfN.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
    F2G_CUDA(cudaMemcpy(dNdet.get(), ndetN.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));

    // canonical configuration space
    std::vector<int64_t> base(n + 2, 0);
    int64_t total = 0;
    for (int nd = 0; nd <= n; ++nd) {
        base[nd] = total;
        const int ns = nel - 2 * nd;
        if (ns < 0 || ns > n - nd)
            continue;
        total += (int64_t)(host_binom(n, nd) * host_binom(n - nd, ns));
    }
    base[n + 1] = total;
    TmpBuf<int64_t> dbase(n + 2, st);
    F2G_CUDA(cudaMemcpyAsync(dbase.get(), base.data(), (n + 2) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    ConfSpace cs{n, nel, dbase.get(), s->binom.get()};

    const DetEnum de = s->dets();
    const int64_t nd_ = s->ndet;
    if (nd_ > 0x7fffffffLL)
        throw Error(1, "CISpinAdapter: more than 2^31 determinants");
    TmpBuf<uint32_t> first(std::max<int64_t>(1, total), st), flag(std::max<int64_t>(1, nd_), st),
        cidx(std::max<int64_t>(1, nd_), st);
    F2G_CUDA(cudaMemsetAsync(first.get(), 0xff, std::max<int64_t>(1, total) * sizeof(uint32_t), st));
    const int T = 256;
    if (nd_ > 0) {
        k_conf_first<<<ceil_div(nd_, T), T, 0, st>>>(de, twoS, cs, first.get());
        F2G_LAUNCH("k_conf_first");
        k_conf_flag<<<ceil_div(nd_, T), T, 0, st>>>(de, twoS, cs, first.get(), flag.get());
        F2G_LAUNCH("k_conf_flag");
        exclusive_scan<uint32_t>(flag.get(), cidx.get(), nd_, st);
        uint32_t last_flag = 0, last_idx = 0;
        F2G_CUDA(cudaMemcpyAsync(&last_flag, flag.get() + nd_ - 1, 4, cudaMemcpyDeviceToHost, st));
        F2G_CUDA(cudaMemcpyAsync(&last_idx, cidx.get() + nd_ - 1, 4, cudaMemcpyDeviceToHost, st));
        F2G_CUDA(cudaStreamSynchronize(st));
        nconf = (int64_t)last_idx + last_flag;
    }
    conf_d.reserve(std::max<int64_t>(1, nconf));
    conf_s.reserve(std::max<int64_t>(1, nconf));
    conf_csf.reserve(nconf + 1);
    conf_slot.reserve(nconf + 1);
    TmpBuf<int64_t> cnc(nconf + 1, st), cns(nconf + 1, st);
    F2G_CUDA(cudaMemsetAsync(cnc.get(), 0, (nconf + 1) * sizeof(int64_t), st));
    F2G_CUDA(cudaMemsetAsync(cns.get(), 0, (nconf + 1) * sizeof(int64_t), st));
    if (nconf > 0) {
        k_conf_fill<<<ceil_div(nd_, T), T, 0, st>>>(de, flag.get(), cidx.get(), dNcsf.get(), dNdet.get(),
                                                   conf_d.get(), conf_s.get(), cnc.get(), cns.get());
        F2G_LAUNCH("k_conf_fill");
    }
    exclusive_scan<int64_t>(cnc.get(), conf_csf.get(), nconf + 1, st);
    exclusive_scan<int64_t>(cns.get(), conf_slot.get(), nconf + 1, st);
    F2G_CUDA(cudaMemcpyAsync(&ncsf, conf_csf.get() + nconf, 8, cudaMemcpyDeviceToHost, st));
    F2G_CUDA(cudaMemcpyAsync(&nslot, conf_slot.get() + nconf, 8, cudaMemcpyDeviceToHost, st));
    F2G_CUDA(cudaStreamSynchronize(st));
    covers_all_dets = nslot == nd_;
    perm.reserve(std::max<int64_t>(1, nslot));
    if (nslot > 0) {
        k_conf_perm<<<ceil_div(nd_, T), T, 0, st>>>(de, twoS, twoMs, cs, first.get(), cidx.get(), conf_slot.get(),
                                                   perm.get());
        F2G_LAUNCH("k_conf_perm");
    }
    // configuration brackets of the 256-element blocks of the transform kernels
    for (int which = 0; which < 2; ++which) {
        const int64_t total = which == 0 ? nslot : ncsf;
        const int64_t nb = (total + kBracket - 1) / kBracket;
        DevBuf<int64_t>& brk = which == 0 ? slot_brk : csf_brk;
        brk.reserve(nb + 1);
        if (total > 0) {
            k_brackets<<<ceil_div(nb + 1, T), T, 0, st>>>(which == 0 ? conf_slot.get() : conf_csf.get(), nconf, total,
                                                          nb, brk.get());
            F2G_LAUNCH("k_brackets");
        }
    }
    // coupling count (non-zero overlaps), as the reference logs it
    TmpBuf<unsigned long long> hist(65, st);
    F2G_CUDA(cudaMemsetAsync(hist.get(), 0, 65 * 8, st));
    if (nconf > 0) {
        k_hist<<<ceil_div(nconf, T), T, 0, st>>>(nconf, conf_s.get(), hist.get());
        F2G_LAUNCH("k_hist");
    }
    std::vector<unsigned long long> h(65);
    F2G_CUDA(cudaMemcpyAsync(h.data(), hist.get(), 65 * 8, cudaMemcpyDeviceToHost, st));
    F2G_CUDA(cudaStreamSynchronize(st));
    ncoupling = 0;
    for (int N = 0; N <= n; ++N)
        ncoupling += (int64_t)h[N] * nnzN[N];
    F2G_CUDA(cudaStreamSynchronize(st));
}

static CsfView view_of(const SpinAdapter& a) {
    return CsfView{a.nconf,       a.conf_s.get(), a.conf_csf.get(), a.conf_slot.get(), a.perm.get(),
                   a.O.get(),     a.dOff.get(),   a.dNcsf.get(),    a.dNdet.get(),     a.O32.get(),
                   a.OT.get(),    a.OT32.get(),   a.slot_brk.get(), a.csf_brk.get()};
}

void SpinAdapter::csf_to_det(const double* csf, double* det, cudaStream_t st, int nvec) const {
    if (nvec <= 0)
        return;
    if (nvec > 65535)
        throw Error(2, "csf_to_det: at most 65535 vectors per call");
    if (!covers_all_dets)
        F2G_CUDA(cudaMemsetAsync(det, 0, (size_t)nvec * s->ndet * sizeof(double), st));
    if (nslot == 0)
        return;
    k_csf_to_det<double><<<dim3((unsigned)ceil_div(nslot, 256), (unsigned)nvec), 256, 0, st>>>(
        nslot, view_of(*this), csf, det, ncsf, s->ndet);
    F2G_LAUNCH("k_csf_to_det");
}

void SpinAdapter::det_to_csf(const double* det, double* csf, cudaStream_t st, int nvec) const {
    if (ncsf == 0 || nvec <= 0)
        return;
    if (nvec > 65535)
        throw Error(2, "det_to_csf: at most 65535 vectors per call");
    k_det_to_csf<false><<<dim3((unsigned)ceil_div(ncsf, 256), (unsigned)nvec), 256, 0, st>>>(ncsf, view_of(*this), det,
                                                                                             csf, s->ndet, ncsf);
    F2G_LAUNCH("k_det_to_csf");
}

// The FP32 transforms (mixed mode): the overlap tables are copied to FP32 once (stream order st).
void SpinAdapter::ensure_fp32_tables(cudaStream_t st) const {
    if (O32.get() || offN.back() == 0)
        return;
    const int64_t nO = offN.back();
    O32.reserve((size_t)nO);
    k_convert_d2f<<<ceil_div(nO, 256), 256, 0, st>>>(nO, O.get(), O32.get());
    F2G_LAUNCH("k_convert_d2f overlaps");
    OT32.reserve((size_t)nO);
    k_convert_d2f<<<ceil_div(nO, 256), 256, 0, st>>>(nO, OT.get(), OT32.get());
    F2G_LAUNCH("k_convert_d2f transposed overlaps");
}

void SpinAdapter::csf_to_det(const float* csf, float* det, cudaStream_t st, int nvec) const {
    if (nvec <= 0)
        return;
    if (nvec > 65535)
        throw Error(2, "csf_to_det: at most 65535 vectors per call");
    ensure_fp32_tables(st);
    if (!covers_all_dets)
        F2G_CUDA(cudaMemsetAsync(det, 0, (size_t)nvec * s->ndet * sizeof(float), st));
    if (nslot == 0)
        return;
    k_csf_to_det<float><<<dim3((unsigned)ceil_div(nslot, 256), (unsigned)nvec), 256, 0, st>>>(
        nslot, view_of(*this), csf, det, ncsf, s->ndet);
    F2G_LAUNCH("k_csf_to_det<float>");
}

void SpinAdapter::det_to_csf(const float* det, float* csf, cudaStream_t st, int nvec) const {
    if (ncsf == 0 || nvec <= 0)
        return;
    if (nvec > 65535)
        throw Error(2, "det_to_csf: at most 65535 vectors per call");
    ensure_fp32_tables(st);
    k_det_to_csf<false, float><<<dim3((unsigned)ceil_div(ncsf, 256), (unsigned)nvec), 256, 0, st>>>(
        ncsf, view_of(*this), det, csf, s->ndet, ncsf);
    F2G_LAUNCH("k_det_to_csf<float>");
}

__global__ void k_convert_f2d(int64_t n, const float* __restrict__ in, double* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = (double)in[i];
}

void CsfSigmaScratch::reserve(const SigmaBuilder& sb, const SpinAdapter& sa, int nvec) {
    const size_t nd = (size_t)std::max<int64_t>(1, sa.s->ndet), nc = (size_t)std::max<int64_t>(1, sa.ncsf);
    if (sb.precision == kFP64) {
        det_in.reserve(nvec * nd);
        det_out.reserve(nvec * nd);
    } else {
        f_csf_in.reserve(nvec * nc);
        f_csf_out.reserve(nvec * nc);
        f_det_in.reserve(nvec * nd);
        f_det_out.reserve(nvec * nd);
    }
    reserved_vec = std::max<int64_t>(reserved_vec, nvec);
}

void sigma_csf(SigmaBuilder& sb, const SpinAdapter& sa, const double* in, double* out, int nvec, cudaStream_t st,
               CsfSigmaScratch& scr, bool graph) {
    if (sa.s != sb.s)
        throw Error(2, "sigma_csf: the spin adapter and the sigma builder use different strings");
    const int64_t nd = sa.s->ndet, nc = sa.ncsf;
    if (nvec <= 0 || nc == 0)
        return;
    if (!graph)
        sb.check_memory();
    const int bs = graph ? nvec : sb.batch_size(nvec);
    if (graph && nvec > scr.reserved_vec)
        throw Error(2, "sigma_csf: more vectors than the graph scratch holds");
    for (int v0 = 0; v0 < nvec; v0 += bs) {
        const int nv = std::min(bs, nvec - v0);
        if (!graph)
            scr.reserve(sb, sa, nv);
        const double* x = in + (int64_t)v0 * nc;
        double* y = out + (int64_t)v0 * nc;
        if (sb.precision == kFP64) {
            sa.csf_to_det(x, scr.det_in.get(), st, nv);
            if (graph)
                sb.apply_untimed(scr.det_in.get(), scr.det_out.get(), st, nv);
            else
                sb.hamiltonian(scr.det_in.get(), scr.det_out.get(), st, nv);
            sa.det_to_csf(scr.det_out.get(), y, st, nv);
        } else {
            const int64_t tc = (int64_t)nv * nc;
            k_convert_d2f<<<ceil_div(tc, 256), 256, 0, st>>>(tc, x, scr.f_csf_in.get());
            F2G_LAUNCH("k_convert_d2f csf");
            sa.csf_to_det(scr.f_csf_in.get(), scr.f_det_in.get(), st, nv);
            sb.apply_f32(scr.f_det_in.get(), scr.f_det_out.get(), st, nv, !graph, graph);
            sa.det_to_csf(scr.f_det_out.get(), scr.f_csf_out.get(), st, nv);
            k_convert_f2d<<<ceil_div(tc, 256), 256, 0, st>>>(tc, scr.f_csf_out.get(), y);
            F2G_LAUNCH("k_convert_f2d csf");
        }
    }
    (void)nd;
}

void SpinAdapter::hdiag(const double* det_energy, double* out, cudaStream_t st) const {
    if (ncsf == 0)
        return;
    k_det_to_csf<true><<<ceil_div(ncsf, 256), 256, 0, st>>>(ncsf, view_of(*this), det_energy, out, 0, 0);
    F2G_LAUNCH("k_hdiag");
}

void SpinAdapter::csf_matrix(const SigmaBuilder& sb, const int64_t* idx, int m, double* out_host) const {
    if (m <= 0)
        return;
    int64_t* didx = mat_idx.reserve(m);
    double* dout = mat_out.reserve((size_t)m * m);
    F2G_CUDA(cudaMemcpy(didx, idx, m * sizeof(int64_t), cudaMemcpyHostToDevice));
    csf_matrix_dev(sb, didx, m, dout, 0);
    F2G_CUDA(cudaMemcpy(out_host, dout, (size_t)m * m * sizeof(double), cudaMemcpyDeviceToHost));
}

void SpinAdapter::csf_matrix_dev(const SigmaBuilder& sb, const int64_t* idx, int m, double* out,
                                 cudaStream_t st) const {
    if (m <= 0)
        return;
    if (m > 65535)
        throw Error(2, "csf_matrix: at most 65535 CSFs per call");
    k_csf_matrix<<<dim3(m, m), 256, 0, st>>>(m, idx, view_of(*this), s->dets(), norb, sb.E, sb.dH.get(), sb.dV.get(),
                                             out);
    F2G_LAUNCH("k_csf_matrix");
}

void SpinAdapter::dump(int64_t* bounds, int64_t* det_idx, double* coeff, int64_t* ranges) const {
    std::vector<int64_t> cc(nconf + 1), cl(nconf + 1);
    std::vector<uint64_t> cs(std::max<int64_t>(1, nconf));
    std::vector<uint32_t> pm(std::max<int64_t>(1, nslot));
    std::vector<double> Oh(std::max<int64_t>(1, offN.back()));
    F2G_CUDA(cudaMemcpy(cc.data(), conf_csf.get(), (nconf + 1) * 8, cudaMemcpyDeviceToHost));
    F2G_CUDA(cudaMemcpy(cl.data(), conf_slot.get(), (nconf + 1) * 8, cudaMemcpyDeviceToHost));
    if (nconf)
        F2G_CUDA(cudaMemcpy(cs.data(), conf_s.get(), nconf * 8, cudaMemcpyDeviceToHost));
    if (nslot)
        F2G_CUDA(cudaMemcpy(pm.data(), perm.get(), nslot * 4, cudaMemcpyDeviceToHost));
    if (offN.back())
        F2G_CUDA(cudaMemcpy(Oh.data(), O.get(), offN.back() * 8, cudaMemcpyDeviceToHost));
    int64_t k = 0, u = 0;
    bounds[0] = 0;
    for (int64_t c = 0; c < nconf; ++c) {
        const int N = popc64(cs[c]);
        const int nd = ndetN[N], nc = ncsfN[N];
        for (int i = 0; i < nc; ++i, ++u) {
            for (int j = 0; j < nd; ++j) {
                const double o = Oh[offN[N] + (int64_t)i * nd + j];
                if (!(std::fabs(o) > 0.0))
                    continue;
                const uint32_t e = pm[cl[c] + j];
                det_idx[k] = e & 0x7fffffffu;
                coeff[k] = (e >> 31) ? -o : o;
                ++k;
            }
            bounds[u + 1] = k;
        }
        ranges[2 * c] = cc[c];
        ranges[2 * c + 1] = cc[c + 1];
    }
}

} // namespace f2g
