// Determinant blocks of a general CI space (point-group irreps, GAS occupation restrictions).
//
// The space and its order are the reference's (forte2/ci/ci_strings.cc:34-184):
//   occupation patterns  every allowed (alpha, beta) electron count per GAS space, from the
//                        ORMAS recursion over the spaces (ci_occupation.cc:35-142): for each space
//                        in turn the alpha count (outer) and the beta count (inner) within the
//                        space's bounds, the last space taking the remaining electrons; distinct
//                        alpha and beta patterns are numbered in order of first appearance;
//   string classes       per spin, (pattern, irrep) with the irreps of one pattern next to each
//                        other (ci_string_class.cc:36-53);
//   strings of a class   the Cartesian product of the per-space strings (first space slowest),
//                        each space's strings in std::next_permutation order of its orbitals,
//                        kept in that order and split by irrep (ci_strings_makers.cc:13-73);
//   blocks               for each allowed pattern pair, for each alpha irrep h: the block
//                        (alpha class (pair.alpha, h), beta class (pair.beta, h ^ symmetry)),
//                        determinants alpha-major inside a block (ci_string_class.cc:56-65,
//                        ci_strings.cc:151-161, 198-206).
//
// The sigma kernels run on the C1 CAS space of the same orbitals and electrons: a vector of the
// blocked space is embedded into a C1 vector (zero outside the space), H is applied there, and
// the space's elements are read back. That is P H P C, what the reference's block loops compute;
// the cost is that of the C1 space.
#include "blocks.cuh"

#include <algorithm>
#include <string>

namespace f2g {

namespace {

using Occ = DetBlocks::Occ;

int index_of(std::vector<Occ>& v, const Occ& o) {
    for (size_t i = 0; i < v.size(); ++i)
        if (v[i] == o)
            return (int)i;
    v.push_back(o);
    return (int)v.size() - 1;
}

struct PatternWalk {
    int nsp;
    Occ lo, hi, size;
    std::vector<Occ>&A, &B;
    std::vector<std::pair<int, int>>& P;

    void walk(int na, int nb, int sp, Occ a, Occ b) {
        if (sp == nsp - 1) {
            // the last space holds what is left
            const int tot = na + nb;
            if (tot <= hi[sp] && tot >= lo[sp] && std::max(na, nb) <= size[sp] && std::min(na, nb) >= 0) {
                a[sp] = na;
                b[sp] = nb;
                const int ia = index_of(A, a), ib = index_of(B, b);
                P.emplace_back(ia, ib);
            }
            return;
        }
        const int amin = std::max(lo[sp] - size[sp], 0), amax = std::min(hi[sp], size[sp]);
        for (int xa = amin; xa <= amax; ++xa) {
            const int bmin = std::max(lo[sp] - xa, 0), bmax = std::min(hi[sp] - xa, size[sp]);
            for (int xb = bmin; xb <= bmax; ++xb) {
                if (xa + xb > hi[sp] || xa + xb < lo[sp])
                    continue;
                a[sp] = xa;
                b[sp] = xb;
                walk(na - xa, nb - xb, sp + 1, a, b);
            }
        }
    }
};

int string_irrep(uint64_t m, const std::vector<int>& orbsym) {
    int h = 0;
    while (m) {
        const int p = __builtin_ctzll(m);
        h ^= orbsym[p];
        m &= m - 1;
    }
    return h;
}

std::vector<uint64_t> host_binom_table() {
    std::vector<uint64_t> t(kBinomLd * kBinomLd, 0);
    for (int a = 0; a < kBinomLd; ++a)
        for (int b = 0; b < kBinomLd; ++b)
            t[a * kBinomLd + b] = host_binom(a, b);
    return t;
}

} // namespace

void DetBlocks::enumerate(int na, int nb, int sym, const std::vector<std::vector<int>>& orbital_symmetry,
                          const std::vector<int>& gas_min, const std::vector<int>& gas_max) {
    symmetry = sym;
    if (gas_min.size() > orbital_symmetry.size() || gas_max.size() > orbital_symmetry.size())
        throw Error(2, "CIStrings: The number of GAS spaces specified by gas_min (" + std::to_string(gas_min.size()) +
                           ") and gas_max (" + std::to_string(gas_max.size()) +
                           ") must be less than or equal to the number of orbital symmetries (" +
                           std::to_string(orbital_symmetry.size()) + ")");
    if (orbital_symmetry.size() > (size_t)kMaxGasSpaces)
        throw Error(2, "CIStrings: at most " + std::to_string(kMaxGasSpaces) + " GAS spaces");
    orbsym.clear();
    gas_size.clear();
    std::vector<int> first; // first orbital of every space
    nirrep = 1;
    for (const auto& sp : orbital_symmetry) {
        first.push_back((int)orbsym.size());
        gas_size.push_back((int)sp.size());
        for (int h : sp) {
            if (h < 0 || h > 7)
                throw Error(2, "CIStrings: orbital irreps must be in 0..7");
            orbsym.push_back(h);
            nirrep = std::max(nirrep, h + 1);
        }
    }
    const int norb = (int)orbsym.size();
    if (norb > kMaxOrb)
        throw Error(2, "CIStrings: the number of active orbitals must be between 0 and 62");
    if (sym < 0 || sym >= nirrep)
        throw Error(2, "CIStrings: the state symmetry " + std::to_string(sym) + " is not an irrep of the orbitals");

    // bounds of the non-empty spaces, indexed like the spaces (ci_occupation.cc:107-141)
    Occ lo{}, hi{}, size{};
    int nsp = 0;
    for (int n = 0; n < kMaxGasSpaces; ++n) {
        const int sz = n < (int)gas_size.size() ? gas_size[n] : 0;
        if (!sz)
            continue;
        int mx = std::min(2 * sz, na + nb);
        if ((int)gas_max.size() > n)
            mx = std::min(gas_max[n], mx);
        hi[n] = mx;
        lo[n] = (int)gas_min.size() > n ? gas_min[n] : 0;
        size[n] = sz;
        ++nsp;
    }
    aocc.clear();
    bocc.clear();
    occ_pairs.clear();
    if (nsp == 0) {
        aocc.push_back(Occ{});
        bocc.push_back(Occ{});
        occ_pairs.emplace_back(0, 0);
        nsp = 1;
    } else {
        PatternWalk w{nsp, lo, hi, size, aocc, bocc, occ_pairs};
        w.walk(na, nb, 0, Occ{}, Occ{});
    }
    nspace = nsp;

    // class strings of both spins
    const std::vector<uint64_t> binom = host_binom_table();
    for (int spin = 0; spin < 2; ++spin) {
        const std::vector<Occ>& pats = spin == 0 ? aocc : bocc;
        str[spin].clear();
        cls_off[spin].assign(1, 0);
        for (const Occ& occ : pats) {
            std::vector<std::vector<uint64_t>> per(nsp);
            bool none = false;
            for (int n = 0; n < nsp; ++n) {
                const int g = n < (int)gas_size.size() ? gas_size[n] : 0, e = occ[n];
                if (e < 0 || e > g) {
                    none = true;
                    continue;
                }
                const uint64_t cnt = host_binom(g, e);
                const int sh = n < (int)first.size() ? first[n] : 0;
                for (uint64_t j = 0; j < cnt; ++j)
                    per[n].push_back(string_unrank(j, g, e, binom.data()) << sh);
            }
            std::vector<std::vector<uint64_t>> byirrep(nirrep);
            if (!none) {
                // odometer over the spaces, the last one fastest
                std::vector<size_t> idx(nsp, 0);
                bool empty = false;
                for (int n = 0; n < nsp; ++n)
                    empty |= per[n].empty();
                while (!empty) {
                    uint64_t m = 0;
                    for (int n = 0; n < nsp; ++n)
                        m |= per[n][idx[n]];
                    byirrep[string_irrep(m, orbsym)].push_back(m);
                    int n = nsp - 1;
                    while (n >= 0 && ++idx[n] == per[n].size()) {
                        idx[n] = 0;
                        --n;
                    }
                    if (n < 0)
                        break;
                }
            }
            for (int h = 0; h < nirrep; ++h) {
                str[spin].insert(str[spin].end(), byirrep[h].begin(), byirrep[h].end());
                cls_off[spin].push_back((int64_t)str[spin].size());
            }
        }
    }

    // blocks
    hblk.clear();
    ndet = 0;
    for (const auto& [ia, ib] : occ_pairs) {
        for (int h = 0; h < nirrep; ++h) {
            const int hb = h ^ sym;
            if (hb >= nirrep)
                throw Error(1, "Block index not found");
            const int ca = ia * nirrep + h, cb = ib * nirrep + hb;
            const int64_t nIa = cls_off[0][ca + 1] - cls_off[0][ca], nIb = cls_off[1][cb + 1] - cls_off[1][cb];
            hblk.insert(hblk.end(), {ca, cb, nIa * nIb, ndet, nIa, nIb});
            ndet += nIa * nIb;
        }
    }
    if (ndet > 0x7fffffffLL)
        throw Error(1, "CIStrings: more than 2^31 determinants in a blocked space");

    // C1 addresses of the class strings
    for (int spin = 0; spin < 2; ++spin) {
        const int k = spin == 0 ? na : nb;
        rank[spin].resize(str[spin].size());
        for (size_t j = 0; j < str[spin].size(); ++j)
            rank[spin][j] = (uint32_t)string_rank(str[spin][j], norb, k, binom.data());
    }
    // trivial: one block over all C1 strings in C1 order
    int nonempty = 0;
    int64_t a0 = 0, b0 = 0;
    for (int b = 0; b < nblk(); ++b) {
        const int64_t* r = hblk.data() + 6 * b;
        if (r[2] == 0)
            continue;
        ++nonempty;
        a0 = cls_off[0][r[0]];
        b0 = cls_off[1][r[1]];
    }
    trivial = false;
    if (nonempty == 1) {
        const int64_t N0a = (int64_t)host_binom(norb, na), N0b = (int64_t)host_binom(norb, nb);
        bool id = ndet == N0a * N0b;
        for (int64_t j = 0; id && j < N0a; ++j)
            id = rank[0][a0 + j] == (uint32_t)j;
        for (int64_t j = 0; id && j < N0b; ++j)
            id = rank[1][b0 + j] == (uint32_t)j;
        trivial = id;
    }
}

void DetBlocks::build(int na, int nb, int sym, const std::vector<std::vector<int>>& orbital_symmetry,
                      const std::vector<int>& gas_min, const std::vector<int>& gas_max) {
    enumerate(na, nb, sym, orbital_symmetry, gas_min, gas_max);
    std::vector<int64_t> dev;
    for (int b = 0; b < nblk(); ++b) {
        const int64_t* r = hblk.data() + 6 * b;
        if (r[2] == 0)
            continue;
        dev.insert(dev.end(), {r[3], r[5], cls_off[0][r[0]], cls_off[1][r[1]]});
    }
    dblk.reserve(std::max<size_t>(dev.size(), 4));
    if (!dev.empty())
        F2G_CUDA(cudaMemcpy(dblk.get(), dev.data(), dev.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    for (int spin = 0; spin < 2; ++spin) {
        const size_t ns = std::max<size_t>(1, str[spin].size());
        dstr[spin].reserve(ns);
        drank[spin].reserve(ns);
        if (!str[spin].empty()) {
            F2G_CUDA(cudaMemcpy(dstr[spin].get(), str[spin].data(), str[spin].size() * 8, cudaMemcpyHostToDevice));
            F2G_CUDA(cudaMemcpy(drank[spin].get(), rank[spin].data(), rank[spin].size() * 4, cudaMemcpyHostToDevice));
        }
    }
}

void DetBlocks::set_c1(int na, int nb, int64_t N0a, int64_t N0b) {
    if (hblk.empty()) {
        symmetry = 0;
        nirrep = 1;
        nspace = 1;
        Occ oa{}, ob{};
        oa[0] = na;
        ob[0] = nb;
        aocc.assign(1, oa);
        bocc.assign(1, ob);
        occ_pairs.assign(1, {0, 0});
        cls_off[0] = {0, N0a};
        cls_off[1] = {0, N0b};
        hblk = {0, 0, N0a * N0b, 0, N0a, N0b};
        ndet = N0a * N0b;
    }
    trivial = true;
    const int64_t one[4] = {0, N0b, 0, 0};
    dblk.reserve(4);
    F2G_CUDA(cudaMemcpy(dblk.get(), one, sizeof(one), cudaMemcpyHostToDevice));
}

void DetBlocks::build_filter(int64_t N0a, int64_t N0b) {
    const int nc[2] = {nclass(0), nclass(1)};
    // allowed (alpha class, beta class) pairs: the non-empty blocks
    std::vector<uint8_t> allowed((size_t)nc[0] * nc[1], 0);
    for (int b = 0; b < nblk(); ++b) {
        const int64_t* r = hblk.data() + 6 * b;
        if (r[2] > 0)
            allowed[(size_t)r[0] * nc[1] + r[1]] = 1;
    }
    for (int spin = 0; spin < 2; ++spin) {
        const int64_t N0 = spin == 0 ? N0a : N0b;
        std::vector<int16_t> cls((size_t)N0, -1);
        std::vector<int32_t> pos((size_t)N0, -1);
        for (int c = 0; c < nc[spin]; ++c)
            for (int64_t j = cls_off[spin][c]; j < cls_off[spin][c + 1]; ++j) {
                cls[rank[spin][j]] = (int16_t)c;
                pos[rank[spin][j]] = (int32_t)(j - cls_off[spin][c]);
            }
        const int m = nc[spin], o = nc[1 - spin];
        std::vector<uint8_t> compat((size_t)m * m, 0);
        for (int c = 0; c < m; ++c)
            for (int c2 = 0; c2 < m; ++c2)
                for (int x = 0; x < o && !compat[(size_t)c * m + c2]; ++x) {
                    const bool a1 = spin == 0 ? allowed[(size_t)c * o + x] : allowed[(size_t)x * m + c];
                    const bool a2 = spin == 0 ? allowed[(size_t)c2 * o + x] : allowed[(size_t)x * m + c2];
                    compat[(size_t)c * m + c2] = a1 && a2;
                }
        dcls[spin].reserve(std::max<int64_t>(1, N0));
        dpos[spin].reserve(std::max<int64_t>(1, N0));
        dcompat[spin].reserve(std::max<size_t>(1, compat.size()));
        if (N0) {
            F2G_CUDA(cudaMemcpy(dcls[spin].get(), cls.data(), (size_t)N0 * sizeof(int16_t), cudaMemcpyHostToDevice));
            F2G_CUDA(cudaMemcpy(dpos[spin].get(), pos.data(), (size_t)N0 * sizeof(int32_t), cudaMemcpyHostToDevice));
        }
        if (!compat.empty())
            F2G_CUDA(cudaMemcpy(dcompat[spin].get(), compat.data(), compat.size(), cudaMemcpyHostToDevice));
    }
}

DetEnum DetBlocks::view(int64_t N0b_c1) const {
    DetEnum d;
    d.ndet = ndet;
    d.nblk = 0;
    for (int b = 0; b < nblk(); ++b)
        d.nblk += hblk[6 * b + 2] > 0;
    d.blk = dblk.get();
    d.amask = dstr[0].get();
    d.bmask = dstr[1].get();
    d.arank = drank[0].get();
    d.brank = drank[1].get();
    d.N0b = N0b_c1;
    return d;
}

template <typename T>
__global__ void k_embed(DetEnum de, int64_t nfull, const T* __restrict__ sub, T* __restrict__ full) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= de.ndet)
        return;
    const int64_t v = blockIdx.y;
    full[v * nfull + de.c1(i)] = sub[v * de.ndet + i];
}

template <typename T> __device__ __forceinline__ void add_to(T& a, const T& b) { a += b; }
template <> __device__ __forceinline__ void add_to<double2>(double2& a, const double2& b) {
    a.x += b.x;
    a.y += b.y;
}

template <typename T>
__global__ void k_extract(DetEnum de, int64_t nfull, const T* __restrict__ full, T* __restrict__ sub, int add) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= de.ndet)
        return;
    const int64_t v = blockIdx.y;
    const T x = full[v * nfull + de.c1(i)];
    if (add)
        add_to(sub[v * de.ndet + i], x);
    else
        sub[v * de.ndet + i] = x;
}

template <typename T>
void blocks_embed(const DetEnum& de, int64_t nfull, const T* sub, T* full, int nvec, cudaStream_t st) {
    if (nvec <= 0 || nfull == 0)
        return;
    if (nvec > 65535)
        throw Error(2, "blocks_embed: at most 65535 vectors per call");
    F2G_CUDA(cudaMemsetAsync(full, 0, (size_t)nvec * nfull * sizeof(T), st));
    if (de.ndet == 0)
        return;
    k_embed<T><<<dim3((unsigned)ceil_div(de.ndet, 256), nvec), 256, 0, st>>>(de, nfull, sub, full);
    F2G_LAUNCH("k_embed");
}

template <typename T>
void blocks_extract(const DetEnum& de, int64_t nfull, const T* full, T* sub, int nvec, cudaStream_t st, bool add) {
    if (nvec <= 0 || de.ndet == 0)
        return;
    if (nvec > 65535)
        throw Error(2, "blocks_extract: at most 65535 vectors per call");
    k_extract<T><<<dim3((unsigned)ceil_div(de.ndet, 256), nvec), 256, 0, st>>>(de, nfull, full, sub, add ? 1 : 0);
    F2G_LAUNCH("k_extract");
}

template void blocks_embed<double>(const DetEnum&, int64_t, const double*, double*, int, cudaStream_t);
template void blocks_embed<float>(const DetEnum&, int64_t, const float*, float*, int, cudaStream_t);
template void blocks_embed<double2>(const DetEnum&, int64_t, const double2*, double2*, int, cudaStream_t);
template void blocks_extract<double2>(const DetEnum&, int64_t, const double2*, double2*, int, cudaStream_t, bool);
template void blocks_extract<double>(const DetEnum&, int64_t, const double*, double*, int, cudaStream_t, bool);
template void blocks_extract<float>(const DetEnum&, int64_t, const float*, float*, int, cudaStream_t, bool);

} // namespace f2g
