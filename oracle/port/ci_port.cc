// Oracle: CPU restatement of the reference's determinant-CI sigma path (test
// infrastructure only; the GPU product never links or calls it).
//
// It restates, for a CAS space in C1 symmetry (one GAS space, one determinant block):
//   * string enumeration and addressing, forte2/ci/ci_strings_makers.cc:13-73 and
//     ci_string_address.cc:6-45 (address = rank of (b0, b1, ..., b_{n-1}) in
//     std::next_permutation order, i.e. lexicographic with false < true);
//   * 1-hole lists (ci_strings_makers.cc:163-241) and 2-hole lists (:243-274), grouped by the
//     hole string K with entries in ascending address of the full string I;
//   * the Harrison-Zarrabian sigma build: H0 (ci_sigma_builder.cc:220-222), H1_hz
//     (ci_sigma_builder_harrison_zarrabian.cc:14-108), H2_hz_same_spin (:110-195) and
//     H2_hz_opposite_spin (:197-308), with the K-block memory contract of
//     ci_sigma_builder_knowles_handy.cc:15-32 and the integral packing of
//     ci_sigma_builder.cc:102-185; dense products go through dgemm_ (oracle/blas_bridge.cc);
//   * Slater-rule determinant energies (determinant/slater_rules.cc:86-121) and the approximate
//     CSF diagonal (ci_sigma_builder.cc:317-370);
//   * the CSF spin adapter (determinant/ci_spin_adapter.cc:23-288): configurations in the order
//     of first appearance over determinants in address order, genealogical spin couplings,
//     Clebsch-Gordan overlaps and the creation-order sign; csf<->det transforms;
//   * reduced density matrices between two determinant vectors: spin-dependent and spin-free
//     1-RDMs (ci_sigma_builder_1rdm.cc:9-84), same-spin packed and mixed-spin 2-RDMs, the
//     spin-free 2-RDM and its cumulant (ci_sigma_builder_2rdm.cc:46-282), and the 3-RDMs
//     (same-spin packed, aab, abb, spin-free) and 3-cumulant (ci_sigma_builder_3rdm.cc:84-542).
//
// Work is spread over host threads (ORACLE_THREADS, default: all hardware threads) the way the
// reference's parallel_for_chunked does (forte2/helpers/parallel.h:140-166).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

extern "C" {
void dgemm_(const char* transA, const char* transB, const int* M, const int* N, const int* K,
            const double* alpha, const double* A, const int* lda, const double* B, const int* ldb,
            const double* beta, double* C, const int* ldc);
}

namespace {

thread_local std::string g_err;

int num_threads() {
    if (const char* e = std::getenv("ORACLE_THREADS")) {
        int n = std::atoi(e);
        if (n > 0)
            return n;
    }
    return std::max(1u, std::thread::hardware_concurrency());
}

template <typename F> void parallel_for(size_t n, F&& f) {
    const size_t nt = std::min<size_t>(num_threads(), n);
    if (nt <= 1 || n < 64) {
        if (n)
            f(size_t(0), n);
        return;
    }
    const size_t block = (n + nt - 1) / nt;
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t) {
        size_t b = t * block, e = std::min(n, b + block);
        if (b < e)
            th.emplace_back([&f, b, e]() { f(b, e); });
    }
    for (auto& x : th)
        x.join();
}

// Row-major C(m x n) = alpha A(m x k) B(k x n) + beta C, through column-major dgemm_ by swapping
// operands (forte2/helpers/blas.h:33-38).
void matmul(int m, int n, int k, double alpha, const double* a, const double* b, double beta,
            double* c) {
    if (m == 0 || n == 0 || k == 0)
        return;
    const char N = 'N';
    dgemm_(&N, &N, &n, &m, &k, &alpha, b, &n, a, &k, &beta, c, &n);
}

uint64_t binom(int n, int k) {
    if (k < 0 || k > n || n < 0)
        return 0;
    uint64_t r = 1;
    for (int i = 1; i <= k; ++i)
        r = r * (uint64_t)(n - k + i) / (uint64_t)i;
    return r;
}

inline int parity_below(uint64_t x, int p) { return __builtin_popcountll(x & ((uint64_t(1) << p) - 1)) & 1; }
inline double sgn(int parity) { return parity ? -1.0 : 1.0; }

// ---- strings -------------------------------------------------------------------------------

struct StringSpace {
    int n = 0, k = 0;        // orbitals, electrons
    std::vector<uint64_t> s; // strings in address order
    std::vector<std::vector<uint64_t>> C; // binomials C[a][b]

    void build(int norb, int nel) {
        n = norb;
        k = nel;
        s.clear();
        C.assign(n + 2, std::vector<uint64_t>(n + 2, 0));
        for (int a = 0; a <= n + 1; ++a)
            for (int b = 0; b <= n + 1; ++b)
                C[a][b] = binom(a, b);
        if (k < 0 || k > n)
            return;
        // next_permutation order over the bool sequence (b0..b_{n-1}) starting at 0..01..1
        std::vector<int> seq(n, 0);
        for (int i = n - k; i < n; ++i)
            seq[i] = 1;
        do {
            uint64_t m = 0;
            for (int i = 0; i < n; ++i)
                if (seq[i])
                    m |= uint64_t(1) << i;
            s.push_back(m);
        } while (std::next_permutation(seq.begin(), seq.end()));
    }
    size_t size() const { return s.size(); }
    // lexicographic rank of (b0..b_{n-1}): each set bit at position i contributes the number of
    // sequences with the same prefix and a 0 at i, C(n-i-1, ones still to place).
    uint64_t rank(uint64_t m) const {
        uint64_t r = 0;
        int left = k;
        for (int i = 0; i < n && left > 0; ++i) {
            if (m >> i & 1) {
                r += C[n - i - 1][left];
                --left;
            }
        }
        return r;
    }
};

struct H1E {
    int16_t sign, p;
    uint32_t I;
};
struct H2E {
    int16_t sign;
    uint8_t p, q;
    uint32_t I;
};

struct H3E {
    int16_t sign;
    uint8_t p, q, r;
    uint32_t I;
};

// 1-hole list grouped by K (N-1 electrons): entries in ascending address of I = K + p.
void make_1h(const StringSpace& S, const StringSpace& S1, std::vector<std::vector<H1E>>& L) {
    L.assign(S1.size(), {});
    if (S.k < 1)
        return;
    for (size_t I = 0; I < S.size(); ++I) {
        const uint64_t m = S.s[I];
        for (int p = 0; p < S.n; ++p) {
            if (!(m >> p & 1))
                continue;
            const uint64_t K = m & ~(uint64_t(1) << p);
            L[S1.rank(K)].push_back({(int16_t)(parity_below(m, p) ? -1 : 1), (int16_t)p, (uint32_t)I});
        }
    }
}

// 2-hole list grouped by K (N-2 electrons), p > q.
void make_2h(const StringSpace& S, const StringSpace& S2, std::vector<std::vector<H2E>>& L) {
    L.assign(S2.size(), {});
    if (S.k < 2)
        return;
    for (size_t I = 0; I < S.size(); ++I) {
        const uint64_t m = S.s[I];
        for (int q = 0; q < S.n; ++q) {
            for (int p = q + 1; p < S.n; ++p) {
                if (!((m >> p & 1) && (m >> q & 1)))
                    continue;
                const uint64_t J = m & ~(uint64_t(1) << q);
                const int qs = parity_below(J, q);
                const uint64_t K = J & ~(uint64_t(1) << p);
                const int ps = parity_below(K, p);
                L[S2.rank(K)].push_back({(int16_t)((qs ^ ps) ? -1 : 1), (uint8_t)p, (uint8_t)q, (uint32_t)I});
            }
        }
    }
}

// 3-hole list grouped by K (N-3 electrons), p > q > r; the sign removes r, then q, then p, each
// with (-1)^{#occupied below it} (ci_strings_makers.cc:276-318).
void make_3h(const StringSpace& S, const StringSpace& S3, std::vector<std::vector<H3E>>& L) {
    L.assign(S3.size(), {});
    if (S.k < 3)
        return;
    for (size_t I = 0; I < S.size(); ++I) {
        const uint64_t m = S.s[I];
        for (int r = 0; r < S.n; ++r)
            for (int q = r + 1; q < S.n; ++q)
                for (int p = q + 1; p < S.n; ++p) {
                    if (!((m >> p & 1) && (m >> q & 1) && (m >> r & 1)))
                        continue;
                    const uint64_t J1 = m & ~(uint64_t(1) << r);
                    const uint64_t J2 = J1 & ~(uint64_t(1) << q);
                    const uint64_t K = J2 & ~(uint64_t(1) << p);
                    const int neg = parity_below(m, r) ^ parity_below(J1, q) ^ parity_below(J2, p);
                    L[S3.rank(K)].push_back({(int16_t)(neg ? -1 : 1), (uint8_t)p, (uint8_t)q, (uint8_t)r, (uint32_t)I});
                }
    }
}

// ---- CSF spin adapter ----------------------------------------------------------------------

double clebsch_gordan(double twoS, double twoM, int dtwoS, double dtwoM) {
    if (dtwoS == 1)
        return std::sqrt(0.5 * (twoS + dtwoM * twoM) / twoS);
    if (dtwoS == -1)
        return -dtwoM * std::sqrt(0.5 * (twoS + 2. - dtwoM * twoM) / (twoS + 2.));
    return 0.0;
}

double csf_overlap(int N, const std::vector<int>& coupling, const std::vector<int>& occ) {
    double o = 1.0;
    int pi = 0, qi = 0;
    for (int i = 0; i < N; ++i) {
        const int dtwoS = 1 - 2 * coupling[i];
        const int dtwoM = 1 - 2 * occ[i];
        pi += dtwoS;
        qi += dtwoM;
        if (std::abs(qi) > pi)
            return 0.0;
        o *= clebsch_gordan(pi, qi, dtwoS, dtwoM);
    }
    return o;
}

std::vector<std::vector<int>> spin_couplings(int N, int twoS) {
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

std::vector<std::vector<int>> det_occupations(int N, int twoMs) {
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

struct SpinAdapter {
    int twoS = 0, twoMs = 0, norb = 0;
    std::vector<int64_t> bounds;  // ncsf + 1
    std::vector<int64_t> det_idx; // ncoupling
    std::vector<double> coeff;
    std::vector<int64_t> conf_ranges; // 2 * nconf
    size_t ncsf() const { return bounds.empty() ? 0 : bounds.size() - 1; }
};

// ---- the sigma builder -----------------------------------------------------------------------

struct Port {
    int n = 0, na = 0, nb = 0;
    StringSpace A, B, A1, B1, A2, B2, A3, B3;
    std::vector<std::vector<H1E>> a1, b1;
    std::vector<std::vector<H2E>> a2, b2;
    std::vector<std::vector<H3E>> a3, b3; // built on first use (3-RDMs)
    bool lists3 = false;

    void build_3h() {
        if (lists3)
            return;
        A3.build(n, na - 3);
        B3.build(n, nb - 3);
        make_3h(A, A3, a3);
        make_3h(B, B3, b3);
        lists3 = true;
    }
    double E = 0.0;
    std::vector<double> h, V; // h[p*n+q], V[((p*n+q)*n+r)*n+s] physicist
    std::vector<double> v_pr_qs, v_pr_qs_a;
    size_t memory = size_t(1) << 30;
    double frac = 1.0; // fraction of K chunks processed (bounded timing samples)

    size_t ndet() const { return A.size() * B.size(); }

    void build_strings() {
        A.build(n, na);
        B.build(n, nb);
        A1.build(n, na - 1);
        B1.build(n, nb - 1);
        A2.build(n, na - 2);
        B2.build(n, nb - 2);
        make_1h(A, A1, a1);
        make_1h(B, B1, b1);
        make_2h(A, A2, a2);
        make_2h(B, B2, b2);
    }

    void set_hamiltonian(double E_, const double* H, const double* Vin) {
        E = E_;
        h.assign(H, H + n * n);
        V.assign(Vin, Vin + (size_t)n * n * n * n);
        const size_t n2 = (size_t)n * n, np = (size_t)n * (n - 1) / 2;
        v_pr_qs.assign(n2 * n2, 0.0);
        v_pr_qs_a.assign(np * np, 0.0);
        auto v = [&](int p, int q, int r, int s) { return V[(((size_t)p * n + q) * n + r) * n + s]; };
        for (int p = 0; p < n; ++p)
            for (int r = 0; r < n; ++r)
                for (int q = 0; q < n; ++q)
                    for (int s = 0; s < n; ++s)
                        v_pr_qs[(p * n + r) * n2 + q * n + s] = v(p, r, q, s);
        for (int p = 1; p < n; ++p)
            for (int r = 0; r < p; ++r)
                for (int q = 1; q < n; ++q)
                    for (int s = 0; s < q; ++s)
                        v_pr_qs_a[(p * (p - 1) / 2 + r) * np + q * (q - 1) / 2 + s] = v(p, r, q, s) - v(p, r, s, q);
    }

    size_t capacity(size_t nrows, size_t ncols) const {
        const size_t maxel = memory / (2 * sizeof(double));
        if (maxel < nrows)
            throw std::runtime_error("The CI builder memory limit (" + std::to_string(memory) +
                                     " bytes) is too small for one K-block column of " +
                                     std::to_string(nrows) + " elements per buffer.");
        return std::min({maxel / nrows, ncols, (size_t)2147483647});
    }

    // number of K strings processed in a bounded timing sample (all of them when frac >= 1)
    size_t chunk_limit(size_t maxK, size_t /*chunk*/) const {
        if (frac >= 1.0)
            return maxK;
        return std::min(maxK, std::max<size_t>(1, (size_t)std::llround(frac * (double)maxK)));
    }

    // C (rows x cols) -> T (cols x rows)
    static void transpose(const double* c, double* t, size_t rows, size_t cols) {
        parallel_for(rows, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i)
                for (size_t j = 0; j < cols; ++j)
                    t[j * rows + i] = c[i * cols + j];
        });
    }

    // One-electron term for one spin on a (rows = strings of this spin) x L matrix tr.
    void h1(const double* tr, double* tl, size_t NI, size_t L, const StringSpace& K1,
            const std::vector<std::vector<H1E>>& lst, int nel) {
        std::fill(tl, tl + NI * L, 0.0);
        if (nel < 1 || L == 0)
            return;
        const size_t maxK = K1.size();
        const size_t chunk = capacity((size_t)n * L, maxK);
        const size_t Kend = chunk_limit(maxK, chunk);
        std::vector<double> D, Eb;
        for (size_t K0 = 0; K0 < Kend; K0 += chunk) {
            const size_t Ks = std::min(chunk, Kend - K0), dimKL = Ks * L;
            D.assign((size_t)n * dimKL, 0.0);
            Eb.assign((size_t)n * dimKL, 0.0);
            parallel_for(Ks, [&](size_t b, size_t e) {
                for (size_t K = b; K < e; ++K)
                    for (const auto& x : lst[K0 + K]) {
                        double* d = &D[x.p * dimKL + K * L];
                        const double* c = &tr[(size_t)x.I * L];
                        for (size_t l = 0; l < L; ++l)
                            d[l] += x.sign * c[l];
                    }
            });
            matmul(n, (int)dimKL, n, 1.0, h.data(), D.data(), 0.0, Eb.data());
            // owner-writes over column ranges of L
            parallel_for(L, [&](size_t lb, size_t le) {
                for (size_t K = 0; K < Ks; ++K)
                    for (const auto& x : lst[K0 + K]) {
                        const double* e = &Eb[x.p * dimKL + K * L];
                        double* t = &tl[(size_t)x.I * L];
                        for (size_t l = lb; l < le; ++l)
                            t[l] += x.sign * e[l];
                    }
            });
        }
    }

    void h2_same(const double* tr, double* tl, size_t NI, size_t L, const StringSpace& K2,
                 const std::vector<std::vector<H2E>>& lst, int nel) {
        std::fill(tl, tl + NI * L, 0.0);
        if (nel < 2 || L == 0)
            return;
        const size_t np = (size_t)n * (n - 1) / 2, maxK = K2.size();
        const size_t chunk = capacity(np * L, maxK);
        const size_t Kend = chunk_limit(maxK, chunk);
        std::vector<double> D, Eb;
        for (size_t K0 = 0; K0 < Kend; K0 += chunk) {
            const size_t Ks = std::min(chunk, Kend - K0), dimKL = Ks * L;
            D.assign(np * dimKL, 0.0);
            Eb.assign(np * dimKL, 0.0);
            parallel_for(Ks, [&](size_t b, size_t e) {
                for (size_t K = b; K < e; ++K)
                    for (const auto& x : lst[K0 + K]) {
                        double* d = &D[(size_t)(x.p * (x.p - 1) / 2 + x.q) * dimKL + K * L];
                        const double* c = &tr[(size_t)x.I * L];
                        for (size_t l = 0; l < L; ++l)
                            d[l] += x.sign * c[l];
                    }
            });
            matmul((int)np, (int)dimKL, (int)np, 1.0, v_pr_qs_a.data(), D.data(), 0.0, Eb.data());
            parallel_for(L, [&](size_t lb, size_t le) {
                for (size_t K = 0; K < Ks; ++K)
                    for (const auto& x : lst[K0 + K]) {
                        const double* e = &Eb[(size_t)(x.p * (x.p - 1) / 2 + x.q) * dimKL + K * L];
                        double* t = &tl[(size_t)x.I * L];
                        for (size_t l = lb; l < le; ++l)
                            t[l] += x.sign * e[l];
                    }
            });
        }
    }

    void h2_opposite(const double* c, double* sigma) {
        if (na < 1 || nb < 1)
            return;
        const size_t n2 = (size_t)n * n, maxKa = A1.size(), maxKb = B1.size(), NIb = B.size();
        const size_t chunk = capacity(n2 * maxKb, maxKa);
        const size_t Kend = chunk_limit(maxKa, chunk);
        std::vector<double> D, Eb;
        for (size_t Ka0 = 0; Ka0 < Kend; Ka0 += chunk) {
            const size_t Kas = std::min(chunk, Kend - Ka0), Kdim = Kas * maxKb;
            D.assign(n2 * Kdim, 0.0);
            Eb.assign(n2 * Kdim, 0.0);
            parallel_for(Kas, [&](size_t b, size_t e) {
                for (size_t Ka = b; Ka < e; ++Ka)
                    for (size_t Kb = 0; Kb < maxKb; ++Kb) {
                        const size_t Kidx = Ka * maxKb + Kb;
                        for (const auto& xa : a1[Ka0 + Ka])
                            for (const auto& xb : b1[Kb])
                                D[(xa.p * n + xb.p) * Kdim + Kidx] =
                                    xa.sign * xb.sign * c[(size_t)xa.I * NIb + xb.I];
                    }
            });
            matmul((int)n2, (int)Kdim, (int)n2, 1.0, v_pr_qs.data(), D.data(), 0.0, Eb.data());
            // owner-writes over stripes of output alpha strings (hz.cc:278-303)
            parallel_for(A.size(), [&](size_t ib, size_t ie) {
                for (size_t Ka = 0; Ka < Kas; ++Ka)
                    for (const auto& xa : a1[Ka0 + Ka]) {
                        if (xa.I < ib || xa.I >= ie)
                            continue;
                        double* s = &sigma[(size_t)xa.I * NIb];
                        for (size_t Kb = 0; Kb < maxKb; ++Kb)
                            for (const auto& xb : b1[Kb])
                                s[xb.I] += xa.sign * xb.sign * Eb[(xa.p * n + xb.p) * Kdim + Ka * maxKb + Kb];
                    }
            });
        }
    }

    // term mask bits: 1 H0, 2 H1a, 4 H1b, 8 aabb, 16 aaaa, 32 bbbb
    void sigma_terms(const double* c, double* sigma, int mask) {
        const size_t NA = A.size(), NB = B.size(), nd = NA * NB;
        std::fill(sigma, sigma + nd, 0.0);
        if (nd == 0)
            return;
        if (mask & 1)
            for (size_t i = 0; i < nd; ++i)
                sigma[i] += E * c[i];
        std::vector<double> tl(nd), ct, tlt;
        if (mask & 2) {
            h1(c, tl.data(), NA, NB, A1, a1, na);
            for (size_t i = 0; i < nd; ++i)
                sigma[i] += tl[i];
        }
        const bool need_t = (mask & (4 | 32)) && nb >= 1;
        if (need_t) {
            ct.resize(nd);
            tlt.resize(nd);
            transpose(c, ct.data(), NA, NB);
        }
        if ((mask & 4) && nb >= 1) {
            h1(ct.data(), tlt.data(), NB, NA, B1, b1, nb);
            transpose(tlt.data(), tl.data(), NB, NA);
            for (size_t i = 0; i < nd; ++i)
                sigma[i] += tl[i];
        }
        if (mask & 8)
            h2_opposite(c, sigma);
        if ((mask & 16) && na >= 2) {
            h2_same(c, tl.data(), NA, NB, A2, a2, na);
            for (size_t i = 0; i < nd; ++i)
                sigma[i] += tl[i];
        }
        if ((mask & 32) && nb >= 2) {
            h2_same(ct.data(), tlt.data(), NB, NA, B2, b2, nb);
            transpose(tlt.data(), tl.data(), NB, NA);
            for (size_t i = 0; i < nd; ++i)
                sigma[i] += tl[i];
        }
    }

    // Slater determinant energy (slater_rules.cc:86-121)
    double det_energy(uint64_t a, uint64_t b) const {
        double e = E;
        auto J = [&](int p, int q) { return V[(((size_t)p * n + q) * n + p) * n + q]; };
        auto K = [&](int p, int q) { return V[(((size_t)p * n + q) * n + q) * n + p]; };
        for (int p = 0; p < n; ++p) {
            if (!(a >> p & 1))
                continue;
            e += h[p * n + p];
            for (int q = 0; q < p; ++q)
                if (a >> q & 1)
                    e += J(q, p) - K(q, p);
            for (int q = 0; q < n; ++q)
                if (b >> q & 1)
                    e += J(p, q);
        }
        for (int p = 0; p < n; ++p) {
            if (!(b >> p & 1))
                continue;
            e += h[p * n + p];
            for (int q = 0; q < p; ++q)
                if (b >> q & 1)
                    e += J(q, p) - K(q, p);
        }
        return e;
    }

    void prepare_csf(SpinAdapter& sa) {
        const size_t NA = A.size(), NB = B.size();
        // configurations in order of first appearance over determinants in address order
        std::unordered_map<uint64_t, int64_t> seen; // key: docc | socc << 32 (n <= 32 here)
        std::vector<std::pair<uint64_t, uint64_t>> confs;
        if (n > 32)
            throw std::runtime_error("oracle port supports at most 32 orbitals");
        for (size_t ia = 0; ia < NA; ++ia)
            for (size_t ib = 0; ib < NB; ++ib) {
                const uint64_t a = A.s[ia], b = B.s[ib];
                const uint64_t d = a & b, s = a ^ b;
                if (__builtin_popcountll(s) < sa.twoS)
                    continue;
                const uint64_t key = d | (s << 32);
                if (seen.emplace(key, (int64_t)confs.size()).second)
                    confs.emplace_back(d, s);
            }
        std::vector<std::vector<std::vector<int>>> cpl(n + 1), occ(n + 1);
        std::vector<std::vector<std::vector<double>>> ovl(n + 1);
        sa.bounds.assign(1, 0);
        sa.det_idx.clear();
        sa.coeff.clear();
        sa.conf_ranges.clear();
        for (const auto& [d, s] : confs) {
            const int N = __builtin_popcountll(s);
            if (cpl[N].empty() && occ[N].empty()) {
                cpl[N] = spin_couplings(N, sa.twoS);
                occ[N] = det_occupations(N, sa.twoMs);
                ovl[N].assign(cpl[N].size(), std::vector<double>(occ[N].size()));
                for (size_t i = 0; i < cpl[N].size(); ++i)
                    for (size_t j = 0; j < occ[N].size(); ++j)
                        ovl[N][i][j] = csf_overlap(N, cpl[N][i], occ[N][j]);
            }
            std::vector<int> socc;
            for (int p = 0; p < n; ++p)
                if (s >> p & 1)
                    socc.push_back(p);
            const int64_t first = (int64_t)sa.ncsf();
            for (size_t i = 0; i < cpl[N].size(); ++i) {
                for (size_t j = 0; j < occ[N].size(); ++j) {
                    const double o = ovl[N][i][j];
                    if (!(std::fabs(o) > 0.0))
                        continue;
                    uint64_t a = d, b = d;
                    double sign = 1.0;
                    for (int k = N - 1; k >= 0; --k) {
                        const int p = socc[k];
                        if (occ[N][j][k]) {
                            sign *= sgn((__builtin_popcountll(a) + parity_below(b, p)) & 1);
                            b |= uint64_t(1) << p;
                        } else {
                            sign *= sgn(parity_below(a, p));
                            a |= uint64_t(1) << p;
                        }
                    }
                    sa.det_idx.push_back((int64_t)(A.rank(a) * NB + B.rank(b)));
                    sa.coeff.push_back(sign * o);
                }
                sa.bounds.push_back((int64_t)sa.det_idx.size());
            }
            sa.conf_ranges.push_back(first);
            sa.conf_ranges.push_back((int64_t)sa.ncsf());
        }
    }
};


// ---- reduced density matrices -----------------------------------------------------------------
//
// Restated from the reference's RDM builders (forte2/ci/ci_sigma_builder_1rdm.cc:9-84 and
// ci_sigma_builder_2rdm.cc:46-282) for one CAS block. A determinant vector holds C(Ia, Ib) at
// Ia * NB + Ib; the spin-s "row" of string I is row I of C for alpha and column I for beta.

// Sum over items [0, n) of per-item contributions into an accumulator of `size` doubles: each
// host thread fills its own buffer, and the buffers are added in thread order (deterministic).
template <typename F> std::vector<double> parallel_sum(size_t n, size_t size, F&& f) {
    const size_t nt = std::max<size_t>(1, std::min<size_t>(num_threads(), n));
    std::vector<std::vector<double>> part(nt, std::vector<double>(size, 0.0));
    const size_t block = n ? (n + nt - 1) / nt : 0;
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t) {
        const size_t b = t * block, e = std::min(n, b + block);
        if (b < e)
            th.emplace_back([&f, &part, t, b, e]() { f(b, e, part[t].data()); });
    }
    for (auto& x : th)
        x.join();
    std::vector<double> out(size, 0.0);
    for (size_t t = 0; t < nt; ++t)
        for (size_t i = 0; i < size; ++i)
            out[i] += part[t][i];
    return out;
}

struct RdmPort {
    const Port& P;
    const double* CL;
    const double* CR;

    // bounded timing samples: only the first fraction P.frac of the hole strings contribute
    size_t items(size_t n) const {
        if (P.frac >= 1.0 || n == 0)
            return n;
        return std::max<size_t>(1, (size_t)std::ceil(P.frac * (double)n));
    }

    size_t NA() const { return P.A.size(); }
    size_t NB() const { return P.B.size(); }
    // <left row I | right row J> over the other spin's strings
    double dot(int spin, size_t I, size_t J) const {
        double acc = 0.0;
        if (spin == 0) {
            const double* a = CL + I * NB();
            const double* b = CR + J * NB();
            for (size_t L = 0; L < NB(); ++L)
                acc += a[L] * b[L];
        } else {
            for (size_t L = 0; L < NA(); ++L)
                acc += CL[L * NB() + I] * CR[L * NB() + J];
        }
        return acc;
    }

    // gamma[p][q] = <L| a+_p a_q |R> for one spin: every string I of the right vector, every
    // occupied q and every p empty in I - q (p = q included) gives J = I - q + p with the sign
    // of a_q on I times the sign of a+_p on I - q (ci_strings_makers.cc:75-110).
    std::vector<double> one(int spin) const {
        const int n = P.n;
        const StringSpace& S = spin == 0 ? P.A : P.B;
        if (S.k < 1 || n < 1)
            return std::vector<double>((size_t)n * n, 0.0);
        return parallel_sum(items(S.size()), (size_t)n * n, [&](size_t b, size_t e, double* g) {
            for (size_t I = b; I < e; ++I) {
                const uint64_t mI = S.s[I];
                for (int q = 0; q < n; ++q) {
                    if (!(mI >> q & 1))
                        continue;
                    const uint64_t mK = mI & ~(uint64_t(1) << q);
                    for (int p = 0; p < n; ++p) {
                        if (mK >> p & 1)
                            continue;
                        const uint64_t mJ = mK | (uint64_t(1) << p);
                        const double sign = sgn(parity_below(mI, q) ^ parity_below(mK, p));
                        g[p * n + q] += sign * dot(spin, S.rank(mJ), I);
                    }
                }
            }
        });
    }

    // gamma[pq][rs] (p > q, r > s, pair index p(p-1)/2 + q) = sum over 2-hole strings K of
    // sign(K; p, q) sign(K; r, s) <row K+p+q | row K+r+s> (ci_sigma_builder_2rdm.cc:46-117).
    std::vector<double> same_spin(int spin) const {
        const int n = P.n;
        const size_t np = n >= 2 ? (size_t)n * (n - 1) / 2 : 0;
        const auto& L2 = spin == 0 ? P.a2 : P.b2;
        const StringSpace& S = spin == 0 ? P.A : P.B;
        if (S.k < 2 || np == 0)
            return std::vector<double>(np * np, 0.0);
        return parallel_sum(items(L2.size()), np * np, [&](size_t b, size_t e, double* g) {
            for (size_t K = b; K < e; ++K) {
                for (const auto& l : L2[K]) {
                    const size_t pq = (size_t)l.p * (l.p - 1) / 2 + l.q;
                    for (const auto& r : L2[K]) {
                        const size_t rs = (size_t)r.p * (r.p - 1) / 2 + r.q;
                        g[pq * np + rs] += l.sign * r.sign * dot(spin, l.I, r.I);
                    }
                }
            }
        });
    }

    // gamma[u][v][x][y] = sum over 1-hole strings Ka, Kb of
    // s(Ka,u) s(Kb,v) CL(Ka+u, Kb+v) s(Ka,x) s(Kb,y) CR(Ka+x, Kb+y) (ci_sigma_builder_2rdm.cc:119-201).
    std::vector<double> mixed() const {
        const size_t n = P.n, n4 = n * n * n * n;
        if (P.na < 1 || P.nb < 1 || n < 1)
            return std::vector<double>(n4, 0.0);
        const size_t nb = NB();
        return parallel_sum(items(P.a1.size()), n4, [&](size_t b, size_t e, double* g) {
            for (size_t Ka = b; Ka < e; ++Ka) {
                for (const auto& u : P.a1[Ka]) {
                    for (const auto& x : P.a1[Ka]) {
                        const double sa = u.sign * x.sign;
                        const double* rl = CL + (size_t)u.I * nb;
                        const double* rr = CR + (size_t)x.I * nb;
                        double* gux = g + (size_t)u.p * n * n * n + (size_t)x.p * n;
                        for (const auto& Kb : P.b1) {
                            for (const auto& v : Kb) {
                                const double lv = sa * v.sign * rl[v.I];
                                for (const auto& y : Kb)
                                    gux[(size_t)v.p * n * n + y.p] += lv * y.sign * rr[y.I];
                            }
                        }
                    }
                }
            }
        });
    }

    // spin-free 2-RDM: ab(p,q,r,s) + ab(q,p,s,r) plus the antisymmetric expansion of aa + bb
    // (ci_sigma_builder_2rdm.cc:203-250)
    std::vector<double> spin_free2() const {
        const size_t n = P.n;
        std::vector<double> sf(n * n * n * n, 0.0);
        if (n < 1)
            return sf;
        const auto ab = mixed();
        auto at = [n](size_t p, size_t q, size_t r, size_t s) { return ((p * n + q) * n + r) * n + s; };
        for (size_t p = 0; p < n; ++p)
            for (size_t q = 0; q < n; ++q)
                for (size_t r = 0; r < n; ++r)
                    for (size_t s = 0; s < n; ++s)
                        sf[at(p, q, r, s)] = ab[at(p, q, r, s)] + ab[at(q, p, s, r)];
        if (n < 2)
            return sf;
        const size_t np = n * (n - 1) / 2;
        for (int spin = 0; spin < 2; ++spin) {
            const auto ss = same_spin(spin);
            for (size_t p = 1; p < n; ++p)
                for (size_t q = 0; q < p; ++q)
                    for (size_t r = 1; r < n; ++r)
                        for (size_t s = 0; s < r; ++s) {
                            const double e = ss[(p * (p - 1) / 2 + q) * np + r * (r - 1) / 2 + s];
                            sf[at(p, q, r, s)] += e;
                            sf[at(q, p, r, s)] -= e;
                            sf[at(p, q, s, r)] -= e;
                            sf[at(q, p, s, r)] += e;
                        }
        }
        return sf;
    }

    // ---- 3-RDMs (ci_sigma_builder_3rdm.cc:84-542); P.build_3h() must have run ----

    // gamma[pqr][stu] (p > q > r, s > t > u, triplet index p(p-1)(p-2)/6 + q(q-1)/2 + r) =
    // sum over 3-hole strings K of sign(K; p,q,r) sign(K; s,t,u) <row K+p+q+r | row K+s+t+u>
    std::vector<double> same_spin3(int spin) const {
        const int n = P.n;
        const size_t nt = n >= 3 ? (size_t)n * (n - 1) * (n - 2) / 6 : 0;
        const auto& L3 = spin == 0 ? P.a3 : P.b3;
        const StringSpace& S = spin == 0 ? P.A : P.B;
        if (S.k < 3 || nt == 0)
            return std::vector<double>(nt * nt, 0.0);
        auto tri = [](size_t p, size_t q, size_t r) { return p * (p - 1) * (p - 2) / 6 + q * (q - 1) / 2 + r; };
        return parallel_sum(items(L3.size()), nt * nt, [&](size_t b, size_t e, double* g) {
            for (size_t K = b; K < e; ++K)
                for (const auto& l : L3[K])
                    for (const auto& r : L3[K])
                        g[tri(l.p, l.q, l.r) * nt + tri(r.p, r.q, r.r)] += l.sign * r.sign * dot(spin, l.I, r.I);
        });
    }

    // gamma[pq][r][st][u] (alpha pairs p > q, s > t; beta r, u) = sum over 2-hole alpha strings Ka
    // and 1-hole beta strings Kb of s(Ka;p,q) s(Kb,r) CL(Ka+p+q, Kb+r) s(Ka;s,t) s(Kb,u) CR(Ka+s+t, Kb+u)
    std::vector<double> aab() const {
        const size_t n = P.n, np = n >= 2 ? n * (n - 1) / 2 : 0, M = np * n;
        if (P.na < 2 || P.nb < 1 || n < 2)
            return std::vector<double>(M * M, 0.0);
        const size_t nb = NB();
        return parallel_sum(items(P.a2.size()), M * M, [&](size_t b, size_t e, double* g) {
            for (size_t Ka = b; Ka < e; ++Ka)
                for (const auto& l : P.a2[Ka])
                    for (const auto& r : P.a2[Ka]) {
                        const double sa = l.sign * r.sign;
                        const double* rl = CL + (size_t)l.I * nb;
                        const double* rr = CR + (size_t)r.I * nb;
                        const size_t row = ((size_t)l.p * (l.p - 1) / 2 + l.q) * n;
                        const size_t col = ((size_t)r.p * (r.p - 1) / 2 + r.q) * n;
                        for (const auto& Kb : P.b1)
                            for (const auto& v : Kb) {
                                const double lv = sa * v.sign * rl[v.I];
                                for (const auto& y : Kb)
                                    g[(row + v.p) * M + col + y.p] += lv * y.sign * rr[y.I];
                            }
                    }
        });
    }

    // gamma[p][qr][s][tu] (alpha p, s; beta pairs q > r, t > u) over 1-hole alpha and 2-hole beta
    std::vector<double> abb() const {
        const size_t n = P.n, np = n >= 2 ? n * (n - 1) / 2 : 0, M = n * np;
        if (P.na < 1 || P.nb < 2 || n < 2)
            return std::vector<double>(M * M, 0.0);
        const size_t nb = NB();
        return parallel_sum(items(P.a1.size()), M * M, [&](size_t b, size_t e, double* g) {
            for (size_t Ka = b; Ka < e; ++Ka)
                for (const auto& l : P.a1[Ka])
                    for (const auto& r : P.a1[Ka]) {
                        const double sa = l.sign * r.sign;
                        const double* rl = CL + (size_t)l.I * nb;
                        const double* rr = CR + (size_t)r.I * nb;
                        for (const auto& Kb : P.b2)
                            for (const auto& v : Kb) {
                                const double lv = sa * v.sign * rl[v.I];
                                const size_t row = (size_t)l.p * np + (size_t)v.p * (v.p - 1) / 2 + v.q;
                                for (const auto& y : Kb)
                                    g[row * M + (size_t)r.p * np + (size_t)y.p * (y.p - 1) / 2 + y.q] +=
                                        lv * y.sign * rr[y.I];
                            }
                    }
        });
    }

    // spin-free 3-RDM G3[p][q][r][s][t][u] = sum over spins of <a+_p a+_q a+_r a_u a_t a_s>: the
    // same-spin blocks with all permutation signs, and each mixed block in its three placements of
    // the odd spin (ci_sigma_builder_3rdm.cc:320-497)
    std::vector<double> spin_free3() const {
        const size_t n = P.n;
        const size_t n6 = n * n * n * n * n * n;
        std::vector<double> sf(n6, 0.0);
        if (n < 2)
            return sf;
        auto at = [n](size_t a, size_t b, size_t c, size_t d, size_t e, size_t f) {
            return ((((a * n + b) * n + c) * n + d) * n + e) * n + f;
        };
        const size_t np = n * (n - 1) / 2;
        // pair variants (x, y, sign): (hi, lo, +1) and (lo, hi, -1)
        auto variants = [](size_t hi, size_t lo, size_t* x, size_t* y, double* sg) {
            x[0] = hi, y[0] = lo, sg[0] = 1.0;
            x[1] = lo, y[1] = hi, sg[1] = -1.0;
        };
        const auto g_aab = aab();
        for (size_t p = 1; p < n; ++p)
            for (size_t q = 0; q < p; ++q)
                for (size_t r = 0; r < n; ++r)
                    for (size_t s = 1; s < n; ++s)
                        for (size_t t = 0; t < s; ++t)
                            for (size_t u = 0; u < n; ++u) {
                                const double el = g_aab[(((p * (p - 1) / 2 + q) * n + r) * np + s * (s - 1) / 2 + t) * n + u];
                                size_t a1[2], a2[2], b1[2], b2[2];
                                double sa[2], sb[2];
                                variants(p, q, a1, a2, sa);
                                variants(s, t, b1, b2, sb);
                                for (int i = 0; i < 2; ++i)
                                    for (int j = 0; j < 2; ++j) {
                                        const double v = sa[i] * sb[j] * el;
                                        sf[at(a1[i], a2[i], r, b1[j], b2[j], u)] += v; // beta third
                                        sf[at(a1[i], r, a2[i], b1[j], u, b2[j])] += v; // beta second
                                        sf[at(r, a1[i], a2[i], u, b1[j], b2[j])] += v; // beta first
                                    }
                            }
        const auto g_abb = abb();
        for (size_t p = 0; p < n; ++p)
            for (size_t q = 1; q < n; ++q)
                for (size_t r = 0; r < q; ++r)
                    for (size_t s = 0; s < n; ++s)
                        for (size_t t = 1; t < n; ++t)
                            for (size_t u = 0; u < t; ++u) {
                                const double el = g_abb[((p * np + q * (q - 1) / 2 + r) * n + s) * np + t * (t - 1) / 2 + u];
                                size_t a1[2], a2[2], b1[2], b2[2];
                                double sa[2], sb[2];
                                variants(q, r, a1, a2, sa);
                                variants(t, u, b1, b2, sb);
                                for (int i = 0; i < 2; ++i)
                                    for (int j = 0; j < 2; ++j) {
                                        const double v = sa[i] * sb[j] * el;
                                        sf[at(p, a1[i], a2[i], s, b1[j], b2[j])] += v; // alpha first
                                        sf[at(a1[i], p, a2[i], b1[j], s, b2[j])] += v; // alpha second
                                        sf[at(a1[i], a2[i], p, b1[j], b2[j], s)] += v; // alpha third
                                    }
                            }
        if (n < 3)
            return sf;
        const size_t nt = n * (n - 1) * (n - 2) / 6;
        // the six orderings of a triple (x, y, z) = (0, 1, 2) with their permutation signs
        const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {2, 0, 1}, {2, 1, 0}, {1, 2, 0}, {1, 0, 2}};
        const double psign[6] = {1, -1, 1, -1, 1, -1};
        for (int spin = 0; spin < 2; ++spin) {
            const auto g = same_spin3(spin);
            for (size_t p = 2, pqr = 0; p < n; ++p)
                for (size_t q = 1; q < p; ++q)
                    for (size_t r = 0; r < q; ++r, ++pqr)
                        for (size_t s = 2, stu = 0; s < n; ++s)
                            for (size_t t = 1; t < s; ++t)
                                for (size_t u = 0; u < t; ++u, ++stu) {
                                    const double el = g[pqr * nt + stu];
                                    const size_t bra[3] = {p, q, r}, ket[3] = {s, t, u};
                                    for (int i = 0; i < 6; ++i)
                                        for (int j = 0; j < 6; ++j)
                                            sf[at(bra[perm[i][0]], bra[perm[i][1]], bra[perm[i][2]], ket[perm[j][0]],
                                                  ket[perm[j][1]], ket[perm[j][2]])] += psign[i] * psign[j] * el;
                                }
        }
        return sf;
    }
};

} // namespace

extern "C" {

const char* port_last_error() { return g_err.c_str(); }

void* port_new(int norb, int na, int nb) {
    try {
        auto* p = new Port();
        p->n = norb;
        p->na = na;
        p->nb = nb;
        p->build_strings();
        return p;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void port_free(void* h) { delete static_cast<Port*>(h); }

/// out: nas, nbs, ndet, n1a, n1b, n2a, n2b
void port_info(void* h, int64_t* out) {
    auto* p = static_cast<Port*>(h);
    out[0] = p->A.size();
    out[1] = p->B.size();
    out[2] = p->ndet();
    out[3] = p->A1.size();
    out[4] = p->B1.size();
    out[5] = p->A2.size();
    out[6] = p->B2.size();
}

void port_strings(void* h, int spin, uint64_t* out) {
    auto* p = static_cast<Port*>(h);
    const auto& S = spin == 0 ? p->A : p->B;
    std::copy(S.s.begin(), S.s.end(), out);
}

/// Rows (0, K, 0, sign, p, I) in the reference's list order; returns the count.
int64_t port_1h(void* h, int spin, int32_t* out) {
    auto* p = static_cast<Port*>(h);
    const auto& L = spin == 0 ? p->a1 : p->b1;
    int64_t k = 0;
    for (size_t K = 0; K < L.size(); ++K)
        for (const auto& x : L[K]) {
            if (out) {
                int32_t* r = out + 6 * k;
                r[0] = 0;
                r[1] = (int32_t)K;
                r[2] = 0;
                r[3] = x.sign;
                r[4] = x.p;
                r[5] = (int32_t)x.I;
            }
            ++k;
        }
    return k;
}

int64_t port_2h(void* h, int spin, int32_t* out) {
    auto* p = static_cast<Port*>(h);
    const auto& L = spin == 0 ? p->a2 : p->b2;
    int64_t k = 0;
    for (size_t K = 0; K < L.size(); ++K)
        for (const auto& x : L[K]) {
            if (out) {
                int32_t* r = out + 7 * k;
                r[0] = 0;
                r[1] = (int32_t)K;
                r[2] = 0;
                r[3] = x.sign;
                r[4] = x.p;
                r[5] = x.q;
                r[6] = (int32_t)x.I;
            }
            ++k;
        }
    return k;
}

void port_set_hamiltonian(void* h, double E, const double* H, const double* V) {
    static_cast<Port*>(h)->set_hamiltonian(E, H, V);
}

/// 0 ok, 2 invalid argument
int port_set_memory(void* h, int mb) {
    if (mb < 0) {
        g_err = "CI builder memory must be non-negative.";
        return 2;
    }
    static_cast<Port*>(h)->memory = (size_t)mb * 1024 * 1024;
    return 0;
}

void port_set_fraction(void* h, double frac) { static_cast<Port*>(h)->frac = frac; }

/// sigma = selected terms applied to c; 0 ok, 1 runtime error (message in port_last_error)
int port_sigma(void* h, const double* c, double* sigma, int mask) {
    try {
        static_cast<Port*>(h)->sigma_terms(c, sigma, mask);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

void port_det_energies(void* h, double* out) {
    auto* p = static_cast<Port*>(h);
    const size_t NB = p->B.size();
    parallel_for(p->A.size(), [&](size_t b, size_t e) {
        for (size_t ia = b; ia < e; ++ia)
            for (size_t ib = 0; ib < NB; ++ib)
                out[ia * NB + ib] = p->det_energy(p->A.s[ia], p->B.s[ib]);
    });
}

void* port_spin_adapter_new(void* h, int twoS, int twoMs) {
    try {
        auto* sa = new SpinAdapter();
        sa->twoS = twoS;
        sa->twoMs = twoMs;
        sa->norb = static_cast<Port*>(h)->n;
        static_cast<Port*>(h)->prepare_csf(*sa);
        return sa;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void port_spin_adapter_free(void* s) { delete static_cast<SpinAdapter*>(s); }

/// out: nconf, ncsf, ncoupling
void port_spin_adapter_info(void* s, int64_t* out) {
    auto* sa = static_cast<SpinAdapter*>(s);
    out[0] = sa->conf_ranges.size() / 2;
    out[1] = sa->ncsf();
    out[2] = sa->det_idx.size();
}

void port_spin_adapter_dump(void* s, int64_t* bounds, int64_t* det_idx, double* coeff, int64_t* ranges) {
    auto* sa = static_cast<SpinAdapter*>(s);
    std::copy(sa->bounds.begin(), sa->bounds.end(), bounds);
    std::copy(sa->det_idx.begin(), sa->det_idx.end(), det_idx);
    std::copy(sa->coeff.begin(), sa->coeff.end(), coeff);
    std::copy(sa->conf_ranges.begin(), sa->conf_ranges.end(), ranges);
}

void port_csf_to_det(void* s, const double* csf, double* det, int64_t ndet) {
    auto* sa = static_cast<SpinAdapter*>(s);
    std::fill(det, det + ndet, 0.0);
    for (size_t i = 0; i < sa->ncsf(); ++i)
        for (int64_t j = sa->bounds[i]; j < sa->bounds[i + 1]; ++j)
            det[sa->det_idx[j]] += sa->coeff[j] * csf[i];
}

void port_det_to_csf(void* s, const double* det, double* csf) {
    auto* sa = static_cast<SpinAdapter*>(s);
    parallel_for(sa->ncsf(), [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            double acc = 0.0;
            for (int64_t j = sa->bounds[i]; j < sa->bounds[i + 1]; ++j)
                acc += sa->coeff[j] * det[sa->det_idx[j]];
            csf[i] = acc;
        }
    });
}

/// Approximate CSF diagonal sum_j c_ij^2 E(det_j) (ci_sigma_builder.cc:331-368).
void port_hdiag_csf(void* h, void* s, double* out) {
    auto* p = static_cast<Port*>(h);
    auto* sa = static_cast<SpinAdapter*>(s);
    const size_t NB = p->B.size();
    parallel_for(sa->ncsf(), [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            double acc = 0.0;
            for (int64_t j = sa->bounds[i]; j < sa->bounds[i + 1]; ++j) {
                const int64_t d = sa->det_idx[j];
                const double c = sa->coeff[j];
                acc += c * c * p->det_energy(p->A.s[d / NB], p->B.s[d % NB]);
            }
            out[i] = acc;
        }
    });
}

/// Reduced density matrices between two determinant vectors (kinds as in the GPU library:
/// 0 a_1rdm, 1 b_1rdm, 2 sf_1rdm, 3 aa_2rdm, 4 bb_2rdm, 5 ab_2rdm, 6 sf_2rdm, 7 sf_2cumulant;
/// and 8 aaa_3rdm, 9 bbb_3rdm, 10 aab_3rdm, 11 abb_3rdm, 12 sf_3rdm, 13 sf_3cumulant).
/// Returns the number of doubles written to out, or -1 for an unknown kind.
int64_t port_rdm(void* h, int kind, const double* CL, const double* CR, double* out) {
    auto& P = *static_cast<Port*>(h);
    if (kind >= 8)
        P.build_3h();
    RdmPort R{P, CL, CR};
    const size_t n = P.n;
    std::vector<double> r;
    switch (kind) {
    case 0: r = R.one(0); break;
    case 1: r = R.one(1); break;
    case 2: {
        r = R.one(0);
        const auto b = R.one(1);
        for (size_t i = 0; i < r.size(); ++i)
            r[i] += b[i];
        break;
    }
    case 3: r = R.same_spin(0); break;
    case 4: r = R.same_spin(1); break;
    case 5: r = R.mixed(); break;
    case 6: r = R.spin_free2(); break;
    case 7: {
        // L2[p,q,r,s] = G2[p,q,r,s] - G1[p,r] G1[q,s] + G1[p,s] G1[q,r] / 2
        // (ci_sigma_builder_2rdm.cc:252-278)
        r = R.spin_free2();
        auto g1 = R.one(0);
        const auto b = R.one(1);
        for (size_t i = 0; i < g1.size(); ++i)
            g1[i] += b[i];
        for (size_t p = 0; p < n; ++p)
            for (size_t q = 0; q < n; ++q)
                for (size_t a = 0; a < n; ++a)
                    for (size_t s = 0; s < n; ++s)
                        r[((p * n + q) * n + a) * n + s] +=
                            -g1[p * n + a] * g1[q * n + s] + 0.5 * g1[p * n + s] * g1[q * n + a];
        break;
    }
    case 8: r = R.same_spin3(0); break;
    case 9: r = R.same_spin3(1); break;
    case 10: r = R.aab(); break;
    case 11: r = R.abb(); break;
    case 12: r = R.spin_free3(); break;
    case 13: {
        // spin-free 3-cumulant (ci_sigma_builder_3rdm.cc:499-540): G3 minus the products of
        // G1 with G2 and of three G1 that the cumulant expansion removes
        r = R.spin_free3();
        if (n < 2)
            break;
        auto g1 = R.one(0);
        const auto b1 = R.one(1);
        for (size_t i = 0; i < g1.size(); ++i)
            g1[i] += b1[i];
        const auto g2 = R.spin_free2();
        auto G1 = [&](size_t a, size_t b) { return g1[a * n + b]; };
        auto G2 = [&](size_t a, size_t b, size_t c, size_t d) { return g2[((a * n + b) * n + c) * n + d]; };
        size_t i = 0;
        for (size_t p = 0; p < n; ++p)
            for (size_t q = 0; q < n; ++q)
                for (size_t a = 0; a < n; ++a)
                    for (size_t s = 0; s < n; ++s)
                        for (size_t t = 0; t < n; ++t)
                            for (size_t u = 0; u < n; ++u, ++i) {
                                double v = -G1(p, s) * G2(q, a, t, u) - G1(q, t) * G2(p, a, s, u) - G1(a, u) * G2(p, q, s, t);
                                v += 0.5 * (G1(p, t) * G2(q, a, s, u) + G1(p, u) * G2(q, a, t, s) + G1(q, s) * G2(p, a, t, u) +
                                            G1(q, u) * G2(p, a, s, t) + G1(a, s) * G2(p, q, u, t) + G1(a, t) * G2(p, q, s, u));
                                v += 2.0 * G1(p, s) * G1(q, t) * G1(a, u) - G1(p, s) * G1(q, u) * G1(a, t) -
                                     G1(p, u) * G1(q, t) * G1(a, s) - G1(p, t) * G1(q, s) * G1(a, u) +
                                     0.5 * (G1(p, t) * G1(q, u) * G1(a, s) + G1(p, u) * G1(q, s) * G1(a, t));
                                r[i] += v;
                            }
        break;
    }
    default: return -1;
    }
    std::copy(r.begin(), r.end(), out);
    return (int64_t)r.size();
}

} // extern "C"
