// Test infrastructure (oracle only): a C-ABI wrapper around the reference's own hot-path
// classes (CIStrings, CISigmaBuilder, CISpinAdapter, SlaterRules), compiled from the
// reference sources by oracle/build_ref.sh into oracle/_ref/libforte2_ref.so. It exists to
// generate golden vectors and to check the CPU restatement in oracle/port; nothing in the GPU
// product links or loads it.
//
// Private HZ terms are reached for per-term golden vectors by widening access in this
// translation unit only (the class layout is unchanged).
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

// Every header the sigma builder pulls in is included first with normal access, so that
// the access widening below touches only the CISigmaBuilder class itself.
#include <complex>
#include <sstream>
#include <span>
#include "helpers/ndarray.h"
#include "helpers/spin.h"
#include "ci/ci_strings.h"
#include "determinant/slater_rules.h"
#include "determinant/ci_spin_adapter.h"
#include "sparse/sparse_state.h"
#define private public
#include "ci/ci_sigma_builder.h"
#undef private
#include "ci/rel_ci_sigma_builder.h"

using namespace forte2;

namespace {
thread_local std::string g_err;

int fail(const std::exception& e, int code) {
    g_err = e.what();
    return code;
}

struct RefStrings {
    CIStrings* lists;
    std::vector<Determinant> dets;
};

struct RefSigma {
    CISigmaBuilder* sb;
    std::vector<double> H, V;
    int norb;
};

np_vector vec_view(double* p, size_t n) {
    size_t shape[1] = {n};
    return np_vector(p, 1, shape);
}

struct RefRelSigma {
    RelCISigmaBuilder* sb;
    std::vector<std::complex<double>> H, V;
    int norb;
};

np_vector_complex cvec_view(double* p, size_t n) {
    size_t shape[1] = {n};
    return np_vector_complex(reinterpret_cast<std::complex<double>*>(p), 1, shape);
}
} // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

/// Build CIStrings. orbsym_flat holds the orbital irreps of all GAS spaces, gas_sizes[g] each.
/// Returns nullptr and sets the error on failure (exception kind in *kind: 1 runtime, 2 invalid).
void* ref_strings_new(int na, int nb, int symmetry, int ngas, const int* gas_sizes,
                      const int* orbsym_flat, int nmin, const int* gas_min, int nmax,
                      const int* gas_max, int* kind) {
    try {
        std::vector<std::vector<int>> orbsym(ngas);
        int k = 0;
        for (int g = 0; g < ngas; ++g)
            for (int i = 0; i < gas_sizes[g]; ++i)
                orbsym[g].push_back(orbsym_flat[k++]);
        std::vector<int> gmin(gas_min, gas_min + nmin), gmax(gas_max, gas_max + nmax);
        auto* s = new RefStrings{new CIStrings(na, nb, symmetry, orbsym, gmin, gmax), {}};
        s->dets = s->lists->make_determinants();
        *kind = 0;
        return s;
    } catch (const std::invalid_argument& e) {
        *kind = fail(e, 2);
    } catch (const std::exception& e) {
        *kind = fail(e, 1);
    }
    return nullptr;
}

void ref_strings_free(void* h) {
    auto* s = static_cast<RefStrings*>(h);
    delete s->lists;
    delete s;
}

/// out: norb, na, nb, nas, nbs, ndet, nirrep, n_alpha_classes, n_beta_classes, n_blocks
void ref_strings_info(void* h, int64_t* out) {
    auto* L = static_cast<RefStrings*>(h)->lists;
    out[0] = L->norb();
    out[1] = L->na();
    out[2] = L->nb();
    out[3] = L->nas();
    out[4] = L->nbs();
    out[5] = L->ndet();
    out[6] = L->nirrep();
    out[7] = L->alpha_address()->nclasses();
    out[8] = L->beta_address()->nclasses();
    out[9] = L->determinant_classes().size();
}

/// Blocks: per block (class_Ia, class_Ib, size, offset).
void ref_strings_blocks(void* h, int64_t* out) {
    auto* L = static_cast<RefStrings*>(h)->lists;
    size_t k = 0;
    for (const auto& [n, ca, cb] : L->determinant_classes()) {
        out[4 * k + 0] = ca;
        out[4 * k + 1] = cb;
        out[4 * k + 2] = L->block_size(n);
        out[4 * k + 3] = L->block_offset(n);
        ++k;
    }
}

/// Strings of one spin (0 alpha, 1 beta) in (class, address) order: bit masks and class ids.
int64_t ref_strings_dump(void* h, int spin, uint64_t* masks, int32_t* classes) {
    auto* L = static_cast<RefStrings*>(h)->lists;
    const auto& strings = spin == 0 ? L->alpha_strings() : L->beta_strings();
    int64_t k = 0;
    for (size_t c = 0; c < strings.size(); ++c) {
        for (const auto& s : strings[c]) {
            if (masks) {
                uint64_t m = 0;
                for (int p = 0; p < (int)L->norb(); ++p)
                    if (s[p])
                        m |= (uint64_t(1) << p);
                masks[k] = m;
                classes[k] = (int32_t)c;
            }
            ++k;
        }
    }
    return k;
}

/// 1-hole lists (list2 form, grouped by K): rows (class_K, K, class_I, sign, p, I).
int64_t ref_1h_dump(void* h, int spin, int32_t* out) {
    auto* L = static_cast<RefStrings*>(h)->lists;
    auto addr1h = spin == 0 ? L->alpha_address_1h() : L->beta_address_1h();
    auto addr = spin == 0 ? L->alpha_address() : L->beta_address();
    int64_t k = 0;
    for (int cK = 0; cK < addr1h->nclasses(); ++cK) {
        for (int cI = 0; cI < addr->nclasses(); ++cI) {
            const auto& l2 = spin == 0 ? L->get_alpha_1h_list2(cK, cI) : L->get_beta_1h_list2(cK, cI);
            for (size_t K = 0; K < l2.size(); ++K) {
                for (const auto& e : l2[K]) {
                    if (out) {
                        int32_t* r = out + 6 * k;
                        r[0] = cK;
                        r[1] = (int32_t)K;
                        r[2] = cI;
                        r[3] = e.sign;
                        r[4] = e.p;
                        r[5] = (int32_t)e.J;
                    }
                    ++k;
                }
            }
        }
    }
    return k;
}

/// Same content through the (class_K, K, class_I)-keyed 1h list used by H1_hz: rows as above.
int64_t ref_1h_dump_keyed(void* h, int spin, int32_t* out) {
    auto* L = static_cast<RefStrings*>(h)->lists;
    auto addr1h = spin == 0 ? L->alpha_address_1h() : L->beta_address_1h();
    auto addr = spin == 0 ? L->alpha_address() : L->beta_address();
    int64_t k = 0;
    for (int cK = 0; cK < addr1h->nclasses(); ++cK) {
        for (size_t K = 0; K < addr1h->strpcls(cK); ++K) {
            for (int cI = 0; cI < addr->nclasses(); ++cI) {
                const auto& l = spin == 0 ? L->get_alpha_1h_list(cK, K, cI) : L->get_beta_1h_list(cK, K, cI);
                for (const auto& e : l) {
                    if (out) {
                        int32_t* r = out + 6 * k;
                        r[0] = cK;
                        r[1] = (int32_t)K;
                        r[2] = cI;
                        r[3] = e.sign;
                        r[4] = e.p;
                        r[5] = (int32_t)e.J;
                    }
                    ++k;
                }
            }
        }
    }
    return k;
}

/// 2-hole lists: rows (class_K, K, class_I, sign, p, q, I).
int64_t ref_2h_dump(void* h, int spin, int32_t* out) {
    auto* L = static_cast<RefStrings*>(h)->lists;
    auto addr2h = spin == 0 ? L->alpha_address_2h() : L->beta_address_2h();
    auto addr = spin == 0 ? L->alpha_address() : L->beta_address();
    int64_t k = 0;
    for (int cK = 0; cK < addr2h->nclasses(); ++cK) {
        for (size_t K = 0; K < addr2h->strpcls(cK); ++K) {
            for (int cI = 0; cI < addr->nclasses(); ++cI) {
                const auto& l = spin == 0 ? L->get_alpha_2h_list(cK, K, cI) : L->get_beta_2h_list(cK, K, cI);
                for (const auto& e : l) {
                    if (out) {
                        int32_t* r = out + 7 * k;
                        r[0] = cK;
                        r[1] = (int32_t)K;
                        r[2] = cI;
                        r[3] = e.sign;
                        r[4] = e.p;
                        r[5] = e.q;
                        r[6] = (int32_t)e.J;
                    }
                    ++k;
                }
            }
        }
    }
    return k;
}

/// Determinants in address order: (alpha mask, beta mask).
void ref_dets_dump(void* h, uint64_t* out) {
    auto* s = static_cast<RefStrings*>(h);
    const int norb = (int)s->lists->norb();
    for (size_t i = 0; i < s->dets.size(); ++i) {
        uint64_t a = 0, b = 0;
        for (int p = 0; p < norb; ++p) {
            if (s->dets[i].na(p))
                a |= (uint64_t(1) << p);
            if (s->dets[i].nb(p))
                b |= (uint64_t(1) << p);
        }
        out[2 * i] = a;
        out[2 * i + 1] = b;
    }
}

void* ref_sigma_new(void* hs, double E, const double* H, const double* V, int norb, int log_level) {
    try {
        auto* s = static_cast<RefStrings*>(hs);
        auto* r = new RefSigma{nullptr, std::vector<double>(H, H + norb * norb),
                               std::vector<double>(V, V + (size_t)norb * norb * norb * norb), norb};
        size_t hs2[2] = {(size_t)norb, (size_t)norb};
        size_t vs4[4] = {(size_t)norb, (size_t)norb, (size_t)norb, (size_t)norb};
        np_matrix Hm(r->H.data(), 2, hs2);
        np_tensor4 Vt(r->V.data(), 4, vs4);
        r->sb = new CISigmaBuilder(*s->lists, E, Hm, Vt, log_level);
        return r;
    } catch (const std::exception& e) {
        fail(e, 1);
    }
    return nullptr;
}

void ref_sigma_free(void* h) {
    auto* r = static_cast<RefSigma*>(h);
    delete r->sb;
    delete r;
}

/// 0 ok, 1 runtime_error, 2 invalid_argument
int ref_sigma_set_algorithm(void* h, const char* name) {
    try {
        static_cast<RefSigma*>(h)->sb->set_algorithm(name);
        return 0;
    } catch (const std::invalid_argument& e) {
        return fail(e, 2);
    } catch (const std::exception& e) {
        return fail(e, 1);
    }
}

int ref_sigma_set_memory(void* h, int mb) {
    try {
        static_cast<RefSigma*>(h)->sb->set_memory(mb);
        return 0;
    } catch (const std::invalid_argument& e) {
        return fail(e, 2);
    } catch (const std::exception& e) {
        return fail(e, 1);
    }
}

int ref_sigma_hamiltonian(void* h, double* basis, double* sigma, int64_t ndet) {
    try {
        static_cast<RefSigma*>(h)->sb->Hamiltonian(vec_view(basis, ndet), vec_view(sigma, ndet));
        return 0;
    } catch (const std::invalid_argument& e) {
        return fail(e, 2);
    } catch (const std::exception& e) {
        return fail(e, 1);
    }
}

/// One HZ term into a zeroed sigma: 0 H0, 1 H1 alpha, 2 H1 beta, 3 opposite spin,
/// 4 same-spin alpha, 5 same-spin beta.
int ref_sigma_term(void* h, int term, double* basis, double* sigma, int64_t ndet) {
    try {
        auto* sb = static_cast<RefSigma*>(h)->sb;
        std::span<double> b(basis, ndet), s(sigma, ndet);
        std::fill(s.begin(), s.end(), 0.0);
        switch (term) {
        case 0:
            sb->H0(b, s);
            break;
        case 1:
            sb->H1_hz(b, s, Spin::Alpha, sb->h_hz);
            break;
        case 2:
            sb->H1_hz(b, s, Spin::Beta, sb->h_hz);
            break;
        case 3:
            sb->H2_hz_opposite_spin(b, s);
            break;
        case 4:
            sb->H2_hz_same_spin(b, s, Spin::Alpha);
            break;
        case 5:
            sb->H2_hz_same_spin(b, s, Spin::Beta);
            break;
        default:
            throw std::runtime_error("unknown term");
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(e, 1);
    }
}

void ref_sigma_avg_build_time(void* h, double* out) {
    auto t = static_cast<RefSigma*>(h)->sb->avg_build_time();
    for (int i = 0; i < 4; ++i)
        out[i] = t[i];
}

/// Slater-rules determinant energies for every determinant of the strings (address order).
void ref_det_energies(void* hsig, void* hs, double* out) {
    auto* r = static_cast<RefSigma*>(hsig);
    auto* s = static_cast<RefStrings*>(hs);
    for (size_t i = 0; i < s->dets.size(); ++i)
        out[i] = r->sb->slater_rules_.energy(s->dets[i]);
}

void* ref_spin_adapter_new(int twoS, int twoMs, int norb) {
    auto* sa = new CISpinAdapter(twoS, twoMs, norb);
    sa->set_log_level(0);
    return sa;
}

void ref_spin_adapter_free(void* h) { delete static_cast<CISpinAdapter*>(h); }

void ref_spin_adapter_prepare(void* h, void* hs) {
    static_cast<CISpinAdapter*>(h)->prepare_couplings(static_cast<RefStrings*>(hs)->dets);
}

/// out: nconf, ncsf, ncoupling
void ref_spin_adapter_info(void* h, int64_t* out) {
    auto* sa = static_cast<CISpinAdapter*>(h);
    out[0] = sa->nconf();
    out[1] = sa->ncsf();
    int64_t nc = 0;
    for (size_t i = 0; i < sa->ncsf(); ++i)
        nc += sa->ndets_in_csf(i);
    out[2] = nc;
}

/// Couplings in CSF order: bounds[ncsf+1], det index and coefficient per coupling,
/// and the CSF range of each configuration (conf_ranges[2*nconf]).
void ref_spin_adapter_dump(void* h, int64_t* bounds, int64_t* det_idx, double* coeff,
                           int64_t* conf_ranges) {
    auto* sa = static_cast<CISpinAdapter*>(h);
    int64_t k = 0;
    bounds[0] = 0;
    for (size_t i = 0; i < sa->ncsf(); ++i) {
        for (const auto& [d, c] : sa->csf(i)) {
            det_idx[k] = d;
            coeff[k] = c;
            ++k;
        }
        bounds[i + 1] = k;
    }
    const auto& rg = sa->conf_to_csfs_range();
    for (size_t c = 0; c < rg.size(); ++c) {
        conf_ranges[2 * c] = rg[c].first;
        conf_ranges[2 * c + 1] = rg[c].second;
    }
}

void ref_csf_to_det(void* h, double* csf, int64_t ncsf, double* det, int64_t ndet) {
    static_cast<CISpinAdapter*>(h)->csf_C_to_det_C(vec_view(csf, ncsf), vec_view(det, ndet));
}

void ref_det_to_csf(void* h, double* det, int64_t ndet, double* csf, int64_t ncsf) {
    static_cast<CISpinAdapter*>(h)->det_C_to_csf_C(vec_view(det, ndet), vec_view(csf, ncsf));
}

void ref_hdiag_csf(void* hsig, void* hsa, void* hs, int full, double* out, int64_t ncsf) {
    auto* r = static_cast<RefSigma*>(hsig);
    auto* sa = static_cast<CISpinAdapter*>(hsa);
    auto* s = static_cast<RefStrings*>(hs);
    auto v = r->sb->form_Hdiag_csf(s->dets, *sa, full != 0);
    std::memcpy(out, v.data(), sizeof(double) * ncsf);
}

double ref_slater_rules_csf(void* hsig, void* hsa, void* hs, int64_t I, int64_t J) {
    auto* r = static_cast<RefSigma*>(hsig);
    auto* sa = static_cast<CISpinAdapter*>(hsa);
    auto* s = static_cast<RefStrings*>(hs);
    return r->sb->slater_rules_csf(s->dets, *sa, I, J);
}


/// Reduced density matrices of the reference (ci_sigma_builder_1rdm.cc:9-84,
/// ci_sigma_builder_2rdm.cc:46-282, ci_sigma_builder_3rdm.cc:84-542) between two determinant
/// vectors, copied into `out`: kind 0 a_1rdm, 1 b_1rdm, 2 sf_1rdm (n*n); 3 aa_2rdm, 4 bb_2rdm
/// (P*P, P = n(n-1)/2); 5 ab_2rdm, 6 sf_2rdm, 7 sf_2cumulant (n^4); 8 aaa_3rdm, 9 bbb_3rdm
/// (T*T, T = n(n-1)(n-2)/6); 10 aab_3rdm (P, n, P, n); 11 abb_3rdm (n, P, n, P); 12 sf_3rdm,
/// 13 sf_3cumulant (n^6). Returns the number of elements written.
int64_t ref_rdm(void* h, int kind, double* CL, double* CR, int64_t ndet, double* out) {
    try {
        auto* sb = static_cast<RefSigma*>(h)->sb;
        auto l = vec_view(CL, ndet), r = vec_view(CR, ndet);
        auto copy = [&](const auto& a) {
            const size_t n = a.size();
            std::memcpy(out, a.data(), n * sizeof(double));
            return (int64_t)n;
        };
        switch (kind) {
        case 0: return copy(sb->compute_a_1rdm(l, r));
        case 1: return copy(sb->compute_b_1rdm(l, r));
        case 2: return copy(sb->compute_sf_1rdm(l, r));
        case 3: return copy(sb->compute_aa_2rdm(l, r));
        case 4: return copy(sb->compute_bb_2rdm(l, r));
        case 5: return copy(sb->compute_ab_2rdm(l, r));
        case 6: return copy(sb->compute_sf_2rdm(l, r));
        case 7: return copy(sb->compute_sf_2cumulant(l, r));
        case 8: return copy(sb->compute_aaa_3rdm(l, r));
        case 9: return copy(sb->compute_bbb_3rdm(l, r));
        case 10: return copy(sb->compute_aab_3rdm(l, r));
        case 11: return copy(sb->compute_abb_3rdm(l, r));
        case 12: return copy(sb->compute_sf_3rdm(l, r));
        case 13: return copy(sb->compute_sf_3cumulant(l, r));
        default: throw std::runtime_error("unknown RDM kind");
        }
    } catch (const std::exception& e) {
        fail(e, 1);
    }
    return -1;
}

/// The reference's two-component sigma builder (rel_ci_sigma_builder*.cc) on a CIStrings with
/// nb == 0. H (n x n) and V (n^4, physicist) are complex, interleaved (re, im) doubles.
void* ref_rel_sigma_new(void* hs, double E, const double* H, const double* V, int norb, int log_level) {
    try {
        auto* s = static_cast<RefStrings*>(hs);
        const size_t n2 = (size_t)norb * norb, n4 = n2 * n2;
        auto* r = new RefRelSigma{nullptr, {}, {}, norb};
        r->H.resize(n2);
        r->V.resize(n4);
        std::memcpy(r->H.data(), H, n2 * sizeof(std::complex<double>));
        std::memcpy(r->V.data(), V, n4 * sizeof(std::complex<double>));
        size_t hs2[2] = {(size_t)norb, (size_t)norb};
        size_t vs4[4] = {(size_t)norb, (size_t)norb, (size_t)norb, (size_t)norb};
        np_matrix_complex Hm(r->H.data(), 2, hs2);
        np_tensor4_complex Vt(r->V.data(), 4, vs4);
        r->sb = new RelCISigmaBuilder(*s->lists, E, Hm, Vt, log_level);
        return r;
    } catch (const std::exception& e) {
        fail(e, 1);
    }
    return nullptr;
}

void ref_rel_sigma_free(void* h) {
    auto* r = static_cast<RefRelSigma*>(h);
    delete r->sb;
    delete r;
}

int ref_rel_sigma_set_algorithm(void* h, const char* name) {
    try {
        static_cast<RefRelSigma*>(h)->sb->set_algorithm(name);
        return 0;
    } catch (const std::exception& e) {
        return fail(e, 1);
    }
}

int ref_rel_sigma_hamiltonian(void* h, double* basis, double* sigma, int64_t ndet) {
    try {
        static_cast<RefRelSigma*>(h)->sb->Hamiltonian(cvec_view(basis, ndet), cvec_view(sigma, ndet));
        return 0;
    } catch (const std::exception& e) {
        return fail(e, 1);
    }
}

/// form_Hdiag(dets) into out (ndet complex, interleaved)
void ref_rel_form_hdiag(void* h, void* hs, double* out) {
    auto* r = static_cast<RefRelSigma*>(h);
    auto* s = static_cast<RefStrings*>(hs);
    auto v = r->sb->form_Hdiag(s->dets);
    std::memcpy(out, v.data(), v.size() * sizeof(std::complex<double>));
}

/// slater_rules(dets, I, J) into out[2]
void ref_rel_slater_rules(void* h, void* hs, int64_t I, int64_t J, double* out) {
    auto* r = static_cast<RefRelSigma*>(h);
    auto* s = static_cast<RefStrings*>(hs);
    const std::complex<double> x = r->sb->slater_rules(s->dets, (size_t)I, (size_t)J);
    out[0] = x.real();
    out[1] = x.imag();
}

/// spin-orbital RDMs between two complex vectors: kind 0 so_1rdm (n^2), 1 so_2rdm (n^4),
/// 2 so_2cumulant (n^4), 3 so_3rdm (n^6), 4 so_3cumulant (n^6); interleaved complex output.
int64_t ref_rel_rdm(void* h, int kind, double* CL, double* CR, int64_t ndet, double* out) {
    try {
        auto* sb = static_cast<RefRelSigma*>(h)->sb;
        auto l = cvec_view(CL, ndet), r = cvec_view(CR, ndet);
        auto copy = [&](const auto& a) {
            const size_t n = a.size();
            std::memcpy(out, a.data(), n * sizeof(std::complex<double>));
            return (int64_t)n;
        };
        switch (kind) {
        case 0: return copy(sb->compute_1rdm(l, r));
        case 1: return copy(sb->compute_2rdm(l, r));
        case 2: return copy(sb->compute_2cumulant(l, r));
        case 3: return copy(sb->compute_3rdm(l, r));
        case 4: return copy(sb->compute_3cumulant(l, r));
        default: throw std::runtime_error("unknown RDM kind");
        }
    } catch (const std::exception& e) {
        fail(e, 1);
    }
    return -1;
}

} // extern "C"
