// C-ABI entry points (include/forte2_gb300.h). Every call catches exceptions and maps them to
// status codes with a thread-local message; nothing here allocates on behalf of the caller's
// vectors (C, sigma, CSF vectors are caller-owned device or host buffers).
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/forte2_gb300.h"
#include "csf.cuh"
#include "rel.cuh"
#include "dgraph.cuh"
#include "rdm.cuh"

namespace f2g {
void dav_dots(const double* A, int na, int64_t lda, const double* B, int nb, int64_t ldb, int64_t n, double* out,
              double* scratch, cudaStream_t st);
int64_t dav_scratch_size(int64_t n);
void dav_lincomb(const double* X, int nx, int64_t ldx, const double* coef, int ny, double* Y, int64_t ldy, double beta,
                 int64_t n, cudaStream_t st);
void dav_residual(const double* B, const double* S, int m, int64_t ld, const double* alpha, const double* lam, int nroot,
                  const double* hdiag, int64_t n, double thresh, double* R, int64_t ldr, double* norms2, double* scratch,
                  cudaStream_t st);
void dav_eigh(int m, const double* G, double* evals, double* evecs, cudaStream_t st);
void dav_dots_noalloc(const double* A, int na, int64_t lda, const double* B, int nb, int64_t ldb, int64_t n,
                      double* out, cudaStream_t st);
void probe_dfma(int blocks, int threads, long long iters, double* out, cudaStream_t st);
} // namespace f2g

using namespace f2g;

namespace {
thread_local std::string g_err;

template <typename F> int guard(F&& f) {
    try {
        f();
        return 0;
    } catch (const Error& e) {
        g_err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_err = "host out of memory";
        return 1;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

inline cudaStream_t S(void* p) { return static_cast<cudaStream_t>(p); }

void need(const void* p, const char* what) {
    if (!p)
        throw Error(2, std::string(what) + " is NULL");
}
} // namespace

extern "C" {

const char* f2g_last_error(void) { return g_err.c_str(); }

const char* f2g_version(void) { return "forte2_gb300 0.1 (sm_103a)"; }

int f2g_strings_create(int na, int nb, int norb, void** out) {
    return guard([&] {
        need(out, "out");
        if (na < 0 || nb < 0)
            throw Error(2, "CIStrings: the number of electrons must be non-negative");
        if (na > norb || nb > norb)
            throw Error(2, "CIStrings: more electrons than orbitals");
        *out = new CIStrings(na, nb, norb);
    });
}

// the reference's (orbital_symmetry, gas_min, gas_max) arguments from flat arrays
struct SpaceArgs {
    std::vector<std::vector<int>> spaces;
    std::vector<int> mn, mx;
    int norb = 0;
};
static SpaceArgs space_args(int na, int nb, int nspace, const int* gas_size, const int* orbsym, int nmin,
                            const int* gas_min, int nmax, const int* gas_max) {
    if (na < 0 || nb < 0)
        throw Error(2, "CIStrings: the number of electrons must be non-negative");
    if (nspace < 0 || nmin < 0 || nmax < 0)
        throw Error(2, "CIStrings: negative list length");
    if ((nspace && !gas_size) || (nmin && !gas_min) || (nmax && !gas_max))
        throw Error(2, "CIStrings: NULL list");
    SpaceArgs a;
    a.spaces.resize(nspace);
    for (int g = 0; g < nspace; ++g) {
        if (gas_size[g] < 0)
            throw Error(2, "CIStrings: negative GAS space size");
        if (gas_size[g] && !orbsym)
            throw Error(2, "CIStrings: NULL orbital irreps");
        for (int i = 0; i < gas_size[g]; ++i)
            a.spaces[g].push_back(orbsym[a.norb++]);
    }
    if (na > a.norb || nb > a.norb)
        throw Error(2, "CIStrings: more electrons than orbitals");
    a.mn.assign(gas_min, gas_min + nmin);
    a.mx.assign(gas_max, gas_max + nmax);
    return a;
}

static void blocks_info(const DetBlocks& B, int64_t nfull, int64_t* out) {
    const int64_t v[16] = {B.trivial ? 1 : 0,
                           B.nirrep,
                           B.nspace,
                           B.nclass(0),
                           B.nclass(1),
                           B.nblk(),
                           B.cls_off[0].back(),
                           B.cls_off[1].back(),
                           nfull,
                           (int64_t)B.aocc.size(),
                           (int64_t)B.bocc.size(),
                           (int64_t)B.occ_pairs.size(),
                           B.symmetry,
                           B.ndet,
                           0,
                           0};
    std::memcpy(out, v, sizeof(v));
}

int f2g_strings_create_general(int na, int nb, int symmetry, int nspace, const int* gas_size, const int* orbsym,
                               int nmin, const int* gas_min, int nmax, const int* gas_max, void** out) {
    return guard([&] {
        need(out, "out");
        const SpaceArgs a = space_args(na, nb, nspace, gas_size, orbsym, nmin, gas_min, nmax, gas_max);
        *out = new CIStrings(na, nb, symmetry, a.spaces, a.mn, a.mx);
    });
}

int f2g_strings_blocks_info(void* h, int64_t* out) {
    return guard([&] {
        need(h, "strings");
        need(out, "out");
        const auto* s = static_cast<CIStrings*>(h);
        blocks_info(s->blocks, s->nfull, out);
    });
}

int f2g_blocks_enumerate(int na, int nb, int symmetry, int nspace, const int* gas_size, const int* orbsym, int nmin,
                         const int* gas_min, int nmax, const int* gas_max, int64_t* info, uint64_t* amasks,
                         int32_t* aclasses, uint64_t* bmasks, int32_t* bclasses, int64_t* blocks) {
    return guard([&] {
        need(info, "info");
        const SpaceArgs a = space_args(na, nb, nspace, gas_size, orbsym, nmin, gas_min, nmax, gas_max);
        DetBlocks B;
        B.enumerate(na, nb, symmetry, a.spaces, a.mn, a.mx);
        blocks_info(B, (int64_t)(host_binom(a.norb, na) * host_binom(a.norb, nb)), info);
        for (int spin = 0; spin < 2; ++spin) {
            uint64_t* m = spin == 0 ? amasks : bmasks;
            int32_t* c = spin == 0 ? aclasses : bclasses;
            if (m)
                std::copy(B.str[spin].begin(), B.str[spin].end(), m);
            if (c)
                for (int k = 0; k < B.nclass(spin); ++k)
                    for (int64_t j = B.cls_off[spin][k]; j < B.cls_off[spin][k + 1]; ++j)
                        c[j] = k;
        }
        if (blocks)
            std::copy(B.hblk.begin(), B.hblk.end(), blocks);
    });
}

int f2g_strings_class_strings(void* h, int spin, uint64_t* host_masks, int32_t* host_classes) {
    return guard([&] {
        need(h, "strings");
        if (spin != 0 && spin != 1)
            throw Error(2, "spin must be 0 or 1");
        const auto* s = static_cast<CIStrings*>(h);
        const DetBlocks& B = s->blocks;
        const int64_t n = B.cls_off[spin].back();
        if (n == 0)
            return;
        need(host_masks, "masks");
        need(host_classes, "classes");
        if (B.str[spin].empty()) // C1 space built without enumeration: the C1 strings, one class
            F2G_CUDA(cudaMemcpy(host_masks, s->spin(spin).str.get(), n * 8, cudaMemcpyDeviceToHost));
        else
            std::memcpy(host_masks, B.str[spin].data(), n * 8);
        for (int c = 0; c < B.nclass(spin); ++c)
            for (int64_t j = B.cls_off[spin][c]; j < B.cls_off[spin][c + 1]; ++j)
                host_classes[j] = c;
    });
}

int f2g_strings_block_table(void* h, int64_t* host_out) {
    return guard([&] {
        need(h, "strings");
        const DetBlocks& B = static_cast<CIStrings*>(h)->blocks;
        if (B.hblk.empty())
            return;
        need(host_out, "out");
        std::memcpy(host_out, B.hblk.data(), B.hblk.size() * sizeof(int64_t));
    });
}

int f2g_strings_occupations(void* h, int32_t* host_aocc, int32_t* host_bocc, int32_t* host_pairs) {
    return guard([&] {
        need(h, "strings");
        const DetBlocks& B = static_cast<CIStrings*>(h)->blocks;
        for (size_t i = 0; host_aocc && i < B.aocc.size(); ++i)
            for (int g = 0; g < kMaxGasSpaces; ++g)
                host_aocc[i * kMaxGasSpaces + g] = B.aocc[i][g];
        for (size_t i = 0; host_bocc && i < B.bocc.size(); ++i)
            for (int g = 0; g < kMaxGasSpaces; ++g)
                host_bocc[i * kMaxGasSpaces + g] = B.bocc[i][g];
        for (size_t i = 0; host_pairs && i < B.occ_pairs.size(); ++i) {
            host_pairs[2 * i] = B.occ_pairs[i].first;
            host_pairs[2 * i + 1] = B.occ_pairs[i].second;
        }
    });
}

int f2g_strings_destroy(void* s) {
    return guard([&] { delete static_cast<CIStrings*>(s); });
}

int f2g_strings_info(void* h, int64_t* out) {
    return guard([&] {
        need(h, "strings");
        auto* s = static_cast<CIStrings*>(h);
        const int64_t v[10] = {s->norb, s->na, s->nb, s->a.N0, s->b.N0, s->ndet, s->a.N1, s->b.N1, s->a.N2, s->b.N2};
        std::memcpy(out, v, sizeof(v));
    });
}

int f2g_strings_masks(void* h, int spin, uint64_t* host_out) {
    return guard([&] {
        need(h, "strings");
        const auto& ss = static_cast<CIStrings*>(h)->spin(spin);
        if (ss.N0)
            F2G_CUDA(cudaMemcpy(host_out, ss.str.get(), ss.N0 * 8, cudaMemcpyDeviceToHost));
    });
}

int f2g_strings_list1h(void* h, int spin, int32_t* rows, int64_t* count) {
    return guard([&] {
        need(h, "strings");
        const auto& ss = static_cast<CIStrings*>(h)->spin(spin);
        const int64_t nent = ss.N1 * ss.m1;
        *count = nent;
        if (!rows || nent == 0)
            return;
        std::vector<uint32_t> e(nent);
        F2G_CUDA(cudaMemcpy(e.data(), ss.up1.get(), nent * 4, cudaMemcpyDeviceToHost));
        for (int64_t K = 0; K < ss.N1; ++K)
            for (int j = 0; j < ss.m1; ++j) {
                const uint32_t x = e[K * ss.m1 + j];
                int32_t* r = rows + 6 * (K * ss.m1 + j);
                r[0] = 0;
                r[1] = (int32_t)K;
                r[2] = 0;
                r[3] = e_neg(x) ? -1 : 1;
                r[4] = e_orb(x);
                r[5] = (int32_t)e_addr(x);
            }
    });
}

int f2g_strings_list2h(void* h, int spin, int32_t* rows, int64_t* count) {
    return guard([&] {
        need(h, "strings");
        auto* s = static_cast<CIStrings*>(h);
        auto& ss = s->spin(spin);
        const int64_t nent = ss.N2 * ss.m2;
        *count = nent;
        if (!rows || nent == 0)
            return;
        ss.build_up2(s->binom.get(), 0);
        std::vector<uint64_t> e(nent);
        F2G_CUDA(cudaMemcpy(e.data(), ss.up2.get(), nent * 8, cudaMemcpyDeviceToHost));
        for (int64_t K = 0; K < ss.N2; ++K)
            for (int j = 0; j < ss.m2; ++j) {
                const uint64_t x = e[K * ss.m2 + j];
                int32_t* r = rows + 7 * (K * ss.m2 + j);
                r[0] = 0;
                r[1] = (int32_t)K;
                r[2] = 0;
                r[3] = (x >> 48 & 1) ? -1 : 1;
                r[4] = (int32_t)(x >> 32 & 0xff);
                r[5] = (int32_t)(x >> 40 & 0xff);
                r[6] = (int32_t)(x & 0xffffffffu);
            }
    });
}

int f2g_sigma_create(void* strings, double E, const double* H, const double* V, int log_level, void** out) {
    return guard([&] {
        need(strings, "strings");
        need(out, "out");
        auto* s = static_cast<CIStrings*>(strings);
        if (s->norb > 0) {
            need(H, "H");
            need(V, "V");
        }
        *out = new SigmaBuilder(s, E, H, V, log_level);
    });
}

int f2g_sigma_destroy(void* sb) {
    return guard([&] { delete static_cast<SigmaBuilder*>(sb); });
}

int f2g_sigma_set_hamiltonian(void* sb, double E, const double* H, const double* V) {
    return guard([&] {
        need(sb, "sigma");
        static_cast<SigmaBuilder*>(sb)->set_hamiltonian(E, H, V);
    });
}

int f2g_sigma_set_algorithm(void* sb, const char* name) {
    return guard([&] {
        need(sb, "sigma");
        need(name, "name");
        const std::string a(name);
        auto* b = static_cast<SigmaBuilder*>(sb);
        if (a == "kh" || a == "knowles-handy")
            b->algorithm = 0;
        else if (a == "hz" || a == "harrison-zarrabian")
            b->algorithm = 1;
        else
            throw Error(1, "CI algorithm " + a + " not valid.");
    });
}

int f2g_sigma_get_algorithm(void* sb, char* buf, int buflen) {
    return guard([&] {
        need(sb, "sigma");
        need(buf, "buf");
        if (buflen <= 0)
            throw Error(2, "buflen must be positive");
        const char* name = static_cast<SigmaBuilder*>(sb)->algorithm == 0 ? "Knowles-Handy" : "Harrison-Zarrabian";
        std::strncpy(buf, name, (size_t)buflen);
        buf[buflen - 1] = 0;
    });
}

int f2g_sigma_set_memory(void* sb, int mb) {
    return guard([&] {
        need(sb, "sigma");
        if (mb < 0)
            throw Error(2, "CI builder memory must be non-negative.");
        static_cast<SigmaBuilder*>(sb)->memory = (size_t)mb * 1024 * 1024;
    });
}

// ---- two-component sigma builder (RelCISigmaBuilder) ----

int f2g_rel_sigma_create(void* strings, double E, const double* H, const double* V, void** out) {
    return guard([&] {
        need(strings, "strings");
        need(out, "out");
        auto* s = static_cast<CIStrings*>(strings);
        const size_t n = (size_t)s->norb;
        if (n && (!H || !V))
            throw Error(2, "NULL integrals");
        *out = new RelSigmaBuilder(s, E, reinterpret_cast<const std::complex<double>*>(H),
                                   reinterpret_cast<const std::complex<double>*>(V));
    });
}

int f2g_rel_sigma_destroy(void* h) {
    return guard([&] { delete static_cast<RelSigmaBuilder*>(h); });
}

int f2g_rel_sigma_set_algorithm(void* h, const char* name) {
    return guard([&] {
        need(h, "rel sigma");
        need(name, "name");
        const std::string a(name);
        auto* b = static_cast<RelSigmaBuilder*>(h);
        if (a == "kh" || a == "knowles-handy")
            b->algorithm = 0;
        else if (a == "hz" || a == "harrison-zarrabian")
            b->algorithm = 1;
        else
            throw Error(1, "CI algorithm " + a + " not valid.");
    });
}

int f2g_rel_sigma_get_algorithm(void* h, char* buf, int buflen) {
    return guard([&] {
        need(h, "rel sigma");
        need(buf, "buf");
        if (buflen <= 0)
            throw Error(2, "buflen must be positive");
        const char* name = static_cast<RelSigmaBuilder*>(h)->algorithm == 0 ? "Knowles-Handy" : "Harrison-Zarrabian";
        std::strncpy(buf, name, (size_t)buflen);
        buf[buflen - 1] = 0;
    });
}

int f2g_rel_sigma_set_memory(void* h, int mb) {
    return guard([&] {
        need(h, "rel sigma");
        if (mb < 0)
            throw Error(2, "CI builder memory must be non-negative.");
        static_cast<RelSigmaBuilder*>(h)->memory = (size_t)mb * 1024 * 1024;
    });
}

int f2g_rel_sigma_apply(void* h, const double* C, double* sigma, int nvec, void* stream) {
    return guard([&] {
        need(h, "rel sigma");
        auto* b = static_cast<RelSigmaBuilder*>(h);
        if (nvec < 0)
            throw Error(2, "nvec must be >= 0");
        if (nvec == 0 || b->s->ndet == 0)
            return;
        need(C, "C");
        need(sigma, "sigma");
        b->hamiltonian(reinterpret_cast<const double2*>(C), reinterpret_cast<double2*>(sigma), S(stream), nvec);
    });
}

int f2g_rel_sigma_hdiag(void* h, double* out, void* stream) {
    return guard([&] {
        need(h, "rel sigma");
        auto* b = static_cast<RelSigmaBuilder*>(h);
        if (b->s->ndet == 0)
            return;
        need(out, "out");
        b->hdiag(reinterpret_cast<double2*>(out), S(stream));
    });
}

int f2g_rel_sigma_element(void* h, int64_t I, int64_t J, double* out) {
    return guard([&] {
        need(h, "rel sigma");
        need(out, "out");
        const std::complex<double> x = static_cast<RelSigmaBuilder*>(h)->element(I, J);
        out[0] = x.real();
        out[1] = x.imag();
    });
}

int64_t f2g_rel_rdm_size(int nspinor, int kind) {
    try {
        if (nspinor < 0 || nspinor > kMaxOrb)
            throw Error(2, "spin-orbital RDM: need 0 <= nspinor <= 62");
        return RelSigmaBuilder::rdm_size(nspinor, kind);
    } catch (const Error& e) {
        g_err = e.what();
        return -1;
    }
}

int f2g_rel_sigma_rdm(void* h, int kind, const double* CL, const double* CR, double* out, void* stream) {
    return guard([&] {
        need(h, "rel sigma");
        auto* b = static_cast<RelSigmaBuilder*>(h);
        const int64_t size = RelSigmaBuilder::rdm_size(b->n, kind);
        if (size == 0)
            return;
        need(out, "out");
        if (b->s->ndet > 0) {
            need(CL, "CL");
            need(CR, "CR");
        }
        b->rdm(kind, reinterpret_cast<const double2*>(CL), reinterpret_cast<const double2*>(CR),
               reinterpret_cast<double2*>(out), S(stream));
    });
}

int f2g_sigma_reset_build_times(void* sb) {
    return guard([&] {
        need(sb, "sigma");
        auto* b = static_cast<SigmaBuilder*>(sb);
        b->reset_timers();
    });
}

int f2g_sigma_set_variant(void* sb, int which, int value) {
    return guard([&] {
        need(sb, "sigma");
        auto* b = static_cast<SigmaBuilder*>(sb);
        if (which == 0)
            b->use_tc = value != 0;
        else if (which == 1)
            b->spmm_narrow = value != 0;
        else if (which == 2)
            b->opposite_persistent = value != 0;
        else if (which == 3) {
            // polls per bounded wait of the tensor-core kernel (0 = the default limit); also clears
            // its error flag. A small limit makes the waits give up: the error path, for tests.
            if (value < 0)
                throw Error(2, "tensor-core wait limit must be >= 0");
            b->tc_poll_limit = value;
            F2G_CUDA(cudaMemset(b->tc_err.get(), 0, sizeof(int)));
        } else if (which == 4)
            b->use_sym = value != 0;
        else if (which == 5) {
            b->use_tma_b = value != 0;
            if (b->use_tma_b && b->precision == kFP32) {
                b->prepare_tma_b(0);
                F2G_CUDA(cudaStreamSynchronize(0));
            }
        } else if (which == 6) {
            if (value && !b->dense_ss_supported())
                throw Error(2, "dense same-spin GEMMs need at most 4096 strings per spin");
            b->use_dense_ss = value != 0;
            if (b->use_dense_ss && b->precision == kFP32)
                b->ensure_fp32();
        } else
            throw Error(2, "variant must be 0 (tensor cores), 1 (narrow same-spin tiles), 2 (persistent opposite "
                           "grid), 3 (tensor-core wait limit), 4 (irrep-aware opposite-spin kernel), 5 "
                           "(TMA-fed tensor-core B tiles) or 6 (FP32 same-spin terms as dense GEMMs)");
    });
}

int f2g_sigma_set_tensor_cores(void* sb, int on, int* available) {
    return guard([&] {
        need(sb, "sigma");
        auto* b = static_cast<SigmaBuilder*>(sb);
        b->use_tc = on != 0;
        if (available)
            *available = b->tensor_cores_available() ? 1 : 0;
    });
}

int f2g_sigma_tc_error(void* sb, int* out) {
    return guard([&] {
        need(sb, "sigma");
        need(out, "out");
        *out = static_cast<SigmaBuilder*>(sb)->tc_error();
    });
}

int f2g_sigma_set_max_blocks(void* sb, int max_blocks) {
    return guard([&] {
        need(sb, "sigma");
        if (max_blocks < 0)
            throw Error(2, "max_blocks must be >= 0");
        static_cast<SigmaBuilder*>(sb)->max_ctas = max_blocks;
    });
}

int f2g_sigma_set_precision(void* sb, int precision) {
    return guard([&] {
        need(sb, "sigma");
        auto* b = static_cast<SigmaBuilder*>(sb);
        if (precision != kFP64 && precision != kFP32)
            throw Error(2, "precision must be 0 (FP64) or 1 (FP32)");
        if (precision != b->precision) {
            b->reset_timers(); // averages per precision; no wait for builds still running
            b->precision = precision;
            if (precision == kFP32)
                b->ensure_fp32();
        }
    });
}

int f2g_sigma_apply(void* sb, const double* C, double* sigma, int nvec, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        auto* b = static_cast<SigmaBuilder*>(sb);
        const int64_t nd = b->s->ndet;
        if (nvec < 0)
            throw Error(2, "nvec must be >= 0");
        if (nvec == 0)
            return;
        if (nd && (!C || !sigma))
            throw Error(2, "NULL vector");
        b->hamiltonian(C, sigma, S(stream), nvec);
    });
}

int f2g_sigma_apply_host(void* sb, const double* C, double* sigma, int nvec) {
    return guard([&] {
        need(sb, "sigma");
        auto* b = static_cast<SigmaBuilder*>(sb);
        const int64_t nd = b->s->ndet;
        if (nvec < 0)
            throw Error(2, "nvec must be >= 0");
        if (nd == 0 || nvec == 0)
            return;
        if (!C || !sigma)
            throw Error(2, "NULL vector");
        double* dc = b->hostC.reserve(nd);
        double* ds = b->hostS.reserve(nd);
        for (int v = 0; v < nvec; ++v) {
            F2G_CUDA(cudaMemcpy(dc, C + v * nd, nd * 8, cudaMemcpyHostToDevice));
            b->hamiltonian(dc, ds, 0);
            F2G_CUDA(cudaMemcpy(sigma + v * nd, ds, nd * 8, cudaMemcpyDeviceToHost));
        }
    });
}

int f2g_sigma_term(void* sb, int term, const double* C, double* sigma, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        if (term < 0 || term > 5)
            throw Error(2, "term must be 0..5");
        if (static_cast<SigmaBuilder*>(sb)->s->ndet && (!C || !sigma))
            throw Error(2, "NULL vector");
        static_cast<SigmaBuilder*>(sb)->term(term, C, sigma, S(stream));
    });
}

int f2g_sigma_avg_build_time(void* sb, double* out) {
    return guard([&] {
        need(sb, "sigma");
        need(out, "out");
        static_cast<SigmaBuilder*>(sb)->avg_build_time(out);
    });
}

int f2g_sigma_det_energies(void* sb, double* out, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        if (static_cast<SigmaBuilder*>(sb)->s->ndet)
            need(out, "out");
        static_cast<SigmaBuilder*>(sb)->det_energies(out, S(stream));
    });
}

int64_t f2g_rdm_size(int norb, int kind) {
    try {
        return rdm_size(norb, kind);
    } catch (const Error& e) {
        g_err = e.what();
        return -1;
    }
}

int f2g_sigma_rdm(void* sb, int kind, const double* CL, const double* CR, double* out, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        compute_rdm(*static_cast<SigmaBuilder*>(sb), kind, CL, CR, out, S(stream));
    });
}

int f2g_rdm_pair_list(int norb, int nel, int force_wide, void* entries, uint16_t* seg_pair, int64_t* counts) {
    return guard([&] {
        need(counts, "counts");
        if (norb < 0 || norb > kMaxOrb || nel < 0 || nel > norb)
            throw Error(2, "RDM pair list: need 0 <= nel <= norb <= 62");
        PairListHost L;
        build_pair_list(norb, nel, force_wide != 0, kRdmSeg, L);
        counts[0] = L.nseg;
        counts[1] = L.nentry;
        counts[2] = L.wide ? 1 : 0;
        counts[3] = L.N0;
        if (entries) {
            if (L.wide)
                std::memcpy(entries, L.e64.data(), L.e64.size() * sizeof(uint64_t));
            else
                std::memcpy(entries, L.e32.data(), L.e32.size() * sizeof(uint32_t));
        }
        if (seg_pair)
            std::memcpy(seg_pair, L.pair.data(), L.pair.size() * sizeof(uint16_t));
    });
}

int f2g_spin_adapter_create(void* strings, int twoS, int twoMs, void** out) {
    return guard([&] {
        need(strings, "strings");
        need(out, "out");
        *out = new SpinAdapter(static_cast<CIStrings*>(strings), twoS, twoMs);
    });
}

int f2g_spin_adapter_destroy(void* sa) {
    return guard([&] { delete static_cast<SpinAdapter*>(sa); });
}

int f2g_spin_adapter_info(void* h, int64_t* out) {
    return guard([&] {
        need(h, "spin adapter");
        auto* a = static_cast<SpinAdapter*>(h);
        out[0] = a->nconf;
        out[1] = a->ncsf;
        out[2] = a->ncoupling;
    });
}

int f2g_sigma_apply_csf(void* sb, void* sa, const double* csf_in, double* csf_out, int nvec, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        need(sa, "spin adapter");
        if (nvec < 0)
            throw Error(2, "nvec must be >= 0");
        auto* a = static_cast<SpinAdapter*>(sa);
        if (nvec > 0 && a->ncsf > 0) {
            need(csf_in, "csf_in");
            need(csf_out, "csf_out");
        }
        if (!a->host_scratch)
            a->host_scratch = std::make_unique<CsfSigmaScratch>();
        sigma_csf(*static_cast<SigmaBuilder*>(sb), *a, csf_in, csf_out, nvec, S(stream), *a->host_scratch, false);
    });
}

int f2g_csf_to_det(void* h, const double* csf, double* det, int nvec, void* stream) {
    return guard([&] {
        need(h, "spin adapter");
        auto* a = static_cast<SpinAdapter*>(h);
        if (nvec < 0)
            throw Error(2, "nvec must be >= 0");
        if (nvec > 0 && a->ncsf > 0)
            need(csf, "csf");
        if (nvec > 0 && a->s->ndet > 0)
            need(det, "det");
        for (int v0 = 0; v0 < nvec; v0 += 65535)
            a->csf_to_det(csf + v0 * a->ncsf, det + v0 * a->s->ndet, S(stream), std::min(65535, nvec - v0));
    });
}

int f2g_det_to_csf(void* h, const double* det, double* csf, int nvec, void* stream) {
    return guard([&] {
        need(h, "spin adapter");
        auto* a = static_cast<SpinAdapter*>(h);
        if (nvec < 0)
            throw Error(2, "nvec must be >= 0");
        if (nvec > 0 && a->s->ndet > 0)
            need(det, "det");
        if (nvec > 0 && a->ncsf > 0)
            need(csf, "csf");
        for (int v0 = 0; v0 < nvec; v0 += 65535)
            a->det_to_csf(det + v0 * a->s->ndet, csf + v0 * a->ncsf, S(stream), std::min(65535, nvec - v0));
    });
}

int f2g_hdiag_csf(void* sb, void* h, double* out, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        need(h, "spin adapter");
        auto* b = static_cast<SigmaBuilder*>(sb);
        auto* a = static_cast<SpinAdapter*>(h);
        if (a->ncsf > 0)
            need(out, "out");
        double* e = b->eDet.reserve(std::max<int64_t>(1, b->s->ndet));
        b->det_energies(e, S(stream));
        a->hdiag(e, out, S(stream));
    });
}

int f2g_csf_matrix(void* sb, void* h, const int64_t* idx, int m, double* out) {
    return guard([&] {
        need(sb, "sigma");
        need(h, "spin adapter");
        auto* a = static_cast<SpinAdapter*>(h);
        if (m < 0)
            throw Error(2, "csf_matrix: negative size");
        if (m > 0) {
            need(idx, "idx");
            need(out, "out");
        }
        for (int i = 0; i < m; ++i)
            if (idx[i] < 0 || idx[i] >= a->ncsf)
                throw Error(2, "CSF index out of range");
        a->csf_matrix(*static_cast<SigmaBuilder*>(sb), idx, m, out);
    });
}

int f2g_csf_matrix_dev(void* sb, void* h, const int64_t* idx, int m, double* out, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        need(h, "spin adapter");
        if (m < 0)
            throw Error(2, "csf_matrix: negative size");
        if (m > 0) {
            need(idx, "idx");
            need(out, "out");
        }
        static_cast<SpinAdapter*>(h)->csf_matrix_dev(*static_cast<SigmaBuilder*>(sb), idx, m, out, S(stream));
    });
}

int f2g_spin_adapter_dump(void* h, int64_t* bounds, int64_t* det_idx, double* coeff, int64_t* ranges) {
    return guard([&] {
        need(h, "spin adapter");
        static_cast<SpinAdapter*>(h)->dump(bounds, det_idx, coeff, ranges);
    });
}

int f2g_probe_dfma(int blocks, int threads, int64_t iters, double* out, void* stream) {
    return guard([&] {
        need(out, "out");
        probe_dfma(blocks, threads, (long long)iters, out, S(stream));
    });
}

int64_t f2g_dav_scratch_size(int64_t n) { return dav_scratch_size(n); }

int f2g_dav_dots(const double* A, int na, int64_t lda, const double* B, int nb, int64_t ldb, int64_t n, double* out,
                 double* scratch, void* stream) {
    return guard([&] {
        if (na < 0 || nb < 0 || n < 0)
            throw Error(2, "dots: negative size");
        if (na > 0 && nb > 0) {
            need(A, "A");
            need(B, "B");
            need(out, "out");
            need(scratch, "scratch");
        }
        dav_dots(A, na, lda, B, nb, ldb, n, out, scratch, S(stream));
    });
}

int f2g_dav_dots_noalloc(const double* A, int na, int64_t lda, const double* B, int nb, int64_t ldb, int64_t n,
                         double* out, void* stream) {
    return guard([&] {
        if (na < 0 || nb < 0 || n < 0)
            throw Error(2, "dots_noalloc: negative size");
        if (na > 0 && nb > 0) {
            need(A, "A");
            need(B, "B");
            need(out, "out");
        }
        dav_dots_noalloc(A, na, lda, B, nb, ldb, n, out, S(stream));
    });
}

int f2g_dav_lincomb(const double* X, int nx, int64_t ldx, const double* coef, int ny, double* Y, int64_t ldy,
                    double beta, int64_t n, void* stream) {
    return guard([&] {
        if (nx < 0 || ny < 0 || n < 0)
            throw Error(2, "lincomb: negative size");
        if (ny > 0 && n > 0) {
            need(Y, "Y");
            if (nx > 0) {
                need(X, "X");
                need(coef, "coef");
            }
        }
        dav_lincomb(X, nx, ldx, coef, ny, Y, ldy, beta, n, S(stream));
    });
}

int f2g_dav_residual(const double* B, const double* Sv, int m, int64_t ld, const double* alpha, const double* lam,
                     int nroot, const double* hdiag, int64_t n, double thresh, double* R, int64_t ldr, double* norms2,
                     double* scratch, void* stream) {
    return guard([&] {
        if (m < 0 || nroot < 0 || n < 0)
            throw Error(2, "residual: negative size");
        if (nroot > 0) {
            need(alpha, "alpha");
            need(lam, "lam");
            need(norms2, "norms2");
            need(scratch, "scratch");
            if (n > 0) {
                need(B, "B");
                need(Sv, "S");
                need(hdiag, "hdiag");
                need(R, "R");
            }
        }
        dav_residual(B, Sv, m, ld, alpha, lam, nroot, hdiag, n, thresh, R, ldr, norms2, scratch, S(stream));
    });
}

int f2g_dav_eigh(int m, const double* G, double* evals, double* evecs, void* stream) {
    return guard([&] {
        if (m < 0)
            throw Error(2, "eigh: negative size");
        if (m > 0) {
            need(G, "G");
            need(evals, "evals");
            need(evecs, "evecs");
        }
        dav_eigh(m, G, evals, evecs, S(stream));
    });
}

int f2g_dav_gs_append(double* B, int64_t ld, int cap, int m0, const double* R, int64_t ldr, int ncand, int64_t n,
                      double discard, double ortho, int min_total, uint64_t seed, int* added, void* stream) {
    return guard([&] {
        need(B, "B");
        need(added, "added");
        if (ncand > 0)
            need(R, "R");
        dav_gs_append(B, ld, cap, m0, R, ldr, ncand, n, discard, ortho, min_total, seed, added, S(stream));
    });
}

int f2g_dgraph_create(void* sb, void* sa, int64_t n, int nroot, int maxm, int collapse_k, int maxiter_cap,
                      uint64_t seed, int iters_per_launch, const double* thresholds, double* b, double* sigma,
                      double* r, double* tmp, int64_t ld, int64_t ldr, int64_t ldt, const double* hdiag, void** out) {
    return guard([&] {
        need(sb, "sigma");
        need(sa, "spin adapter");
        need(thresholds, "thresholds");
        need(out, "out");
        need(b, "b");
        need(sigma, "sigma rows");
        need(r, "r");
        need(tmp, "tmp");
        need(hdiag, "hdiag");
        if (ld < n || ldr < n || ldt < n)
            throw Error(2, "dgraph: leading dimensions must be at least n");
        DGParams P{};
        P.n = n;
        P.nroot = nroot;
        P.maxm = maxm;
        P.collapse_k = collapse_k;
        P.maxiter_cap = maxiter_cap;
        P.precond_thresh = thresholds[0];
        P.discard = thresholds[1];
        P.ortho = thresholds[2];
        P.seed = seed;
        auto g = std::make_unique<DavGraph>(static_cast<SigmaBuilder*>(sb), static_cast<SpinAdapter*>(sa), P,
                                            iters_per_launch, b, sigma, r, tmp, ld, ldr, ldt, hdiag);
        *out = g.release();
    });
}

int f2g_dgraph_destroy(void* g) {
    return guard([&] { delete static_cast<DavGraph*>(g); });
}

int f2g_dgraph_set_correction(void* g, const double* X, const double* D, int64_t ldx, const double* Mxd, int k) {
    return guard([&] {
        need(g, "dgraph");
        if (k > 0) {
            need(X, "X");
            need(D, "D");
            need(Mxd, "Mxd");
        }
        static_cast<DavGraph*>(g)->set_correction(X, D, ldx, Mxd, k);
    });
}

int f2g_dgraph_reset(void* g, int m, int sigma_size, const int32_t* dev_m, const double* dev_S, int ldS,
                     const double* lam_old, int nlam, double e_tol, double r_tol, int maxiter, int stall_window,
                     double stall_floor, void* stream) {
    return guard([&] {
        need(g, "dgraph");
        DGReset rs{};
        rs.m = m;
        rs.sigma_size = sigma_size;
        rs.dev_m = dev_m;
        rs.S = dev_S;
        rs.ldS = ldS;
        if (dev_S && ldS < m)
            throw Error(2, "dgraph: ldS must be at least m");
        rs.nlam = nlam;
        rs.maxiter = maxiter;
        rs.stall_window = stall_window;
        rs.e_tol = e_tol;
        rs.r_tol = r_tol;
        rs.stall_floor = stall_floor;
        if (nlam < 0 || nlam > 64)
            throw Error(2, "dgraph: 0 to 64 previous roots");
        if (nlam)
            need(lam_old, "lam_old");
        for (int i = 0; i < nlam; ++i)
            rs.lam_old[i] = lam_old[i];
        static_cast<DavGraph*>(g)->reset(rs, S(stream));
    });
}

int f2g_dgraph_launch(void* g, void* stream) {
    return guard([&] {
        need(g, "dgraph");
        static_cast<DavGraph*>(g)->launch(S(stream));
    });
}

int f2g_dgraph_state(void* g, int32_t* host_ints, double* host_dbl) {
    return guard([&] {
        need(g, "dgraph");
        need(host_ints, "ints");
        need(host_dbl, "doubles");
        const DGState& s = *static_cast<DavGraph*>(g)->host_state;
        const int32_t iv[8] = {s.m, s.sigma_size, s.iter, s.status, s.collapse, s.added, s.m_eig, 0};
        std::memcpy(host_ints, iv, sizeof(iv));
        host_dbl[0] = s.max_de;
        host_dbl[1] = s.max_r;
        std::memcpy(host_dbl + 2, s.lam, sizeof(s.lam));
        std::memcpy(host_dbl + 66, s.lam_old, sizeof(s.lam_old));
        host_dbl[130] = s.ortho_dev;
    });
}

int f2g_dgraph_ritz(void* g, double* out, int64_t ldo, void* stream) {
    return guard([&] {
        need(g, "dgraph");
        need(out, "out");
        static_cast<DavGraph*>(g)->ritz(out, ldo, S(stream));
    });
}

int f2g_dgraph_history(void* g, double* host_out, int count) {
    return guard([&] {
        need(g, "dgraph");
        need(host_out, "out");
        static_cast<DavGraph*>(g)->history(host_out, count);
    });
}

int f2g_dgraph_serial(void* g, uint64_t* out) {
    return guard([&] {
        need(g, "dgraph");
        need(out, "out");
        *out = static_cast<DavGraph*>(g)->serial;
    });
}

int f2g_dgraph_batch_create(void* const* graphs, int count, void** out) {
    return guard([&] {
        need(graphs, "graphs");
        need(out, "out");
        std::vector<DavGraph*> v((size_t)std::max(count, 0));
        for (int i = 0; i < count; ++i)
            v[(size_t)i] = static_cast<DavGraph*>(graphs[i]);
        auto b = std::make_unique<DavBatch>(v.data(), count);
        *out = b.release();
    });
}

int f2g_dgraph_batch_destroy(void* b) {
    return guard([&] { delete static_cast<DavBatch*>(b); });
}

int f2g_dgraph_batch_launch(void* b, void* stream) {
    return guard([&] {
        need(b, "dgraph batch");
        static_cast<DavBatch*>(b)->launch(S(stream));
    });
}

int f2g_dgraph_batch_nodes(void* b, int* out) {
    return guard([&] {
        need(b, "dgraph batch");
        need(out, "out");
        *out = static_cast<DavBatch*>(b)->nodes;
    });
}

int f2g_sigma_set_hamiltonian_async(void* sb, double E, const double* H, const double* V, void* stream) {
    return guard([&] {
        need(sb, "sigma");
        static_cast<SigmaBuilder*>(sb)->set_hamiltonian_async(E, H, V, S(stream));
    });
}

} // extern "C"
