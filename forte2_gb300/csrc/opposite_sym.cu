// Opposite-spin sigma (FP64) of a point-group-blocked space: the determinants (Ia, Ib) with
// irrep(Ia) ^ irrep(Ib) = S, embedded in the C1 vector (zero elsewhere).
//
// The term is the one of k_opposite (sigma.cu): for an output alpha string Ja, an orbital p of
// Ja (Ka = Ja - p) and a beta 1-hole string Kb,
//   E[r] = sum_{q not in Ka, s not in Kb} V[p,r,q,s] sgn C(Ka + q, Kb + s),   sigma(Ja, Kb + r) += sgn E[r].
// In the blocked space C(Ka + q, Kb + s) is zero unless irrep(q) ^ irrep(s) = t with
// t = S ^ irrep(Ka) ^ irrep(Kb), and sigma(Ja, Kb + r) is needed only when
// irrep(r) = u = S ^ irrep(Ja) ^ irrep(Kb). So for each q only the orbitals s of irrep t ^ irrep(q)
// are gathered, and E is formed only for the orbitals r of irrep u: about 1/nirrep^2 of the C1
// kernel's multiply-adds. The beta 1-hole strings are processed sorted by irrep (each irrep's group
// padded to whole warps), so t, u and the orbital loops are the same for every lane of a warp and
// the FP64 pipe runs only the needed multiply-adds; a lane whose string occupies s gathers a zero.
// Writes follow the C1 kernel's owner-ordered phases (one phase per created orbital r, a_r^+
// one-to-one on the strings of a round): every sigma element is summed in a fixed order. With few
// multiply-adds left per gathered value the kernel is latency-bound, so the sigma row stays in
// global memory (one CTA owns it) and three 256-thread CTAs share an SM.
#include "opposite_sym.cuh"

namespace f2g {

namespace {

__device__ __forceinline__ double flip_sign(double x, uint32_t neg) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x) ^ ((unsigned long long)neg << 63);
    return __longlong_as_double((long long)bits);
}

constexpr uint32_t kNoEntry = 0xffffffffu;
constexpr int kSymThreads = 256;
constexpr int kSymBlocksPerSM = 3;

} // namespace

template <int RM>
__global__ void __launch_bounds__(kSymThreads, kSymBlocksPerSM)
    k_opposite_sym(int64_t N0a, int n, int na, int N0b, int64_t nkb, int ma, int mb, const uint32_t* __restrict__ down_a,
                   const uint32_t* __restrict__ up_a, const uint32_t* __restrict__ up_b,
                   const int32_t* __restrict__ kb_sorted, const int8_t* __restrict__ kb_h,
                   const uint64_t* __restrict__ astr, OrbSym os, const double* __restrict__ V,
                   const double* __restrict__ C, double* sig) {
    extern __shared__ unsigned char smem_raw[];
    double* vs = reinterpret_cast<double*>(smem_raw);          // [n][ma][n]: V[p, r, q_i, s]
    uint32_t* ua = reinterpret_cast<uint32_t*>(vs + (size_t)n * ma * n); // [ma]
    uint32_t* tbl = ua + ((ma + 3) & ~3);                       // [n][kSymThreads]: this thread's 1-hole entries by orbital
    double* dsm = reinterpret_cast<double*>(tbl + (size_t)n * kSymThreads); // [RM][kSymThreads]: gathered values
    const int tid = threadIdx.x;
    C += blockIdx.y * N0a * N0b;
    sig += blockIdx.y * N0a * N0b;
    for (int64_t Ja = blockIdx.x; Ja < N0a; Ja += gridDim.x) {
        // the sigma row stays in global memory (L2): the owner-ordered phases give every element
        // one writer per phase, so plain read-modify-writes are exact and ordered
        double* srow = sig + Ja * (int64_t)N0b;
        int hJa = 0;
        for (uint64_t m = astr[Ja]; m; m &= m - 1)
            hJa ^= os.h[__ffsll((long long)m) - 1];
        for (int pi = 0; pi < na; ++pi) {
            __syncthreads(); // previous slice fully consumed
            const uint32_t ep = down_a[Ja * na + pi];
            const int64_t Ka = e_addr(ep);
            const int p = e_orb(ep);
            const uint32_t negp = (uint32_t)e_neg(ep);
            const int hKa = hJa ^ os.h[p];
            for (int i = tid; i < ma; i += blockDim.x)
                ua[i] = up_a[Ka * ma + i];
            __syncthreads();
            const int nslice = n * ma * n;
            for (int idx = tid; idx < nslice; idx += blockDim.x) {
                const int r = idx / (ma * n);
                const int rem = idx - r * (ma * n);
                const int qi = rem / n;
                const int s = rem - qi * n;
                const int q = e_orb(ua[qi]);
                vs[idx] = V[(((size_t)p * n + r) * n + q) * n + s];
            }
            __syncthreads();
            for (int64_t base = 0; base < nkb; base += blockDim.x) {
                const int64_t idx = base + tid;
                const int32_t Kb = idx < nkb ? kb_sorted[idx] : -1;
                const bool active = Kb >= 0;
                const int hKb = idx < nkb ? kb_h[idx] : 0;
                for (int o = 0; o < n; ++o)
                    tbl[o * kSymThreads + tid] = kNoEntry;
                if (active)
                    for (int si = 0; si < mb; ++si) {
                        const uint32_t e = __ldg(up_b + (int64_t)Kb * mb + si);
                        tbl[e_orb(e) * kSymThreads + tid] = e;
                    }
                const int t = os.S ^ hKa ^ hKb, u = os.S ^ hJa ^ hKb;
                const int nr = os.cnt[u];
                double acc[RM];
#pragma unroll
                for (int j = 0; j < RM; ++j)
                    acc[j] = 0.0;
                for (int qi = 0; qi < ma; ++qi) {
                    const uint32_t eq = ua[qi];
                    const int q = e_orb(eq);
                    const double* crow = C + (int64_t)e_addr(eq) * N0b;
                    const uint32_t negq = (uint32_t)e_neg(eq);
                    const int tq = t ^ os.h[q];
                    const int ns = os.cnt[tq];
                    // gathers into this thread's column of dsm, then exactly nr x ns multiply-adds
                    // (warp-uniform trip counts: no predicated-off FP64 instruction)
                    for (int js = 0; js < ns; ++js) {
                        const uint32_t es = tbl[os.list[tq][js] * kSymThreads + tid];
                        double d = 0.0;
                        if (es != kNoEntry)
                            d = flip_sign(__ldg(crow + e_addr(es)), negq ^ (uint32_t)e_neg(es));
                        dsm[js * kSymThreads + tid] = d;
                    }
#pragma unroll
                    for (int j = 0; j < RM; ++j) {
                        if (j < nr) {
                            const double* vr = vs + ((size_t)os.list[u][j] * ma + qi) * n;
                            double a = acc[j];
                            for (int js = 0; js < ns; ++js)
                                a += vr[os.list[tq][js]] * dsm[js * kSymThreads + tid];
                            acc[j] = a;
                        }
                    }
                }
                // owner-ordered writes, one phase per created orbital r
                for (int r = 0; r < n; ++r) {
                    __syncthreads();
                    if (active && os.h[r] == u) {
                        const uint32_t er = tbl[r * kSymThreads + tid];
                        if (er != kNoEntry) {
                            const int jr = os.pos[r];
                            double v = 0.0;
#pragma unroll
                            for (int j = 0; j < RM; ++j)
                                if (j == jr)
                                    v = acc[j];
                            double* dst = srow + e_addr(er);
                            *dst += flip_sign(v, negp ^ (uint32_t)e_neg(er));
                        }
                    }
                }
            }
        }
    }
}

int64_t opposite_sym_smem(int n, int ma, int64_t N0b, int rm) {
    (void)N0b;
    return (int64_t)n * ma * n * 8 + (int64_t)((ma + 3) & ~3) * 4 + (int64_t)n * kSymThreads * 4 +
           (int64_t)rm * kSymThreads * 8;
}

static int sym_rm(int maxper) { return maxper <= 2 ? 2 : maxper <= 4 ? 4 : maxper <= 8 ? 8 : 16; }

bool opposite_sym_supported(const CIStrings* s) {
    const DetBlocks& B = s->blocks;
    if (!s->blocked() || B.nirrep < 2 || s->norb > 62 || s->na < 1 || s->nb < 1)
        return false;
    // every C1 string in exactly one class, the classes being the irreps: no GAS restriction
    if (B.nclass(0) != B.nirrep || B.nclass(1) != B.nirrep || B.cls_off[0].back() != s->a.N0 ||
        B.cls_off[1].back() != s->b.N0)
        return false;
    int maxper = 0;
    for (int h = 0; h < B.nirrep; ++h) {
        int c = 0;
        for (int x : B.orbsym)
            c += x == h;
        maxper = std::max(maxper, c);
    }
    if (maxper > 16)
        return false; // the per-irrep orbital loops are unrolled up to 16
    int optin = 0, dev = 0;
    F2G_CUDA(cudaGetDevice(&dev));
    F2G_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    return opposite_sym_smem(s->norb, s->a.m1, s->b.N0, sym_rm(maxper)) <= optin;
}

void OppositeSym::build(const CIStrings* s) {
    const DetBlocks& B = s->blocks;
    const int n = s->norb;
    os = OrbSym{};
    os.nirrep = B.nirrep;
    os.S = B.symmetry;
    for (int p = 0; p < n; ++p) {
        const int h = B.orbsym[p];
        os.h[p] = (int8_t)h;
        os.pos[p] = os.cnt[h];
        os.list[h][os.cnt[h]++] = (int8_t)p;
    }
    maxper = 0;
    for (int h = 0; h < 8; ++h)
        maxper = std::max(maxper, (int)os.cnt[h]);
    // beta 1-hole strings by irrep, every irrep's group padded to whole warps
    const int kb1 = s->nb - 1;
    const int64_t N1b = s->b.N1;
    std::vector<uint64_t> bt(kBinomLd * kBinomLd);
    for (int a = 0; a < kBinomLd; ++a)
        for (int b = 0; b < kBinomLd; ++b)
            bt[a * kBinomLd + b] = host_binom(a, b);
    std::vector<std::vector<int32_t>> groups(8);
    for (int64_t K = 0; K < N1b; ++K) {
        int h = 0;
        for (uint64_t m = string_unrank((uint64_t)K, n, kb1, bt.data()); m; m &= m - 1)
            h ^= os.h[__builtin_ctzll(m)];
        groups[h].push_back((int32_t)K);
    }
    std::vector<int32_t> order;
    std::vector<int8_t> hs;
    for (int h = 0; h < 8; ++h) {
        if (groups[h].empty())
            continue;
        const size_t padded = (groups[h].size() + 31) / 32 * 32;
        for (size_t i = 0; i < padded; ++i) {
            order.push_back(i < groups[h].size() ? groups[h][i] : -1);
            hs.push_back((int8_t)h);
        }
    }
    nkb = (int64_t)order.size();
    kb_sorted.reserve(std::max<size_t>(1, order.size()));
    kb_h.reserve(std::max<size_t>(1, hs.size()));
    if (nkb) {
        F2G_CUDA(cudaMemcpy(kb_sorted.get(), order.data(), order.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        F2G_CUDA(cudaMemcpy(kb_h.get(), hs.data(), hs.size(), cudaMemcpyHostToDevice));
    }
    ready = true;
}

template <int RM>
static void launch_sym_rm(const CIStrings* s, const OppositeSym& t, const double* V, const double* C, double* sig,
                          cudaStream_t st, int nvec, int max_ctas) {
    const int n = s->norb, ma = s->a.m1, mb = s->b.m1;
    const int64_t smem = opposite_sym_smem(n, ma, s->b.N0, RM);
    F2G_CUDA(cudaFuncSetAttribute(k_opposite_sym<RM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t gx = s->a.N0;
    if (max_ctas > 0)
        gx = std::min<int64_t>(gx, max_ctas);
    k_opposite_sym<RM><<<dim3((unsigned)gx, (unsigned)nvec), kSymThreads, smem, st>>>(
        s->a.N0, n, s->na, (int)s->b.N0, t.nkb, ma, mb, s->a.down1.get(), s->a.up1.get(), s->b.up1.get(),
        t.kb_sorted.get(), t.kb_h.get(), s->a.str.get(), t.os, V, C, sig);
    F2G_LAUNCH("k_opposite_sym");
}

void launch_opposite_sym(const CIStrings* s, const OppositeSym& t, const double* V, const double* C, double* sig,
                         cudaStream_t st, int nvec, int max_ctas) {
    if (s->na < 1 || s->nb < 1 || s->a.N0 == 0 || t.nkb == 0)
        return;
    if (nvec > 65535)
        throw Error(2, "opposite-spin kernel: at most 65535 vectors per launch");
    if (t.maxper <= 2)
        launch_sym_rm<2>(s, t, V, C, sig, st, nvec, max_ctas);
    else if (t.maxper <= 4)
        launch_sym_rm<4>(s, t, V, C, sig, st, nvec, max_ctas);
    else if (t.maxper <= 8)
        launch_sym_rm<8>(s, t, V, C, sig, st, nvec, max_ctas);
    else
        launch_sym_rm<16>(s, t, V, C, sig, st, nvec, max_ctas);
}

} // namespace f2g
