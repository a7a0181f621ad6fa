// Two-component (relativistic) sigma: the reference's RelCISigmaBuilder
// (forte2/ci/rel_ci_sigma_builder.cc, rel_ci_sigma_builder_harrison_zarrabian.cc). All electrons
// are alpha spinors (nb = 0), so sigma = E C + H1 + H2 acting within one string space with complex
// integrals. Its operator is the same-spin string Hamiltonian of the real builder:
//   <J| sum_pq h_pq a+_p a_q + sum_{p>r, q>s} (<pr|qs> - <pr|sq>) a+_r a+_p a_q a_s |I>,
// every element a signed sum of integral elements, so its real and imaginary parts are the real
// builder's rows for Re(h, V) and Im(h, V) (the constant E on the real diagonal). sigma(J) is
// then a complex sparse row product, one warp per row J summing its entries in a fixed order (a
// shuffle tree): bitwise reproducible. As in the reference, the default algorithm (Knowles-Handy)
// only applies E (its two-component KH branch is empty); "hz" applies the full operator.
#include "rel.cuh"
#include "rdm.cuh"

#include <algorithm>
#include <string>

namespace f2g {

__global__ void k_rel_spmv(int64_t N0, int nnz, const int32_t* __restrict__ col, const double* __restrict__ vr,
                           const double* __restrict__ vi, const double2* __restrict__ C, double2* __restrict__ S,
                           int64_t vstride) {
    const int64_t J = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (J >= N0)
        return;
    C += blockIdx.y * vstride;
    S += blockIdx.y * vstride;
    double ar = 0.0, ai = 0.0;
    for (int k = lane; k < nnz; k += 32) {
        const int64_t e = J * nnz + k;
        const double hr = vr[e], hi = vi[e];
        const double2 c = C[col[e]];
        ar += hr * c.x - hi * c.y;
        ai += hr * c.y + hi * c.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ar += __shfl_down_sync(0xffffffffu, ar, o);
        ai += __shfl_down_sync(0xffffffffu, ai, o);
    }
    if (lane == 0)
        S[J] = make_double2(ar, ai);
}

__global__ void k_rel_scale(int64_t n, double E, const double2* __restrict__ C, double2* __restrict__ S) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 c = C[i];
        S[i] = make_double2(E * c.x, E * c.y);
    }
}

__global__ void k_rel_diag(int64_t N0, int nnz, const double* __restrict__ vr, const double* __restrict__ vi,
                           double2* __restrict__ out) {
    const int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (J < N0)
        out[J] = make_double2(vr[J * nnz], vi[J * nnz]);
}

RelSigmaBuilder::RelSigmaBuilder(CIStrings* s_, double E_, const std::complex<double>* H_,
                                 const std::complex<double>* V_)
    : s(s_), n(s_->norb) {
    if (s->nb != 0)
        throw Error(1, "RelCISigmaBuilder requires nb == 0 (two-component CI treats all electrons as alpha spinors).");
    set_hamiltonian(E_, H_, V_);
}

void RelSigmaBuilder::set_hamiltonian(double E_, const std::complex<double>* H_, const std::complex<double>* V_) {
    E = E_;
    const size_t n2 = (size_t)n * n, n4 = n2 * n2;
    H.assign(H_, H_ + n2);
    V.assign(V_, V_ + n4);
    std::vector<double> hr(n2), hi(n2), vr(n4), vi(n4);
    for (size_t i = 0; i < n2; ++i) {
        hr[i] = H[i].real();
        hi[i] = H[i].imag();
    }
    for (size_t i = 0; i < n4; ++i) {
        vr[i] = V[i].real();
        vi[i] = V[i].imag();
    }
    hre.reserve(std::max<size_t>(1, n2));
    him.reserve(std::max<size_t>(1, n2));
    vre.reserve(std::max<size_t>(1, n4));
    vim.reserve(std::max<size_t>(1, n4));
    if (n2) {
        F2G_CUDA(cudaMemcpy(hre.get(), hr.data(), n2 * 8, cudaMemcpyHostToDevice));
        F2G_CUDA(cudaMemcpy(him.get(), hi.data(), n2 * 8, cudaMemcpyHostToDevice));
        F2G_CUDA(cudaMemcpy(vre.get(), vr.data(), n4 * 8, cudaMemcpyHostToDevice));
        F2G_CUDA(cudaMemcpy(vim.get(), vi.data(), n4 * 8, cudaMemcpyHostToDevice));
    }
    const SpinStrings& a = s->a;
    nnz = ss_row_nnz(n, a.k);
    if (a.N0 == 0 || nnz == 0)
        return;
    const size_t total = (size_t)a.N0 * nnz;
    col.reserve(total);
    valr.reserve(total);
    vali.reserve(total);
    build_ss_values(n, a.k, a.N0, nnz, a.str.get(), s->binom.get(), hre.get(), vre.get(), E, col.get(), valr.get(), 0);
    build_ss_values(n, a.k, a.N0, nnz, a.str.get(), s->binom.get(), him.get(), vim.get(), 0.0, col.get(), vali.get(),
                    0);
    F2G_CUDA(cudaStreamSynchronize(0));
}

// The reference's K-block contract (rel_ci_sigma_builder_harrison_zarrabian.cc:28-60): one complex
// column of norb (H1) or norb(norb-1)/2 (H2) elements must fit each of its two buffers.
void RelSigmaBuilder::check_memory() const {
    const size_t maxel = memory / (2 * sizeof(std::complex<double>));
    auto need = [&](size_t nrows) {
        if (nrows && maxel < nrows)
            throw Error(1, "The CI builder memory limit (" + std::to_string(memory) +
                               " bytes) is too small for one complex K-block column of " + std::to_string(nrows) +
                               " elements per buffer.");
    };
    if (algorithm == 1) {
        if (s->na >= 1)
            need((size_t)n);
        if (s->na >= 2)
            need((size_t)n * (n - 1) / 2);
    }
}

void RelSigmaBuilder::hamiltonian(const double2* C, double2* S, cudaStream_t st, int nvec) {
    const int64_t nd = s->ndet, nf = s->nfull;
    if (nd == 0 || nvec <= 0)
        return;
    if (nvec > 65535)
        throw Error(2, "RelCISigmaBuilder: at most 65535 vectors per call");
    check_memory();
    if (algorithm == 0) {
        k_rel_scale<<<1024, 256, 0, st>>>((int64_t)nvec * nd, E, C, S);
        F2G_LAUNCH("k_rel_scale");
        return;
    }
    const double2* c = C;
    double2* o = S;
    const DetEnum de = s->dets();
    if (s->blocked()) {
        double2* xc = xC.reserve((size_t)nvec * nf);
        double2* xs = xS.reserve((size_t)nvec * nf);
        blocks_embed<double2>(de, nf, C, xc, nvec, st);
        c = xc;
        o = xs;
    }
    const int64_t rows = s->a.N0;
    k_rel_spmv<<<dim3((unsigned)ceil_div(rows * 32, 256), (unsigned)nvec), 256, 0, st>>>(
        rows, nnz, col.get(), valr.get(), vali.get(), c, o, nf);
    F2G_LAUNCH("k_rel_spmv");
    if (s->blocked())
        blocks_extract<double2>(de, nf, o, S, nvec, st, false);
}

void RelSigmaBuilder::hdiag(double2* out, cudaStream_t st) {
    const int64_t nd = s->ndet, nf = s->nfull;
    if (nd == 0)
        return;
    double2* d = out;
    if (s->blocked())
        d = xS.reserve((size_t)nf);
    k_rel_diag<<<ceil_div(nf, 256), 256, 0, st>>>(nf, nnz, valr.get(), vali.get(), d);
    F2G_LAUNCH("k_rel_diag");
    if (s->blocked())
        blocks_extract<double2>(s->dets(), nf, d, out, 1, st, false);
}

std::complex<double> RelSigmaBuilder::element(int64_t I, int64_t J) {
    if (I < 0 || J < 0 || I >= s->ndet || J >= s->ndet)
        throw Error(2, "determinant index out of range");
    // C1 addresses (nb = 0: the beta string is the vacuum, the C1 address is the alpha rank)
    auto c1 = [&](int64_t i) -> int64_t {
        if (!s->blocked())
            return i;
        const DetBlocks& B = s->blocks;
        for (int b = 0; b < B.nblk(); ++b) {
            const int64_t* r = B.hblk.data() + 6 * b;
            if (r[2] > 0 && i >= r[3] && i < r[3] + r[2]) {
                const int64_t ja = B.cls_off[0][r[0]] + (i - r[3]) / r[5];
                return (int64_t)B.rank[0][ja];
            }
        }
        throw Error(1, "determinant index not in a block");
    };
    const int64_t a = c1(I), b = c1(J);
    std::vector<int32_t> cols(nnz);
    std::vector<double> re(nnz), im(nnz);
    F2G_CUDA(cudaMemcpy(cols.data(), col.get() + a * nnz, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
    F2G_CUDA(cudaMemcpy(re.data(), valr.get() + a * nnz, nnz * sizeof(double), cudaMemcpyDeviceToHost));
    F2G_CUDA(cudaMemcpy(im.data(), vali.get() + a * nnz, nnz * sizeof(double), cudaMemcpyDeviceToHost));
    for (int k = 0; k < nnz; ++k)
        if (cols[k] == b)
            return {re[k], im[k]};
    return {0.0, 0.0};
}

// ---- spin-orbital RDMs -----------------------------------------------------------------------

__global__ void k_split_planes(int64_t n, const double2* __restrict__ x, double* __restrict__ re,
                               double* __restrict__ im) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = x[i];
        re[i] = v.x;
        im[i] = v.y;
    }
}

// out = (a + b) + i (c - d)
__global__ void k_combine(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                          const double* __restrict__ c, const double* __restrict__ d, double2* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_double2(a[i] + b[i], c[i] - d[i]);
}

__device__ __forceinline__ int so_pair(int a, int b) { return a > b ? a * (a - 1) / 2 + b : b * (b - 1) / 2 + a; }
__device__ __forceinline__ int so_trip(int a, int b, int c) {
    const int x = max(a, max(b, c)), z = min(a, min(b, c)), y = a + b + c - x - z;
    return x * (x - 1) * (x - 2) / 6 + y * (y - 1) / 2 + z;
}
__device__ __forceinline__ double so_sign3(int a, int b, int c) {
    return (((a < b) + (a < c) + (b < c)) & 1) ? -1.0 : 1.0;
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// packed [pq][rs] (p > q, r > s) to [p][q][r][s], antisymmetric in p, q and in r, s
__global__ void k_expand2(int n, const double2* __restrict__ pk, double2* __restrict__ out) {
    const int64_t np = (int64_t)n * (n - 1) / 2, n2 = (int64_t)n * n, total = n2 * n2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / (n2 * n)), q = (int)(i / n2 % n), r = (int)(i / n % n), s = (int)(i % n);
        double2 v = make_double2(0.0, 0.0);
        if (p != q && r != s) {
            v = pk[(int64_t)so_pair(p, q) * np + so_pair(r, s)];
            if ((p > q) != (r > s)) {
                v.x = -v.x;
                v.y = -v.y;
            }
        }
        out[i] = v;
    }
}

// packed [pqr][stu] to n^6, antisymmetric in each index triple
__global__ void k_expand3(int n, const double2* __restrict__ pk, double2* __restrict__ out) {
    const int64_t nt = (int64_t)n * (n - 1) * (n - 2) / 6, n3 = (int64_t)n * n * n, total = n3 * n3;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a3 = i / n3, b3 = i % n3;
        const int o1 = (int)(a3 / (n * n)), o2 = (int)(a3 / n % n), o3 = (int)(a3 % n);
        const int o4 = (int)(b3 / (n * n)), o5 = (int)(b3 / n % n), o6 = (int)(b3 % n);
        double2 v = make_double2(0.0, 0.0);
        if (o1 != o2 && o1 != o3 && o2 != o3 && o4 != o5 && o4 != o6 && o5 != o6) {
            v = pk[(int64_t)so_trip(o1, o2, o3) * nt + so_trip(o4, o5, o6)];
            const double sg = so_sign3(o1, o2, o3) * so_sign3(o4, o5, o6);
            v.x *= sg;
            v.y *= sg;
        }
        out[i] = v;
    }
}

// L2 = G2 - G1[p][r] G1[q][s] + G1[p][s] G1[q][r] (rel_ci_sigma_builder_rdm.cc, compute_2cumulant)
__global__ void k_so_cum2(int n, const double2* __restrict__ g1, double2* __restrict__ l2) {
    const int64_t n2 = (int64_t)n * n, total = n2 * n2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / (n2 * n)), q = (int)(i / n2 % n), r = (int)(i / n % n), s = (int)(i % n);
        const double2 a = cmul(g1[p * n + r], g1[q * n + s]), b = cmul(g1[p * n + s], g1[q * n + r]);
        double2 v = l2[i];
        v.x += -a.x + b.x;
        v.y += -a.y + b.y;
        l2[i] = v;
    }
}

// the spin-orbital 3-cumulant in place (rel_ci_sigma_builder_rdm.cc, compute_3cumulant)
__global__ void k_so_cum3(int n, const double2* __restrict__ g1, const double2* __restrict__ g2, double2* __restrict__ l3) {
    const int64_t n2 = (int64_t)n * n, n3 = n2 * n, total = n3 * n3;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / (n3 * n2)), q = (int)(i / (n3 * n) % n), r = (int)(i / n3 % n);
        const int s = (int)(i / n2 % n), t = (int)(i / n % n), u = (int)(i % n);
        auto G1 = [&](int a, int b) { return g1[a * n + b]; };
        auto G2 = [&](int a, int b, int c, int d) { return g2[(((int64_t)a * n + b) * n + c) * n + d]; };
        double2 v = l3[i];
        auto add = [&](double w, double2 x) {
            v.x += w * x.x;
            v.y += w * x.y;
        };
        add(-1.0, cmul(G1(p, s), G2(q, r, t, u)));
        add(-1.0, cmul(G1(q, t), G2(p, r, s, u)));
        add(-1.0, cmul(G1(r, u), G2(p, q, s, t)));
        add(1.0, cmul(G1(p, t), G2(q, r, s, u)));
        add(1.0, cmul(G1(p, u), G2(q, r, t, s)));
        add(1.0, cmul(G1(q, s), G2(p, r, t, u)));
        add(1.0, cmul(G1(q, u), G2(p, r, s, t)));
        add(1.0, cmul(G1(r, s), G2(p, q, u, t)));
        add(1.0, cmul(G1(r, t), G2(p, q, s, u)));
        add(2.0, cmul(cmul(G1(p, s), G1(q, t)), G1(r, u)));
        add(-2.0, cmul(cmul(G1(p, s), G1(q, u)), G1(r, t)));
        add(-2.0, cmul(cmul(G1(p, u), G1(q, t)), G1(r, s)));
        add(-2.0, cmul(cmul(G1(p, t), G1(q, s)), G1(r, u)));
        add(2.0, cmul(cmul(G1(p, t), G1(q, u)), G1(r, s)));
        add(2.0, cmul(cmul(G1(p, u), G1(q, s)), G1(r, t)));
        l3[i] = v;
    }
}

int64_t RelSigmaBuilder::rdm_size(int n, int kind) {
    const int64_t n2 = (int64_t)n * n;
    switch (kind) {
    case 0:
        return n2;
    case 1:
    case 2:
        return n2 * n2;
    case 3:
    case 4:
        return n2 * n2 * n2;
    default:
        throw Error(2, "spin-orbital RDM kind must be between 0 and 4");
    }
}

static int ew_grid(int64_t total) { return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 4096)); }

void RelSigmaBuilder::rdm(int kind, const double2* CL, const double2* CR, double2* out, cudaStream_t st) {
    const int64_t size = rdm_size(n, kind);
    if (size == 0)
        return;
    F2G_CUDA(cudaMemsetAsync(out, 0, (size_t)size * sizeof(double2), st));
    const int64_t nd = s->ndet;
    if (nd == 0 || s->na < 1)
        return;
    if (!rsb)
        rsb = std::make_unique<SigmaBuilder>(s, SigmaBuilder::RdmOnly{});
    double* P = planes.reserve((size_t)4 * nd);
    double *lr = P, *li = P + nd, *rr = P + 2 * nd, *ri = P + 3 * nd;
    k_split_planes<<<ew_grid(nd), 256, 0, st>>>(nd, CL, lr, li);
    k_split_planes<<<ew_grid(nd), 256, 0, st>>>(nd, CR, rr, ri);
    F2G_LAUNCH("k_split_planes");
    // the complex contraction of one real kind from four real ones
    auto complex_kind = [&](int rk, double2* dst) {
        const int64_t m = f2g::rdm_size(n, rk);
        double* R = parts.reserve((size_t)4 * std::max<int64_t>(1, m));
        compute_rdm(*rsb, rk, lr, rr, R, st);
        compute_rdm(*rsb, rk, li, ri, R + m, st);
        compute_rdm(*rsb, rk, lr, ri, R + 2 * m, st);
        compute_rdm(*rsb, rk, li, rr, R + 3 * m, st);
        k_combine<<<ew_grid(m), 256, 0, st>>>(m, R, R + m, R + 2 * m, R + 3 * m, dst);
        F2G_LAUNCH("k_combine");
    };
    const int64_t n2 = (int64_t)n * n, n4 = n2 * n2;
    switch (kind) {
    case 0:
        complex_kind(kRdmA1, out);
        break;
    case 1:
    case 2: {
        if (s->na >= 2 && n >= 2) {
            double2* pk = packed.reserve((size_t)f2g::rdm_size(n, kRdmAA));
            complex_kind(kRdmAA, pk);
            k_expand2<<<ew_grid(n4), 256, 0, st>>>(n, pk, out);
            F2G_LAUNCH("k_expand2");
        }
        if (kind == 2) {
            double2* G1 = g1.reserve((size_t)n2);
            complex_kind(kRdmA1, G1);
            k_so_cum2<<<ew_grid(n4), 256, 0, st>>>(n, G1, out);
            F2G_LAUNCH("k_so_cum2");
        }
        break;
    }
    case 3:
    case 4: {
        if (s->na >= 3 && n >= 3) {
            double2* pk = packed.reserve((size_t)f2g::rdm_size(n, kRdmAAA));
            complex_kind(kRdmAAA, pk);
            k_expand3<<<ew_grid(size), 256, 0, st>>>(n, pk, out);
            F2G_LAUNCH("k_expand3");
        }
        if (kind == 4) {
            double2* G1 = g1.reserve((size_t)n2);
            double2* G2 = g2.reserve((size_t)n4);
            complex_kind(kRdmA1, G1);
            F2G_CUDA(cudaMemsetAsync(G2, 0, (size_t)n4 * sizeof(double2), st));
            if (s->na >= 2 && n >= 2) {
                double2* pk = packed.reserve((size_t)std::max(f2g::rdm_size(n, kRdmAA), f2g::rdm_size(n, kRdmAAA)));
                complex_kind(kRdmAA, pk);
                k_expand2<<<ew_grid(n4), 256, 0, st>>>(n, pk, G2);
                F2G_LAUNCH("k_expand2");
            }
            k_so_cum3<<<ew_grid(size), 256, 0, st>>>(n, G1, G2, out);
            F2G_LAUNCH("k_so_cum3");
        }
        break;
    }
    }
}

} // namespace f2g
