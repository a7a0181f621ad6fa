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

} // namespace f2g
