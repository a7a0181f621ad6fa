// FP32 same-spin sigma terms as dense GEMMs on the tensor cores (the mixed-precision mode's option
// for large spaces).
//
// Operator: sigma_aa(Ja, Ib) = sum_Ia Ha[Ja][Ia] C(Ia, Ib) and sigma_bb(Ia, Jb) = sum_Ib
// Hb[Jb][Ib] C(Ia, Ib), with Ha, Hb the same-spin string Hamiltonians (the reference's H1_hz +
// H2_hz_same_spin of one spin, forte2/ci/ci_sigma_builder_harrison_zarrabian.cc:20-150; Ha also
// carries E on its diagonal). Each string Hamiltonian row has 1 + k(n-k) + C(k,2) C(n-k,2)
// couplings (347 of 3,432 at CAS(14,14)), so the dense product does about 10 times the
// multiply-adds of the sparse row kernel; on the tensor cores it still takes a fraction of the
// time of the sparse kernel, which is bound by re-reading whole rows of C from L2 (CAS(14,14):
// 0.21 ms per spin against 1.31 ms). Spaces of at most kDenseSsMaxStrings strings per spin: at
// CAS(16,16) (12,870 strings) the dense product is slower than the sparse kernel (44 against
// 33 ms per spin) and the FP32 accumulation over K = 12,870 loses accuracy (4e-6 relative).
//
// Accuracy: H (per spin) and C (per vector) are scaled by powers of two into [2^14, 2^15) and
// split x = hi + lo into two FP16 parts; each product is H_hi C_hi + H_lo C_hi + H_hi C_lo, three
// cuBLAS FP16 GEMMs accumulating in FP32 (22 significant bits per operand, as the tensor-core
// opposite-spin kernel), unscaled exactly by the power-of-two alpha. The contraction is cut into
// chunks of kDssChunk along K, each its own GEMM added in FP32, which bounds the accumulation error
// of the tensor cores' FP32 sums (it grows with K). Leading dimensions of the FP16 operands are
// padded to multiples of 8 (16-byte rows). The scales live in device
// memory (pointer mode device), so captured graphs follow new integrals and vectors.
//
// Determinism: one GEMM call per vector and product, in a fixed order; cuBLAS gives the same bits
// for the same call on the same device, so sigma is bitwise the same for every batch shape.
#include <cublas_v2.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <memory>
#include <string>

#include "sigma.cuh"

namespace f2g {

struct DenseSameSpin {
    cublasHandle_t handle = nullptr;
    DevBuf<char> workspace;
    int64_t N0[2] = {0, 0};
    int64_t ld[2] = {0, 0};        // padded row length of the FP16 operands of each spin
    DevBuf<__half> hhi[2], hlo[2]; // dense H of each spin [J][I], scaled
    DevBuf<unsigned int> hmax;     // [2] largest |H| of each spin (FP32 bits)
    // per call set (0 direct, 1 graph): split vectors, their largest magnitudes, alpha values
    DevBuf<__half> chi[2], clo[2];
    DevBuf<unsigned int> cmax[2];
    DevBuf<float> alpha[2];        // [spin][v]
    DevBuf<float> consts;          // {0, 1}: the beta values
    ~DenseSameSpin() {
        if (handle)
            cublasDestroy(handle);
    }
};

namespace {

constexpr size_t kWorkspaceBytes = size_t(32) << 20;
constexpr int64_t kDssChunk = 1024; // K per GEMM

void cublas_check(cublasStatus_t s, const char* what) {
    if (s != CUBLAS_STATUS_SUCCESS)
        throw Error(3, std::string("dense same-spin sigma: ") + what + " failed with cuBLAS status " +
                           std::to_string((int)s));
}

// 2^e as a float for -126 <= e <= 127
__device__ __forceinline__ float p2(int e) { return __int_as_float((e + 127) << 23); }

// exponent that maps a largest magnitude m into [2^14, 2^15) (0 for m = 0 or not finite)
__device__ __forceinline__ int scale_exponent(float m) {
    if (!(m > 0.0f) || !(m <= 3.0e38f))
        return 0;
    int ex = 0;
    (void)frexpf(m, &ex);
    const int e = 15 - ex;
    return e < -120 ? -120 : (e > 120 ? 120 : e);
}

__device__ __forceinline__ void split_half(float x, __half& hi, __half& lo) {
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

// out[v] = largest |x| of vector v (FP32 bits; non-negative floats order like their bits); zeroed first
__global__ void k_dss_absmax(int64_t n, const float* __restrict__ x, unsigned int* __restrict__ out) {
    x += blockIdx.y * n;
    float m = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[32];
    if ((threadIdx.x & 31) == 0)
        wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0)
            atomicMax(out + blockIdx.y, __float_as_uint(m));
    }
}

// dense H[J][I] (zeroed before) from the string Hamiltonian rows: row J lists (I, value); every I
// appears at most once per row with a non-zero value (padding entries carry 0 and are skipped)
__global__ void k_dss_fill(int64_t N0, int64_t ld, int nnz, const int32_t* __restrict__ col,
                           const float* __restrict__ val, const unsigned int* __restrict__ hmax,
                           __half* __restrict__ hi, __half* __restrict__ lo) {
    const float f = p2(scale_exponent(__uint_as_float(*hmax)));
    const int64_t total = N0 * nnz;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const float v = val[t];
        if (v == 0.0f)
            continue;
        const int64_t J = t / nnz, I = col[t];
        __half h, l;
        split_half(v * f, h, l);
        hi[J * ld + I] = h;
        lo[J * ld + I] = l;
    }
}

// the split parts of nvec vectors, each scaled by its own power of two
// (rows x cols vectors; row pitch ldc of the split parts, whose padding columns are zero)
__global__ void k_dss_split(int64_t rows, int64_t cols, int64_t ldc, const float* __restrict__ C,
                            const unsigned int* __restrict__ cmax, __half* __restrict__ hi, __half* __restrict__ lo) {
    const int v = blockIdx.y;
    const float f = p2(scale_exponent(__uint_as_float(cmax[v])));
    C += v * rows * cols;
    hi += v * rows * ldc;
    lo += v * rows * ldc;
    const int64_t total = rows * ldc;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / ldc, c = i - r * ldc;
        __half h = __float2half_rn(0.0f), l = h;
        if (c < cols)
            split_half(C[r * cols + c] * f, h, l);
        hi[i] = h;
        lo[i] = l;
    }
}

// alpha[spin][v] = 2^-(eh[spin] + ec[v]): the exact unscaling of the products
__global__ void k_dss_alpha(int nvec, const unsigned int* __restrict__ hmax, const unsigned int* __restrict__ cmax,
                            float* __restrict__ alpha) {
    const int v = threadIdx.x;
    if (v >= nvec)
        return;
    const int ec = scale_exponent(__uint_as_float(cmax[v]));
    for (int spin = 0; spin < 2; ++spin) {
        const int e = scale_exponent(__uint_as_float(hmax[spin])) + ec;
        // e <= 240: split the unscaling into two normal factors' product, exact for powers of two
        alpha[spin * nvec + v] = p2(-(e / 2)) * p2(-(e - e / 2));
    }
}

} // namespace

// (Re)build the dense split string Hamiltonians from the FP32 rows, on st. The first call
// allocates them (2 x N0^2 halves per spin: 1.32 GB at CAS(16,16)) and the cuBLAS handle.
void dense_ss_build(const CIStrings* s, const StringHamiltonian* sh[2], std::shared_ptr<DenseSameSpin>& d,
                    cudaStream_t st) {
    if (!d) {
        auto t = std::make_shared<DenseSameSpin>();
        cublas_check(cublasCreate(&t->handle), "cublasCreate");
        cublas_check(cublasSetPointerMode(t->handle, CUBLAS_POINTER_MODE_DEVICE), "cublasSetPointerMode");
        t->workspace.reserve(kWorkspaceBytes);
        cublas_check(cublasSetWorkspace(t->handle, t->workspace.get(), kWorkspaceBytes), "cublasSetWorkspace");
        t->hmax.reserve(2);
        t->consts.reserve(2);
        const float c01[2] = {0.0f, 1.0f};
        F2G_CUDA(cudaMemcpy(t->consts.get(), c01, sizeof(c01), cudaMemcpyHostToDevice));
        for (int spin = 0; spin < 2; ++spin) {
            t->N0[spin] = s->spin(spin).N0;
            t->ld[spin] = (t->N0[spin] + 7) / 8 * 8;
            const size_t m = (size_t)std::max<int64_t>(1, t->N0[spin] * t->ld[spin]);
            t->hhi[spin].reserve(m);
            t->hlo[spin].reserve(m);
        }
        d = t;
    }
    F2G_CUDA(cudaMemsetAsync(d->hmax.get(), 0, 2 * sizeof(unsigned int), st));
    for (int spin = 0; spin < 2; ++spin) {
        const int64_t N0 = d->N0[spin];
        if (N0 == 0)
            continue;
        F2G_CUDA(cudaMemsetAsync(d->hhi[spin].get(), 0, (size_t)N0 * d->ld[spin] * sizeof(__half), st));
        F2G_CUDA(cudaMemsetAsync(d->hlo[spin].get(), 0, (size_t)N0 * d->ld[spin] * sizeof(__half), st));
        const StringHamiltonian& h = *sh[spin];
        const int64_t total = N0 * h.nnz;
        if (total == 0)
            continue;
        k_dss_absmax<<<dim3(256, 1), 256, 0, st>>>(total, h.valf.get(), d->hmax.get() + spin);
        F2G_LAUNCH("k_dss_absmax H");
        const int grid = (int)std::min<int64_t>((total + 255) / 256, 8192);
        k_dss_fill<<<grid, 256, 0, st>>>(N0, d->ld[spin], h.nnz, h.col.get(), h.valf.get(), d->hmax.get() + spin,
                                         d->hhi[spin].get(), d->hlo[spin].get());
        F2G_LAUNCH("k_dss_fill");
    }
}

// Scratch of dense_ss_split / dense_ss_term for nvec vectors of one set (graph captures must not
// allocate: the set of captured graphs is reserved before a capture)
void dense_ss_reserve(const CIStrings* s, DenseSameSpin& d, int nvec, int set) {
    const int64_t NA = s->a.N0, ldb = d.ld[1];
    d.chi[set].reserve((size_t)std::max<int64_t>(1, nvec * NA * ldb));
    d.clo[set].reserve((size_t)std::max<int64_t>(1, nvec * NA * ldb));
    d.cmax[set].reserve((size_t)std::max(1, nvec));
    d.alpha[set].reserve((size_t)2 * std::max(1, nvec));
}

// The split parts of nvec vectors of the C1 space (scales and alpha values in device memory), for
// the GEMMs of dense_ss_term. set: 0 direct calls, 1 captured graphs (separate scratch).
void dense_ss_split(const CIStrings* s, DenseSameSpin& d, const float* C, int nvec, int set, cudaStream_t st) {
    const int64_t NA = s->a.N0, NB = s->b.N0, nd = NA * NB, ldb = d.ld[1];
    if (nvec > 1024)
        throw Error(2, "dense same-spin sigma: at most 1024 vectors per call");
    dense_ss_reserve(s, d, nvec, set);
    F2G_CUDA(cudaMemsetAsync(d.cmax[set].get(), 0, (size_t)nvec * sizeof(unsigned int), st));
    if (nd == 0)
        return;
    k_dss_absmax<<<dim3(256, (unsigned)nvec), 256, 0, st>>>(nd, C, d.cmax[set].get());
    F2G_LAUNCH("k_dss_absmax C");
    k_dss_split<<<dim3(1024, (unsigned)nvec), 256, 0, st>>>(NA, NB, ldb, C, d.cmax[set].get(), d.chi[set].get(),
                                                            d.clo[set].get());
    F2G_LAUNCH("k_dss_split");
    k_dss_alpha<<<1, 1024, 0, st>>>(nvec, d.hmax.get(), d.cmax[set].get(), d.alpha[set].get());
    F2G_LAUNCH("k_dss_alpha");
}

// sigma (nvec FP32 vectors) <- (accumulate: +=) the same-spin term of one spin (0 alpha, 1 beta),
// from the split vectors of the last dense_ss_split of the same set
void dense_ss_term(const CIStrings* s, DenseSameSpin& d, float* sig, int spin, bool accumulate, int nvec, int set,
                   cudaStream_t st) {
    const int64_t NA = s->a.N0, NB = s->b.N0, nd = NA * NB;
    if (nd == 0)
        return;
    const int64_t lda = d.ld[0], ldb = d.ld[1]; // padded rows of Ha and of Hb and the split vectors
    cublas_check(cublasSetStream(d.handle, st), "cublasSetStream");
    const float* zero = d.consts.get();
    const float* one = d.consts.get() + 1;
    const int64_t K = spin ? NB : NA;
    for (int v = 0; v < nvec; ++v) {
        const __half* chi = d.chi[set].get() + (size_t)v * NA * ldb;
        const __half* clo = d.clo[set].get() + (size_t)v * NA * ldb;
        float* S = sig + (size_t)v * nd;
        const float* al = d.alpha[set].get() + (size_t)spin * nvec + v;
        bool first = !accumulate;
        for (int p = 0; p < 3; ++p) {
            for (int64_t k0 = 0; k0 < K; k0 += kDssChunk) {
                const int kc = (int)std::min<int64_t>(kDssChunk, K - k0);
                const float* be = first ? zero : one;
                first = false;
                if (spin == 1) {
                    // S^T (NB x NA, column-major) = Hb C^T: Hb stored [Jb][Ib] is (Hb)^T column-major;
                    // the chunk takes Ib in [k0, k0 + kc)
                    const __half* A = (p == 1 ? d.hlo[1].get() : d.hhi[1].get()) + k0;
                    const __half* B = (p == 2 ? clo : chi) + k0;
                    cublas_check(cublasGemmEx(d.handle, CUBLAS_OP_T, CUBLAS_OP_N, (int)NB, (int)NA, kc, al, A,
                                              CUDA_R_16F, (int)ldb, B, CUDA_R_16F, (int)ldb, be, S, CUDA_R_32F,
                                              (int)NB, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT),
                                 "cublasGemmEx (beta spin)");
                } else {
                    // S^T (NB x NA) = C^T Ha^T: C stored [Ia][Ib] is C^T column-major, Ha [Ja][Ia] is
                    // Ha^T; the chunk takes Ia in [k0, k0 + kc)
                    const __half* A = (p == 2 ? clo : chi) + k0 * ldb;
                    const __half* B = (p == 1 ? d.hlo[0].get() : d.hhi[0].get()) + k0;
                    cublas_check(cublasGemmEx(d.handle, CUBLAS_OP_N, CUBLAS_OP_N, (int)NB, (int)NA, kc, al, A,
                                              CUDA_R_16F, (int)ldb, B, CUDA_R_16F, (int)lda, be, S, CUDA_R_32F,
                                              (int)NB, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT),
                                 "cublasGemmEx (alpha spin)");
                }
            }
        }
    }
}

} // namespace f2g
