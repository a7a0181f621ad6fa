// Device kernels for the Davidson-Liu solver (forte2/helpers/davidsonliu.py:184-484), FP64.
// Vectors are stored as rows: X_i = X + i * ld, i.e. the transpose of the reference's (size, m)
// column blocks, so that every vector is contiguous.
//
//   dots      out[i * nb + j] = <A_i, B_j>       (subspace matrix B^T S, projections, overlaps)
//   lincomb   Y_j = beta Y_j + sum_i coef[i, j] X_i   (collapse, final eigenvectors, projections)
//   residual  R_r = S alpha_r - lambda_r B alpha_r, ||R_r||^2, then R_r / (lambda_r - Hdiag) where
//             |lambda_r - Hdiag| > threshold, else 0 (davidsonliu.py:271-293)
//   eigh      cyclic Jacobi on the small subspace matrix, eigenvalues ascending (replaces eigh,
//             davidsonliu.py:259)
// All reductions are two-stage with a fixed order, so results are bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "common.cuh"

namespace f2g {

constexpr int kTile = 256;

__global__ void __launch_bounds__(256) k_dots_partial(const double* __restrict__ A, int na, int64_t lda,
                                                      const double* __restrict__ B, int nb, int64_t ldb, int64_t n,
                                                      double* __restrict__ partial) {
    extern __shared__ double sm[];
    double* As = sm;                       // [na][kTile + 1]
    double* Bs = sm + (size_t)na * (kTile + 1); // [nb][kTile + 1]
    const int npair = na * nb;
    double acc[4] = {0, 0, 0, 0};
    for (int64_t base = (int64_t)blockIdx.x * kTile; base < n; base += (int64_t)gridDim.x * kTile) {
        __syncthreads();
        for (int t = threadIdx.x; t < na * kTile; t += blockDim.x) {
            const int i = t / kTile, e = t % kTile;
            As[i * (kTile + 1) + e] = base + e < n ? A[i * lda + base + e] : 0.0;
        }
        for (int t = threadIdx.x; t < nb * kTile; t += blockDim.x) {
            const int i = t / kTile, e = t % kTile;
            Bs[i * (kTile + 1) + e] = base + e < n ? B[i * ldb + base + e] : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < 4; ++k) {
            const int pr = threadIdx.x + k * blockDim.x;
            if (pr >= npair)
                break;
            const double* a = As + (pr / nb) * (kTile + 1);
            const double* b = Bs + (pr % nb) * (kTile + 1);
            double s = 0.0;
#pragma unroll 8
            for (int e = 0; e < kTile; ++e)
                s += a[e] * b[e];
            acc[k] += s;
        }
    }
    for (int k = 0; k < 4; ++k) {
        const int pr = threadIdx.x + k * blockDim.x;
        if (pr < npair)
            partial[(int64_t)blockIdx.x * npair + pr] = acc[k];
    }
}

__global__ void k_reduce_partials(int nblocks, int npair, const double* partial, double* out) {
    const int pr = blockIdx.x * blockDim.x + threadIdx.x;
    if (pr >= npair)
        return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b)
        s += partial[(int64_t)b * npair + pr];
    out[pr] = s;
}

__global__ void k_lincomb(const double* __restrict__ X, int nx, int64_t ldx, const double* __restrict__ coef, int ny,
                          double* __restrict__ Y, int64_t ldy, double beta, int64_t n) {
    extern __shared__ double sc[];
    for (int t = threadIdx.x; t < nx * ny; t += blockDim.x)
        sc[t] = coef[t];
    __syncthreads();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        double x[64];
        const int nxx = nx < 64 ? nx : 64;
        for (int i = 0; i < nxx; ++i)
            x[i] = X[i * ldx + e];
        for (int j = 0; j < ny; ++j) {
            double s = beta == 0.0 ? 0.0 : beta * Y[j * ldy + e];
            for (int i = 0; i < nxx; ++i)
                s += sc[i * ny + j] * x[i];
            Y[j * ldy + e] = s;
        }
    }
}

__global__ void __launch_bounds__(256) k_residual(const double* __restrict__ B, const double* __restrict__ S, int m,
                                                  int64_t ld, const double* __restrict__ alpha, const double* __restrict__ lam,
                                                  int nroot, const double* __restrict__ hdiag, int64_t n, double thresh,
                                                  double* __restrict__ R, int64_t ldr, double* __restrict__ partial) {
    __shared__ double sa[64 * 16];
    __shared__ double sl[16];
    __shared__ double red[16][256];
    for (int t = threadIdx.x; t < m * nroot; t += blockDim.x)
        sa[t] = alpha[t];
    for (int t = threadIdx.x; t < nroot; t += blockDim.x)
        sl[t] = lam[t];
    __syncthreads();
    double nrm[16];
    for (int r = 0; r < nroot; ++r)
        nrm[r] = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const double hd = hdiag[e];
        double bv[64], sv[64];
        for (int i = 0; i < m; ++i) {
            bv[i] = B[i * ld + e];
            sv[i] = S[i * ld + e];
        }
        for (int r = 0; r < nroot; ++r) {
            double ba = 0.0, sa_ = 0.0;
            for (int i = 0; i < m; ++i) {
                ba += bv[i] * sa[i * nroot + r];
                sa_ += sv[i] * sa[i * nroot + r];
            }
            const double res = sa_ - ba * sl[r];
            nrm[r] += res * res;
            const double den = sl[r] - hd;
            R[r * ldr + e] = fabs(den) > thresh ? res / den : 0.0;
        }
    }
    for (int r = 0; r < nroot; ++r)
        red[r][threadIdx.x] = nrm[r];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int r = 0; r < nroot; ++r)
                red[r][threadIdx.x] += red[r][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < nroot)
        partial[(int64_t)blockIdx.x * nroot + threadIdx.x] = red[threadIdx.x][0];
}

// Cyclic Jacobi for a symmetric m x m matrix (m <= 64), one block. Output: eigenvalues ascending,
// eigenvectors as columns of V (row-major V[i * m + j]).
__global__ void k_jacobi(int m, const double* __restrict__ G, double* __restrict__ evals, double* __restrict__ V,
                         int max_sweeps) {
    __shared__ double A[64][65];
    __shared__ double Q[64][65];
    __shared__ double cs[2];
    __shared__ double off_red[128];
    __shared__ int stop;
    const int t = threadIdx.x;
    // Hermitize on load: A = (G + G^T) / 2 (davidsonliu.py:258)
    for (int k = t; k < m * m; k += blockDim.x) {
        const int i = k / m, j = k % m;
        A[i][j] = 0.5 * (G[i * m + j] + G[j * m + i]);
        Q[i][j] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int k = t; k < m * m; k += blockDim.x) {
            const int i = k / m, j = k % m;
            const double a2 = A[i][j] * A[i][j];
            tot += a2;
            if (i != j)
                off += a2;
        }
        off_red[t] = off;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (t < w)
                off_red[t] += off_red[t + w];
            __syncthreads();
        }
        const double offsum = off_red[0];
        __syncthreads();
        off_red[t] = tot;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (t < w)
                off_red[t] += off_red[t + w];
            __syncthreads();
        }
        if (t == 0)
            stop = (offsum <= 1e-32 * off_red[0]) || offsum == 0.0;
        __syncthreads();
        if (stop)
            break;
        for (int p = 0; p < m - 1; ++p) {
            for (int q = p + 1; q < m; ++q) {
                if (t == 0) {
                    const double apq = A[p][q];
                    double c = 1.0, s = 0.0;
                    if (apq != 0.0) {
                        const double tau = (A[q][q] - A[p][p]) / (2.0 * apq);
                        const double tt = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        c = 1.0 / sqrt(1.0 + tt * tt);
                        s = tt * c;
                    }
                    cs[0] = c;
                    cs[1] = s;
                }
                __syncthreads();
                const double c = cs[0], s = cs[1];
                if (s != 0.0) {
                    if (t < m) {
                        const double akp = A[t][p], akq = A[t][q];
                        A[t][p] = c * akp - s * akq;
                        A[t][q] = s * akp + c * akq;
                        const double vkp = Q[t][p], vkq = Q[t][q];
                        Q[t][p] = c * vkp - s * vkq;
                        Q[t][q] = s * vkp + c * vkq;
                    }
                    __syncthreads();
                    if (t < m) {
                        const double apk = A[p][t], aqk = A[q][t];
                        A[p][t] = c * apk - s * aqk;
                        A[q][t] = s * apk + c * aqk;
                    }
                }
                __syncthreads();
            }
        }
    }
    __syncthreads();
    if (t == 0) {
        // selection sort of eigenpairs, ascending
        int order[64];
        double w[64];
        for (int i = 0; i < m; ++i) {
            order[i] = i;
            w[i] = A[i][i];
        }
        for (int i = 0; i < m; ++i) {
            int b = i;
            for (int j = i + 1; j < m; ++j)
                if (w[j] < w[b])
                    b = j;
            const double tw = w[i];
            w[i] = w[b];
            w[b] = tw;
            const int to = order[i];
            order[i] = order[b];
            order[b] = to;
        }
        for (int i = 0; i < m; ++i)
            evals[i] = w[i];
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j)
                V[i * m + j] = Q[i][order[j]];
    }
}

// ---- host wrappers ----------------------------------------------------------------------------

static int dots_blocks(int64_t n) {
    const int64_t b = (n + kTile - 1) / kTile;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 1216));
}

void dav_dots(const double* A, int na, int64_t lda, const double* B, int nb, int64_t ldb, int64_t n, double* out,
              double* scratch, cudaStream_t st) {
    if (na * nb == 0)
        return;
    if (nb > 64 || na > 64)
        throw Error(2, "dots: at most 64 vectors per operand");
    // rows of A in chunks so that one launch holds at most 1024 pairs (4 per thread)
    const int chunk = std::max(1, std::min(na, std::min(32, 1024 / nb)));
    const int nbk = dots_blocks(n);
    for (int i0 = 0; i0 < na; i0 += chunk) {
        const int ni = std::min(chunk, na - i0);
        const size_t smem = (size_t)(ni + nb) * (kTile + 1) * sizeof(double);
        if (smem > 48 * 1024)
            F2G_CUDA(cudaFuncSetAttribute(k_dots_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_dots_partial<<<nbk, 256, smem, st>>>(A + (int64_t)i0 * lda, ni, lda, B, nb, ldb, n, scratch);
        F2G_LAUNCH("k_dots_partial");
        k_reduce_partials<<<ceil_div(ni * nb, 128), 128, 0, st>>>(nbk, ni * nb, scratch, out + (int64_t)i0 * nb);
        F2G_LAUNCH("k_reduce_partials");
    }
}

int64_t dav_scratch_size(int64_t n) { return (int64_t)dots_blocks(n) * 4 * 256 + 64; }

// ---- dots without a caller-provided scratch buffer --------------------------------------------
// Some callers cannot allocate device memory when they need these dot products: a host program
// whose device memory is handed out by its own pool (cudaMalloc would bypass the pool, and fails
// once the pool has reserved the GPU's memory), or one that must not add the device-wide
// synchronisation a cudaMalloc/cudaFree can cause in the middle of its iteration loop. For them
// the per-block partial sums live in this file-scope static array instead of a caller buffer.
// It is 304 blocks x 256 vector pairs of doubles (608 KB); every GPU that loads the library holds
// it until the process exits. Each call overwrites exactly the partials it then reads, so nothing
// has to start at zero. All calls share the array: calls that overlap on the GPU (different
// streams, or several host threads) race on it and must be serialised by the caller.
constexpr int kStaticBlocks = 304;
constexpr int kStaticPairs = 256;
static __device__ __align__(256) double g_static_partials[kStaticBlocks * kStaticPairs];

namespace {
std::mutex g_static_mu;
double* g_static_ptr[128] = {};
} // namespace

// Device address of g_static_partials on the current device. In host code the array's name is only
// a host-side stand-in, so the address is looked up once per device with that device current; the
// first call on a device therefore does this set-up (it should come before any stream capture).
static double* static_partials() {
    int dev = 0;
    F2G_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128)
        throw Error(1, "dots_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_partials);
        if (e != cudaSuccess || p == nullptr)
            throw Error(3, std::string("dots_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        g_static_ptr[dev] = static_cast<double*>(p);
    }
    return g_static_ptr[dev];
}

void dav_dots_noalloc(const double* A, int na, int64_t lda, const double* B, int nb, int64_t ldb, int64_t n,
                      double* out, cudaStream_t st) {
    if (na < 0 || nb < 0 || n < 0)
        throw Error(2, "dots_noalloc: negative size");
    if (na * nb == 0)
        return;
    if (na > 64 || nb > 64)
        throw Error(2, "dots_noalloc: at most 64 vectors per operand");
    if ((int64_t)na * nb > kStaticPairs)
        throw Error(2, "dots_noalloc: na * nb = " + std::to_string((int64_t)na * nb) +
                           " vector pairs exceeds the static scratch limit of " + std::to_string(kStaticPairs) +
                           " pairs per call");
    double* partial = static_partials();
    const int nbk = (int)std::max<int64_t>(1, std::min<int64_t>((n + kTile - 1) / kTile, kStaticBlocks));
    const size_t smem = (size_t)(na + nb) * (kTile + 1) * sizeof(double);
    if (smem > 48 * 1024)
        F2G_CUDA(cudaFuncSetAttribute(k_dots_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_dots_partial<<<nbk, 256, smem, st>>>(A, na, lda, B, nb, ldb, n, partial);
    F2G_LAUNCH("k_dots_partial (static scratch)");
    k_reduce_partials<<<ceil_div(na * nb, 128), 128, 0, st>>>(nbk, na * nb, partial, out);
    F2G_LAUNCH("k_reduce_partials (static scratch)");
}

void dav_lincomb(const double* X, int nx, int64_t ldx, const double* coef, int ny, double* Y, int64_t ldy, double beta,
                 int64_t n, cudaStream_t st) {
    if (nx > 64 || ny > 64)
        throw Error(2, "lincomb: at most 64 vectors");
    if (ny == 0 || n == 0)
        return;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
    k_lincomb<<<blocks, 256, (size_t)nx * ny * sizeof(double), st>>>(X, nx, ldx, coef, ny, Y, ldy, beta, n);
    F2G_LAUNCH("k_lincomb");
}

void dav_residual(const double* B, const double* S, int m, int64_t ld, const double* alpha, const double* lam, int nroot,
                  const double* hdiag, int64_t n, double thresh, double* R, int64_t ldr, double* norms2, double* scratch,
                  cudaStream_t st) {
    if (m > 64 || nroot > 16)
        throw Error(2, "residual: at most 64 basis vectors and 16 roots");
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8));
    k_residual<<<blocks, 256, 0, st>>>(B, S, m, ld, alpha, lam, nroot, hdiag, n, thresh, R, ldr, scratch);
    F2G_LAUNCH("k_residual");
    k_reduce_partials<<<1, 32, 0, st>>>(blocks, nroot, scratch, norms2);
    F2G_LAUNCH("k_reduce_partials");
}

void dav_eigh(int m, const double* G, double* evals, double* evecs, cudaStream_t st) {
    if (m > 64)
        throw Error(2, "eigh: subspace larger than 64");
    k_jacobi<<<1, 128, 0, st>>>(m, G, evals, evecs, 100);
    F2G_LAUNCH("k_jacobi");
}

} // namespace f2g
