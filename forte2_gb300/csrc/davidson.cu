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

#include "davidson.cuh"

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

// Jacobi eigensolver for a symmetric m x m matrix (m <= 64), one block of at least 32 threads.
// Output: eigenvalues ascending, eigenvectors as columns of V (row-major V[i * ldv + j]).
// Parallel cyclic ordering (Brent and Luk, 1985; round-robin tournament): each sweep has
// m' - 1 steps (m' = m rounded up to even) and each step rotates m'/2 disjoint pairs at once, so
// the rotations of a step commute and are applied as one row pass and one column pass. Each
// rotation zeroes A[p][q] with t = sgn(tau) / (|tau| + sqrt(1 + tau^2)), tau = (A_qq - A_pp) /
// (2 A_pq), c = 1 / sqrt(1 + t^2), s = t c. Sweeps stop when the off-diagonal squared norm is at
// most 1e-32 of the total.
template <int MAXM>
__device__ void jacobi_block(int m, const double* __restrict__ G, int ldg, double* __restrict__ evals,
                             double* __restrict__ V, int ldv, int max_sweeps) {
    __shared__ double A[MAXM][MAXM + 1];
    __shared__ double Q[MAXM][MAXM + 1];
    __shared__ double rc[MAXM / 2], rs[MAXM / 2];
    __shared__ int rp[MAXM / 2], rq[MAXM / 2];
    __shared__ double red[2][32];
    __shared__ int order[MAXM];
    __shared__ int rotated; // a rotation was applied in this sweep
    const int t = threadIdx.x, nt = blockDim.x;
    const int M = m + (m & 1), npair = M / 2;
    // Hermitize on load: A = (G + G^T) / 2 (davidsonliu.py:258)
    for (int k = t; k < m * m; k += nt) {
        const int i = k / m, j = k % m;
        A[i][j] = 0.5 * (G[i * ldg + j] + G[j * ldg + i]);
        Q[i][j] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int sweep = 0; sweep < max_sweeps && m > 1; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int k = t; k < m * m; k += nt) {
            const int i = k / m, j = k % m;
            const double a2 = A[i][j] * A[i][j];
            tot += a2;
            if (i != j)
                off += a2;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_down_sync(0xffffffffu, off, o);
            tot += __shfl_down_sync(0xffffffffu, tot, o);
        }
        if ((t & 31) == 0) {
            red[0][t >> 5] = off;
            red[1][t >> 5] = tot;
        }
        __syncthreads();
        double offsum = 0.0, totsum = 0.0;
        for (int w = 0; w < (nt + 31) / 32; ++w) {
            offsum += red[0][w];
            totsum += red[1][w];
        }
        __syncthreads();
        if (offsum <= 1e-32 * totsum || offsum == 0.0)
            break;
        if (t == 0)
            rotated = 0;
        __syncthreads();
        for (int step = 0; step < M - 1; ++step) {
            if (t < npair) {
                // players 0..M-1: 0 stays, 1..M-1 rotate; pair t is (r(t), r(M-1-t))
                const int a_ = t == 0 ? 0 : (t - 1 + step) % (M - 1) + 1;
                const int b_ = (M - 1 - t - 1 + step) % (M - 1) + 1;
                const int p = min(a_, b_), q = max(a_, b_);
                double c = 1.0, sn = 0.0;
                if (q < m) {
                    const double apq = A[p][q];
                    // an element below 1e-17 of both diagonal elements moves no eigenvalue or
                    // vector at FP64 precision: left, so that the sweeps end when none is left
                    if (apq != 0.0 && !(fabs(apq) <= 1e-17 * fmax(fabs(A[p][p]), fabs(A[q][q])))) {
                        rotated = 1;
                        const double tau = (A[q][q] - A[p][p]) / (2.0 * apq);
                        const double tt = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        c = 1.0 / sqrt(1.0 + tt * tt);
                        sn = tt * c;
                    }
                }
                rp[t] = p;
                rq[t] = q < m ? q : -1;
                rc[t] = c;
                rs[t] = sn;
            }
            __syncthreads();
            // columns: A <- A J, Q <- Q J
            for (int k = t; k < npair * m; k += nt) {
                const int pr = k / m, i = k % m, q = rq[pr];
                if (q < 0 || rs[pr] == 0.0)
                    continue;
                const int p = rp[pr];
                const double c = rc[pr], sn = rs[pr];
                const double aip = A[i][p], aiq = A[i][q];
                A[i][p] = c * aip - sn * aiq;
                A[i][q] = sn * aip + c * aiq;
                const double vip = Q[i][p], viq = Q[i][q];
                Q[i][p] = c * vip - sn * viq;
                Q[i][q] = sn * vip + c * viq;
            }
            __syncthreads();
            // rows: A <- J^T A
            for (int k = t; k < npair * m; k += nt) {
                const int pr = k / m, j = k % m, q = rq[pr];
                if (q < 0 || rs[pr] == 0.0)
                    continue;
                const int p = rp[pr];
                const double c = rc[pr], sn = rs[pr];
                const double apj = A[p][j], aqj = A[q][j];
                A[p][j] = c * apj - sn * aqj;
                A[q][j] = sn * apj + c * aqj;
            }
            __syncthreads();
        }
        if (!rotated)
            break; // every off-diagonal element is negligible
    }
    // ascending order by rank (ties by index), then gather
    for (int i = t; i < m; i += nt) {
        const double w = A[i][i];
        int r = 0;
        for (int j = 0; j < m; ++j) {
            const double x = A[j][j];
            r += (x < w) || (x == w && j < i);
        }
        order[r] = i;
    }
    __syncthreads();
    for (int i = t; i < m; i += nt)
        evals[i] = A[order[i]][order[i]];
    for (int k = t; k < m * m; k += nt) {
        const int i = k / m, j = k % m;
        V[i * ldv + j] = Q[i][order[j]];
    }
}

__global__ void k_jacobi(int m, const double* __restrict__ G, double* __restrict__ evals, double* __restrict__ V,
                         int max_sweeps) {
    jacobi_block<64>(m, G, m, evals, V, m, max_sweeps);
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
// The address is kept for the life of the process: a cudaDeviceReset (or any reset of the device's
// primary context) unloads the module that holds the array, so this entry point must not be called
// again after one.
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


// ---- Gram-Schmidt with on-device acceptance ----------------------------------------------------
// The acceptance rule is the reference's (davidsonliu.py:438-484): each candidate is cycled (at
// most 10 times) through v -= sum_i <B_i,v> B_i, rejected when |v| < discard, v /= |v|, and
// accepted once max_i |<B_i,v>| < ortho and |<v,v> - 1| < ortho. One CTA runs the whole sequence,
// so the decisions never leave the device; it suits the short vectors (up to a few 10^4) for which
// host round trips, not bandwidth, bound the iteration.
constexpr int kGsChunk = 8;
constexpr int kGsThreads = 1024;

// out[j] = <B_{i0+j}, v> for j < cnt (cnt <= kGsChunk); whole-CTA reduction in a fixed order.
__device__ void gs_block_dots(const double* B, int64_t ld, int i0, int cnt, const double* v, int64_t n,
                              double (*red)[kGsChunk], double* out) {
    double acc[kGsChunk];
#pragma unroll
    for (int j = 0; j < kGsChunk; ++j)
        acc[j] = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const double x = v[e];
#pragma unroll
        for (int j = 0; j < kGsChunk; ++j)
            if (j < cnt)
                acc[j] += B[(int64_t)(i0 + j) * ld + e] * x;
    }
#pragma unroll
    for (int j = 0; j < kGsChunk; ++j)
        for (int off = 16; off > 0; off >>= 1)
            acc[j] += __shfl_down_sync(0xffffffffu, acc[j], off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < kGsChunk; ++j)
            red[warp][j] = acc[j];
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            s += red[w][threadIdx.x];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

// Uniform deviate in [-1, 1) from a counter (SplitMix64 output function, Steele, Lea and Flood,
// OOPSLA 2014), for the random vectors that replace rejected candidates.
__device__ __forceinline__ double gs_uniform(uint64_t seed, uint64_t stream, uint64_t e) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (stream * 0x100000001B3ull + e + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53 * 2.0 - 1.0;
}

struct GsShared {
    double red[kGsThreads / 32][kGsChunk];
    double dv[72];
    double scal[2];
};

// Orthonormalise row s of B (already holding the candidate) against rows [0, s). Returns 1 if
// accepted. Every thread returns the same value (decisions read shared values after a barrier).
__device__ int gs_one(double* B, int64_t ld, int s, int64_t n, double discard, double ortho, GsShared& sh) {
    double* v = B + (int64_t)s * ld;
    for (int cycle = 0; cycle < 10; ++cycle) {
        for (int i0 = 0; i0 < s; i0 += kGsChunk)
            gs_block_dots(B, ld, i0, min(kGsChunk, s - i0), v, n, sh.red, sh.dv + i0);
        if (s > 0) {
            for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
                double x = v[e];
                for (int i = 0; i < s; ++i)
                    x -= sh.dv[i] * B[(int64_t)i * ld + e];
                v[e] = x;
            }
            __syncthreads();
        }
        gs_block_dots(v, 0, 0, 1, v, n, sh.red, sh.scal);
        const double nrm = sqrt(fmax(sh.scal[0], 0.0));
        if (nrm < discard)
            return 0;
        const double inv = 1.0 / nrm;
        for (int64_t e = threadIdx.x; e < n; e += blockDim.x)
            v[e] *= inv;
        __syncthreads();
        for (int i0 = 0; i0 < s; i0 += kGsChunk)
            gs_block_dots(B, ld, i0, min(kGsChunk, s - i0), v, n, sh.red, sh.dv + i0);
        gs_block_dots(v, 0, 0, 1, v, n, sh.red, sh.scal + 1);
        double mo = 0.0;
        for (int i = 0; i < s; ++i)
            mo = fmax(mo, fabs(sh.dv[i]));
        if (mo < ortho && fabs(sh.scal[1] - 1.0) < ortho)
            return 1;
    }
    return 0;
}

// Append candidates R_c (c < ncand) to B[0, m0), then random rows until m0 + added >= min_total
// (at most 10 tries per missing row). Rows are written in place, so B needs cap >= m0 + ncand and
// cap >= min_total rows (checked on the host).
__global__ void __launch_bounds__(kGsThreads) k_gs_append(double* B, int64_t ld, int m0, const double* R,
                                                          int64_t ldr, int ncand, int64_t n, double discard,
                                                          double ortho, int min_total, uint64_t seed, int* added) {
    __shared__ GsShared sh;
    int nadd = 0;
    for (int c = 0; c < ncand; ++c) {
        double* v = B + (int64_t)(m0 + nadd) * ld;
        const double* rc = R + (int64_t)c * ldr;
        for (int64_t e = threadIdx.x; e < n; e += blockDim.x)
            v[e] = rc[e];
        __syncthreads();
        nadd += gs_one(B, ld, m0 + nadd, n, discard, ortho, sh);
    }
    const int missing = min_total - m0 - nadd;
    for (int t = 0; t < 10 * missing && m0 + nadd < min_total; ++t) {
        double* v = B + (int64_t)(m0 + nadd) * ld;
        for (int64_t e = threadIdx.x; e < n; e += blockDim.x)
            v[e] = gs_uniform(seed, (uint64_t)t, (uint64_t)e);
        __syncthreads();
        nadd += gs_one(B, ld, m0 + nadd, n, discard, ortho, sh);
    }
    if (threadIdx.x == 0)
        *added = nadd;
}

// Threads of the one-block Gram-Schmidt: about 8 elements per thread, 64 to 1024 (whole warps),
// so that short vectors do not pay for barriers across idle warps.
static int gs_threads(int64_t n) {
    const int64_t t = ((n / 8 + 31) / 32) * 32;
    return (int)std::max<int64_t>(64, std::min<int64_t>(kGsThreads, t));
}

void dav_gs_append(double* B, int64_t ld, int cap, int m0, const double* R, int64_t ldr, int ncand, int64_t n,
                   double discard, double ortho, int min_total, uint64_t seed, int* added, cudaStream_t st) {
    if (m0 < 0 || ncand < 0 || n < 0)
        throw Error(2, "gs_append: negative size");
    if (cap > 64 || m0 + ncand > cap || min_total > cap)
        throw Error(2, "gs_append: the basis holds at most min(64, cap) vectors");
    k_gs_append<<<1, gs_threads(n), 0, st>>>(B, ld, m0, R, ldr, ncand, n, discard, ortho, min_total, seed, added);
    F2G_LAUNCH("k_gs_append");
}

// ---- device-driven iteration -------------------------------------------------------------------
// Each kernel returns at once unless the solve is running, so a captured run of iterations stops
// doing work as soon as one of them converges. Sizes that change during the solve (basis size,
// collapse) come from the state; grids are sized for the largest case.

__global__ void k_dg_reset(DGState* st, DGReset r) {
    int m = r.m;
    if (r.dev_m)
        m = max(0, min(r.m, *r.dev_m));
    st->m = m;
    st->sigma_size = r.sigma_size < 0 ? m : min(r.sigma_size, m);
    st->iter = 0;
    st->status = kDGRunning;
    st->collapse = 0;
    st->added = 0;
    st->m_eig = 0;
    st->g_size = 0;
    st->maxiter = r.maxiter;
    st->stall_window = r.stall_window;
    st->e_tol = r.e_tol;
    st->r_tol = r.r_tol;
    st->stall_floor = r.stall_floor;
    st->max_de = st->max_r = 0.0;
    st->ortho_dev = 0.0;
    for (int i = 0; i < 64; ++i) {
        st->lam_old[i] = i < r.nlam ? r.lam_old[i] : 0.0;
        st->lam[i] = 0.0;
    }
    if (r.S) {
        // np.allclose(S, I, atol=1e-11) of the starting basis (the check at the start of the
        // reference's solve); the deviation reported is max |S - I|
        bool ok = true;
        double dev = 0.0;
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) {
                const double d = i == j ? 1.0 : 0.0;
                const double x = fabs(r.S[i * r.ldS + j] - d);
                dev = fmax(dev, x);
                if (!(x <= 1e-11 + 1e-5 * d))
                    ok = false;
            }
        st->ortho_dev = dev;
        if (!ok)
            st->status = kDGNotOrthoStart;
    }
    if (m == 0)
        st->status = kDGNotOrthoStart;
}

void dg_reset(DGState* st, const DGReset& r, cudaStream_t s) {
    k_dg_reset<<<1, 1, 0, s>>>(st, r);
    F2G_LAUNCH("k_dg_reset");
}

__global__ void k_dg_stage(const DGState* st, const double* __restrict__ b, int64_t ld, int R, int64_t n,
                           double* __restrict__ out) {
    if (st->status != kDGRunning)
        return;
    const int lo = st->sigma_size, m = st->m;
    const int64_t total = (int64_t)R * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / n);
        const int64_t e = t - (int64_t)r * n;
        out[t] = lo + r < m ? b[(int64_t)(lo + r) * ld + e] : 0.0;
    }
}

static int dg_grid(int64_t work) { return (int)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, 152 * 8)); }

void dg_stage(const DGState* st, const double* b, int64_t ld, int R, int64_t n, double* out, cudaStream_t s) {
    k_dg_stage<<<dg_grid((int64_t)R * n), 256, 0, s>>>(st, b, ld, R, n, out);
    F2G_LAUNCH("k_dg_stage");
}

// Bodies shared by the one-kernel-per-step iteration and the fused one-block iteration. Loops are
// grid-stride, so a body called from a one-block kernel covers everything with that block.

__device__ void dg_unstage_body(const DGState* st, const double* __restrict__ in, int R, int64_t n,
                                double* __restrict__ sigma, int64_t ld) {
    const int lo = st->sigma_size, m = st->m;
    const int64_t total = (int64_t)R * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / n);
        const int64_t e = t - (int64_t)r * n;
        if (lo + r < m)
            sigma[(int64_t)(lo + r) * ld + e] = in[t];
    }
}

__global__ void k_dg_unstage(const DGState* st, const double* __restrict__ in, int R, int64_t n,
                             double* __restrict__ sigma, int64_t ld) {
    if (st->status != kDGRunning)
        return;
    dg_unstage_body(st, in, R, n, sigma, ld);
}

void dg_unstage(const DGState* st, const double* in, int R, int64_t n, double* sigma, int64_t ld, cudaStream_t s) {
    k_dg_unstage<<<dg_grid((int64_t)R * n), 256, 0, s>>>(st, in, R, n, sigma, ld);
    F2G_LAUNCH("k_dg_unstage");
}

// One CTA per (i, j) pair of a grid of ni x nj; pairs outside the current sizes return.
__global__ void __launch_bounds__(256) k_dg_dots(const DGState* st, int which, const double* __restrict__ A,
                                                 int64_t lda, const double* __restrict__ B, int64_t ldb, int64_t n,
                                                 int ni, int nj, double* __restrict__ out, int ldo) {
    if (st->status != kDGRunning)
        return;
    if ((which == 1 || which == 2) && !st->collapse)
        return;
    const int i = blockIdx.x / nj, j = blockIdx.x % nj;
    int li = ni, lj = nj;
    if (which == 0 || which == 1 || which == 5)
        li = lj = st->m;
    else if (which == 3)
        li = st->m;
    if (i >= li || j >= lj)
        return;
    if (which == 5 && i < st->g_size && j < st->g_size)
        return; // still current
    const double* a = A + (int64_t)i * lda;
    const double* bb = B + (int64_t)j * ldb;
    double acc = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x)
        acc += a[e] * bb[e];
    __shared__ double red[8];
    for (int off = 16; off > 0; off >>= 1)
        acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            s += red[w];
        out[i * ldo + j] = s;
    }
}

// Long vectors: every block takes a strided share of the elements for 8 pairs at a time; partial
// sums per block, added in block order by k_dg_dots_reduce (the same pair selection as k_dg_dots).
__device__ __forceinline__ void dg_pair_limits(const DGState* st, int which, int ni, int nj, int& li, int& lj) {
    li = ni;
    lj = nj;
    if (which == 0 || which == 1 || which == 5)
        li = lj = st->m;
    else if (which == 3)
        li = st->m;
}

// Pairs of a launch: all li x lj, or for which == 5 (the subspace matrix after new sigma rows)
// only those outside the g x g block that is still current: rows i < g with j >= g, then every
// pair of the rows i >= g. Each pair's sum does not depend on which other pairs a launch holds,
// so the matrix is bitwise the one a full computation gives.
__device__ __forceinline__ int dg_pair_count(const DGState* st, int which, int li, int lj) {
    if (which != 5)
        return li * lj;
    const int g = min(st->g_size, li);
    return li * lj - g * g;
}
__device__ __forceinline__ void dg_pair(const DGState* st, int which, int pr, int li, int lj, int& i, int& j) {
    if (which != 5) {
        i = pr / lj;
        j = pr % lj;
        return;
    }
    const int g = min(st->g_size, li), w = lj - g;
    if (pr < g * w) {
        i = pr / w;
        j = g + pr % w;
    } else {
        pr -= g * w;
        i = g + pr / lj;
        j = pr % lj;
    }
}

__global__ void __launch_bounds__(256) k_dg_dots_partial(const DGState* st, int which, const double* __restrict__ A,
                                                         int64_t lda, const double* __restrict__ B, int64_t ldb,
                                                         int64_t n, int ni, int nj, double* __restrict__ partial) {
    if (st->status != kDGRunning)
        return;
    if ((which == 1 || which == 2) && !st->collapse)
        return;
    int li, lj;
    dg_pair_limits(st, which, ni, nj, li, lj);
    const int np = dg_pair_count(st, which, li, lj);
    const int64_t e0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, step = (int64_t)gridDim.x * blockDim.x;
    __shared__ double red[8][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int p0 = 0; p0 < np; p0 += 8) {
        double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int cnt = min(8, np - p0);
        const double* ap[8];
        const double* bp[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            int i = 0, j = 0;
            if (q < cnt)
                dg_pair(st, which, p0 + q, li, lj, i, j);
            ap[q] = A + (int64_t)i * lda;
            bp[q] = B + (int64_t)j * ldb;
        }
        for (int64_t e = e0; e < n; e += step)
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q < cnt)
                    a[q] += ap[q][e] * bp[q][e];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            double x = a[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0)
                red[w][q] = x;
        }
        __syncthreads();
        if (threadIdx.x < cnt) {
            double t = 0.0;
            for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww)
                t += red[ww][threadIdx.x];
            partial[(int64_t)blockIdx.x * 4096 + p0 + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

__global__ void k_dg_dots_reduce(const DGState* st, int which, int ni, int nj, int nblocks,
                                 const double* __restrict__ partial, double* __restrict__ out, int ldo) {
    if (st->status != kDGRunning)
        return;
    if ((which == 1 || which == 2) && !st->collapse)
        return;
    int li, lj;
    dg_pair_limits(st, which, ni, nj, li, lj);
    const int pr = blockIdx.x * blockDim.x + threadIdx.x;
    if (pr >= dg_pair_count(st, which, li, lj))
        return;
    double t = 0.0;
    for (int bk = 0; bk < nblocks; ++bk)
        t += partial[(int64_t)bk * 4096 + pr];
    int i, j;
    dg_pair(st, which, pr, li, lj, i, j);
    out[i * ldo + j] = t;
}

void dg_dots_long(const DGState* st, int which, const double* A, int64_t lda, const double* B, int64_t ldb, int64_t n,
                  int ni, int nj, double* out, int ldo, double* partial, cudaStream_t s) {
    if (ni <= 0 || nj <= 0 || ni > 64 || nj > 64)
        throw Error(2, "dg_dots: 1 to 64 vectors per operand");
    const int blocks = dg_gsm_blocks(n);
    k_dg_dots_partial<<<blocks, 256, 0, s>>>(st, which, A, lda, B, ldb, n, ni, nj, partial);
    F2G_LAUNCH("k_dg_dots_partial");
    k_dg_dots_reduce<<<ceil_div(ni * nj, 128), 128, 0, s>>>(st, which, ni, nj, blocks, partial, out, ldo);
    F2G_LAUNCH("k_dg_dots_reduce");
}

void dg_dots(const DGState* st, int which, const double* A, int64_t lda, const double* B, int64_t ldb, int64_t n,
             int ni, int nj, double* out, int ldo, cudaStream_t s) {
    if (ni <= 0 || nj <= 0 || ni > 64 || nj > 64)
        throw Error(2, "dg_dots: 1 to 64 vectors per operand");
    k_dg_dots<<<ni * nj, 256, 0, s>>>(st, which, A, lda, B, ldb, n, ni, nj, out, ldo);
    F2G_LAUNCH("k_dg_dots");
}

// out[i * ldo + j] = <A_i, B_j> for i < ni, j < nj inside one block: one warp per pair.
__device__ void warp_pair_dots(const double* __restrict__ A, int64_t lda, const double* __restrict__ B,
                               int64_t ldb, int64_t n, int ni, int nj, double* __restrict__ out, int ldo) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int p = warp; p < ni * nj; p += nw) {
        const int i = p / nj, j = p % nj;
        const double* a = A + (int64_t)i * lda;
        const double* bb = B + (int64_t)j * ldb;
        double acc = 0.0;
        for (int64_t e = lane; e < n; e += 32)
            acc += a[e] * bb[e];
        for (int off = 16; off > 0; off >>= 1)
            acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0)
            out[i * ldo + j] = acc;
    }
}

__global__ void k_dg_eigh(DGState* st, const double* G, int ldg, double* evals, double* V, int ldv) {
    if (st->status != kDGRunning)
        return;
    const int m = st->m;
    jacobi_block<64>(m, G, ldg, evals, V, ldv, 100);
    __syncthreads();
    if (threadIdx.x == 0) {
        st->m_eig = m;
        st->sigma_size = m;
        st->g_size = m;
    }
}

void dg_eigh(DGState* st, const double* G, int ldg, double* evals, double* V, int ldv, cudaStream_t s) {
    k_dg_eigh<<<1, 128, 0, s>>>(st, G, ldg, evals, V, ldv);
    F2G_LAUNCH("k_dg_eigh");
}

// Residuals of the first nroot Ritz pairs, as k_residual, with m and alpha (columns of V) taken
// from the device; per-block partial squared norms (the total when the grid is one block).
__device__ void dg_residual_body(const DGState* st, const DGParams& P, const double* __restrict__ B,
                                 const double* __restrict__ S, int64_t ld, const double* __restrict__ V, int ldv,
                                 const double* __restrict__ lam, const double* __restrict__ hdiag,
                                 double* __restrict__ R, int64_t ldr, double* __restrict__ partial) {
    const int m = st->m, nroot = P.nroot;
    __shared__ double sa[64 * 16];
    __shared__ double sl[16];
    __shared__ double red[32][16];
    for (int t = threadIdx.x; t < m * nroot; t += blockDim.x)
        sa[t] = V[(t / nroot) * ldv + (t % nroot)];
    for (int t = threadIdx.x; t < nroot; t += blockDim.x)
        sl[t] = lam[t];
    __syncthreads();
    double nrm[16];
    for (int r = 0; r < nroot; ++r)
        nrm[r] = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P.n; e += (int64_t)gridDim.x * blockDim.x) {
        const double hd = hdiag[e];
        for (int r = 0; r < nroot; ++r) {
            double ba = 0.0, sa_ = 0.0;
            for (int i = 0; i < m; ++i) {
                ba += B[i * ld + e] * sa[i * nroot + r];
                sa_ += S[i * ld + e] * sa[i * nroot + r];
            }
            const double res = sa_ - ba * sl[r];
            nrm[r] += res * res;
            const double den = sl[r] - hd;
            R[r * ldr + e] = fabs(den) > P.precond_thresh ? res / den : 0.0;
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = 0; r < nroot; ++r) {
        double v = nrm[r];
        for (int off = 16; off > 0; off >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0)
            red[warp][r] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < nroot) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            v += red[w][threadIdx.x];
        partial[(int64_t)blockIdx.x * nroot + threadIdx.x] = v;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256) k_dg_residual(const DGState* st, DGParams P, const double* __restrict__ B,
                                                     const double* __restrict__ S, int64_t ld,
                                                     const double* __restrict__ V, int ldv,
                                                     const double* __restrict__ lam, const double* __restrict__ hdiag,
                                                     double* __restrict__ R, int64_t ldr, double* __restrict__ partial) {
    if (st->status != kDGRunning)
        return;
    dg_residual_body(st, P, B, S, ld, V, ldv, lam, hdiag, R, ldr, partial);
}

__global__ void k_dg_reduce(const DGState* st, int nblocks, int npair, const double* partial, double* out) {
    if (st->status != kDGRunning)
        return;
    const int pr = threadIdx.x;
    if (pr >= npair)
        return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b)
        s += partial[(int64_t)b * npair + pr];
    out[pr] = s;
}

int dg_residual_blocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 4)); }

void dg_residual(const DGState* st, const DGParams& P, const double* B, const double* S, int64_t ld, const double* V,
                 int ldv, const double* evals, const double* hdiag, double* R, int64_t ldr, double* norms2,
                 double* partial, cudaStream_t s) {
    if (P.nroot > 16 || P.maxm > 64)
        throw Error(2, "dg_residual: at most 16 roots and 64 basis vectors");
    const int blocks = dg_residual_blocks(P.n);
    k_dg_residual<<<blocks, 256, 0, s>>>(st, P, B, S, ld, V, ldv, evals, hdiag, R, ldr, partial);
    F2G_LAUNCH("k_dg_residual");
    k_dg_reduce<<<1, 32, 0, s>>>(st, blocks, P.nroot, partial, norms2);
    F2G_LAUNCH("k_dg_reduce");
}

// Convergence and control decisions of one iteration (davidsonliu.py:295-336), one thread.
// hist holds 4 doubles per iteration: mean root energy, max |dE|, max |r|, basis size.
__device__ void dg_check_body(DGState* st, const DGParams& P, const double* norms2, const double* evals,
                              double* hist) {
    const int nroot = P.nroot, m = st->m, it = st->iter;
    double max_de = 0.0, max_r = 0.0, mean = 0.0;
    for (int r = 0; r < nroot; ++r) {
        const double lam = evals[r];
        st->lam[r] = lam;
        mean += lam;
        max_de = fmax(max_de, fabs(lam - st->lam_old[r]));
        max_r = fmax(max_r, sqrt(fmax(norms2[r], 0.0)));
    }
    for (int r = nroot; r < m; ++r)
        st->lam[r] = evals[r];
    st->max_de = max_de;
    st->max_r = max_r;
    st->iter = it + 1;
    hist[4 * it + 0] = mean / nroot;
    hist[4 * it + 1] = max_de;
    hist[4 * it + 2] = max_r;
    hist[4 * it + 3] = m;
    if ((max_de < st->e_tol && max_r < st->r_tol) || (int64_t)m == P.n) {
        st->status = kDGConverged;
        return;
    }
    const int w = st->stall_window;
    if (w > 0 && it + 1 > w) {
        double recent = hist[4 * (it - w + 1) + 2], before = hist[2];
        for (int k = it - w + 1; k <= it; ++k)
            recent = fmin(recent, hist[4 * k + 2]);
        for (int k = 0; k <= it - w; ++k)
            before = fmin(before, hist[4 * k + 2]);
        if (recent > 0.5 * before && recent < st->stall_floor) {
            st->status = kDGStalled;
            return;
        }
    }
    if (it >= st->maxiter - 1) {
        st->status = kDGMaxIter;
        return;
    }
    for (int r = 0; r < nroot; ++r)
        st->lam_old[r] = evals[r];
    st->collapse = m + nroot > P.maxm;
}

__global__ void k_dg_check(DGState* st, DGParams P, const double* norms2, const double* evals, double* hist) {
    if (st->status != kDGRunning)
        return;
    dg_check_body(st, P, norms2, evals, hist);
}

void dg_check(DGState* st, const DGParams& P, const double* norms2, const double* evals, double* hist, cudaStream_t s) {
    k_dg_check<<<1, 1, 0, s>>>(st, P, norms2, evals, hist);
    F2G_LAUNCH("k_dg_check");
}

// np.allclose(S, I, atol=1e-11) on the basis overlap (davidsonliu.py:391-411): |S_ij - d_ij| <=
// 1e-11 + 1e-5 d_ij. After a passing post-collapse check the basis size becomes collapse_k.
// Block-level; ends with a barrier.
__device__ void dg_orthocheck_body(DGState* st, const DGParams& P, const double* G, int ldg, int after) {
    const int m = after ? P.collapse_k : st->m;
    __shared__ int bad;
    if (threadIdx.x == 0)
        bad = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
        const int i = t / m, j = t % m;
        const double d = i == j ? 1.0 : 0.0;
        if (!(fabs(G[i * ldg + j] - d) <= 1e-11 + 1e-5 * d))
            bad = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (bad) {
            st->status = after ? kDGNotOrthoAfter : kDGNotOrthoBefore;
        } else if (after) {
            st->m = P.collapse_k;
            st->sigma_size = P.collapse_k;
            st->collapse = 0;
            st->g_size = 0; // a new basis: the next subspace matrix is computed in full
        }
    }
    __syncthreads();
}

__global__ void k_dg_orthocheck(DGState* st, DGParams P, const double* G, int ldg, int after) {
    if (st->status != kDGRunning || !st->collapse)
        return;
    dg_orthocheck_body(st, P, G, ldg, after);
}

void dg_orthocheck(DGState* st, const DGParams& P, const double* G, int ldg, int after, cudaStream_t s) {
    k_dg_orthocheck<<<1, 256, 0, s>>>(st, P, G, ldg, after);
    F2G_LAUNCH("k_dg_orthocheck");
}

// tmp[j] = sum_i V[i, j] b_i and tmp[k + j] = sum_i V[i, j] sigma_i for j < k = collapse_k
// (davidsonliu.py:389-411), summed in the order of k_lincomb.
__device__ void dg_collapse_lc_body(const DGState* st, const DGParams& P, const double* __restrict__ b,
                                    const double* __restrict__ sigma, int64_t ld, const double* __restrict__ V,
                                    int ldv, double* __restrict__ tmp, int64_t ldt) {
    const int m = st->m, k = P.collapse_k;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P.n; e += (int64_t)gridDim.x * blockDim.x) {
        for (int j = 0; j < k; ++j) {
            double sb = 0.0, ss = 0.0;
            for (int i = 0; i < m; ++i) {
                const double c = V[i * ldv + j];
                sb += c * b[i * ld + e];
                ss += c * sigma[i * ld + e];
            }
            tmp[j * ldt + e] = sb;
            tmp[(k + j) * ldt + e] = ss;
        }
    }
}

__device__ void dg_collapse_copy_body(const DGParams& P, double* __restrict__ b, double* __restrict__ sigma,
                                      int64_t ld, const double* __restrict__ tmp, int64_t ldt) {
    const int k = P.collapse_k;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P.n; e += (int64_t)gridDim.x * blockDim.x)
        for (int j = 0; j < k; ++j) {
            b[j * ld + e] = tmp[j * ldt + e];
            sigma[j * ld + e] = tmp[(k + j) * ldt + e];
        }
}

__global__ void k_dg_collapse_lc(const DGState* st, DGParams P, const double* __restrict__ b,
                                 const double* __restrict__ sigma, int64_t ld, const double* __restrict__ V, int ldv,
                                 double* __restrict__ tmp, int64_t ldt) {
    if (st->status != kDGRunning || !st->collapse)
        return;
    dg_collapse_lc_body(st, P, b, sigma, ld, V, ldv, tmp, ldt);
}

__global__ void k_dg_collapse_copy(const DGState* st, DGParams P, double* __restrict__ b, double* __restrict__ sigma,
                                   int64_t ld, const double* __restrict__ tmp, int64_t ldt) {
    if (st->status != kDGRunning || !st->collapse)
        return;
    dg_collapse_copy_body(P, b, sigma, ld, tmp, ldt);
}

void dg_collapse(const DGState* st, const DGParams& P, double* b, double* sigma, int64_t ld, const double* V, int ldv,
                 double* tmp, int64_t ldt, cudaStream_t s) {
    const int g = dg_grid(P.n);
    k_dg_collapse_lc<<<g, 256, 0, s>>>(st, P, b, sigma, ld, V, ldv, tmp, ldt);
    F2G_LAUNCH("k_dg_collapse_lc");
    k_dg_collapse_copy<<<g, 256, 0, s>>>(st, P, b, sigma, ld, tmp, ldt);
    F2G_LAUNCH("k_dg_collapse_copy");
}

// r_j -= sum_i D[i, j] b_i for i < m, j < nroot (projection of the new directions out of the basis).
__device__ void dg_project_body(const DGState* st, const DGParams& P, const double* __restrict__ b, int64_t ld,
                                const double* __restrict__ D, double* __restrict__ r, int64_t ldr) {
    const int m = st->m, nroot = P.nroot;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P.n; e += (int64_t)gridDim.x * blockDim.x)
        for (int j = 0; j < nroot; ++j) {
            double s = r[j * ldr + e];
            for (int i = 0; i < m; ++i)
                s += -D[i * nroot + j] * b[i * ld + e];
            r[j * ldr + e] = s;
        }
}

__global__ void k_dg_project(const DGState* st, DGParams P, const double* __restrict__ b, int64_t ld,
                             const double* __restrict__ D, double* __restrict__ r, int64_t ldr) {
    if (st->status != kDGRunning)
        return;
    dg_project_body(st, P, b, ld, D, r, ldr);
}

void dg_project(const DGState* st, const DGParams& P, const double* b, int64_t ld, const double* D, double* r,
                int64_t ldr, cudaStream_t s) {
    k_dg_project<<<dg_grid(P.n), 256, 0, s>>>(st, P, b, ld, D, r, ldr);
    F2G_LAUNCH("k_dg_project");
}

// Append the preconditioned residuals to the basis (davidsonliu.py:338-366): to_add = min(nroot,
// maxm - m) candidates; if some are rejected, as many random vectors are tried once each.
// Block-level (one block).
__device__ void dg_gs_body(DGState* st, const DGParams& P, double* b, int64_t ld, const double* r, int64_t ldr,
                           GsShared& sh) {
    const int m0 = st->m, it = st->iter;
    const int to_add = min(P.nroot, P.maxm - m0);
    if (to_add <= 0) {
        if (threadIdx.x == 0)
            st->status = kDGConverged;
        return;
    }
    int nadd = 0;
    for (int c = 0; c < to_add; ++c) {
        double* v = b + (int64_t)(m0 + nadd) * ld;
        const double* rc = r + (int64_t)c * ldr;
        for (int64_t e = threadIdx.x; e < P.n; e += blockDim.x)
            v[e] = rc[e];
        __syncthreads();
        nadd += gs_one(b, ld, m0 + nadd, P.n, P.discard, P.ortho, sh);
    }
    const int refill = to_add - nadd;
    for (int t = 0; t < refill; ++t) {
        double* v = b + (int64_t)(m0 + nadd) * ld;
        for (int64_t e = threadIdx.x; e < P.n; e += blockDim.x)
            v[e] = gs_uniform(P.seed, (uint64_t)it * 64 + t, (uint64_t)e);
        __syncthreads();
        nadd += gs_one(b, ld, m0 + nadd, P.n, P.discard, P.ortho, sh);
    }
    if (threadIdx.x == 0) {
        st->m = m0 + nadd;
        st->added = nadd;
    }
}

__global__ void __launch_bounds__(kGsThreads) k_dg_gs(DGState* st, DGParams P, double* b, int64_t ld,
                                                      const double* r, int64_t ldr) {
    __shared__ GsShared sh;
    __shared__ int go;
    if (threadIdx.x == 0)
        go = st->status == kDGRunning;
    __syncthreads();
    if (!go)
        return;
    dg_gs_body(st, P, b, ld, r, ldr, sh);
}

void dg_gs(DGState* st, const DGParams& P, double* b, int64_t ld, const double* r, int64_t ldr, cudaStream_t s) {
    k_dg_gs<<<1, gs_threads(P.n), 0, s>>>(st, P, b, ld, r, ldr);
    F2G_LAUNCH("k_dg_gs");
}

// ---- multi-block Gram-Schmidt (graph-captured iterations on long vectors) ----------------------
// Partial sums use a fixed element order per block and are added over blocks in block order, so
// every decision is the same on every run.
constexpr int kGsmCycles = 10;  // the reference's cycle limit per vector
constexpr int kGsmStride = 65;  // partial slots per block: 64 overlaps and the squared norm

int dg_gsm_blocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 1023) / 1024, 152 * 4)); }

__global__ void k_gsm_init(DGState* st, DGParams P, GsmState* g) {
    g->active = 0;
    g->kind = 0;
    if (st->status != kDGRunning) {
        g->to_add = 0;
        return;
    }
    g->m0 = st->m;
    g->to_add = min(P.nroot, P.maxm - st->m);
    g->nadd = g->cand = g->refill_tried = 0;
    g->refill_total = -1;
    if (g->to_add <= 0)
        st->status = kDGConverged;
}

// next slot: the next candidate residual, then (once the candidates are done) as many random vectors
// as candidates were rejected, each tried once
__global__ void k_gsm_pick(const DGState* st, GsmState* g) {
    g->active = 0;
    g->kind = 0;
    if (st->status != kDGRunning || g->to_add <= 0)
        return;
    if (g->cand < g->to_add) {
        g->kind = 1;
        g->src = g->cand++;
    } else {
        if (g->refill_total < 0)
            g->refill_total = g->to_add - g->nadd;
        if (g->refill_tried >= g->refill_total)
            return;
        g->kind = 2;
        g->src = g->refill_tried++;
    }
    g->s = g->m0 + g->nadd;
    g->active = 1;
}

__global__ void k_gsm_load(const DGState* st, DGParams P, const GsmState* g, double* b, int64_t ld,
                           const double* __restrict__ r, int64_t ldr) {
    if (!g->active)
        return;
    double* v = b + (int64_t)g->s * ld;
    const int kind = g->kind, src = g->src;
    const uint64_t stream = (uint64_t)st->iter * 64 + src;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P.n; e += (int64_t)gridDim.x * blockDim.x)
        v[e] = kind == 1 ? r[(int64_t)src * ldr + e] : gs_uniform(P.seed, stream, e);
}

// block sums of 8 values per thread into partial[blockIdx.x * kGsmStride + slot0 + i], fixed order
__device__ void gsm_block_sum8(const double (&a)[8], int cnt, double* partial, int slot0) {
    __shared__ double red[8][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        double x = a[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0)
            red[w][i] = x;
    }
    __syncthreads();
    if (threadIdx.x < cnt) {
        double t = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww)
            t += red[ww][threadIdx.x];
        partial[(int64_t)blockIdx.x * kGsmStride + slot0 + threadIdx.x] = t;
    }
    __syncthreads();
}

// mode 0: overlaps of v with rows 0..s-1; mode 1: v -= sum dv_i b_i, then |v|^2;
// mode 2: v *= inv, then overlaps and |v|^2
__global__ void __launch_bounds__(256) k_gsm_pass(DGParams P, const GsmState* g, double* b, int64_t ld, int mode,
                                                  double* __restrict__ partial) {
    if (!g->active)
        return;
    __shared__ double dv[64];
    const int s = g->s;
    double* v = b + (int64_t)s * ld;
    const int64_t e0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, step = (int64_t)gridDim.x * blockDim.x;
    if (mode == 1) {
        for (int i = threadIdx.x; i < s; i += blockDim.x)
            dv[i] = g->dv[i];
        __syncthreads();
        double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int64_t e = e0; e < P.n; e += step) {
            double x = v[e];
            for (int i = 0; i < s; ++i)
                x -= dv[i] * b[(int64_t)i * ld + e];
            v[e] = x;
            a[0] += x * x;
        }
        gsm_block_sum8(a, 1, partial, 64);
        return;
    }
    if (mode == 2) {
        const double inv = g->inv;
        for (int64_t e = e0; e < P.n; e += step)
            v[e] *= inv;
    }
    for (int i0 = 0; i0 < s; i0 += 8) {
        double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int cnt = min(8, s - i0);
        for (int64_t e = e0; e < P.n; e += step) {
            const double x = v[e];
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (i < cnt)
                    a[i] += b[(int64_t)(i0 + i) * ld + e] * x;
        }
        gsm_block_sum8(a, cnt, partial, i0);
    }
    if (mode == 2) {
        double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int64_t e = e0; e < P.n; e += step)
            a[0] += v[e] * v[e];
        gsm_block_sum8(a, 1, partial, 64);
    }
}

// Sums the block partials in block order and decides (one block of 64 threads).
// mode 0: overlaps -> dv; mode 1: norm -> reject (below the discard threshold) or inv;
// mode 2: overlaps and norm of the normalised vector -> accept, or another cycle
__global__ void k_gsm_decide(DGParams P, GsmState* g, int nblocks, int mode, const double* __restrict__ partial) {
    if (!g->active)
        return;
    __shared__ double tot[kGsmStride];
    const int s = g->s;
    for (int i = threadIdx.x; i < kGsmStride; i += blockDim.x) {
        const bool used = (i < s && mode != 1) || (i == 64 && mode != 0);
        double t = 0.0;
        if (used)
            for (int bk = 0; bk < nblocks; ++bk)
                t += partial[(int64_t)bk * kGsmStride + i];
        tot[i] = t;
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    if (mode == 0) {
        for (int i = 0; i < s; ++i)
            g->dv[i] = tot[i];
    } else if (mode == 1) {
        const double nrm = sqrt(fmax(tot[64], 0.0));
        if (nrm < P.discard)
            g->active = 0; // rejected
        else
            g->inv = 1.0 / nrm;
    } else {
        double mo = 0.0;
        for (int i = 0; i < s; ++i)
            mo = fmax(mo, fabs(tot[i]));
        if (mo < P.ortho && fabs(tot[64] - 1.0) < P.ortho) {
            g->active = 0; // accepted
            g->nadd += 1;
        }
    }
}

__global__ void k_gsm_end_slot(GsmState* g) { g->active = 0; } // cycles exhausted: rejected

__global__ void k_gsm_end(DGState* st, const GsmState* g) {
    if (st->status != kDGRunning || g->to_add <= 0)
        return;
    st->m = g->m0 + g->nadd;
    st->added = g->nadd;
}

void dg_gs_multi(DGState* st, const DGParams& P, double* b, int64_t ld, const double* r, int64_t ldr, GsmState* g,
                 double* partial, cudaStream_t s) {
    const int blocks = dg_gsm_blocks(P.n);
    k_gsm_init<<<1, 1, 0, s>>>(st, P, g);
    F2G_LAUNCH("k_gsm_init");
    for (int slot = 0; slot < 2 * P.nroot; ++slot) {
        k_gsm_pick<<<1, 1, 0, s>>>(st, g);
        F2G_LAUNCH("k_gsm_pick");
        k_gsm_load<<<dg_grid(P.n), 256, 0, s>>>(st, P, g, b, ld, r, ldr);
        F2G_LAUNCH("k_gsm_load");
        for (int cycle = 0; cycle < kGsmCycles; ++cycle) {
            for (int mode = 0; mode < 3; ++mode) {
                k_gsm_pass<<<blocks, 256, 0, s>>>(P, g, b, ld, mode, partial);
                F2G_LAUNCH("k_gsm_pass");
                k_gsm_decide<<<1, 64, 0, s>>>(P, g, blocks, mode, partial);
                F2G_LAUNCH("k_gsm_decide");
            }
        }
        k_gsm_end_slot<<<1, 1, 0, s>>>(g);
        F2G_LAUNCH("k_gsm_end_slot");
    }
    k_gsm_end<<<1, 1, 0, s>>>(st, g);
    F2G_LAUNCH("k_gsm_end");
}

// Everything of one iteration after the sigma build, in one block: for short vectors the
// iteration is bound by the launches of the separate steps, not by their work. Same steps and
// decisions as the separate kernels (unstage, subspace matrix, Jacobi, residuals, convergence,
// collapse with its checks, projection, Gram-Schmidt); dot products are one warp per pair.
template <int MAXM>
__global__ void __launch_bounds__(256) k_dg_small_iter(DGState* st, DGParams P, const double* __restrict__ stage_s,
                                                       int R, double* b, double* sigma, int64_t ld, double* r,
                                                       int64_t ldr, const double* __restrict__ hdiag, double* G,
                                                       double* evals, double* V, double* Dp, double* tmp, int64_t ldt,
                                                       double* hist, double* norms2) {
    __shared__ GsShared gsh;
    __shared__ int flag;
    if (threadIdx.x == 0)
        flag = st->status == kDGRunning;
    __syncthreads();
    if (!flag)
        return;
    dg_unstage_body(st, stage_s, R, P.n, sigma, ld);
    __syncthreads();
    const int m = st->m;
    warp_pair_dots(b, ld, sigma, ld, P.n, m, m, G, P.maxm);
    __syncthreads();
    jacobi_block<MAXM>(m, G, P.maxm, evals, V, P.maxm, 100);
    __syncthreads();
    if (threadIdx.x == 0) {
        st->m_eig = m;
        st->sigma_size = m;
        st->g_size = m;
    }
    dg_residual_body(st, P, b, sigma, ld, V, P.maxm, evals, hdiag, r, ldr, norms2);
    if (threadIdx.x == 0) {
        dg_check_body(st, P, norms2, evals, hist);
        flag = st->status != kDGRunning ? 0 : (st->collapse ? 2 : 1);
    }
    __syncthreads();
    if (flag == 0)
        return;
    if (flag == 2) {
        warp_pair_dots(b, ld, b, ld, P.n, m, m, G, P.maxm);
        __syncthreads();
        dg_orthocheck_body(st, P, G, P.maxm, 0);
        if (st->status != kDGRunning)
            return;
        dg_collapse_lc_body(st, P, b, sigma, ld, V, P.maxm, tmp, ldt);
        __syncthreads();
        dg_collapse_copy_body(P, b, sigma, ld, tmp, ldt);
        __syncthreads();
        warp_pair_dots(b, ld, b, ld, P.n, P.collapse_k, P.collapse_k, G, P.maxm);
        __syncthreads();
        dg_orthocheck_body(st, P, G, P.maxm, 1);
        if (st->status != kDGRunning)
            return;
    }
    const int m2 = st->m;
    warp_pair_dots(b, ld, r, ldr, P.n, m2, P.nroot, Dp, P.nroot);
    __syncthreads();
    dg_project_body(st, P, b, ld, Dp, r, ldr);
    __syncthreads();
    dg_gs_body(st, P, b, ld, r, ldr, gsh);
}

bool dg_small_ok(const DGParams& P) { return P.n <= kDGSmallN && P.maxm <= 32 && P.nroot <= 16; }

void dg_small_iter(DGState* st, const DGParams& P, const double* stage_s, int R, double* b, double* sigma, int64_t ld,
                   double* r, int64_t ldr, const double* hdiag, double* G, double* evals, double* V, double* Dp,
                   double* tmp, int64_t ldt, double* hist, double* norms2, cudaStream_t s) {
    if (!dg_small_ok(P))
        throw Error(2, "dg_small_iter: vectors too long or basis too large for the one-block iteration");
    // one warp for the shortest vectors: its barriers are nearly free, and the work is small
    const int threads = P.n <= 1024 ? 32 : P.n <= 2048 ? 64 : 128;
    if (P.maxm <= 16)
        k_dg_small_iter<16><<<1, threads, 0, s>>>(st, P, stage_s, R, b, sigma, ld, r, ldr, hdiag, G, evals, V, Dp,
                                                 tmp, ldt, hist, norms2);
    else
        k_dg_small_iter<32><<<1, threads, 0, s>>>(st, P, stage_s, R, b, sigma, ld, r, ldr, hdiag, G, evals, V, Dp,
                                                 tmp, ldt, hist, norms2);
    F2G_LAUNCH("k_dg_small_iter");
}

// Defect correction of the mixed-precision operator on R staged rows: S_r += D A_r + X (Bd_r - Mxd A_r)
// with A = X B^T, Bd = D B^T (k x R, from dg_dots) and the symmetric k x k matrix Mxd.
__global__ void k_dg_correct(const DGState* st, const double* __restrict__ X, const double* __restrict__ D,
                             int64_t ldx, const double* __restrict__ Mxd, const double* __restrict__ A,
                             const double* __restrict__ Bd, int k, int R, int64_t n, double* __restrict__ S) {
    if (st->status != kDGRunning)
        return;
    __shared__ double c1[16 * 16], c2[16 * 16];
    for (int t = threadIdx.x; t < k * R; t += blockDim.x) {
        const int i = t / R, r = t % R;
        double s = Bd[t];
        for (int l = 0; l < k; ++l)
            s -= Mxd[i * k + l] * A[l * R + r];
        c1[t] = A[t];
        c2[t] = s;
    }
    __syncthreads();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        for (int r = 0; r < R; ++r) {
            double s = S[r * n + e];
            for (int i = 0; i < k; ++i)
                s += D[i * ldx + e] * c1[i * R + r] + X[i * ldx + e] * c2[i * R + r];
            S[r * n + e] = s;
        }
}

void dg_correct(const DGState* st, const double* X, const double* D, int64_t ldx, const double* Mxd, const double* A,
                const double* Bd, int k, int R, int64_t n, double* S, cudaStream_t s) {
    if (k > 16 || R > 16)
        throw Error(2, "dg_correct: at most 16 corrected vectors and 16 staged rows");
    k_dg_correct<<<dg_grid(n), 256, 0, s>>>(st, X, D, ldx, Mxd, A, Bd, k, R, n, S);
    F2G_LAUNCH("k_dg_correct");
}

// Final Ritz vectors out_j = sum_{i < m} V[i, j] b_i, j < nroot (davidsonliu.py:380-387).
__global__ void k_dg_ritz(const DGState* st, DGParams P, const double* __restrict__ b, int64_t ld,
                          const double* __restrict__ V, int ldv, double* __restrict__ out, int64_t ldo) {
    const int m = st->m;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P.n; e += (int64_t)gridDim.x * blockDim.x)
        for (int j = 0; j < P.nroot; ++j) {
            double s = 0.0;
            for (int i = 0; i < m; ++i)
                s += V[i * ldv + j] * b[i * ld + e];
            out[j * ldo + e] = s;
        }
}

void dg_ritz(const DGState* st, const DGParams& P, const double* b, int64_t ld, const double* V, int ldv, double* out,
             int64_t ldo, cudaStream_t s) {
    k_dg_ritz<<<dg_grid(P.n), 256, 0, s>>>(st, P, b, ld, V, ldv, out, ldo);
    F2G_LAUNCH("k_dg_ritz");
}

} // namespace f2g
