// Test infrastructure (oracle only). Provides the LP64 Fortran BLAS symbols that the
// reference's sigma builder calls (dgemm_, daxpy_, ddot_; forte2/helpers/blas.h:12-26) and
// forwards them to the ILP64 OpenBLAS bundled with numpy (exported as scipy_dgemm_64_ etc.),
// which is opened at run time with oracle_blas_open(path). Without a library the calls fall
// back to plain loops, which are exact but slow; the oracle's CPU timing always opens one.
#include <dlfcn.h>

#include <atomic>
#include <cstdint>
#include <cstring>

extern "C" {

typedef void (*dgemm64_t)(const char*, const char*, const int64_t*, const int64_t*, const int64_t*,
                          const double*, const double*, const int64_t*, const double*,
                          const int64_t*, const double*, double*, const int64_t*, size_t, size_t);
typedef void (*daxpy64_t)(const int64_t*, const double*, const double*, const int64_t*, double*,
                          const int64_t*);
typedef double (*ddot64_t)(const int64_t*, const double*, const int64_t*, const double*,
                           const int64_t*);
typedef void (*setthreads_t)(int);
typedef void (*zgemm64_t)(const char*, const char*, const int64_t*, const int64_t*, const int64_t*,
                          const double*, const double*, const int64_t*, const double*,
                          const int64_t*, const double*, double*, const int64_t*, size_t, size_t);
typedef void (*zaxpy64_t)(const int64_t*, const double*, const double*, const int64_t*, double*,
                          const int64_t*);

static zgemm64_t g_zgemm = nullptr;
static zaxpy64_t g_zaxpy = nullptr;
static dgemm64_t g_dgemm = nullptr;
static daxpy64_t g_daxpy = nullptr;
static ddot64_t g_ddot = nullptr;
static setthreads_t g_setthreads = nullptr;

/// Open an ILP64 OpenBLAS (numpy's bundled scipy-openblas). Returns 0 on success.
int oracle_blas_open(const char* path) {
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h)
        return 1;
    g_dgemm = (dgemm64_t)dlsym(h, "scipy_dgemm_64_");
    g_daxpy = (daxpy64_t)dlsym(h, "scipy_daxpy_64_");
    g_ddot = (ddot64_t)dlsym(h, "scipy_ddot_64_");
    g_setthreads = (setthreads_t)dlsym(h, "scipy_openblas_set_num_threads64_");
    g_zgemm = (zgemm64_t)dlsym(h, "scipy_zgemm_64_");
    g_zaxpy = (zaxpy64_t)dlsym(h, "scipy_zaxpy_64_");
    if (!g_dgemm || !g_daxpy || !g_ddot) {
        g_dgemm = nullptr;
        g_daxpy = nullptr;
        g_ddot = nullptr;
        return 2;
    }
    return 0;
}

int oracle_blas_is_open() { return g_dgemm != nullptr; }

void oracle_blas_set_threads(int n) {
    if (g_setthreads)
        g_setthreads(n);
}

// Column-major C = alpha op(A) op(B) + beta C, as the Fortran interface defines it.
static void naive_dgemm(char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
                        const double* a, int64_t lda, const double* b, int64_t ldb, double beta,
                        double* c, int64_t ldc) {
    const bool tA = (ta == 'T' || ta == 't');
    const bool tB = (tb == 'T' || tb == 't');
    for (int64_t j = 0; j < n; ++j) {
        for (int64_t i = 0; i < m; ++i) {
            double s = 0.0;
            for (int64_t l = 0; l < k; ++l) {
                const double av = tA ? a[l + i * lda] : a[i + l * lda];
                const double bv = tB ? b[j + l * ldb] : b[l + j * ldb];
                s += av * bv;
            }
            c[i + j * ldc] = (beta == 0.0 ? 0.0 : beta * c[i + j * ldc]) + alpha * s;
        }
    }
}

void dgemm_(const char* transA, const char* transB, const int* M, const int* N, const int* K,
            const double* alpha, const double* A, const int* lda, const double* B, const int* ldb,
            const double* beta, double* C, const int* ldc) {
    if (g_dgemm) {
        const int64_t m = *M, n = *N, k = *K, la = *lda, lb = *ldb, lc = *ldc;
        g_dgemm(transA, transB, &m, &n, &k, alpha, A, &la, B, &lb, beta, C, &lc, 1, 1);
    } else {
        naive_dgemm(*transA, *transB, *M, *N, *K, *alpha, A, *lda, B, *ldb, *beta, C, *ldc);
    }
}

void daxpy_(int* length, double* a, const double* x, int* inc_x, double* y, int* inc_y) {
    if (g_daxpy) {
        const int64_t n = *length, ix = *inc_x, iy = *inc_y;
        g_daxpy(&n, a, x, &ix, y, &iy);
    } else {
        for (int i = 0; i < *length; ++i)
            y[(int64_t)i * *inc_y] += *a * x[(int64_t)i * *inc_x];
    }
}

double ddot_(int* n, const double* x, int* incx, const double* y, int* incy) {
    if (g_ddot) {
        const int64_t nn = *n, ix = *incx, iy = *incy;
        return g_ddot(&nn, x, &ix, y, &iy);
    }
    double s = 0.0;
    for (int i = 0; i < *n; ++i)
        s += x[(int64_t)i * *incx] * y[(int64_t)i * *incy];
    return s;
}

// complex (interleaved re, im) counterparts for the reference's relativistic sigma builder
// (forte2/helpers/blas.h:14-24): forwarded when the library has them, plain loops otherwise
void zgemm_(const char* transA, const char* transB, const int* M, const int* N, const int* K, const double* alpha,
            const double* A, const int* lda, const double* B, const int* ldb, const double* beta, double* C,
            const int* ldc) {
    if (g_zgemm) {
        const int64_t m = *M, n = *N, k = *K, la = *lda, lb = *ldb, lc = *ldc;
        g_zgemm(transA, transB, &m, &n, &k, alpha, A, &la, B, &lb, beta, C, &lc, 1, 1);
        return;
    }
    const char ta = *transA, tb = *transB;
    for (int64_t j = 0; j < *N; ++j)
        for (int64_t i = 0; i < *M; ++i) {
            double sr = 0.0, si = 0.0;
            for (int64_t l = 0; l < *K; ++l) {
                const int64_t ia = (ta == 'N' || ta == 'n') ? i + l * *lda : l + i * *lda;
                const int64_t ib = (tb == 'N' || tb == 'n') ? l + j * *ldb : j + l * *ldb;
                double ar = A[2 * ia], ai = A[2 * ia + 1], br = B[2 * ib], bi = B[2 * ib + 1];
                if (ta == 'C' || ta == 'c')
                    ai = -ai;
                if (tb == 'C' || tb == 'c')
                    bi = -bi;
                sr += ar * br - ai * bi;
                si += ar * bi + ai * br;
            }
            double* c = C + 2 * (i + j * *ldc);
            double cr = 0.0, ci = 0.0;
            if (beta[0] != 0.0 || beta[1] != 0.0) {
                cr = beta[0] * c[0] - beta[1] * c[1];
                ci = beta[0] * c[1] + beta[1] * c[0];
            }
            c[0] = cr + alpha[0] * sr - alpha[1] * si;
            c[1] = ci + alpha[0] * si + alpha[1] * sr;
        }
}

void zaxpy_(int* length, double* a, const double* x, int* inc_x, double* y, int* inc_y) {
    if (g_zaxpy) {
        const int64_t n = *length, ix = *inc_x, iy = *inc_y;
        g_zaxpy(&n, a, x, &ix, y, &iy);
        return;
    }
    for (int64_t i = 0; i < *length; ++i) {
        const double* xv = x + 2 * i * *inc_x;
        double* yv = y + 2 * i * *inc_y;
        yv[0] += a[0] * xv[0] - a[1] * xv[1];
        yv[1] += a[0] * xv[1] + a[1] * xv[0];
    }
}

} // extern "C"
