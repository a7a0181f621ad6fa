// Davidson-Liu device kernels: plain launchers (host-driven iterations) and the device-driven
// iteration used by the graph-captured solver (dgraph.cuh).
#pragma once

#include <cstdint>

#include "common.cuh"

namespace f2g {

void dav_dots(const double* A, int na, int64_t lda, const double* B, int nb, int64_t ldb, int64_t n, double* out,
              double* scratch, cudaStream_t st);
int64_t dav_scratch_size(int64_t n);
void dav_lincomb(const double* X, int nx, int64_t ldx, const double* coef, int ny, double* Y, int64_t ldy, double beta,
                 int64_t n, cudaStream_t st);
void dav_gs_append(double* B, int64_t ld, int cap, int m0, const double* R, int64_t ldr, int ncand, int64_t n,
                   double discard, double ortho, int min_total, uint64_t seed, int* added, cudaStream_t st);

// State of one device-driven Davidson-Liu solve. Every iteration kernel reads its sizes and
// decisions from here, so a captured sequence of iterations needs no host decisions; the host
// reads a copy after each launch. The layout is part of the C ABI (f2g_dgraph_state).
struct DGState {
    int32_t m;          // basis size
    int32_t sigma_size; // basis rows whose sigma is current
    int32_t iter;       // iterations completed in this solve
    int32_t status;     // DGStatus
    int32_t collapse;   // this iteration collapses the basis
    int32_t added;      // vectors appended by the last Gram-Schmidt
    int32_t m_eig;      // basis size of the last subspace eigenproblem
    int32_t maxiter;    // iteration limit of this solve
    int32_t stall_window;
    int32_t g_size;     // leading rows and columns of the subspace matrix still current (0 after a collapse)
    double e_tol, r_tol, stall_floor;
    double max_de, max_r;
    double ortho_dev;   // largest |S - I| of the starting basis (checked at reset when S is given)
    double lam[64];     // eigenvalues of the last subspace eigenproblem (first nroot are the roots)
    double lam_old[64]; // roots of the previous iteration
};

enum DGStatus : int32_t {
    kDGRunning = 0,
    kDGConverged = 1,    // converged, or the basis spans the space, or no room to add vectors
    kDGMaxIter = 2,      // the iteration limit was reached
    kDGStalled = 3,      // stall rule fired (residual stopped decreasing below the floor)
    kDGNotOrthoBefore = 4, // basis failed the orthonormality check before a collapse
    kDGNotOrthoAfter = 5,  // collapsed basis failed the orthonormality check
    kDGNotOrthoStart = 6,  // starting basis failed the orthonormality check
};

// Fixed for the lifetime of a captured graph.
struct DGParams {
    int64_t n; // vector length
    int32_t nroot, maxm, collapse_k, maxiter_cap;
    double precond_thresh, discard, ortho;
    uint64_t seed;
};

// Start of a solve: sizes, previous roots and this solve's tolerances.
struct DGReset {
    int32_t m, sigma_size, nlam, maxiter, stall_window, pad;
    const int32_t* dev_m; // if set: basis size read on the device (m is an upper bound); sigma_size < 0 = m
    const double* S;      // if set: overlap of the starting basis (leading dimension ldS) to check
    int32_t ldS, pad2;
    double e_tol, r_tol, stall_floor;
    double lam_old[64];
};

void dg_reset(DGState* st, const DGReset& r, cudaStream_t s);
void dg_stage(const DGState* st, const double* b, int64_t ld, int R, int64_t n, double* out, cudaStream_t s);
void dg_unstage(const DGState* st, const double* in, int R, int64_t n, double* sigma, int64_t ld, cudaStream_t s);
// which: 0 <A_i,B_j> i,j < m; 1 the same only when collapsing; 2 i,j < ni only when collapsing;
// 3 i < m, j < nj; 4 i < ni, j < nj (fixed)
void dg_dots(const DGState* st, int which, const double* A, int64_t lda, const double* B, int64_t ldb, int64_t n,
             int ni, int nj, double* out, int ldo, cudaStream_t s);
void dg_eigh(DGState* st, const double* G, int ldg, double* evals, double* V, int ldv, cudaStream_t s);
int dg_residual_blocks(int64_t n);
void dg_residual(const DGState* st, const DGParams& P, const double* B, const double* S, int64_t ld, const double* V,
                 int ldv, const double* evals, const double* hdiag, double* R, int64_t ldr, double* norms2,
                 double* partial, cudaStream_t s);
void dg_check(DGState* st, const DGParams& P, const double* norms2, const double* evals, double* hist, cudaStream_t s);
void dg_orthocheck(DGState* st, const DGParams& P, const double* G, int ldg, int after, cudaStream_t s);
void dg_collapse(const DGState* st, const DGParams& P, double* b, double* sigma, int64_t ld, const double* V, int ldv,
                 double* tmp, int64_t ldt, cudaStream_t s);
void dg_project(const DGState* st, const DGParams& P, const double* b, int64_t ld, const double* D, double* r,
                int64_t ldr, cudaStream_t s);
void dg_gs(DGState* st, const DGParams& P, double* b, int64_t ld, const double* r, int64_t ldr, cudaStream_t s);
// The same Gram-Schmidt step (the reference's acceptance rule, davidsonliu.py:338-366 and 438-484)
// with every pass over the vectors spread over the whole GPU: a fixed sequence of kernels whose
// decisions (accept, reject, next candidate, random refill) live in a GsmState on the device, so it
// can be captured in a graph. For long vectors, where one block would stream them alone.
struct GsmState {
    int32_t m0, to_add, nadd;       // basis size before the step, candidates, vectors added so far
    int32_t cand, refill_total, refill_tried;
    int32_t kind, src, s, active;   // current slot: 1 candidate src / 2 random refill src; its row s
    double inv;                      // 1 / norm of the projected vector
    double dv[64];                   // its overlaps with the basis rows
};
constexpr int64_t kGsOneBlockMaxN = 1 << 15; // longer vectors use the multi-block Gram-Schmidt
int dg_gsm_blocks(int64_t n);
// dg_dots for long vectors: all SMs share every pair (partial: dg_gsm_blocks(n) x 4096 doubles)
void dg_dots_long(const DGState* st, int which, const double* A, int64_t lda, const double* B, int64_t ldb, int64_t n,
                  int ni, int nj, double* out, int ldo, double* partial, cudaStream_t s);
void dg_gs_multi(DGState* st, const DGParams& P, double* b, int64_t ld, const double* r, int64_t ldr, GsmState* g,
                 double* partial, cudaStream_t s);
void dg_correct(const DGState* st, const double* X, const double* D, int64_t ldx, const double* Mxd, const double* A,
                const double* Bd, int k, int R, int64_t n, double* S, cudaStream_t s);
// One-block iteration after the sigma build, for vectors up to kDGSmallN and bases up to 32.
constexpr int64_t kDGSmallN = 4096;
bool dg_small_ok(const DGParams& P);
void dg_small_iter(DGState* st, const DGParams& P, const double* stage_s, int R, double* b, double* sigma, int64_t ld,
                   double* r, int64_t ldr, const double* hdiag, double* G, double* evals, double* V, double* Dp,
                   double* tmp, int64_t ldt, double* hist, double* norms2, cudaStream_t s);
void dg_ritz(const DGState* st, const DGParams& P, const double* b, int64_t ld, const double* V, int ldv, double* out,
             int64_t ldo, cudaStream_t s);

} // namespace f2g
