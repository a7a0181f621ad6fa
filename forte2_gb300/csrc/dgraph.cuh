// Graph-captured Davidson-Liu iterations (forte2/helpers/davidsonliu.py:184-387 with the CSF sigma
// closure of forte2/ci/ci.py:221-235).
//
// One solve's iteration is captured once into a CUDA graph: stage the new basis rows, CSF -> det,
// sigma, det -> CSF (plus the defect correction in the mixed-precision phase), the subspace matrix
// and its Jacobi eigendecomposition, residuals, the convergence decision, collapse, projection and
// Gram-Schmidt. Every size and decision lives in a DGState on the device, so K iterations replay
// with no host involvement; the graph ends by copying the state to pinned host memory, which the
// host reads after its next synchronisation. Kernels return at once when the state says the solve
// has stopped, so a launch that converges early costs only empty launches for the rest.
//
// The captured addresses (basis, sigma and residual rows, the diagonal, the sigma builder's and the
// spin adapter's tables) must stay valid while the graph exists; reusing one graph for a new solve
// of the same shape only needs new integrals (SigmaBuilder::set_hamiltonian_async), a new
// diagonal and guess written to the same buffers, and dg_reset.
#pragma once

#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "csf.cuh"
#include "davidson.cuh"

namespace f2g {

// Pinned host slots for the state copies of all graphs, carved from 64-slot chunks: page-locked
// allocation synchronises the device, so it happens once per 64 graphs, not per graph.
class PinnedStateSlots {
  public:
    static PinnedStateSlots& get() {
        static PinnedStateSlots inst;
        return inst;
    }
    DGState* take() {
        std::lock_guard<std::mutex> lock(mu_);
        if (free_.empty()) {
            DGState* chunk = nullptr;
            F2G_CUDA(cudaMallocHost(reinterpret_cast<void**>(&chunk), 64 * sizeof(DGState)));
            for (int i = 63; i >= 0; --i)
                free_.push_back(chunk + i);
        }
        DGState* p = free_.back();
        free_.pop_back();
        std::memset(p, 0, sizeof(DGState));
        return p;
    }
    void give(DGState* p) {
        std::lock_guard<std::mutex> lock(mu_);
        free_.push_back(p);
    }

  private:
    std::mutex mu_;
    std::vector<DGState*> free_; // chunks stay allocated until the process exits
};

// One stream for all captures (a capture only records work), created once; captures are serialised.
inline cudaStream_t capture_stream(std::unique_lock<std::mutex>& lock) {
    static std::mutex mu;
    static cudaStream_t st = nullptr;
    lock = std::unique_lock<std::mutex>(mu);
    if (!st)
        F2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    return st;
}

// Serial numbers of captured iteration contents: a new one at creation and whenever the captured
// work changes (a new defect correction), so a batch built from older contents is never reused.
inline uint64_t next_graph_serial() {
    static std::atomic<uint64_t> c{0};
    return ++c;
}

struct DavGraph {
    SigmaBuilder* sb;
    SpinAdapter* sa;
    DGParams P;
    int R;     // staged rows per iteration
    int iters; // iterations per launch
    double *b, *sigma, *r, *tmp;
    int64_t ld, ldr, ldt;
    const double* hdiag;

    DevBuf<DGState> st;
    DevBuf<double> G, G2, evals, V, norms2, partial, Dp, hist, stage_c, stage_s, cA, cB;
    bool long_vectors = false;    // multi-block dot products and Gram-Schmidt
    DevBuf<GsmState> gsm;
    DevBuf<double> gsm_partial, dots_partial;
    CsfSigmaScratch scr; // determinant-space scratch of the captured sigma (reserved at capture)
    DGState* host_state = nullptr;

    const double *X = nullptr, *D = nullptr, *Mxd = nullptr;
    int64_t ldx = 0;
    int kc = 0;

    cudaGraphExec_t exec = nullptr;
    std::shared_ptr<int> users; // the sigma builder's count of graphs using its graph scratch
    uint64_t serial = next_graph_serial();

    DavGraph(SigmaBuilder* sb_, SpinAdapter* sa_, const DGParams& p, int iters_, double* b_, double* sigma_, double* r_,
             double* tmp_, int64_t ld_, int64_t ldr_, int64_t ldt_, const double* hdiag_)
        : sb(sb_), sa(sa_), P(p), iters(iters_), b(b_), sigma(sigma_), r(r_), tmp(tmp_), ld(ld_), ldr(ldr_), ldt(ldt_),
          hdiag(hdiag_) {
        if (P.nroot < 1 || P.nroot > 16)
            throw Error(2, "dgraph: 1 to 16 roots");
        if (P.maxm < P.nroot || P.maxm > 64)
            throw Error(2, "dgraph: basis size must be in [nroot, 64]");
        if (P.collapse_k < 1 || P.collapse_k > P.maxm)
            throw Error(2, "dgraph: collapse size must be in [1, maxm]");
        if (P.n != sa->ncsf)
            throw Error(2, "dgraph: vector length differs from the spin adapter's CSF count");
        if (P.maxiter_cap < 1 || iters < 1)
            throw Error(2, "dgraph: maxiter and iterations per launch must be positive");
        R = P.nroot;
        const int64_t n = P.n, nd = sa->s->ndet;
        st.reserve(1);
        G.reserve(64 * 64);
        G2.reserve(64 * 64);
        evals.reserve(64);
        V.reserve(64 * 64);
        norms2.reserve(16);
        partial.reserve((size_t)dg_residual_blocks(n) * 16);
        Dp.reserve(64 * 16);
        hist.reserve((size_t)4 * P.maxiter_cap);
        stage_c.reserve((size_t)R * n);
        stage_s.reserve((size_t)R * n);
        long_vectors = n > kGsOneBlockMaxN;
        if (long_vectors) {
            gsm.reserve(1);
            gsm_partial.reserve((size_t)dg_gsm_blocks(n) * 65);
            dots_partial.reserve((size_t)dg_gsm_blocks(n) * 4096);
        }
        host_state = PinnedStateSlots::get().take();
    }

    ~DavGraph() {
        if (users)
            --*users;
        if (exec)
            cudaGraphExecDestroy(exec);
        if (host_state)
            PinnedStateSlots::get().give(host_state);
    }

    void set_correction(const double* X_, const double* D_, int64_t ldx_, const double* Mxd_, int k) {
        if (k < 0 || k > 16)
            throw Error(2, "dgraph: at most 16 corrected vectors");
        X = X_;
        D = D_;
        ldx = ldx_;
        Mxd = Mxd_;
        kc = k;
        if (k) {
            cA.reserve((size_t)k * R);
            cB.reserve((size_t)k * R);
        }
        drop();
        serial = next_graph_serial();
    }

    void drop() {
        if (exec)
            cudaGraphExecDestroy(exec);
        exec = nullptr;
    }

    void iteration(cudaStream_t s) {
        const int64_t n = P.n, nd = sa->s->ndet;
        const int mm = P.maxm;
        DGState* S = st.get();
        // dot products: one block per pair for short vectors, all SMs on every pair for long ones
        auto dots = [&](int which, const double* A, int64_t lda, const double* B, int64_t ldb, int ni, int nj,
                        double* out, int ldo) {
            if (long_vectors)
                dg_dots_long(S, which, A, lda, B, ldb, n, ni, nj, out, ldo, dots_partial.get(), s);
            else
                dg_dots(S, which, A, lda, B, ldb, n, ni, nj, out, ldo, s);
        };
        dg_stage(S, b, ld, R, n, stage_c.get(), s);
        sigma_csf(*sb, *sa, stage_c.get(), stage_s.get(), R, s, scr, true);
        if (kc) {
            dots(4, X, ldx, stage_c.get(), n, kc, R, cA.get(), R);
            dots(4, D, ldx, stage_c.get(), n, kc, R, cB.get(), R);
            dg_correct(S, X, D, ldx, Mxd, cA.get(), cB.get(), kc, R, n, stage_s.get(), s);
        }
        if (dg_small_ok(P)) {
            dg_small_iter(S, P, stage_s.get(), R, b, sigma, ld, r, ldr, hdiag, G.get(), evals.get(), V.get(), Dp.get(),
                          tmp, ldt, hist.get(), norms2.get(), s);
            return;
        }
        dg_unstage(S, stage_s.get(), R, n, sigma, ld, s);
        dots(5, b, ld, sigma, ld, mm, mm, G.get(), mm); // the pairs with a new basis or sigma row
        dg_eigh(S, G.get(), mm, evals.get(), V.get(), mm, s);
        dg_residual(S, P, b, sigma, ld, V.get(), mm, evals.get(), hdiag, r, ldr, norms2.get(), partial.get(), s);
        dg_check(S, P, norms2.get(), evals.get(), hist.get(), s);
        dots(1, b, ld, b, ld, mm, mm, G2.get(), mm);
        dg_orthocheck(S, P, G2.get(), mm, 0, s);
        dg_collapse(S, P, b, sigma, ld, V.get(), mm, tmp, ldt, s);
        dots(2, b, ld, b, ld, P.collapse_k, P.collapse_k, G2.get(), mm);
        dg_orthocheck(S, P, G2.get(), mm, 1, s);
        dots(3, b, ld, r, ldr, mm, P.nroot, Dp.get(), P.nroot);
        dg_project(S, P, b, ld, Dp.get(), r, ldr, s);
        if (long_vectors)
            dg_gs_multi(S, P, b, ld, r, ldr, gsm.get(), gsm_partial.get(), s);
        else
            dg_gs(S, P, b, ld, r, ldr, s);
    }

    // everything a capture of the iterations needs allocated and current (a capture cannot allocate)
    void prepare() {
        sb->prepare_untimed(R);
        if (sb->precision == kFP32) {
            sb->prepare_graph_fp32(R);
            sa->ensure_fp32_tables(0);
        }
        scr.reserve(*sb, *sa, R);
        F2G_CUDA(cudaStreamSynchronize(0)); // set-up work of the legacy stream done before the capture
        sb->flush_timers();
    }

    void capture() {
        drop();
        prepare();
        std::unique_lock<std::mutex> lock;
        cudaStream_t cap = capture_stream(lock);
        F2G_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        cudaGraph_t g = nullptr;
        try {
            for (int i = 0; i < iters; ++i)
                iteration(cap);
            F2G_CUDA(cudaMemcpyAsync(host_state, st.get(), sizeof(DGState), cudaMemcpyDeviceToHost, cap));
        } catch (...) {
            cudaStreamEndCapture(cap, &g);
            if (g)
                cudaGraphDestroy(g);
            cudaGetLastError();
            throw;
        }
        F2G_CUDA(cudaStreamEndCapture(cap, &g));
        const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            exec = nullptr;
            throw Error(3, std::string("dgraph: graph instantiation failed: ") + cudaGetErrorString(e));
        }
        if (!users) {
            users = sb->graph_users;
            ++*users;
        }
    }

    void reset(const DGReset& rs, cudaStream_t s) {
        if (rs.m < 0 || rs.m > P.maxm || rs.sigma_size > rs.m || rs.nlam < 0 || rs.nlam > 64)
            throw Error(2, "dgraph: reset sizes out of range");
        if (rs.sigma_size < 0 && !rs.dev_m)
            throw Error(2, "dgraph: sigma_size < 0 needs a device basis size");
        if (rs.sigma_size >= 0 && rs.m - rs.sigma_size > R)
            throw Error(2, "dgraph: at most nroot basis rows may lack sigma when the iterations start");
        if (rs.maxiter < 1 || rs.maxiter > P.maxiter_cap)
            throw Error(2, "dgraph: maxiter must be in [1, the limit given at creation]");
        host_state->status = kDGRunning;
        dg_reset(st.get(), rs, s);
    }

    void launch(cudaStream_t s) {
        if (!exec)
            capture();
        F2G_CUDA(cudaGraphLaunch(exec, s));
    }

    const DGState* state_dev() const { return st.get(); }

    void ritz(double* out, int64_t ldo, cudaStream_t s) { dg_ritz(st.get(), P, b, ld, V.get(), P.maxm, out, ldo, s); }

    void history(double* host_out, int count) {
        if (count < 0 || count > P.maxiter_cap)
            throw Error(2, "dgraph: history count out of range");
        if (count)
            F2G_CUDA(cudaMemcpy(host_out, hist.get(), (size_t)4 * count * sizeof(double), cudaMemcpyDeviceToHost));
    }
};

// Many solves' iterations in ONE graph launch. The parent graph holds one branch per solve: a
// memset of the branch's loop counter, then a conditional WHILE node whose body is one captured
// iteration of that solve followed by k_dg_continue, which keeps the loop going while the solve's
// state says it is running (and the counter is below the iteration limit + 2, so every loop ends
// even if a state were never set), then a copy of the state to the solve's pinned host slot.
// Branches are independent, so the solves run concurrently and each stops at its own
// convergence; the launch ends when the last one has stopped. The solves must use distinct sigma
// builders (each branch uses its builder's scratch).
struct DavBatch {
    std::vector<DavGraph*> g;
    std::vector<uint64_t> serials;
    DevBuf<int32_t> loops;
    cudaGraphExec_t exec = nullptr;
    int nodes = 0; // kernel, memset and memcpy nodes captured (for reporting)

    DavBatch(DavGraph* const* graphs, int count);
    ~DavBatch() {
        if (exec)
            cudaGraphExecDestroy(exec);
    }
    void build();
    void launch(cudaStream_t s);
};

} // namespace f2g
