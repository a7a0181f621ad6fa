// The sigma builder: sigma = H C for one or more determinant vectors, resident on the device.
#pragma once

#include <memory>
#include <vector>

#include "strings.cuh"

namespace f2g {

enum Precision : int { kFP64 = 0, kFP32 = 1 };

struct RdmScratch; // rdm.cuh

// Same-spin string Hamiltonian of one spin: for every string J the list of (I, value) with
// value = <J| sum_pq h_pq a+_p a_q + sum_{p>r,q>s} <pr||qs> a+_r a+_p a_q a_s |I>, i.e. the
// reference's H1_hz + H2_hz_same_spin operator restricted to one spin's strings.
struct StringHamiltonian {
    int nnz = 0; // entries per row
    DevBuf<int32_t> col;
    DevBuf<double> val;
    DevBuf<float> valf;
    // FP32 row groups (large spaces): rows g*kSsGroup .. +kSsGroup read the union of their input
    // rows once; gcol[goff[g] .. goff[g+1]) is that union in ascending order and gval holds, per
    // union row, the kSsGroup values of the group's rows (0 where a row has no entry). The layout
    // depends on the strings only: later integrals refill gval in place.
    int64_t ngroups = 0;
    DevBuf<int64_t> goff;
    DevBuf<int32_t> gcol;
    DevBuf<float> gval;
};

constexpr int kSsGroup = 8;            // rows per group of the grouped FP32 same-spin kernel
constexpr int64_t kSsGroupMinRows = 2048; // strings per spin from which the FP32 build uses groups
constexpr int kSsGroupMaxSort = 16384; // kSsGroup * entries per row must fit one block's sort
constexpr int64_t kDenseSsMaxStrings = 4096; // dense same-spin GEMMs up to this many strings per spin
constexpr int64_t kDenseSsMinStrings = 512;  // ... and by default from this many

struct SigmaBuilder {
    CIStrings* s;
    int n;
    double E = 0.0;
    std::vector<double> H, V; // host copies (row-major h[p*n+q], physicist V[p][q][r][s])
    DevBuf<double> dH, dV;
    DevBuf<float> fV;
    StringHamiltonian ha, hb;
    int ss_nnz_filtered[2] = {-1, -1}; // blocked spaces: kept couplings per string-Hamiltonian row
    int algorithm = 0;       // 0 Knowles-Handy (the C++ default, ci_sigma_builder.h:288),
                             // 1 Harrison-Zarrabian (what the Python driver selects)
    size_t memory = size_t(1) << 30;
    int precision = kFP64;
    int max_ctas = 0; // cap on the opposite-spin grid (0 = one CTA per alpha string)
    // kernel variants picked by the autotuner (same results): opposite-spin grid of one CTA per
    // SM looping over the alpha strings; same-spin kernel with half the columns per thread
    bool opposite_persistent = false;
    int spmm_narrow = 0;
    // FP32 opposite-spin term on the tensor cores (split-FP16 products, opposite_tc.cu) when the
    // space allows it
    bool use_tc = true;
    // FP64 opposite-spin term of a space blocked by irreps alone through the irrep-aware kernel
    // (opposite_sym.cu); off: the C1 kernel on the embedding (same sigma up to rounding)
    bool use_sym = true;
    std::shared_ptr<struct OppositeSym> osym; // set when the space allows it
    // such a space's same-spin terms on its own vectors: class-local string Hamiltonians (rows in
    // the space's string order, columns as positions inside the class), rebuilt with the integrals
    DevBuf<int32_t> lcol[2];
    DevBuf<double> lval[2];
    void build_local_ss(cudaStream_t st);
    bool blocked_sym_path() const;
    void run_blocked_sym(const double* C, double* S, cudaStream_t st, int nvec, bool timed, bool graph);
    // the tensor-core kernel's B tiles prebuilt for every alpha string and fed to it by TMA
    // (k_build_bops, rebuilt with the integrals); off: each CTA builds B itself (same sigma)
    bool use_tma_b = true;
    bool tc_b_ready = false;
    std::shared_ptr<struct TcBOperands> tc_b;
    void prepare_tma_b(cudaStream_t st);
    // FP32 same-spin terms as dense GEMMs on the tensor cores (dense_ss.cu; split FP16, three
    // products) for spaces of kDenseSsMinStrings to kDenseSsMaxStrings strings per spin by default;
    // the autotuner times both
    bool use_dense_ss = false;
    bool dss_ready = false;
    std::shared_ptr<struct DenseSameSpin> dss;
    bool dense_ss_supported() const;
    void prepare_dense_ss(cudaStream_t st);
    void prepare_graph_fp32(int nvec);
    DevBuf<uint32_t> beta_exc; // beta single excitations per string for its scatter
    DevBuf<int> tc_err;        // set by the tensor-core kernel if a bounded wait gave up
    DevBuf<unsigned int> tc_cmax; // per-vector largest |C| of a tensor-core launch (its operand scale)
    DevBuf<unsigned int> tc_vmax; // largest |V| of the FP32 integrals (the FP16 split's scale)
    long long tc_poll_limit = 0; // polls per bounded wait in the tensor-core kernel (0: the default)
    bool tensor_cores_available() const;
    int tc_error() const;
    int log_level = 3;

    // scratch (grown on demand)
    DevBuf<double> Ct, Tt;
    DevBuf<float> fC, fCt, fTt, fS;
    DevBuf<double> hostC, hostS; // device staging for host-buffer calls
    DevBuf<double> eA, eB, eJ, eDet; // determinant-energy scratch (string energies, exchange rows, energies)
    std::shared_ptr<RdmScratch> rdm;  // reduced-density-matrix lists and scratch, made on first use

    // timing: [total, aabb, aaaa, bbbb] accumulated from CUDA events
    double t_acc[4] = {0, 0, 0, 0};
    int builds = 0;
    // build timing without host waits: a ring of event sets; finished builds are harvested in
    // order when they are found complete, and the host waits only when all slots are pending
    static constexpr int kTimerSlots = 8;
    cudaEvent_t ev[kTimerSlots][4] = {};
    int ev_nvec[kTimerSlots] = {}; // vectors covered by a slot's build
    int ev_gen[kTimerSlots] = {};  // timer generation the slot was recorded in
    int ev_head = 0, ev_count = 0; // oldest pending slot, number pending
    int timer_gen = 0;             // bumped by reset_timers(): older pending builds are dropped
    cudaEvent_t* cur_ev = nullptr; // events of the build being recorded
    void timer_begin();
    void timer_end(int nvec);
    void poll_timers(bool wait);
    void reset_timers();

    SigmaBuilder(CIStrings* s, double E, const double* H, const double* V, int log_level);
    // A builder without a Hamiltonian: the strings and scratch of the RDM kernels only
    struct RdmOnly {};
    SigmaBuilder(CIStrings* s, RdmOnly) : s(s), n(s->norb) {}
    ~SigmaBuilder();
    void set_hamiltonian(double E, const double* H, const double* V);
    void ensure_fp32();
    bool fp32_ready = false;
    void check_memory() const;
    // nvec vectors back to back; built in batches of batch_size(nvec) vectors
    void hamiltonian(const double* C, double* sigma, cudaStream_t st, int nvec = 1);
    int batch_size(int nvec) const;
    // Stream-ordered variants for solves that share the device with others: no device-wide
    // synchronisation, no timers, no allocation (prepare_untimed() allocates the scratch first),
    // so the calls can be captured into a CUDA graph.
    void set_hamiltonian_async(double E, const double* H, const double* V, cudaStream_t st);
    // FP32 vectors in and out (the mixed mode's CSF-space sigma): timed like hamiltonian, or
    // untimed on the graph scratch
    void apply_f32(const float* C, float* S, cudaStream_t st, int nvec, bool timed, bool graph);
    // (all public calls take vectors of the space; a blocked space's are embedded into C1 vectors)
    void prepare_untimed(int nvec);
    void apply_untimed(const double* C, double* sigma, cudaStream_t st, int nvec);
    int untimed_nvec = 0;
    // captured graphs that reference the graph scratch (shared so that a graph outliving the
    // builder can still release its count)
    std::shared_ptr<int> graph_users = std::make_shared<int>(0);
    DevBuf<double> gCt, gTt;
    DevBuf<float> gfC, gfS, gfCt, gfTt;
    // C1-sized copies of a blocked space's vectors (timed / host calls, and the graph scratch)
    DevBuf<double> xC, xS, gxC, gxS;
    DevBuf<float> xfC, xfS, gxfC, gxfS;
    // one HZ term into sigma (overwrites): 0 H0, 1 H1 alpha, 2 H1 beta, 3 opposite spin (aabb),
    // 4 alpha same-spin two-electron part alone (aaaa), 5 beta same-spin two-electron part (bbbb)
    void term(int which, const double* C, double* sigma, cudaStream_t st);
    void det_energies(double* out, cudaStream_t st);
    void flush_timers();
    void avg_build_time(double* out);

  private:
    void build_string_hamiltonian(int spin, StringHamiltonian& sh, bool with_e0, cudaStream_t st);
    void build_groups(int spin, StringHamiltonian& sh, cudaStream_t st);
    template <typename T>
    void run(const T* C, T* sig, cudaStream_t st, int mask, bool timed, int nvec, T* Ct_, T* Tt_, bool graph);
    void apply_batch(const double* C, double* sigma, cudaStream_t st, int nvec, bool timed, bool graph);
    void apply_f32_c1(const float* C, float* S, cudaStream_t st, int nvec, bool timed, bool graph, size_t tot);
    void term_c1(int which, const double* C, double* sigma, cudaStream_t st);
};

int ss_row_nnz(int n, int k);
// String-Hamiltonian rows (columns and values) of one spin's strings for integrals h, V and
// diagonal offset e0: the H1 + same-spin H2 operator, nnz = ss_row_nnz(n, k) entries per row,
// the diagonal first. Every value is a signed sum of integral elements, so complex integrals give
// the real and imaginary parts from two calls.
void build_ss_values(int n, int k, int64_t N0, int nnz, const uint64_t* str, const uint64_t* binom, const double* h,
                     const double* V, double e0, int32_t* col, double* val, cudaStream_t st);

} // namespace f2g
