// CSF spin adaptation on the device (see csf.cu).
#pragma once

#include <memory>
#include <vector>

#include "sigma.cuh"

namespace f2g {

struct SpinAdapter {
    const CIStrings* s;
    int twoS, twoMs, norb;
    int64_t nconf = 0, ncsf = 0, nslot = 0, ncoupling = 0;
    bool covers_all_dets = true;
    // per number of open shells N: CSF count, determinant-pattern count, dense overlap table
    std::vector<int> ncsfN, ndetN;
    std::vector<int64_t> offN;             // offset of table N in O
    DevBuf<double> O;                      // concatenated [ncsfN][ndetN] tables
    DevBuf<double> OT;                     // the same tables transposed, [ndetN][ncsfN]
    DevBuf<int64_t> dOff;                  // offN on the device
    DevBuf<int> dNcsf, dNdet;
    DevBuf<uint64_t> conf_d, conf_s;       // [nconf] doubly / singly occupied masks (insertion order)
    DevBuf<int64_t> conf_csf, conf_slot;   // [nconf + 1] exclusive offsets
    DevBuf<uint32_t> perm;                 // [nslot] determinant address | negative sign << 31
    DevBuf<int64_t> slot_brk, csf_brk;     // configuration of every 256th slot / CSF (and of the last)

    SpinAdapter(const CIStrings* s, int twoS, int twoMs);
    // nvec vectors back to back (strides ncsf and ndet), one launch
    void csf_to_det(const double* csf, double* det, cudaStream_t st, int nvec = 1) const;
    void det_to_csf(const double* det, double* csf, cudaStream_t st, int nvec = 1) const;
    // FP32 transforms (the mixed mode's FP32 sigma): FP32 overlap tables made on first use
    void csf_to_det(const float* csf, float* det, cudaStream_t st, int nvec = 1) const;
    void det_to_csf(const float* det, float* csf, cudaStream_t st, int nvec = 1) const;
    void ensure_fp32_tables(cudaStream_t st) const;
    mutable DevBuf<float> O32, OT32;
    mutable std::unique_ptr<struct CsfSigmaScratch> host_scratch; // for host calls of sigma_csf
    void hdiag(const double* det_energy, double* out, cudaStream_t st) const;
    // dense <I|H|J> over CSFs idx[0..m) (slater_rules_csf, ci_sigma_builder.cc:278-297)
    void csf_matrix(const SigmaBuilder& sb, const int64_t* idx, int m, double* out_host) const;
    // the same with device indices and output, ordered on st
    void csf_matrix_dev(const SigmaBuilder& sb, const int64_t* idx, int m, double* out, cudaStream_t st) const;
    mutable DevBuf<int64_t> mat_idx; // staging of csf_matrix (kept: no allocation per call)
    mutable DevBuf<double> mat_out;
    void dump(int64_t* bounds, int64_t* det_idx, double* coeff, int64_t* ranges) const;
};

// Scratch of sigma_csf: determinant vectors (FP64, or FP32 with FP32 CSF vectors).
struct CsfSigmaScratch {
    DevBuf<double> det_in, det_out;
    DevBuf<float> f_csf_in, f_csf_out, f_det_in, f_det_out;
    int64_t reserved_vec = 0; // vectors reserved (graph use: never grown after a capture)
    void reserve(const SigmaBuilder& sb, const SpinAdapter& sa, int nvec);
};

// sigma in the CSF basis, out = P^T H P in for nvec vectors back to back (the sigma closure of
// forte2/ci/ci.py:221-235 as one call). In FP32 precision the CSF transforms run in FP32 too, so
// the mixed mode's FP32 operator is the same wherever it is applied. graph = untimed, no
// allocation (scratch reserved beforehand), capturable.
void sigma_csf(SigmaBuilder& sb, const SpinAdapter& sa, const double* in, double* out, int nvec, cudaStream_t st,
               CsfSigmaScratch& scr, bool graph);

} // namespace f2g
