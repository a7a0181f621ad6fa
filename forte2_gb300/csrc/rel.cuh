// Two-component (relativistic) sigma builder on the device (see rel.cu).
#pragma once

#include <complex>
#include <memory>
#include <vector>

#include "sigma.cuh"

namespace f2g {

struct RelSigmaBuilder {
    CIStrings* s;
    int n;
    double E = 0.0;
    int algorithm = 0; // 0 Knowles-Handy (the reference's default: sigma = E C), 1 Harrison-Zarrabian
    size_t memory = size_t(1) << 30;
    std::vector<std::complex<double>> H, V; // host copies
    DevBuf<double> hre, him, vre, vim;      // real and imaginary parts of the integrals
    // string Hamiltonian of the spinor strings: common columns, real and imaginary values
    int nnz = 0;
    DevBuf<int32_t> col;
    DevBuf<double> valr, vali;
    DevBuf<double2> xC, xS; // C1-sized copies for blocked spaces

    RelSigmaBuilder(CIStrings* s, double E, const std::complex<double>* H, const std::complex<double>* V);
    void set_hamiltonian(double E, const std::complex<double>* H, const std::complex<double>* V);
    void check_memory() const;
    // nvec vectors of the space (complex, interleaved) back to back, overwritten
    void hamiltonian(const double2* C, double2* S, cudaStream_t st, int nvec);
    void hdiag(double2* out, cudaStream_t st);
    std::complex<double> element(int64_t I, int64_t J); // <I|H|J> of two determinants of the space

    // Spin-orbital RDMs between two complex vectors (compute_1rdm ... compute_3cumulant,
    // rel_ci_sigma_builder_rdm.cc): kind 0 so_1rdm (n^2), 1 so_2rdm (n^4), 2 so_2cumulant (n^4),
    // 3 so_3rdm (n^6), 4 so_3cumulant (n^6), complex, bra conjugated. The real RDM kernels give
    // each complex sum as Re = g(Lr, Rr) + g(Li, Ri), Im = g(Lr, Ri) - g(Li, Rr).
    void rdm(int kind, const double2* CL, const double2* CR, double2* out, cudaStream_t st);
    static int64_t rdm_size(int n, int kind);
    std::unique_ptr<SigmaBuilder> rsb; // real builder over the same strings: its RDM kernels and scratch
    DevBuf<double> planes, parts;      // real / imaginary planes of the vectors; real RDM results
    DevBuf<double2> packed, g1, g2;    // complex packed RDM, 1- and 2-RDM of the cumulants
};

} // namespace f2g
