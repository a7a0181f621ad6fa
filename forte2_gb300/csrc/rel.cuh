// Two-component (relativistic) sigma builder on the device (see rel.cu).
#pragma once

#include <complex>
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
};

} // namespace f2g
