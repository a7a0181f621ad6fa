// Opposite-spin sigma of a point-group-blocked space (see opposite_sym.cu).
#pragma once

#include "strings.cuh"

namespace f2g {

// Orbital irreps in a kernel argument: irrep of every orbital, the orbitals of every irrep (in
// orbital order), their counts, and every orbital's position in its irrep's list.
struct OrbSym {
    int8_t h[64];
    int8_t pos[64];
    int8_t list[8][64];
    int8_t cnt[8];
    int nirrep, S;
};

// Set-up of the kernel for one set of strings: beta 1-hole strings sorted by irrep (groups padded
// to whole warps with -1).
struct OppositeSym {
    bool ready = false;
    OrbSym os{};
    int maxper = 0;
    int64_t nkb = 0;
    DevBuf<int32_t> kb_sorted;
    DevBuf<int8_t> kb_h;
    void build(const CIStrings* s);
};

// The space is blocked by irreps only (no GAS restriction) and the kernel's shared memory fits.
bool opposite_sym_supported(const CIStrings* s);
int64_t opposite_sym_smem(int n, int ma, int64_t N0b, int rm);
// sigma += the opposite-spin term for nvec C1-embedded vectors back to back
void launch_opposite_sym(const CIStrings* s, const OppositeSym& t, const double* V, const double* C, double* sig,
                         cudaStream_t st, int nvec, int max_ctas);

} // namespace f2g
