// Sigma = H C on the device for a CAS space (C1, one determinant block), FP64 or FP32.
//
// The operator is the reference's Harrison-Zarrabian split (CISigmaBuilder::Hamiltonian,
// forte2/ci/ci_sigma_builder.cc:187-218): H0 + H1(alpha) + H1(beta) + H2(alpha beta)
// + H2(alpha alpha) + H2(beta beta), with the same coupling-list sign conventions, organised for
// the GPU as follows (C and sigma are row-major: index Ia * N0b + Ib):
//
// * Same spin, alpha: the one-electron and same-spin two-electron operators restricted to alpha
//   strings form a sparse "string Hamiltonian" Haa(Ja, Ia) with 1 + k(n-k) + C(k,2)C(n-k,2)
//   entries per row (diagonal, single and double replacements). Its values are built once per
//   set of integrals from the HZ lists' signs (hz.cc:14-195): a single Ja <- Ia (p <- q) carries
//   s1(Ja,p) s1(Ia,q) h_pq + sum_t s2(Ja;p,t) s2(Ia;q,t) <(p,t)||(q,t)>, a double carries
//   s2(Ja;p,r) s2(Ia;q,s) <pr||qs>, with s1/s2 the 1-hole/2-hole list signs. The scalar energy E
//   (H0) is folded into the alpha diagonal. sigma(Ja,:) += sum_k Haa(Ja,Ia_k) C(Ia_k,:) is a row
//   SpMM with coalesced row reads.
// * Same spin, beta: the same SpMM on the transposed vector (the reference's gather_block /
//   scatter_block transposes, ci_sigma_builder.cc:224-276).
// * Opposite spin (hz.cc:197-308): one CTA owns an output alpha row Ja and keeps sigma(Ja,:) in
//   shared memory. For each p in Ja (Ka = Ja - p) it stages the integral slice V[p, r, q, s]
//   (q unoccupied in Ka) and, per beta 1-hole string Kb, gathers D[q][s] = sgn C(Ka+q, Kb+s),
//   forms E[r] = sum_{q,s} V[p,r,q,s] D[q][s] for the (n - nb + 1) r unoccupied in Kb and adds
//   sgn E[r] to sigma(Ja, Kb+r) in one phase per orbital r (a_r^+ is one-to-one on the Kb of a
//   round, so the adds of a phase never collide). Only the non-zero rows of the reference's
//   D([qs],[Ka Kb]) are touched, so the FLOP count is 2 N1a N1b (ma mb)^2 with ma = n-na+1,
//   mb = n-nb+1 (10x fewer than the dense n^2 x n^2 product). Owner-writes over Ja rows and no
//   atomics: every sigma element is summed in a fixed order (bitwise reproducible).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "sigma.cuh"
#include "opposite_sym.cuh"

namespace f2g {

int ss_row_nnz(int n, int k) {
    if (k < 0 || k > n)
        return 0;
    return int(1 + (int64_t)k * (n - k) + host_binom(k, 2) * host_binom(n - k, 2));
}

// ---- same-spin string Hamiltonian ------------------------------------------------------------

__device__ inline double vphys(const double* V, int n, int p, int q, int r, int s) {
    return V[(((size_t)p * n + q) * n + r) * n + s];
}
// <ab||cd> = V[a,b,c,d] - V[a,b,d,c]
__device__ inline double vanti(const double* V, int n, int a, int b, int c, int d) {
    return vphys(V, n, a, b, c, d) - vphys(V, n, a, b, d, c);
}
// 2-hole list sign <X - hi - lo| a_hi a_lo |X> (ci_strings_makers.cc:255-262)
__device__ inline int s2neg(uint64_t X, int hi, int lo) {
    return parity_below(X, lo) ^ parity_below(X & ~(uint64_t(1) << lo), hi);
}

// parts: bit 0 one-electron, bit 1 same-spin two-electron; e0 is added to the diagonal.
template <typename T>
__global__ void k_build_ss(int n, int k, int64_t N0, int nnz, const uint64_t* str, const uint64_t* binom,
                           const double* h, const double* V, double e0, int parts, int32_t* col,
                           T* val) {
    const int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (J >= N0)
        return;
    const uint64_t mJ = str[J];
    const bool one = parts & 1, two = parts & 2;
    int32_t* c = col + J * (int64_t)nnz;
    T* v = val + J * (int64_t)nnz;
    int e = 0;
    // diagonal
    double d = e0;
    for (int t = 0; t < n; ++t) {
        if (!(mJ >> t & 1))
            continue;
        if (one)
            d += h[t * n + t];
        if (two)
            for (int u = 0; u < t; ++u)
                if (mJ >> u & 1)
                    d += vanti(V, n, t, u, t, u);
    }
    c[e] = (int32_t)J;
    v[e] = (T)d;
    ++e;
    // single replacements Ja <- Ia: p in J, q not in J
    for (int p = 0; p < n; ++p) {
        if (!(mJ >> p & 1))
            continue;
        for (int q = 0; q < n; ++q) {
            if (mJ >> q & 1)
                continue;
            const uint64_t mI = (mJ & ~(uint64_t(1) << p)) | (uint64_t(1) << q);
            double x = 0.0;
            if (one) {
                const int neg = parity_below(mJ, p) ^ parity_below(mI, q);
                x = neg ? -h[p * n + q] : h[p * n + q];
            }
            if (two) {
                for (int t = 0; t < n; ++t) {
                    if (t == p || !(mJ >> t & 1))
                        continue;
                    const int ph = p > t ? p : t, pl = p > t ? t : p;
                    const int qh = q > t ? q : t, ql = q > t ? t : q;
                    const int neg = s2neg(mJ, ph, pl) ^ s2neg(mI, qh, ql);
                    const double a = vanti(V, n, ph, pl, qh, ql);
                    x += neg ? -a : a;
                }
            }
            c[e] = (int32_t)string_rank(mI, n, k, binom);
            v[e] = (T)x;
            ++e;
        }
    }
    // double replacements: p > r in J, q > s not in J
    for (int p = 0; p < n; ++p) {
        if (!(mJ >> p & 1))
            continue;
        for (int r = 0; r < p; ++r) {
            if (!(mJ >> r & 1))
                continue;
            for (int q = 0; q < n; ++q) {
                if (mJ >> q & 1)
                    continue;
                for (int s = 0; s < q; ++s) {
                    if (mJ >> s & 1)
                        continue;
                    const uint64_t mI =
                        (mJ & ~((uint64_t(1) << p) | (uint64_t(1) << r))) | (uint64_t(1) << q) | (uint64_t(1) << s);
                    double x = 0.0;
                    if (two) {
                        const int neg = s2neg(mJ, p, r) ^ s2neg(mI, q, s);
                        const double a = vanti(V, n, p, r, q, s);
                        x = neg ? -a : a;
                    }
                    c[e] = (int32_t)string_rank(mI, n, k, binom);
                    v[e] = (T)x;
                    ++e;
                }
            }
        }
    }
}

// Y[J, :] = (accumulate ? Y[J, :] : 0) + sum_k val[J,k] X[col[J,k], :]
// grid (rows, column tiles of blockDim * VEC); the row's (col, val) list is staged in shared memory.
template <typename T, int VEC>
__global__ void __launch_bounds__(128) k_spmm_rows(int64_t nrows, int ncols, int nnz, const int32_t* col,
                                                   const T* val, const T* X, T* Y, int accumulate, int64_t vstride) {
    extern __shared__ unsigned char smem_raw[];
    X += blockIdx.z * vstride; // vector blockIdx.z of a batch
    Y += blockIdx.z * vstride;
    T* sval = reinterpret_cast<T*>(smem_raw);
    int32_t* scol = reinterpret_cast<int32_t*>(sval + nnz);
    const int64_t J = blockIdx.x;
    for (int i = threadIdx.x; i < nnz; i += blockDim.x) {
        sval[i] = val[J * nnz + i];
        scol[i] = col[J * nnz + i];
    }
    __syncthreads();
    const int c0 = blockIdx.y * (blockDim.x * VEC) + threadIdx.x;
    T acc[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j)
        acc[j] = T(0);
#pragma unroll 4
    for (int i = 0; i < nnz; ++i) {
        const T v = sval[i];
        const T* x = X + (int64_t)scol[i] * ncols;
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const int c = c0 + j * blockDim.x;
            if (c < ncols)
                acc[j] += v * __ldg(x + c);
        }
    }
    T* y = Y + J * (int64_t)ncols;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        const int c = c0 + j * blockDim.x;
        if (c < ncols)
            y[c] = accumulate ? y[c] + acc[j] : acc[j];
    }
}

// ---- grouped FP32 same-spin SpMM -------------------------------------------------------------
// Output rows are taken kSsGroup at a time: consecutive strings share most of the strings within
// two replacements of them (at CAS(16,16) the union of 8 rows' 849 inputs is ~42% of 8 x 849), so
// the group reads each input row once and applies it to all its rows. The same-spin term is bound
// by these row reads (L2), not by arithmetic.

// Build pass (one block per group): the group's (input row, slot) keys sorted in shared memory
// (bitonic), slot = j * nnz + k for entry k of row g*G + j. fill = 0 counts the distinct input
// rows into count[g]; fill = 1 writes gcol and gval from goff.
__global__ void k_group_build(int64_t nrows, int nnz, const int32_t* __restrict__ col, const float* __restrict__ valf,
                              int S, int fill, int64_t* __restrict__ count, const int64_t* __restrict__ goff,
                              int32_t* __restrict__ gcol, float* __restrict__ gval) {
    extern __shared__ unsigned long long keys[]; // S keys, then S floats
    float* vals = reinterpret_cast<float*>(keys + S);
    __shared__ int part[1024];
    const int64_t g = blockIdx.x, J0 = g * kSsGroup;
    const int tid = threadIdx.x, T = blockDim.x;
    for (int i = tid; i < S; i += T) {
        const int j = i / nnz, k = i - j * nnz;
        if (j < kSsGroup && J0 + j < nrows) {
            keys[i] = ((unsigned long long)(uint32_t)col[(J0 + j) * nnz + k] << 32) | (unsigned)i;
            vals[i] = valf[(J0 + j) * nnz + k];
        } else {
            keys[i] = ~0ull;
        }
    }
    __syncthreads();
    for (int k = 2; k <= S; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < S; i += T) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = keys[i], b = keys[ixj];
                    if ((a > b) == ((i & k) == 0)) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    // a new input row starts where the row index changes; each thread scans a contiguous segment
    const int seg = (S + T - 1) / T, i0 = tid * seg;
    int n_new = 0;
    for (int i = i0; i < i0 + seg && i < S; ++i)
        n_new += keys[i] != ~0ull && (i == 0 || (keys[i] >> 32) != (keys[i - 1] >> 32));
    part[tid] = n_new;
    __syncthreads();
    if (!fill) {
        if (tid == 0) {
            int64_t c = 0;
            for (int t = 0; t < T; ++t)
                c += part[t];
            count[g] = c;
        }
        return;
    }
    int before = 0; // exclusive prefix over the threads before this one
    for (int t = 0; t < tid; ++t)
        before += part[t];
    const int64_t base = goff[g], nu = goff[g + 1] - base;
    for (int64_t e = tid; e < nu * kSsGroup; e += T)
        gval[base * kSsGroup + e] = 0.0f;
    __syncthreads();
    int u = before - 1;
    for (int i = i0; i < i0 + seg && i < S; ++i) {
        const unsigned long long key = keys[i];
        if (key == ~0ull)
            break;
        if (i == 0 || (key >> 32) != (keys[i - 1] >> 32)) { // else: continues the row started before
            ++u;
            gcol[base + u] = (int32_t)(key >> 32);
        }
        const int slot = (int)(key & 0xffffffffu);
        gval[(base + u) * kSsGroup + slot / nnz] = vals[slot];
    }
}

// Y[J, :] = (accumulate ? Y[J, :] : 0) + sum_u gval[u][J - g G] X[gcol[u], :] for the rows J of
// group g = blockIdx.x; the input rows in ascending order (a fixed summation order). The group's
// (row, values) list is staged in shared memory chunk by chunk, and the loads of kSsUnroll input
// rows are issued before their multiply-adds (the kernel is bound by load latency, not bandwidth).
constexpr int kSsChunk = 512, kSsUnroll = 4;
template <int VEC>
__global__ void __launch_bounds__(128) k_spmm_group(int64_t nrows, int ncols, const int64_t* __restrict__ goff,
                                                    const int32_t* __restrict__ gcol, const float* __restrict__ gval,
                                                    const float* __restrict__ X, float* __restrict__ Y, int accumulate,
                                                    int64_t vstride) {
    __shared__ int32_t scol[kSsChunk];
    __shared__ __align__(16) float sval[kSsChunk * kSsGroup];
    X += blockIdx.z * vstride;
    Y += blockIdx.z * vstride;
    const int64_t g = blockIdx.x, u0 = goff[g], u1 = goff[g + 1];
    const int c0 = blockIdx.y * (blockDim.x * VEC) + threadIdx.x;
    float acc[kSsGroup][VEC];
#pragma unroll
    for (int j = 0; j < kSsGroup; ++j)
#pragma unroll
        for (int v = 0; v < VEC; ++v)
            acc[j][v] = 0.0f;
    for (int64_t base = u0; base < u1; base += kSsChunk) {
        const int cnt = (int)(u1 - base < kSsChunk ? u1 - base : kSsChunk);
        __syncthreads(); // the previous chunk is consumed
        for (int t = threadIdx.x; t < cnt; t += blockDim.x)
            scol[t] = gcol[base + t];
        for (int t = threadIdx.x; t < cnt * kSsGroup / 4; t += blockDim.x)
            reinterpret_cast<float4*>(sval)[t] = __ldg(reinterpret_cast<const float4*>(gval + base * kSsGroup) + t);
        // rows past the chunk's end: read row 0 with zero weights (no branch in the unrolled loop)
        for (int t = cnt + threadIdx.x; t < ((cnt + kSsUnroll - 1) / kSsUnroll) * kSsUnroll; t += blockDim.x) {
            scol[t] = 0;
#pragma unroll
            for (int j = 0; j < kSsGroup; ++j)
                sval[t * kSsGroup + j] = 0.0f;
        }
        __syncthreads();
        for (int u = 0; u < cnt; u += kSsUnroll) {
            float x[kSsUnroll][VEC];
#pragma unroll
            for (int q = 0; q < kSsUnroll; ++q) {
                const float* xr = X + (int64_t)scol[u + q] * ncols;
#pragma unroll
                for (int v = 0; v < VEC; ++v) {
                    const int c = c0 + v * blockDim.x;
                    x[q][v] = c < ncols ? __ldg(xr + c) : 0.0f;
                }
            }
#pragma unroll
            for (int q = 0; q < kSsUnroll; ++q) {
                float w[kSsGroup];
#pragma unroll
                for (int h = 0; h < kSsGroup / 4; ++h) {
                    const float4 t = reinterpret_cast<const float4*>(sval)[(u + q) * (kSsGroup / 4) + h];
                    w[4 * h] = t.x;
                    w[4 * h + 1] = t.y;
                    w[4 * h + 2] = t.z;
                    w[4 * h + 3] = t.w;
                }
#pragma unroll
                for (int j = 0; j < kSsGroup; ++j)
#pragma unroll
                    for (int v = 0; v < VEC; ++v)
                        acc[j][v] = fmaf(w[j], x[q][v], acc[j][v]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kSsGroup; ++j) {
        const int64_t J = g * kSsGroup + j;
        if (J >= nrows)
            break;
        float* y = Y + J * (int64_t)ncols;
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const int c = c0 + v * blockDim.x;
            if (c < ncols)
                y[c] = accumulate ? y[c] + acc[j][v] : acc[j][v];
        }
    }
}

// out (cols x rows) = in (rows x cols)^T, 32x32 tiles
template <typename T>
__global__ void k_transpose(int64_t rows, int64_t cols, const T* __restrict__ in, T* __restrict__ out) {
    __shared__ T tile[32][33];
    in += blockIdx.z * rows * cols; // vector blockIdx.z of a batch
    out += blockIdx.z * rows * cols;
    const int64_t bx = (int64_t)blockIdx.x * 32, by = (int64_t)blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t r = by + j, c = bx + threadIdx.x;
        if (r < rows && c < cols)
            tile[j][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t c = bx + j, r = by + threadIdx.x;
        if (r < rows && c < cols)
            out[c * rows + r] = tile[threadIdx.x][j];
    }
}

// One block of a blocked space's vectors transposed: in (rows x cols, vector z at z * ldv) to
// out (cols x rows, vector z at z * ldv_out), overwritten
__global__ void k_transpose_blk(int64_t rows, int64_t cols, const double* __restrict__ in, int64_t ldv,
                                double* __restrict__ out, int64_t ldv_out) {
    __shared__ double tile[32][33];
    in += blockIdx.z * ldv;
    out += blockIdx.z * ldv_out;
    const int64_t bx = (int64_t)blockIdx.x * 32, by = (int64_t)blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t r = by + j, c = bx + threadIdx.x;
        if (r < rows && c < cols)
            tile[j][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t c = bx + j, r = by + threadIdx.x;
        if (r < rows && c < cols)
            out[c * rows + r] = tile[threadIdx.x][j];
    }
}

// Class-local string Hamiltonian of a space blocked by irreps: row j is the class string j (classes
// back to back, the space's string order), its entries the filtered row of its C1 string with the
// column turned into the position inside the class (a symmetric space keeps same-irrep couplings)
__global__ void k_ss_local(int64_t nrows, int nnz, const uint32_t* __restrict__ rank, const int32_t* __restrict__ pos,
                           const int32_t* __restrict__ col, const double* __restrict__ val, int32_t* __restrict__ lcol,
                           double* __restrict__ lval) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nrows)
        return;
    const int64_t J = rank[j];
    for (int k = 0; k < nnz; ++k) {
        lcol[j * nnz + k] = pos[col[J * nnz + k]];
        lval[j * nnz + k] = val[J * nnz + k];
    }
}

template <typename TI, typename TO> __global__ void k_convert(int64_t n, const TI* in, TO* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (TO)in[i];
}

__global__ void k_scale(int64_t n, double a, const double* in, double* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a * in[i];
}

// ---- opposite spin ----------------------------------------------------------------------------
// x with its sign flipped when neg is 1, by an integer XOR of the sign bit: the FP64 pipe (the
// bound of the FP64 kernel) is left to the multiply-adds
__device__ __forceinline__ double flip(double x, int neg) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)neg << 63));
}
__device__ __forceinline__ float flip(float x, int neg) {
    return __uint_as_float(__float_as_uint(x) ^ ((unsigned)neg << 31));
}

// One CTA per output alpha string Ja. MB bounds mb = n - nb + 1 (beta holes per 1-hole string).
// SMROW: sigma(Ja,:) lives in shared memory; otherwise the phased updates go to global memory.
template <typename T, int MB, bool SMROW>
__global__ void __launch_bounds__(512, 1)
    k_opposite(int64_t N0a, int n, int na, int N0b, int64_t N1b, int ma, int mb, const uint32_t* __restrict__ down_a,
               const uint32_t* __restrict__ up_a, const uint32_t* __restrict__ up_b, const T* __restrict__ V,
               const T* __restrict__ C, T* sig) {
    extern __shared__ unsigned char smem_raw[];
    T* vs = reinterpret_cast<T*>(smem_raw);                 // [n][ma][n]: V[p, r, q_i, s]
    T* row = vs + (size_t)n * ma * n;                       // [N0b] (SMROW)
    uint32_t* ua = reinterpret_cast<uint32_t*>(row + (SMROW ? N0b : 0)); // [ma]
    C += blockIdx.y * N0a * N0b; // vector blockIdx.y of a batch
    sig += blockIdx.y * N0a * N0b;
    // grid-stride over the output alpha strings: a grid smaller than N0a leaves SMs free for other work
    for (int64_t Ja = blockIdx.x; Ja < N0a; Ja += gridDim.x) {
    T* srow = sig + Ja * (int64_t)N0b;
    __syncthreads(); // the previous row is written back
    if (SMROW) {
        for (int c = threadIdx.x; c < N0b; c += blockDim.x)
            row[c] = srow[c];
    }
    for (int pi = 0; pi < na; ++pi) {
        __syncthreads(); // previous slice fully consumed
        const uint32_t ep = down_a[Ja * na + pi];
        const int64_t Ka = e_addr(ep);
        const int p = e_orb(ep);
        const int negp = e_neg(ep);
        for (int i = threadIdx.x; i < ma; i += blockDim.x)
            ua[i] = up_a[Ka * ma + i];
        __syncthreads();
        const int nslice = n * ma * n;
        for (int idx = threadIdx.x; idx < nslice; idx += blockDim.x) {
            const int r = idx / (ma * n);
            const int rem = idx - r * (ma * n);
            const int qi = rem / n;
            const int s = rem - qi * n;
            const int q = e_orb(ua[qi]);
            vs[idx] = V[(((size_t)p * n + r) * n + q) * n + s];
        }
        __syncthreads();
        // every thread runs the same number of Kb rounds: the scatter below has barriers
        for (int64_t Kb0 = 0; Kb0 < N1b; Kb0 += blockDim.x) {
            const int64_t Kb = Kb0 + threadIdx.x;
            const bool active = Kb < N1b;
            uint32_t ub[MB];
            int so[MB];
            T acc[MB];
#pragma unroll
            for (int si = 0; si < MB; ++si) {
                ub[si] = (active && si < mb) ? __ldg(up_b + Kb * mb + si) : 0u;
                so[si] = (active && si < mb) ? e_orb(ub[si]) : -1;
                acc[si] = T(0);
            }
            // the gathered C values of excitation qi + 1 are requested before the products of qi,
            // so every warp hides its own gather latency (warps leave each round's barriers together)
            T dn[MB];
#pragma unroll
            for (int si = 0; si < MB; ++si)
                dn[si] = (active && si < mb) ? __ldg(C + (int64_t)e_addr(ua[0]) * N0b + e_addr(ub[si])) : T(0);
            for (int qi = 0; active && qi < ma; ++qi) {
                const int negq = e_neg(ua[qi]);
                T d[MB];
#pragma unroll
                for (int si = 0; si < MB; ++si)
                    d[si] = flip(dn[si], negq ^ e_neg(ub[si]));
                if (qi + 1 < ma) {
                    const T* crow = C + (int64_t)e_addr(ua[qi + 1]) * N0b;
#pragma unroll
                    for (int si = 0; si < MB; ++si)
                        if (si < mb)
                            dn[si] = __ldg(crow + e_addr(ub[si]));
                }
                const T* vq = vs + qi * n;
#pragma unroll
                for (int ri = 0; ri < MB; ++ri) {
                    if (ri < mb) {
                        const T* vr = vq + so[ri] * (ma * n);
                        T a = acc[ri];
#pragma unroll
                        for (int si = 0; si < MB; ++si)
                            if (si < mb)
                                a += vr[so[si]] * d[si];
                        acc[ri] = a;
                    }
                }
            }
            // Ordered scatter, one phase per created orbital r: within a phase Kb -> Kb + r is
            // one-to-one, so no two adds of a phase reach the same element, and every sigma
            // element receives its contributions in the fixed order (Kb round, r): the result is
            // bitwise the same for every launch shape and batch. The adds are shared-memory atomics
            // only because those run in the memory unit, not on the FP64 pipe that bounds this kernel.
            for (int r = 0; r < n; ++r) {
                __syncthreads();
#pragma unroll
                for (int ri = 0; ri < MB; ++ri) {
                    if (so[ri] == r)
                        atomicAdd((SMROW ? row : srow) + e_addr(ub[ri]), flip(acc[ri], negp ^ e_neg(ub[ri])));
                }
            }
        }
    }
    if (SMROW) {
        __syncthreads();
        for (int c = threadIdx.x; c < N0b; c += blockDim.x)
            srow[c] = row[c];
    }
    }
}

// ---- determinant energies (Slater rules diagonal, slater_rules.cc:86-121) -----------------------
// Per string: e_same = sum_{p in X} h_pp + sum_{q<p in X} (<pq|pq> - <pq|qp>); per alpha string the
// Coulomb row jrow[q] = sum_{p in Ia} <pq|pq>. E(Ia,Ib) = E0 + ea + eb + sum_{q in Ib} jrow_a[q].
__global__ void k_string_energy(int n, int64_t N0, const uint64_t* str, const double* h, const double* V,
                                double* e_same, double* jrow) {
    const int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= N0)
        return;
    const uint64_t m = str[I];
    double e = 0.0;
    for (int p = 0; p < n; ++p) {
        if (!(m >> p & 1))
            continue;
        e += h[p * n + p];
        for (int q = 0; q < p; ++q)
            if (m >> q & 1)
                e += vphys(V, n, q, p, q, p) - vphys(V, n, q, p, p, q);
    }
    e_same[I] = e;
    if (jrow) {
        for (int q = 0; q < n; ++q) {
            double j = 0.0;
            for (int p = 0; p < n; ++p)
                if (m >> p & 1)
                    j += vphys(V, n, p, q, p, q);
            jrow[I * n + q] = j;
        }
    }
}

__global__ void k_det_energy(int n, int64_t N0a, int64_t N0b, double E0, const uint64_t* strb, const double* ea,
                             const double* eb, const double* jrow, double* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N0a * N0b)
        return;
    const int64_t Ia = i / N0b, Ib = i - Ia * N0b;
    uint64_t mb = strb[Ib];
    double e = E0 + ea[Ia] + eb[Ib];
    const double* jr = jrow + Ia * n;
    while (mb) {
        const int q = __ffsll((long long)mb) - 1;
        e += jr[q];
        mb &= mb - 1;
    }
    out[i] = e;
}

// ---- host side ---------------------------------------------------------------------------------

static int sm_count() {
    int dev = 0, sms = 0;
    F2G_CUDA(cudaGetDevice(&dev));
    F2G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return sms;
}

size_t opposite_tc_smem(int N0b);
bool opposite_tc_supported(const CIStrings* s);
void build_beta_exc(const CIStrings* s, DevBuf<uint32_t>& exc, cudaStream_t st);
void opposite_tc_vmax(const float* V, int64_t count, unsigned int* vmax, cudaStream_t st);
void launch_opposite_tc(const CIStrings* s, const uint32_t* exc, const float* V, const unsigned int* vmax,
                        const float* C, float* sig, unsigned int* cmax, int* err, long long poll_limit, int max_ctas,
                        cudaStream_t st, int nvec, const TcBOperands* tb);
void opposite_tc_build_b(const CIStrings* s, const float* V, const unsigned int* vmax,
                         std::shared_ptr<TcBOperands>& tb, cudaStream_t st);
void dense_ss_build(const CIStrings* s, const StringHamiltonian* sh[2], std::shared_ptr<DenseSameSpin>& d,
                    cudaStream_t st);
void dense_ss_split(const CIStrings* s, DenseSameSpin& d, const float* C, int nvec, int set, cudaStream_t st);
void dense_ss_reserve(const CIStrings* s, DenseSameSpin& d, int nvec, int set);
void dense_ss_term(const CIStrings* s, DenseSameSpin& d, float* sig, int spin, bool accumulate, int nvec, int set,
                   cudaStream_t st);

SigmaBuilder::SigmaBuilder(CIStrings* s_, double E_, const double* H_, const double* V_, int ll)
    : s(s_), n(s_->norb), log_level(ll) {
    for (auto& slot : ev)
        for (auto& e : slot)
            F2G_CUDA(cudaEventCreate(&e));
    tc_err.reserve(1);
    F2G_CUDA(cudaMemsetAsync(tc_err.get(), 0, sizeof(int), 0));
    if (opposite_sym_supported(s)) {
        osym = std::make_shared<OppositeSym>();
        osym->build(s);
    }
    if (opposite_tc_supported(s)) {
        build_beta_exc(s, beta_exc, 0); // ordered before set_hamiltonian's wait on the legacy stream
        tc_cmax.reserve(2 * 65536);      // one word per vector of a batch (grid y <= 65535), two sets
        tc_vmax.reserve(1);
    }
    // FP32 same-spin terms as dense tensor-core GEMMs by default where they were measured faster than
    // the sparse row kernel (CAS(12,12): 0.08 vs 0.13 ms per spin; CAS(14,14): 0.35 vs 1.31 ms)
    use_dense_ss = dense_ss_supported() && std::max(s->a.N0, s->b.N0) >= kDenseSsMinStrings;
    set_hamiltonian(E_, H_, V_);
}

bool SigmaBuilder::tensor_cores_available() const { return beta_exc.get() != nullptr; }

int SigmaBuilder::tc_error() const {
    int h = 0;
    F2G_CUDA(cudaMemcpy(&h, tc_err.get(), sizeof(int), cudaMemcpyDeviceToHost));
    return h;
}

SigmaBuilder::~SigmaBuilder() {
    for (auto& slot : ev)
        for (auto& e : slot)
            if (e)
                cudaEventDestroy(e);
}

// Blocked spaces: the entries of each string-Hamiltonian row that can reach the space (the class
// pair of row and column is compatible, see DetBlocks::build_filter), in list order, padded to
// nnz_out with (J, 0) entries; count mode (ocol == nullptr) records the largest kept count.
template <typename T>
__global__ void k_filter_ss(int64_t N0, int nnz, const int32_t* __restrict__ col, const T* __restrict__ val,
                            const int16_t* __restrict__ cls, const uint8_t* __restrict__ compat, int ncls,
                            int nnz_out, int32_t* __restrict__ ocol, T* __restrict__ oval, int* maxcount) {
    const int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (J >= N0)
        return;
    const int cj = cls[J];
    int cnt = 0;
    if (cj >= 0) {
        for (int k = 0; k < nnz; ++k) {
            const int32_t I = col[J * nnz + k];
            const int ci = cls[I];
            if (ci < 0 || !compat[cj * ncls + ci])
                continue;
            if (ocol && cnt < nnz_out) {
                ocol[J * nnz_out + cnt] = I;
                oval[J * nnz_out + cnt] = val[J * nnz + k];
            }
            ++cnt;
        }
    }
    if (maxcount)
        atomicMax(maxcount, cnt);
    if (ocol)
        for (; cnt < nnz_out; ++cnt) {
            ocol[J * nnz_out + cnt] = (int32_t)J;
            oval[J * nnz_out + cnt] = T(0);
        }
}

void SigmaBuilder::build_string_hamiltonian(int spin, StringHamiltonian& sh, bool with_e0, cudaStream_t st) {
    const SpinStrings& ss = s->spin(spin);
    const int nnz_full = ss_row_nnz(n, ss.k);
    sh.nnz = nnz_full;
    if (ss.N0 == 0 || nnz_full == 0)
        return;
    const size_t total = (size_t)ss.N0 * nnz_full;
    if (!s->blocked()) {
        sh.col.reserve(total);
        sh.val.reserve(total);
        k_build_ss<double><<<ceil_div(ss.N0, 128), 128, 0, st>>>(n, ss.k, ss.N0, nnz_full, ss.str.get(),
                                                                s->binom.get(), dH.get(), dV.get(), with_e0 ? E : 0.0,
                                                                3, sh.col.get(), sh.val.get());
        F2G_LAUNCH("k_build_ss");
        return;
    }
    // blocked space: full rows in stream-ordered scratch, then only the couplings the space can use
    // (a symmetric space keeps about 1/nirrep of them); the layout depends on the strings alone
    TmpBuf<int32_t> fc(total, st);
    TmpBuf<double> fv(total, st);
    k_build_ss<double><<<ceil_div(ss.N0, 128), 128, 0, st>>>(n, ss.k, ss.N0, nnz_full, ss.str.get(), s->binom.get(),
                                                            dH.get(), dV.get(), with_e0 ? E : 0.0, 3, fc.get(),
                                                            fv.get());
    F2G_LAUNCH("k_build_ss");
    const DetBlocks& B = s->blocks;
    if (ss_nnz_filtered[spin] < 0) {
        TmpBuf<int> mx(1, st);
        F2G_CUDA(cudaMemsetAsync(mx.get(), 0, sizeof(int), st));
        k_filter_ss<double><<<ceil_div(ss.N0, 128), 128, 0, st>>>(ss.N0, nnz_full, fc.get(), fv.get(),
                                                                 B.dcls[spin].get(), B.dcompat[spin].get(),
                                                                 B.nclass(spin), 0, nullptr, nullptr, mx.get());
        F2G_LAUNCH("k_filter_ss count");
        int h = 0;
        F2G_CUDA(cudaMemcpyAsync(&h, mx.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
        F2G_CUDA(cudaStreamSynchronize(st));
        ss_nnz_filtered[spin] = std::max(1, h);
    }
    sh.nnz = ss_nnz_filtered[spin];
    const size_t kept = (size_t)ss.N0 * sh.nnz;
    sh.col.reserve(kept);
    sh.val.reserve(kept);
    k_filter_ss<double><<<ceil_div(ss.N0, 128), 128, 0, st>>>(ss.N0, nnz_full, fc.get(), fv.get(),
                                                             B.dcls[spin].get(), B.dcompat[spin].get(),
                                                             B.nclass(spin), sh.nnz, sh.col.get(), sh.val.get(),
                                                             nullptr);
    F2G_LAUNCH("k_filter_ss");
}

bool SigmaBuilder::blocked_sym_path() const { return osym && use_sym && precision == kFP64; }

void SigmaBuilder::build_local_ss(cudaStream_t st) {
    if (!osym)
        return;
    const DetBlocks& B = s->blocks;
    for (int spin = 0; spin < 2; ++spin) {
        const StringHamiltonian& sh = spin == 0 ? ha : hb;
        const int64_t nrows = B.cls_off[spin].back();
        if (nrows == 0 || sh.nnz == 0)
            continue;
        lcol[spin].reserve((size_t)nrows * sh.nnz);
        lval[spin].reserve((size_t)nrows * sh.nnz);
        k_ss_local<<<ceil_div(nrows, 128), 128, 0, st>>>(nrows, sh.nnz, B.drank[spin].get(), B.dpos[spin].get(),
                                                         sh.col.get(), sh.val.get(), lcol[spin].get(),
                                                         lval[spin].get());
        F2G_LAUNCH("k_ss_local");
    }
}

void build_ss_values(int n, int k, int64_t N0, int nnz, const uint64_t* str, const uint64_t* binom, const double* h,
                     const double* V, double e0, int32_t* col, double* val, cudaStream_t st) {
    if (N0 == 0 || nnz == 0)
        return;
    k_build_ss<double><<<ceil_div(N0, 128), 128, 0, st>>>(n, k, N0, nnz, str, binom, h, V, e0, 3, col, val);
    F2G_LAUNCH("k_build_ss");
}

// FP32 copies of the string-Hamiltonian values, made once per set of integrals on first use.
// The TMA-fed B operands of the tensor-core kernel, when it is in use and they are not current.
void SigmaBuilder::prepare_tma_b(cudaStream_t st) {
    if (!use_tc || !use_tma_b || !tensor_cores_available() || tc_b_ready)
        return;
    opposite_tc_build_b(s, fV.get(), tc_vmax.get(), tc_b, st);
    tc_b_ready = true;
}

bool SigmaBuilder::dense_ss_supported() const {
    return s->a.N0 <= kDenseSsMaxStrings && s->b.N0 <= kDenseSsMaxStrings && s->a.N0 * s->b.N0 > 0;
}

// The dense split string Hamiltonians, when the dense same-spin GEMMs are in use and they are not
// current (needs the FP32 rows).
void SigmaBuilder::prepare_dense_ss(cudaStream_t st) {
    if (!use_dense_ss || dss_ready || !fp32_ready)
        return;
    const StringHamiltonian* sh[2] = {&ha, &hb};
    dense_ss_build(s, sh, dss, st);
    dss_ready = true;
}

void SigmaBuilder::ensure_fp32() {
    if (!tc_b_ready && use_tc && use_tma_b && tensor_cores_available()) {
        prepare_tma_b(0);
        F2G_CUDA(cudaStreamSynchronize(0)); // built on the legacy stream: wait for it alone
    }
    if (fp32_ready) {
        if (use_dense_ss && !dss_ready) {
            prepare_dense_ss(0);
            F2G_CUDA(cudaStreamSynchronize(0));
        }
        return;
    }
    for (StringHamiltonian* sh : {&ha, &hb}) {
        const int s_ = sh == &ha ? 0 : 1;
        const size_t total = (size_t)s->spin(s_).N0 * sh->nnz;
        if (total == 0)
            continue;
        sh->valf.reserve(total);
        k_convert<double, float><<<1024, 256>>>((int64_t)total, sh->val.get(), sh->valf.get());
        F2G_LAUNCH("k_convert string Hamiltonian");
        build_groups(s_, *sh, 0);
    }
    F2G_CUDA(cudaStreamSynchronize(0)); // the conversions ran on the legacy stream: wait for them alone
    fp32_ready = true;
    if (use_dense_ss && !dss_ready) {
        prepare_dense_ss(0);
        F2G_CUDA(cudaStreamSynchronize(0));
    }
}

// The grouped layout of one spin's FP32 string Hamiltonian, for spaces of kSsGroupMinRows strings
// or more. The first call sizes it (one host read of the total); later calls (new integrals, same
// strings) refill it in place on stream st.
void SigmaBuilder::build_groups(int spin, StringHamiltonian& sh, cudaStream_t st) {
    const int64_t N0 = s->spin(spin).N0;
    int S = 1;
    while (S < kSsGroup * sh.nnz)
        S <<= 1;
    if (N0 < kSsGroupMinRows || sh.nnz == 0 || S > kSsGroupMaxSort)
        return;
    const size_t smem = (size_t)S * (sizeof(unsigned long long) + sizeof(float));
    F2G_CUDA(cudaFuncSetAttribute(k_group_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t ng = (N0 + kSsGroup - 1) / kSsGroup;
    if (sh.ngroups == 0) {
        DevBuf<int64_t> cnt;
        cnt.reserve(ng + 1);
        F2G_CUDA(cudaMemsetAsync(cnt.get(), 0, (ng + 1) * sizeof(int64_t), st));
        k_group_build<<<(unsigned)ng, 1024, smem, st>>>(N0, sh.nnz, sh.col.get(), sh.valf.get(), S, 0, cnt.get(),
                                                        nullptr, nullptr, nullptr);
        F2G_LAUNCH("k_group_build count");
        std::vector<int64_t> c(ng + 1, 0), off(ng + 1, 0);
        F2G_CUDA(cudaMemcpyAsync(c.data(), cnt.get(), ng * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        F2G_CUDA(cudaStreamSynchronize(st));
        for (int64_t g = 0; g < ng; ++g)
            off[g + 1] = off[g] + c[g];
        sh.goff.reserve(ng + 1);
        sh.gcol.reserve((size_t)std::max<int64_t>(1, off[ng]));
        sh.gval.reserve((size_t)std::max<int64_t>(1, off[ng]) * kSsGroup);
        F2G_CUDA(cudaMemcpyAsync(sh.goff.get(), off.data(), (ng + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        F2G_CUDA(cudaStreamSynchronize(st));
        sh.ngroups = ng;
    }
    k_group_build<<<(unsigned)ng, 1024, smem, st>>>(N0, sh.nnz, sh.col.get(), sh.valf.get(), S, 1, nullptr,
                                                    sh.goff.get(), sh.gcol.get(), sh.gval.get());
    F2G_LAUNCH("k_group_build fill");
}

void SigmaBuilder::set_hamiltonian(double E_, const double* H_, const double* V_) {
    E = E_;
    H.assign(H_, H_ + (size_t)n * n);
    V.assign(V_, V_ + (size_t)n * n * n * n);
    dH.reserve(std::max<size_t>(1, H.size()));
    dV.reserve(std::max<size_t>(1, V.size()));
    if (!H.empty())
        F2G_CUDA(cudaMemcpy(dH.get(), H.data(), H.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (!V.empty())
        F2G_CUDA(cudaMemcpy(dV.get(), V.data(), V.size() * sizeof(double), cudaMemcpyHostToDevice));
    fV.reserve(std::max<size_t>(1, V.size()));
    if (!V.empty()) {
        k_convert<double, float><<<64, 256>>>((int64_t)V.size(), dV.get(), fV.get());
        F2G_LAUNCH("k_convert V");
    }
    if (tc_vmax.get())
        opposite_tc_vmax(fV.get(), (int64_t)V.size(), tc_vmax.get(), 0);
    tc_b_ready = false;
    if (tc_b) // built before: refilled in place for the new integrals
        prepare_tma_b(0);
    build_string_hamiltonian(0, ha, true, 0);
    build_string_hamiltonian(1, hb, false, 0);
    build_local_ss(0);
    F2G_CUDA(cudaStreamSynchronize(0)); // set-up ran on the legacy stream: wait for it alone
    fp32_ready = false;
    dss_ready = false;
    if (precision == kFP32 || (dss && use_dense_ss))
        ensure_fp32(); // (dense same-spin operands built before are refilled in place)
}

// Same result as set_hamiltonian, ordered on stream st: the host arrays are copied into the
// builder's own host vectors first, so the caller may reuse them at once. The FP32 copies are
// refreshed too, so a later switch to FP32 needs no synchronisation. Buffers keep their addresses
// when the orbital count is unchanged, which keeps captured graphs valid.
void SigmaBuilder::set_hamiltonian_async(double E_, const double* H_, const double* V_, cudaStream_t st) {
    E = E_;
    H.assign(H_, H_ + (size_t)n * n);
    V.assign(V_, V_ + (size_t)n * n * n * n);
    dH.reserve(std::max<size_t>(1, H.size()));
    dV.reserve(std::max<size_t>(1, V.size()));
    fV.reserve(std::max<size_t>(1, V.size()));
    if (!H.empty())
        F2G_CUDA(cudaMemcpyAsync(dH.get(), H.data(), H.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    if (!V.empty()) {
        F2G_CUDA(cudaMemcpyAsync(dV.get(), V.data(), V.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        k_convert<double, float><<<64, 256, 0, st>>>((int64_t)V.size(), dV.get(), fV.get());
        F2G_LAUNCH("k_convert V");
    }
    if (tc_vmax.get())
        opposite_tc_vmax(fV.get(), (int64_t)V.size(), tc_vmax.get(), st);
    tc_b_ready = false;
    if (tc_b) // built before: refilled in place, in stream order, so captured graphs follow
        prepare_tma_b(st);
    build_string_hamiltonian(0, ha, true, st);
    build_string_hamiltonian(1, hb, false, st);
    build_local_ss(st);
    for (StringHamiltonian* sh : {&ha, &hb}) {
        const int s_ = sh == &ha ? 0 : 1;
        const size_t total = (size_t)s->spin(s_).N0 * sh->nnz;
        if (total == 0)
            continue;
        sh->valf.reserve(total);
        k_convert<double, float><<<1024, 256, 0, st>>>((int64_t)total, sh->val.get(), sh->valf.get());
        F2G_LAUNCH("k_convert string Hamiltonian");
        build_groups(s_, *sh, st);
    }
    fp32_ready = true;
    dss_ready = false;
    if (dss) // built before: refilled in place, in stream order, so captured graphs follow
        prepare_dense_ss(st);
}

// Reserves the graph scratch for nvec vectors in both precisions. Captured graphs hold its
// addresses, so once graph_users > 0 it may not grow (a larger request is an error).
void SigmaBuilder::prepare_untimed(int nvec) {
    nvec = std::max(1, nvec);
    if (nvec <= untimed_nvec)
        return;
    if (*graph_users > 0)
        throw Error(2, "sigma builder: captured graphs use its graph scratch for " + std::to_string(untimed_nvec) +
                           " vectors; a graph of " + std::to_string(nvec) + " vectors needs a new builder");
    const size_t tot = (size_t)nvec * std::max<int64_t>(1, s->nfull);
    gCt.reserve(tot);
    gTt.reserve(tot);
    gfC.reserve(tot);
    gfS.reserve(tot);
    gfCt.reserve(tot);
    gfTt.reserve(tot);
    if (s->blocked()) {
        gxC.reserve(tot);
        gxS.reserve(tot);
        gxfC.reserve(tot);
        gxfS.reserve(tot);
    }
    untimed_nvec = nvec;
}

// Before a capture of FP32 sigma builds of nvec vectors: the dense same-spin operands and their
// graph scratch (a capture cannot allocate)
void SigmaBuilder::prepare_graph_fp32(int nvec) {
    ensure_fp32();
    if (use_dense_ss && dss)
        dense_ss_reserve(s, *dss, std::max(1, nvec), 1);
}

void SigmaBuilder::apply_f32(const float* C, float* S, cudaStream_t st, int nvec, bool timed, bool graph) {
    const int64_t nd = s->nfull;
    if (s->ndet == 0 || nvec <= 0)
        return;
    if (!fp32_ready)
        throw Error(1, "apply_f32: FP32 Hamiltonian copies are not ready (select FP32 precision first)");
    const size_t tot = (size_t)nvec * nd;
    if (s->blocked()) {
        if (graph && nvec > untimed_nvec)
            throw Error(2, "apply_f32: more vectors than prepared");
        float* xc = graph ? gxfC.get() : xfC.reserve(tot);
        float* xs = graph ? gxfS.get() : xfS.reserve(tot);
        const DetEnum de = s->dets();
        blocks_embed<float>(de, nd, C, xc, nvec, st);
        apply_f32_c1(xc, xs, st, nvec, timed, graph, tot);
        blocks_extract<float>(de, nd, xs, S, nvec, st);
        return;
    }
    apply_f32_c1(C, S, st, nvec, timed, graph, tot);
}

void SigmaBuilder::apply_f32_c1(const float* C, float* S, cudaStream_t st, int nvec, bool timed, bool graph,
                                size_t tot) {
    float *ct, *tt;
    if (graph) {
        if (nvec > untimed_nvec)
            throw Error(2, "apply_f32: more vectors than prepared");
        ct = gfCt.get();
        tt = gfTt.get();
    } else {
        ct = fCt.reserve(tot);
        tt = fTt.reserve(tot);
    }
    if (timed)
        timer_begin();
    run<float>(C, S, st, 7, timed, nvec, ct, tt, graph);
    if (timed)
        timer_end(nvec);
}

void SigmaBuilder::apply_untimed(const double* C, double* sigma, cudaStream_t st, int nvec) {
    if (s->ndet == 0 || nvec <= 0)
        return;
    if (nvec > untimed_nvec)
        throw Error(2, "apply_untimed: more vectors than prepared");
    if (precision == kFP32 && !fp32_ready)
        throw Error(1, "apply_untimed: FP32 Hamiltonian copies are not ready");
    if (blocked_sym_path()) {
        run_blocked_sym(C, sigma, st, nvec, false, true);
        return;
    }
    if (s->blocked()) {
        const DetEnum de = s->dets();
        blocks_embed<double>(de, s->nfull, C, gxC.get(), nvec, st);
        apply_batch(gxC.get(), gxS.get(), st, nvec, false, true);
        blocks_extract<double>(de, s->nfull, gxS.get(), sigma, nvec, st);
        return;
    }
    apply_batch(C, sigma, st, nvec, false, true);
}

// The reference's K-block memory contract (ci_sigma_builder_knowles_handy.cc:15-32): every term
// needs at least one K-block column of nrows doubles in each of its two buffers. The device path
// keeps the same validation and error text; its own scratch is two determinant vectors.
void SigmaBuilder::check_memory() const {
    const int64_t NA = s->a.N0, NB = s->b.N0;
    const size_t maxel = memory / (2 * sizeof(double));
    auto need = [&](int64_t nrows, int64_t ncols) {
        if (nrows == 0 || ncols == 0)
            return;
        if (maxel < (size_t)nrows)
            throw Error(1, "The CI builder memory limit (" + std::to_string(memory) +
                               " bytes) is too small for one K-block column of " + std::to_string(nrows) +
                               " elements per buffer.");
    };
    const int64_t npairs = (int64_t)n * (n - 1) / 2;
    if (algorithm == 1) {
        if (s->na >= 1)
            need((int64_t)n * NB, s->a.N1);
        if (s->nb >= 1)
            need((int64_t)n * NA, s->b.N1);
        if (s->na >= 1 && s->nb >= 1)
            need((int64_t)n * n * s->b.N1, s->a.N1);
        if (s->na >= 2)
            need(npairs * NB, s->a.N2);
        if (s->nb >= 2)
            need(npairs * NA, s->b.N2);
    } else {
        // Knowles-Handy: one (n(n+1)/2 x N(1h1p beta)) block per Ka chunk (kh.cc:88-171)
        const int64_t ngeq = (int64_t)n * (n + 1) / 2;
        need(ngeq * NB, NA);
    }
}

template <typename T> static int64_t opposite_smem(int n, int ma, int N0b, bool smrow) {
    return (int64_t)n * ma * n * sizeof(T) + (smrow ? (int64_t)N0b * sizeof(T) : 0) + (int64_t)ma * 4 + 16;
}

// All launchers take nvec vectors stored back to back (stride = the determinant count) and cover
// them in one launch.
// max_ctas > 0 caps the grid (one CTA per SM at 512 threads): the kernel then loops over the alpha
// strings and leaves the other SMs to concurrent work.
static thread_local int g_opposite_max_ctas = 0;

template <typename T, int MB, bool SMROW>
static void launch_opposite_mb(const CIStrings* s, const T* V, const T* C, T* sig, cudaStream_t st, int nvec) {
    const int n = s->norb, ma = s->a.m1, mb = s->b.m1;
    const int64_t smem = opposite_smem<T>(n, ma, (int)s->b.N0, SMROW);
    auto kern = k_opposite<T, MB, SMROW>;
    F2G_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t gx = s->a.N0;
    if (g_opposite_max_ctas > 0)
        gx = std::min<int64_t>(gx, g_opposite_max_ctas);
    kern<<<dim3((unsigned)gx, (unsigned)nvec), 512, smem, st>>>(s->a.N0, n, s->na, (int)s->b.N0, s->b.N1, ma, mb,
                                                               s->a.down1.get(), s->a.up1.get(), s->b.up1.get(), V,
                                                               C, sig);
    F2G_LAUNCH("k_opposite");
}

template <typename T, bool SMROW>
static void launch_opposite_r(const CIStrings* s, const T* V, const T* C, T* sig, cudaStream_t st, int nvec) {
    const int mb = s->b.m1;
    if (mb <= 4)
        launch_opposite_mb<T, 4, SMROW>(s, V, C, sig, st, nvec);
    else if (mb <= 8)
        launch_opposite_mb<T, 8, SMROW>(s, V, C, sig, st, nvec);
    else if (mb <= 9)
        launch_opposite_mb<T, 9, SMROW>(s, V, C, sig, st, nvec);
    else if (mb <= 12)
        launch_opposite_mb<T, 12, SMROW>(s, V, C, sig, st, nvec);
    else if (mb <= 16)
        launch_opposite_mb<T, 16, SMROW>(s, V, C, sig, st, nvec);
    else if (mb <= 24)
        launch_opposite_mb<T, 24, SMROW>(s, V, C, sig, st, nvec);
    else
        throw Error(1, "opposite-spin kernel supports at most 24 beta holes per 1-hole string");
}

template <typename T>
static void launch_opposite(const CIStrings* s, const T* V, const T* C, T* sig, cudaStream_t st, int nvec = 1) {
    if (s->na < 1 || s->nb < 1 || s->a.N0 == 0 || s->b.N1 == 0)
        return;
    const bool smrow = opposite_smem<T>(s->norb, s->a.m1, (int)s->b.N0, true) <= 200 * 1024;
    if (smrow)
        launch_opposite_r<T, true>(s, V, C, sig, st, nvec);
    else
        launch_opposite_r<T, false>(s, V, C, sig, st, nvec);
}

// columns per thread of the same-spin kernel: 0 = the default (4 FP64 / 8 FP32), 1 = half of it
// (more thread blocks for short rows); chosen by the autotuner (SigmaBuilder::spmm_narrow)
static thread_local int g_spmm_narrow = 0;

template <typename T, int VEC>
static void launch_spmm_v(const StringHamiltonian& sh, const T* val, int64_t nrows, int ncols, const T* X, T* Y,
                          bool accumulate, cudaStream_t st, int nvec) {
    const int tile = 128 * VEC;
    const size_t smem = (size_t)sh.nnz * (sizeof(T) + sizeof(int32_t));
    if (smem > 48 * 1024)
        F2G_CUDA(cudaFuncSetAttribute(k_spmm_rows<T, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)nrows, (unsigned)ceil_div(ncols, tile), (unsigned)nvec);
    k_spmm_rows<T, VEC><<<grid, 128, smem, st>>>(nrows, ncols, sh.nnz, sh.col.get(), val, X, Y, accumulate ? 1 : 0,
                                                 nrows * (int64_t)ncols);
    F2G_LAUNCH("k_spmm_rows");
}

template <typename T>
static void launch_spmm(const StringHamiltonian& sh, const T* val, int64_t nrows, int ncols, const T* X, T* Y,
                        bool accumulate, cudaStream_t st, int nvec = 1) {
    if (nrows == 0 || ncols == 0 || sh.nnz == 0)
        return;
    if constexpr (sizeof(T) == 4) {
        if (sh.ngroups > 0) {
            constexpr int VEC = 4;
            dim3 grid((unsigned)sh.ngroups, (unsigned)ceil_div(ncols, 128 * VEC), (unsigned)nvec);
            k_spmm_group<VEC><<<grid, 128, 0, st>>>(nrows, ncols, sh.goff.get(), sh.gcol.get(), sh.gval.get(), X, Y,
                                                    accumulate ? 1 : 0, nrows * (int64_t)ncols);
            F2G_LAUNCH("k_spmm_group");
            return;
        }
    }
    constexpr int VEC = sizeof(T) == 8 ? 4 : 8;
    if (g_spmm_narrow)
        launch_spmm_v<T, VEC / 2>(sh, val, nrows, ncols, X, Y, accumulate, st, nvec);
    else
        launch_spmm_v<T, VEC>(sh, val, nrows, ncols, X, Y, accumulate, st, nvec);
}

template <typename T>
static void launch_transpose(int64_t rows, int64_t cols, const T* in, T* out, cudaStream_t st, int nvec = 1) {
    if (rows == 0 || cols == 0)
        return;
    dim3 grid((unsigned)ceil_div(cols, 32), (unsigned)ceil_div(rows, 32), (unsigned)nvec);
    k_transpose<T><<<grid, dim3(32, 8), 0, st>>>(rows, cols, in, out);
    F2G_LAUNCH("k_transpose");
}

void transpose_f64(int64_t rows, int64_t cols, const double* in, double* out, cudaStream_t st) {
    launch_transpose<double>(rows, cols, in, out, st);
}

// mask bits: 1 alpha same-spin (+H0 +H1a), 2 beta same-spin (+H1b), 4 opposite spin
// Ct_, Tt_: transposition scratch of nvec * ndet elements.

template <typename T>
void SigmaBuilder::run(const T* C, T* sig, cudaStream_t st, int mask, bool timed, int nvec, T* Ct_, T* Tt_,
                       bool graph) {
    const int64_t NA = s->a.N0, NB = s->b.N0, nd = NA * NB;
    g_opposite_max_ctas = max_ctas > 0 ? max_ctas : (opposite_persistent ? sm_count() : 0);
    g_spmm_narrow = spmm_narrow;
    const T* valb = nullptr;
    const T* vala = nullptr;
    const T* Vt = nullptr;
    if constexpr (sizeof(T) == 8) {
        vala = ha.val.get();
        valb = hb.val.get();
        Vt = dV.get();
    } else {
        vala = ha.valf.get();
        valb = hb.valf.get();
        Vt = fV.get();
    }
    if (timed)
        F2G_CUDA(cudaEventRecord(cur_ev[0], st));
    bool dense = false;
    if constexpr (sizeof(T) == 4) {
        if (use_dense_ss && dss_ready && (mask & 3)) {
            // same-spin terms as dense tensor-core GEMMs on split FP16 operands
            const int set = graph ? 1 : 0;
            dense_ss_split(s, *dss, C, nvec, set, st);
            if ((mask & 2) && s->nb >= 1)
                dense_ss_term(s, *dss, sig, 1, false, nvec, set, st);
            else
                F2G_CUDA(cudaMemsetAsync(sig, 0, (size_t)nvec * nd * sizeof(T), st));
            if (timed)
                F2G_CUDA(cudaEventRecord(cur_ev[1], st));
            if (mask & 1)
                dense_ss_term(s, *dss, sig, 0, true, nvec, set, st);
            dense = true;
        }
    }
    // beta same spin: sigma = (Hbb C^T)^T
    if (dense) {
    } else if ((mask & 2) && s->nb >= 1) {
        launch_transpose<T>(NA, NB, C, Ct_, st, nvec);
        launch_spmm<T>(hb, valb, NB, (int)NA, Ct_, Tt_, false, st, nvec);
        launch_transpose<T>(NB, NA, Tt_, sig, st, nvec);
    } else {
        F2G_CUDA(cudaMemsetAsync(sig, 0, (size_t)nvec * nd * sizeof(T), st));
    }
    if (timed && !dense)
        F2G_CUDA(cudaEventRecord(cur_ev[1], st));
    // alpha same spin + H0
    if ((mask & 1) && !dense)
        launch_spmm<T>(ha, vala, NA, (int)NB, C, sig, true, st, nvec);
    if (timed)
        F2G_CUDA(cudaEventRecord(cur_ev[2], st));
    if (mask & 4) {
        bool done = false;
        if constexpr (sizeof(T) == 4) {
            if (use_tc && tensor_cores_available()) {
                // graph launches use their own half of the scale scratch, so a captured solve and a
                // direct call on the same builder never share it
                unsigned int* cmax = tc_cmax.get() + (graph ? 65536 : 0);
                launch_opposite_tc(s, beta_exc.get(), Vt, tc_vmax.get(), C, sig, cmax, tc_err.get(), tc_poll_limit,
                                   max_ctas, st, nvec, (use_tma_b && tc_b_ready) ? tc_b.get() : nullptr);
                done = true;
            }
        }
        if constexpr (sizeof(T) == 8) {
            if (!done && use_sym && osym) {
                launch_opposite_sym(s, *osym, Vt, C, sig, st, nvec, g_opposite_max_ctas);
                done = true;
            }
        }
        if (!done)
            launch_opposite<T>(s, Vt, C, sig, st, nvec);
    }
    if (timed)
        F2G_CUDA(cudaEventRecord(cur_ev[3], st));
}

// Row SpMM on raw operands: Y[J] (+)= sum_k val[J][k] X[col[J][k]] for J < nrows, vectors at z * vstride.
static void spmm_rows_raw(int64_t nrows, int ncols, int nnz, const int32_t* col, const double* val, const double* X,
                          double* Y, bool accumulate, int64_t vstride, int nvec, cudaStream_t st) {
    if (nrows == 0 || ncols == 0 || nnz == 0 || nvec <= 0)
        return;
    constexpr int VEC = 4;
    const size_t smem = (size_t)nnz * (sizeof(double) + sizeof(int32_t));
    if (smem > 48 * 1024)
        F2G_CUDA(cudaFuncSetAttribute(k_spmm_rows<double, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)nrows, (unsigned)ceil_div(ncols, 128 * VEC), (unsigned)nvec);
    k_spmm_rows<double, VEC><<<grid, 128, smem, st>>>(nrows, ncols, nnz, col, val, X, Y, accumulate ? 1 : 0, vstride);
    F2G_LAUNCH("k_spmm_rows block");
}

// FP64 sigma of a space blocked by irreps alone on its own vectors (ndet elements each): the same-
// spin terms block by block with the class-local string Hamiltonians (a block's rows only meet the
// columns of its own beta class: the C1 path reads all of them), the opposite-spin term through
// the irrep-aware kernel on the embedding. Event slots as in run(): beta, alpha, opposite spin.
void SigmaBuilder::run_blocked_sym(const double* C, double* S, cudaStream_t st, int nvec, bool timed, bool graph) {
    const DetBlocks& B = s->blocks;
    const int64_t nd = s->ndet, nf = s->nfull;
    double* xc = graph ? gxC.get() : xC.reserve((size_t)nvec * nf);
    double* xs = graph ? gxS.get() : xS.reserve((size_t)nvec * nf);
    if (timed)
        F2G_CUDA(cudaEventRecord(cur_ev[0], st));
    // beta same spin: per block transpose (Ia x Ib -> Ib x Ia), beta SpMM, transpose back (overwrites S)
    for (int b = 0; b < B.nblk(); ++b) {
        const int64_t* r = B.hblk.data() + 6 * b;
        const int64_t off = r[3], nIa = r[4], nIb = r[5];
        if (r[2] == 0)
            continue;
        const int cb = (int)r[1];
        k_transpose_blk<<<dim3((unsigned)ceil_div(nIb, 32), (unsigned)ceil_div(nIa, 32), (unsigned)nvec), dim3(32, 8), 0,
                          st>>>(nIa, nIb, C + off, nd, xc + off, nd);
        F2G_LAUNCH("k_transpose_blk");
        spmm_rows_raw(nIb, (int)nIa, hb.nnz, lcol[1].get() + B.cls_off[1][cb] * hb.nnz,
                      lval[1].get() + B.cls_off[1][cb] * hb.nnz, xc + off, xs + off, false, nd, nvec, st);
        k_transpose_blk<<<dim3((unsigned)ceil_div(nIa, 32), (unsigned)ceil_div(nIb, 32), (unsigned)nvec), dim3(32, 8), 0,
                          st>>>(nIb, nIa, xs + off, nd, S + off, nd);
        F2G_LAUNCH("k_transpose_blk");
    }
    if (timed)
        F2G_CUDA(cudaEventRecord(cur_ev[1], st));
    // alpha same spin + H0, accumulated
    for (int b = 0; b < B.nblk(); ++b) {
        const int64_t* r = B.hblk.data() + 6 * b;
        const int64_t off = r[3], nIa = r[4], nIb = r[5];
        if (r[2] == 0)
            continue;
        const int ca = (int)r[0];
        spmm_rows_raw(nIa, (int)nIb, ha.nnz, lcol[0].get() + B.cls_off[0][ca] * ha.nnz,
                      lval[0].get() + B.cls_off[0][ca] * ha.nnz, C + off, S + off, true, nd, nvec, st);
    }
    if (timed)
        F2G_CUDA(cudaEventRecord(cur_ev[2], st));
    // opposite spin on the embedding, added into S
    const DetEnum de = s->dets();
    blocks_embed<double>(de, nf, C, xc, nvec, st);
    F2G_CUDA(cudaMemsetAsync(xs, 0, (size_t)nvec * nf * sizeof(double), st));
    launch_opposite_sym(s, *osym, dV.get(), xc, xs, st, nvec, max_ctas > 0 ? max_ctas : 0);
    blocks_extract<double>(de, nf, xs, S, nvec, st, true);
    if (timed)
        F2G_CUDA(cudaEventRecord(cur_ev[3], st));
}

// Harvest finished timed builds, oldest first; with wait, all of them.
void SigmaBuilder::poll_timers(bool wait) {
    while (ev_count > 0) {
        cudaEvent_t* e = ev[ev_head];
        if (wait) {
            F2G_CUDA(cudaEventSynchronize(e[3]));
        } else {
            const cudaError_t r = cudaEventQuery(e[3]);
            if (r == cudaErrorNotReady) {
                if (cudaPeekAtLastError() == cudaErrorNotReady)
                    (void)cudaGetLastError(); // "not ready" is a status, not an error: do not leave it behind
                break;
            }
            F2G_CUDA(r);
        }
        if (ev_gen[ev_head] == timer_gen) {
            float bb = 0, aa = 0, ab = 0;
            F2G_CUDA(cudaEventElapsedTime(&bb, e[0], e[1]));
            F2G_CUDA(cudaEventElapsedTime(&aa, e[1], e[2]));
            F2G_CUDA(cudaEventElapsedTime(&ab, e[2], e[3]));
            t_acc[0] += (bb + aa + ab) * 1e-3;
            t_acc[1] += ab * 1e-3;
            t_acc[2] += aa * 1e-3;
            t_acc[3] += bb * 1e-3;
            builds += ev_nvec[ev_head];
        }
        ev_head = (ev_head + 1) % kTimerSlots;
        --ev_count;
    }
}

void SigmaBuilder::flush_timers() { poll_timers(true); }

// The slot for the next timed build; the host waits only if every slot is still pending.
void SigmaBuilder::timer_begin() {
    poll_timers(false);
    if (ev_count == kTimerSlots) {
        F2G_CUDA(cudaEventSynchronize(ev[ev_head][3]));
        poll_timers(false);
    }
    cur_ev = ev[(ev_head + ev_count) % kTimerSlots];
}

void SigmaBuilder::timer_end(int nvec) {
    const int slot = (ev_head + ev_count) % kTimerSlots;
    ev_nvec[slot] = nvec;
    ev_gen[slot] = timer_gen;
    ++ev_count;
}

// Restart the averages without waiting: builds still pending belong to the old generation.
void SigmaBuilder::reset_timers() {
    ++timer_gen;
    for (double& t : t_acc)
        t = 0.0;
    builds = 0;
}

void SigmaBuilder::avg_build_time(double* out) {
    flush_timers();
    for (int i = 0; i < 4; ++i)
        out[i] = builds ? t_acc[i] / builds : 0.0;
}

// Vectors are built in batches of at most kBatchElems determinants (one launch per term for the
// whole batch); the transposition scratch grows with the batch.
constexpr int64_t kBatchElems = int64_t(1) << 24;

int SigmaBuilder::batch_size(int nvec) const {
    const int64_t nd = std::max<int64_t>(1, s->nfull);
    return (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)nvec, kBatchElems / nd, 65535}));
}

void SigmaBuilder::hamiltonian(const double* C, double* sigma, cudaStream_t st, int nvec) {
    check_memory();
    const int64_t nd = s->ndet, nf = s->nfull;
    if (nd == 0 || nvec <= 0)
        return;
    const int bs = batch_size(nvec);
    const DetEnum de = s->dets();
    for (int v0 = 0; v0 < nvec; v0 += bs) {
        const int nv = std::min(bs, nvec - v0);
        const double* c = C + (int64_t)v0 * nd;
        double* sg = sigma + (int64_t)v0 * nd;
        if (blocked_sym_path()) {
            timer_begin();
            run_blocked_sym(c, sg, st, nv, true, false);
            timer_end(nv);
            continue;
        }
        if (s->blocked()) {
            // the space's vectors embedded into C1 vectors (zero elsewhere), sigma read back
            double* xc = xC.reserve((size_t)nv * nf);
            double* xs = xS.reserve((size_t)nv * nf);
            blocks_embed<double>(de, nf, c, xc, nv, st);
            timer_begin();
            apply_batch(xc, xs, st, nv, true, false);
            timer_end(nv);
            blocks_extract<double>(de, nf, xs, sg, nv, st);
            continue;
        }
        timer_begin();
        apply_batch(c, sg, st, nv, true, false);
        timer_end(nv);
    }
}

// graph: use the scratch set reserved by prepare_untimed (never reallocated while graphs captured
// with it exist); otherwise the growable scratch.
void SigmaBuilder::apply_batch(const double* C, double* sigma, cudaStream_t st, int nvec, bool timed, bool graph) {
    const int64_t nd = s->nfull;
    const size_t tot = (size_t)nvec * nd;
    if (precision == kFP64) {
        double* ct = graph ? gCt.get() : Ct.reserve(tot);
        double* tt = graph ? gTt.get() : Tt.reserve(tot);
        run<double>(C, sigma, st, 7, timed, nvec, ct, tt, graph);
    } else {
        float* c = graph ? gfC.get() : fC.reserve(tot);
        float* sg = graph ? gfS.get() : fS.reserve(tot);
        float* ct = graph ? gfCt.get() : fCt.reserve(tot);
        float* tt = graph ? gfTt.get() : fTt.reserve(tot);
        k_convert<double, float><<<1024, 256, 0, st>>>((int64_t)tot, C, c);
        F2G_LAUNCH("k_convert C");
        run<float>(c, sg, st, 7, timed, nvec, ct, tt, graph);
        k_convert<float, double><<<1024, 256, 0, st>>>((int64_t)tot, sg, sigma);
        F2G_LAUNCH("k_convert sigma");
    }
}

void SigmaBuilder::term(int which, const double* C, double* sigma, cudaStream_t st) {
    if (s->ndet == 0)
        return;
    if (s->blocked()) {
        const DetEnum de = s->dets();
        double* xc = xC.reserve(s->nfull);
        double* xs = xS.reserve(s->nfull);
        blocks_embed<double>(de, s->nfull, C, xc, 1, st);
        term_c1(which, xc, xs, st);
        blocks_extract<double>(de, s->nfull, xs, sigma, 1, st);
        F2G_CUDA(cudaStreamSynchronize(st));
        return;
    }
    term_c1(which, C, sigma, st);
}

void SigmaBuilder::term_c1(int which, const double* C, double* sigma, cudaStream_t st) {
    const int64_t nd = s->nfull;
    if (which == 0) {
        k_scale<<<1024, 256, 0, st>>>(nd, E, C, sigma);
        F2G_LAUNCH("k_scale");
        return;
    }
    if (which == 3) {
        F2G_CUDA(cudaMemsetAsync(sigma, 0, nd * sizeof(double), st));
        launch_opposite<double>(s, dV.get(), C, sigma, st);
        return;
    }
    // one-electron or same-spin two-electron part alone, through a temporary string Hamiltonian
    const int spin = (which == 1 || which == 4) ? 0 : 1;
    const int parts = (which == 1 || which == 2) ? 1 : 2;
    const SpinStrings& ss = s->spin(spin);
    StringHamiltonian tmp;
    tmp.nnz = ss_row_nnz(n, ss.k);
    F2G_CUDA(cudaMemsetAsync(sigma, 0, nd * sizeof(double), st));
    if (ss.k < 1 || tmp.nnz == 0)
        return;
    const size_t total = (size_t)ss.N0 * tmp.nnz;
    tmp.col.reserve(total);
    tmp.val.reserve(total);
    k_build_ss<double><<<ceil_div(ss.N0, 128), 128, 0, st>>>(n, ss.k, ss.N0, tmp.nnz, ss.str.get(), s->binom.get(),
                                                            dH.get(), dV.get(), 0.0, parts, tmp.col.get(),
                                                            tmp.val.get());
    F2G_LAUNCH("k_build_ss term");
    const int64_t NA = s->a.N0, NB = s->b.N0;
    if (spin == 0) {
        launch_spmm<double>(tmp, tmp.val.get(), NA, (int)NB, C, sigma, false, st);
    } else {
        double* ct = Ct.reserve(nd);
        double* tt = Tt.reserve(nd);
        launch_transpose<double>(NA, NB, C, ct, st);
        launch_spmm<double>(tmp, tmp.val.get(), NB, (int)NA, ct, tt, false, st);
        launch_transpose<double>(NB, NA, tt, sigma, st);
    }
    F2G_CUDA(cudaStreamSynchronize(st));
}

// Stream-ordered; the string-energy scratch is kept by the builder (no allocation after the first
// call, so no implicit device synchronisation).
void SigmaBuilder::det_energies(double* out, cudaStream_t st) {
    const int64_t NA = s->a.N0, NB = s->b.N0;
    if (NA * NB == 0 || s->ndet == 0)
        return;
    double* full = out;
    if (s->blocked())
        full = xS.reserve(NA * NB); // C1 energies, then the space's
    double* ea = eA.reserve(NA);
    double* eb = eB.reserve(NB);
    double* jr = eJ.reserve((size_t)NA * std::max(1, n));
    k_string_energy<<<ceil_div(NA, 128), 128, 0, st>>>(n, NA, s->a.str.get(), dH.get(), dV.get(), ea, jr);
    k_string_energy<<<ceil_div(NB, 128), 128, 0, st>>>(n, NB, s->b.str.get(), dH.get(), dV.get(), eb, nullptr);
    k_det_energy<<<ceil_div(NA * NB, 256), 256, 0, st>>>(n, NA, NB, E, s->b.str.get(), ea, eb, jr, full);
    F2G_LAUNCH("k_det_energy");
    if (s->blocked())
        blocks_extract<double>(s->dets(), NA * NB, full, out, 1, st);
}

} // namespace f2g
