// Opposite-spin sigma on the 5th-generation tensor cores (tcgen05, split-FP16 products with FP32
// accumulation in tensor memory), for the FP32 sigma of the mixed-precision mode.
//
// Operator (forte2/ci/ci_sigma_builder_harrison_zarrabian.cc:197-308, written per alpha string):
//   sigma(Ja, Jb) += sum_{(p,q)} sum_{(r,s)} V[p][r][q][s] <Ja|E^a_pq|Ia> <Jb|E^b_rs|Ib> C(Ia, Ib)
// with V the physicist integrals (pr|qs). For one output alpha string Ja the K = na * (n - na + 1)
// alpha excitations (p in Ja, q not in Ja - p) give the rows T[k][Ib] = sign_k C(Ia_k, Ib) of C
// (whole rows, gathered), and
//   U[Ib][(r,s)] = sum_k T[k][Ib] V'[(r,s)][k],   V'[(r,s)][k] = V[p_k][r][q_k][s]
// is a dense GEMM (M = 128 beta strings per tile, N = 8 values of s x 16 of r per pass, K padded to a
// multiple of 16). Each beta string Ib then scatters its 8 x 9 valid (s in Ib, r not in Ib - s)
// entries into sigma(Ja, Jb = Ib - s + r) with the beta signs.
//
// Accuracy: both operands are scaled by powers of two (C by its largest magnitude per vector, V by
// its largest magnitude) into [2^14, 2^15) and split x = hi + lo with hi, lo FP16 (round to
// nearest); D += A_hi B_hi + A_lo B_hi + A_hi B_lo on kind::f16 (22 significant bits per operand,
// the dropped lo*lo term is below FP32 rounding). The error against the FP64 sigma is that of an
// FP32 evaluation (1e-7 relative).
//
// Determinism: sigma(Ja, :) is accumulated in shared memory as 64-bit fixed point. Every product
// sum is bounded by construction (|A|, |B| < 2^15, K <= 72, so |U| < 2^37 in scaled units), is
// truncated to a multiple of 2^-18 of the scaled unit by integer arithmetic, and at most
// nb (n - nb + 1) <= 72 of them reach one element, so the sum stays below 2^62 and is exact.
// Integer addition does not depend on the order of the shared-memory atomics: the sigma of a vector
// is bitwise the same for every grid, batch and run. The row is converted back and added to the
// same-spin terms in FP32 once per alpha string.
//
// One CTA per SM (persistent over Ja), 1024 threads: all threads gather the operand tiles into
// shared memory in the canonical K-major no-swizzle layout (8-row x 16-byte core matrices), one
// thread issues the MMAs into one of two 128-lane x 128-column FP32 accumulators in tensor memory
// and commits them to an mbarrier, and while they run all 32 warps read the previous tile's
// accumulator back (the 8 warps w = q mod 4 share lanes 32 q .. +31 and take one s column block
// each) for its scatter. Waits are bounded: a wait that gives up sets the error flag, the CTA stops
// issuing work, waits (bounded again) for the MMAs it has committed and releases its tensor memory.
// An error flag of 1 means that the sigma of that call is not valid.
#include <cuda_fp16.h>

#include <cmath>
#include <cstdint>

#include "sigma.cuh"

namespace f2g {

namespace {

constexpr int kTcThreads = 1024;
constexpr int kQuarterWarps = kTcThreads / 128;      // warps sharing one 32-lane quarter of the accumulator
constexpr int kChunksPerWarp = 8 / kQuarterWarps;    // s columns (16 accumulator columns each) per warp
constexpr int kTcM = 128;      // beta strings per tile (accumulator lanes)
constexpr int kTcN = 128;      // 8 values of s x 16 values of r per pass
constexpr int kTcMaxK = 80;    // padded alpha-excitation count (na * (n - na + 1) <= 72 for n <= 16)
constexpr int kTcCols = 256;   // tensor-memory columns allocated: two 128-column accumulators
constexpr int kFixShift = 18;  // fixed-point fraction bits (in units of the scaled product)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row, k) in a K-major, no-swizzle 16-bit operand of kp columns: core
// matrices of 8 rows x 8 FP16 (16 B per row, 128 B each); adjacent core matrices along K are 128 B
// apart (leading byte offset), along rows (kp / 8) * 128 B apart (stride byte offset)
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int kp) {
    return (uint32_t)(((row >> 3) * (kp >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// tcgen05 shared-memory matrix descriptor: start >> 4 [0,14), leading byte offset >> 4 [16,30),
// stride byte offset >> 4 [32,46), version 1 [46,48), base offset 0, no swizzle [61,64) = 0
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D F32 [4,6) = 1, A F16 [7,10) = 0, B F16 [10,13) = 0, both
// K-major (bits 15, 16 = 0), N >> 3 at [17,23), M >> 4 at [24,29)
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :
                 : "r"(tmem_d), "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// bounded wait for the phase `parity` of an mbarrier; returns false if it gave up after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit) {
    for (long long it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(mbar), "r"(parity)
                     : "memory");
        if (done)
            return true;
    }
    return false;
}

// 16 consecutive accumulator columns of this warp's 32 lanes; complete after tmem_wait_ld()
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 2^e as a float for -126 <= e <= 127
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

// scale exponent that maps a largest magnitude m into [2^14, 2^15) (0 for m = 0 or not finite),
// clamped so that 2^e and 2^-e are normal floats
__host__ __device__ inline int split_exponent(float m) {
    if (!(m > 0.0f) || !(m <= 3.0e38f))
        return 0;
    int ex = 0;
    (void)frexpf(m, &ex); // m = f 2^ex, f in [0.5, 1): m < 2^ex
    const int e = 15 - ex;
    return e < -120 ? -120 : (e > 120 ? 120 : e);
}

// x (FP32 bits, |x| < 2^37) times 2^kFixShift, truncated toward zero, as a two's-complement 64-bit
// integer, negated when `neg` is set. Integer operations only: the same bits on every run.
__device__ __forceinline__ unsigned long long fixed_point(uint32_t b, uint32_t neg) {
    const uint32_t e = (b >> 23) & 0xFFu;
    const uint32_t m = (b & 0x7FFFFFu) | 0x800000u;
    int sh = (int)e - (127 + 23 - kFixShift); // x 2^kFixShift = m 2^sh
    sh = sh > 40 ? 40 : sh;                    // only for values outside the bound (not finite)
    unsigned long long q = sh >= 0 ? ((unsigned long long)m << sh) : (sh > -24 ? (unsigned long long)(m >> -sh) : 0ull);
    q = e ? q : 0ull; // zero or subnormal: below the resolution
    return (((b >> 31) ^ neg) & 1u) ? (0ull - q) : q;
}

struct TcShared {
    // operands, K-major no-swizzle core-matrix layout (16-byte aligned)
    alignas(128) __half a_hi[kTcM * kTcMaxK];
    alignas(128) __half a_lo[kTcM * kTcMaxK];
    alignas(128) __half b_hi[kTcN * kTcMaxK];
    alignas(128) __half b_lo[kTcN * kTcMaxK];
    uint32_t ia[kTcMaxK];  // alpha string of excitation k
    float sgn[kTcMaxK];    // its sign
    int pk[kTcMaxK], qk[kTcMaxK];
    alignas(8) uint64_t mbar;
    uint32_t tmem_base;
    int abort;
};

// two FP16 parts of 8 scaled values, stored as one 16-byte row of a core matrix each
__device__ __forceinline__ void split_store(const float (&x)[8], __half* hi_dst, __half* lo_dst) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const __half2 hh = __floats2half2_rn(x[2 * j], x[2 * j + 1]);
        const float2 hf = __half22float2(hh);
        const __half2 ll = __floats2half2_rn(x[2 * j] - hf.x, x[2 * j + 1] - hf.y);
        h[j] = *reinterpret_cast<const uint32_t*>(&hh);
        l[j] = *reinterpret_cast<const uint32_t*>(&ll);
    }
    *reinterpret_cast<uint4*>(hi_dst) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(lo_dst) = make_uint4(l[0], l[1], l[2], l[3]);
}

} // namespace

// exc[Ib][i][r] for the i-th occupied orbital s of Ib and r < 16: Jb | negative << 31 for the beta
// string Jb = Ib - s + r (r not in Ib - s), 0x00FFFFFF otherwise.
__global__ void k_build_beta_exc(int n, int k, int64_t N0, const uint64_t* __restrict__ str,
                                 const uint64_t* __restrict__ binom, uint32_t* __restrict__ exc) {
    const int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= N0)
        return;
    const uint64_t mI = str[I];
    int i = 0;
    for (int s = 0; s < n; ++s) {
        if (!(mI >> s & 1))
            continue;
        const uint64_t mK = mI & ~(uint64_t(1) << s);
        const int neg_s = parity_below(mK, s);
        for (int r = 0; r < 16; ++r) {
            uint32_t e = 0x00FFFFFFu;
            if (r < n && !(mK >> r & 1)) {
                const uint64_t mJ = mK | (uint64_t(1) << r);
                const uint32_t J = (uint32_t)string_rank(mJ, n, k, binom);
                e = J | ((uint32_t)(parity_below(mK, r) ^ neg_s) << 31);
            }
            exc[(I * k + i) * 16 + r] = e;
        }
        ++i;
    }
}

// Largest magnitude of each of nvec vectors of nd elements, as FP32 bits (non-negative floats order
// like their bit patterns). out[v] must be zero on entry.
__global__ void k_absmax(int64_t nd, const float* __restrict__ x, unsigned int* __restrict__ out) {
    x += blockIdx.y * nd;
    float m = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[32];
    if ((threadIdx.x & 31) == 0)
        wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0)
            atomicMax(out + blockIdx.y, __float_as_uint(m));
    }
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_opposite_tc(int n, int na, int nb, int ma, int64_t N0a, int N0b, const uint32_t* __restrict__ down_a,
                  const uint32_t* __restrict__ up_a, const uint64_t* __restrict__ str_b,
                  const uint32_t* __restrict__ exc_b, const float* __restrict__ V, int eb,
                  const unsigned int* __restrict__ cmax, const float* __restrict__ C, float* __restrict__ sig,
                  int* __restrict__ err, long long poll_limit) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcShared& sh = *reinterpret_cast<TcShared*>(smem_raw);
    // sigma(Ja, :) in 64-bit fixed point, N0b elements
    unsigned long long* row = reinterpret_cast<unsigned long long*>(smem_raw + sizeof(TcShared));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = na * ma, kp = (K + 15) & ~15;
    C += blockIdx.y * N0a * (int64_t)N0b; // vector blockIdx.y of a batch
    sig += blockIdx.y * N0a * (int64_t)N0b;
    const uint32_t mbar = smem_u32(&sh.mbar);
    // operand scales 2^ea (C) and 2^eb (V); the fixed-point row is in units of 2^-(ea + eb + kFixShift)
    const int ea = split_exponent(__uint_as_float(cmax[blockIdx.y]));
    const float fa = pow2f(ea), fb = pow2f(eb);
    const float unscale0 = pow2f(-kFixShift), unscale1 = pow2f(-ea), unscale2 = pow2f(-eb);

    if (tid == 0) {
        mbar_init(mbar, 1);
        sh.abort = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh.tmem_base)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh.tmem_base;
    uint32_t phase = 0;
    bool in_flight = false; // a commit this thread has not yet seen complete
    const uint32_t lbo = 128, sbo = (uint32_t)(kp >> 3) * 128;

    // scatter of one finished tile: warp w reads lanes 32 (w % 4) + [0, 32) = beta strings ib0 + that;
    // the warps sharing a lane quarter take every kQuarterWarps-th s of the pass. The excitation
    // entries are requested first, then the accumulator columns, then one wait for both, so their
    // latencies overlap.
    auto scatter = [&](int ib0, uint32_t acc, int s0) {
        const int m = (warp & 3) * 32 + lane;
        const int Ib = ib0 + m;
        const bool valid = Ib < N0b;
        const uint64_t mI = valid ? str_b[Ib] : 0;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        uint4 e4[kChunksPerWarp][4];
        bool has[kChunksPerWarp];
#pragma unroll
        for (int i = 0; i < kChunksPerWarp; ++i) {
            const int s = s0 + (warp >> 2) + kQuarterWarps * i;
            has[i] = valid && s < n && (mI >> s & 1);
            if (has[i]) {
                const int si = popc64(mI & ((uint64_t(1) << s) - 1));
                const uint4* src = reinterpret_cast<const uint4*>(exc_b + ((int64_t)Ib * nb + si) * 16);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    e4[i][q] = __ldg(src + q);
            }
        }
        uint32_t v[kChunksPerWarp][16];
        __syncwarp();
#pragma unroll
        for (int i = 0; i < kChunksPerWarp; ++i)
            tmem_ld16(acc + lane_base + (uint32_t)(((warp >> 2) + kQuarterWarps * i) * 16), v[i]);
        tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < kChunksPerWarp; ++i) {
            if (!has[i])
                continue;
            const uint32_t e[16] = {e4[i][0].x, e4[i][0].y, e4[i][0].z, e4[i][0].w, e4[i][1].x, e4[i][1].y,
                                    e4[i][1].z, e4[i][1].w, e4[i][2].x, e4[i][2].y, e4[i][2].z, e4[i][2].w,
                                    e4[i][3].x, e4[i][3].y, e4[i][3].z, e4[i][3].w};
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const uint32_t jb = e[r] & 0x00FFFFFFu;
                if (jb != 0x00FFFFFFu) // the sign bit of the entry flips the sign of the value
                    atomicAdd(row + jb, fixed_point(v[i][r], e[r] >> 31));
            }
        }
    };

    for (int64_t Ja = blockIdx.x; Ja < N0a && !sh.abort; Ja += gridDim.x) {
        float* srow = sig + Ja * (int64_t)N0b;
        for (int c = tid; c < N0b; c += kTcThreads)
            row[c] = 0ull;
        // alpha excitations of Ja: k = pi * ma + qi
        if (tid < K) {
            const int pi = tid / ma, qi = tid % ma;
            const uint32_t ep = down_a[Ja * na + pi];
            const uint32_t eq = up_a[(int64_t)e_addr(ep) * ma + qi];
            sh.ia[tid] = e_addr(eq);
            sh.sgn[tid] = (e_neg(ep) ^ e_neg(eq)) ? -1.0f : 1.0f;
            sh.pk[tid] = e_orb(ep);
            sh.qk[tid] = e_orb(eq);
        }
        __syncthreads();
        for (int s0 = 0; s0 < n && !sh.abort; s0 += 8) {
            // B = V'[(s, r)][k] 2^eb for s in [s0, s0 + 8), r < 16 (zero outside the space); the alpha
            // sign of excitation k is folded into column k. One 16-byte row of 8 k per task.
            for (int t = tid; t < kTcN * (kp >> 3); t += kTcThreads) {
                const int nn = t / (kp >> 3), k0 = (t % (kp >> 3)) * 8;
                const int s = s0 + (nn >> 4), r = nn & 15;
                float x[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int kk = k0 + j;
                    x[j] = (kk < K && s < n && r < n)
                               ? sh.sgn[kk] * fb * V[(((size_t)sh.pk[kk] * n + r) * n + sh.qk[kk]) * n + s]
                               : 0.0f;
                }
                const uint32_t off = kmajor_off(nn, k0, kp) >> 1;
                split_store(x, sh.b_hi + off, sh.b_lo + off);
            }
            int prev_ib0 = -1, tile = 0;
            uint32_t prev_acc = 0;
            for (int ib0 = 0; ib0 < N0b && !sh.abort; ib0 += kTcM) {
                // A = T[Ib][k] 2^ea = C(Ia_k, Ib) 2^ea for Ib in [ib0, ib0 + 128): each thread takes one
                // Ib and groups of 8 consecutive k (one 16-byte row of a core matrix); for fixed k a
                // warp reads 32 consecutive floats. All loads of a thread are issued first.
                {
                    constexpr int kRowThreads = kTcThreads / kTcM;              // threads per beta string
                    constexpr int kGroups = (kTcMaxK / 8 + kRowThreads - 1) / kRowThreads;
                    const int m = tid & (kTcM - 1);
                    const int Ib = ib0 + m;
                    const int g0 = tid >> 7;
                    const bool in = Ib < N0b;
                    float x[kGroups][8];
#pragma unroll
                    for (int j = 0; j < kGroups; ++j)
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            const int kk = 8 * (g0 + j * kRowThreads) + c;
                            x[j][c] = (kk < K && in) ? fa * __ldg(C + (int64_t)sh.ia[kk] * N0b + Ib) : 0.0f;
                        }
#pragma unroll
                    for (int j = 0; j < kGroups; ++j) {
                        const int g = g0 + j * kRowThreads;
                        if (8 * g < kp) {
                            const uint32_t off = kmajor_off(m, 8 * g, kp) >> 1;
                            split_store(x[j], sh.a_hi + off, sh.a_lo + off);
                        }
                    }
                }
                // make the generic-proxy shared-memory writes visible to the tensor cores
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncthreads();
                // two accumulators: the MMAs of this tile run while the previous tile is scattered
                const uint32_t acc = tmem + (uint32_t)(tile & 1) * kTcN;
                if (tid == 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t ahi = smem_u32(sh.a_hi), alo = smem_u32(sh.a_lo);
                    const uint32_t bhi = smem_u32(sh.b_hi), blo = smem_u32(sh.b_lo);
                    for (int t = 0; t < kp / 16; ++t) {
                        const uint32_t adv = (uint32_t)t * 2 * lbo; // 16 FP16 = two core matrices along K
                        mma_f16(acc, smem_desc(ahi + adv, lbo, sbo), smem_desc(bhi + adv, lbo, sbo), t > 0);
                        mma_f16(acc, smem_desc(alo + adv, lbo, sbo), smem_desc(bhi + adv, lbo, sbo), 1);
                        mma_f16(acc, smem_desc(ahi + adv, lbo, sbo), smem_desc(blo + adv, lbo, sbo), 1);
                    }
                    mma_commit(mbar);
                }
                in_flight = true;
                if (prev_ib0 >= 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    scatter(prev_ib0, prev_acc, s0);
                }
                const bool ok = mbar_wait(mbar, phase, poll_limit);
                if (ok) {
                    in_flight = false;
                    phase ^= 1;
                } else {
                    if (lane == 0)
                        atomicExch(err, 1);
                    sh.abort = 1;
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncthreads();
                prev_ib0 = ib0;
                prev_acc = acc;
                ++tile;
            }
            if (prev_ib0 >= 0 && !sh.abort) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                scatter(prev_ib0, prev_acc, s0);
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            }
            __syncthreads();
        }
        __syncthreads();
        if (!sh.abort)
            for (int c = tid; c < N0b; c += kTcThreads) {
                const float x = __ll2float_rn((long long)row[c]) * unscale0 * unscale1 * unscale2;
                srow[c] += x;
            }
        __syncthreads();
    }
    // after a wait that gave up, the MMAs of that commit may still be running: wait for them (bounded)
    // before the tensor memory they write is released
    if (in_flight)
        (void)mbar_wait(mbar, phase, (1ll << 26));
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
}

size_t opposite_tc_smem(int N0b) { return sizeof(TcShared) + (size_t)N0b * sizeof(unsigned long long); }

bool opposite_tc_supported(const CIStrings* s) {
    const int n = s->norb;
    if (n > 16 || s->na < 1 || s->nb < 1 || s->a.N1 == 0 || s->b.N1 == 0)
        return false;
    // K <= 72 and at most 72 contributions per sigma element keep the fixed-point row exact
    if (s->na * (n - s->na + 1) > 72 || s->nb * (n - s->nb + 1) > 72)
        return false;
    return opposite_tc_smem((int)s->b.N0) <= 227 * 1024;
}

void build_beta_exc(const CIStrings* s, DevBuf<uint32_t>& exc, cudaStream_t st) {
    const SpinStrings& b = s->b;
    exc.reserve((size_t)std::max<int64_t>(1, b.N0 * b.k * 16));
    k_build_beta_exc<<<ceil_div(b.N0, 128), 128, 0, st>>>(s->norb, b.k, b.N0, b.str.get(), s->binom.get(), exc.get());
    F2G_LAUNCH("k_build_beta_exc");
}

int opposite_tc_v_exponent(float vmax) { return split_exponent(vmax); }

// cmax: nvec words of scratch (the per-vector largest |C|), written here before the kernel runs.
void launch_opposite_tc(const CIStrings* s, const uint32_t* exc, const float* V, int eb, const float* C, float* sig,
                        unsigned int* cmax, int* err, long long poll_limit, int max_ctas, cudaStream_t st, int nvec) {
    const int64_t nd = s->a.N0 * s->b.N0;
    F2G_CUDA(cudaMemsetAsync(cmax, 0, (size_t)nvec * sizeof(unsigned int), st));
    k_absmax<<<dim3(256, (unsigned)nvec), 256, 0, st>>>(nd, C, cmax);
    F2G_LAUNCH("k_absmax");
    const size_t smem = opposite_tc_smem((int)s->b.N0);
    F2G_CUDA(cudaFuncSetAttribute(k_opposite_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0;
    F2G_CUDA(cudaGetDevice(&dev));
    F2G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int64_t gx = std::min<int64_t>(s->a.N0, sms);
    if (max_ctas > 0)
        gx = std::min<int64_t>(gx, max_ctas);
    k_opposite_tc<<<dim3((unsigned)gx, (unsigned)nvec), kTcThreads, smem, st>>>(
        s->norb, s->na, s->nb, s->a.m1, s->a.N0, (int)s->b.N0, s->a.down1.get(), s->a.up1.get(), s->b.str.get(), exc,
        V, eb, cmax, C, sig, err, poll_limit > 0 ? poll_limit : (1ll << 26));
    F2G_LAUNCH("k_opposite_tc");
}

} // namespace f2g
