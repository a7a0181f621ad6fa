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
// Determinism: sigma(Ja, :) is accumulated in shared memory in fixed point, as two 32-bit integer
// rows. Every product sum is bounded by construction (|A|, |B| <= 2^15 with FP16 low parts below
// 2^-10 of that, K <= 72, so |U| < 72 2^30 (1 + 2^-9) < 2^36.2 in scaled units) and is rounded to
// a multiple of 2^-7 scaled units, split exactly into a high part
// (units of 2^15) and a low part (units of 2^-7), each below 2^21.2 in magnitude; at most
// nb (n - nb + 1) <= 72 of them reach one element, so both sums stay below 2^28 and are exact.
// Integer addition does not depend on the order of the shared-memory atomics: the sigma of a vector
// is bitwise the same for every grid, batch and run. The row is converted back and added to the
// same-spin terms in FP32 once per alpha string.
//
// One CTA per SM (persistent over Ja), 24 warps in three roles that hand tiles to each other
// through mbarriers (every wait bounded):
//  * 8 producer warps: threads m and m + 128 own the two halves (k < 40, k >= 40) of row m (beta
//    string ib0 + m) of the A tile. They request the gathered values of the next tile into
//    registers while the tensor cores work on the current one, then (once those MMAs have released
//    the A buffer) scale, split and store them in the canonical K-major no-swizzle layout (8-row x
//    16-byte core matrices) and arrive on A_full.
//  * MMA issue (thread 0, after its own row): the 3 x kp/16 MMAs of a tile (M = 128, N = 256: all
//    16 s x 16 r columns in one instruction, so A is gathered once per tile) into one of two
//    256-column FP32 accumulators in tensor memory, committed to A_empty and ACC_full.
//  * 16 scatter warps (four per 32-lane quarter of the accumulator, each taking every fourth s):
//    read the finished accumulator with tcgen05.ld, add the fixed-point contributions into the
//    sigma row and arrive on ACC_empty, so the MMAs of tile t + 1 overlap the scatter of tile t.
//    An r slot runs only if some lane of the warp has it (uniform branch: neighbouring strings
//    mostly agree on the low orbitals).
// B = V' for the alpha string is built by all warps between alpha strings. A wait that gives up
// sets the error flag and the CTA leaves its loops, waits (bounded again) for the MMAs it has
// committed and releases its tensor memory. An error flag of 1 means that the sigma of that call
// is not valid.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstdint>
#include <memory>
#include <mutex>
#include <string>

#include "sigma.cuh"

namespace f2g {

namespace {

constexpr int kProdWarps = 8;   // producer warps: two threads per row of the A tile (thread 0 issues the MMAs)
constexpr int kScatWarps = 16;  // scatter warps: four per lane quarter of the accumulator
constexpr int kTcThreads = (kProdWarps + kScatWarps) * 32; // 24 warps: 6 per SM sub-partition, 80 registers
constexpr int kProdHalf = 40;   // k values per producer thread (half of the padded K)
constexpr int kTcM = 128;      // beta strings per tile (accumulator lanes)
constexpr int kTcN = 256;      // 16 values of s x 16 values of r
constexpr int kTcMaxK = 80;    // padded alpha-excitation count (na * (n - na + 1) <= 72 for n <= 16)
constexpr int kTcCols = 512;   // tensor-memory columns allocated: two 256-column accumulators

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

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// bounded wait for the phase `parity` of an mbarrier; returns false if it gave up after `limit` polls.
// A poll is a try_wait (which may suspend the thread for a while); limits below kProbeLimit (a test
// setting) poll with the non-suspending test_wait instead, so that they give up after that many probes.
// With `abort`, the wait also gives up once another thread of the CTA has set that flag.
constexpr long long kProbeLimit = 4096;
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit,
                                          const volatile int* abort = nullptr) {
    for (long long it = 0; it < limit; ++it) {
        if (abort && (it & 63) == 63 && *abort)
            return false;
        uint32_t done;
        if (limit >= kProbeLimit)
            asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                         "selp.u32 %0, 1, 0, p;\n\t}\n"
                         : "=r"(done)
                         : "r"(mbar), "r"(parity)
                         : "memory");
        else
            asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
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
__device__ __forceinline__ int split_exponent(float m) {
    if (!(m > 0.0f) || !(m <= 3.0e38f))
        return 0;
    int ex = 0;
    (void)frexpf(m, &ex); // m = f 2^ex, f in [0.5, 1): m < 2^ex
    const int e = 15 - ex;
    return e < -120 ? -120 : (e > 120 ? 120 : e);
}

// Adds x (FP32 bits, |x| < 2^36.2 in scaled units; sign flipped when neg is 1) to the fixed-point
// element jb as two exact integers: hi = round(x / 2^15) into row_hi and lo = round((x - hi 2^15)
// 2^7) into row_lo, so the element holds (hi 2^22 + lo) 2^-7. Both parts come from FP32
// multiply-adds on a 1.5 2^23 offset (the float bits of C + y are C's bits + y for an integer
// |y| < 2^22); |hi|, |lo| < 2^21.2, so up to 72 of them sum exactly in 32 bits.
__device__ __forceinline__ void add_fixed(int* row_hi, int* row_lo, uint32_t jb, uint32_t b, uint32_t neg) {
    const float C = 12582912.0f; // 1.5 2^23
    const float x = __uint_as_float(b ^ (neg << 31));
    const float t = fmaf(x, 0x1p-15f, C);                  // C + round(x / 2^15)
    const float rem = fmaf(-(t - C), 32768.0f, x);          // x - hi 2^15, exact, |rem| <= 2^14
    const float u = fmaf(rem, 128.0f, C);                    // C + round(rem 2^7)
    atomicAdd(row_hi + jb, __float_as_int(t) - __float_as_int(C));
    atomicAdd(row_lo + jb, __float_as_int(u) - __float_as_int(C));
}

struct TcShared {
    // operands, K-major no-swizzle core-matrix layout (16-byte aligned)
    alignas(128) __half a_hi[kTcM * kTcMaxK];
    alignas(128) __half a_lo[kTcM * kTcMaxK];
    alignas(128) __half b_hi[kTcN * kTcMaxK];
    alignas(128) __half b_lo[kTcN * kTcMaxK];
    const float* rowp[kTcMaxK]; // row of C of alpha excitation k
    float sfa[kTcMaxK];         // its sign times the C scale 2^ea
    int pk[kTcMaxK], qk[kTcMaxK];
    alignas(8) uint64_t a_full, a_empty, b_full, acc_full[2], acc_empty[2];
    uint32_t tmem_base;
    volatile int abort;
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

// B = V'[(s, r)][k] 2^eb of the K excitations (pk[k], qk[k]) of one alpha string (zero outside the
// space), K-major core matrices, by the threads of one block
__device__ __forceinline__ void build_b(int n, int K, int kp, float fb, const float* __restrict__ V, const int* pk,
                                        const int* qk, __half* b_hi, __half* b_lo, int tid, int nthreads) {
    for (int t = tid; t < kTcN * (kp >> 3); t += nthreads) {
        const int nn = t / (kp >> 3), k0 = (t % (kp >> 3)) * 8;
        const int s = nn >> 4, r = nn & 15;
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int kk = k0 + j;
            x[j] = (kk < K && s < n && r < n) ? fb * V[(((size_t)pk[kk] * n + r) * n + qk[kk]) * n + s] : 0.0f;
        }
        const uint32_t off = kmajor_off(nn, k0, kp) >> 1;
        split_store(x, b_hi + off, b_lo + off);
    }
}

// 2D tensor copy of one box into shared memory, completing on an mbarrier (transaction bytes)
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t mbar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
                 : "memory");
}

} // namespace

// The B operands of every alpha string (the tensor-core kernel's B tiles, fed to it by TMA):
// out[Ja] = {hi, lo}, each kTcN * kp halves in the kernel's shared-memory layout.
__global__ void k_build_bops(int n, int na, int ma, int64_t N0a, const uint32_t* __restrict__ down_a,
                             const uint32_t* __restrict__ up_a, const float* __restrict__ V,
                             const unsigned int* __restrict__ vmax, __half* __restrict__ out) {
    __shared__ int pk[kTcMaxK], qk[kTcMaxK];
    const int K = na * ma, kp = (K + 15) & ~15;
    const float fb = pow2f(split_exponent(__uint_as_float(vmax[0])));
    for (int64_t Ja = blockIdx.x; Ja < N0a; Ja += gridDim.x) {
        __syncthreads(); // the previous string's excitations are no longer read
        if ((int)threadIdx.x < K) {
            const int pi = threadIdx.x / ma, qi = threadIdx.x % ma;
            const uint32_t ep = down_a[Ja * na + pi];
            const uint32_t eq = up_a[(int64_t)e_addr(ep) * ma + qi];
            pk[threadIdx.x] = e_orb(ep);
            qk[threadIdx.x] = e_orb(eq);
        }
        __syncthreads();
        __half* hi = out + (size_t)Ja * 2 * kTcN * kp;
        build_b(n, K, kp, fb, V, pk, qk, hi, hi + (size_t)kTcN * kp, threadIdx.x, blockDim.x);
    }
}

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
                  const uint32_t* __restrict__ exc_b, const float* __restrict__ V,
                  const unsigned int* __restrict__ vmax, const unsigned int* __restrict__ cmax,
                  const float* __restrict__ C, float* __restrict__ sig, int* __restrict__ err,
                  long long poll_limit, const __grid_constant__ CUtensorMap bmap, int tma_b) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcShared& sh = *reinterpret_cast<TcShared*>(smem_raw);
    // sigma(Ja, :) in fixed point: high and low 32-bit parts, N0b elements each
    int* row_hi = reinterpret_cast<int*>(smem_raw + sizeof(TcShared));
    int* row_lo = row_hi + N0b;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = na * ma, kp = (K + 15) & ~15;
    const int ntile = (N0b + kTcM - 1) / kTcM;
    C += blockIdx.y * N0a * (int64_t)N0b; // vector blockIdx.y of a batch
    sig += blockIdx.y * N0a * (int64_t)N0b;
    // operand scales 2^ea (C) and 2^eb (V) from the largest magnitudes, read from device memory (so
    // captured graphs follow new vectors and integrals); the fixed-point row is in units of
    // 2^-(ea + eb + 7)
    const int ea = split_exponent(__uint_as_float(cmax[blockIdx.y]));
    const int eb = split_exponent(__uint_as_float(vmax[0]));
    const float fa = pow2f(ea), fb = pow2f(eb);
    const float unscale0 = pow2f(-7), unscale1 = pow2f(-ea), unscale2 = pow2f(-eb);
    const uint32_t a_full = smem_u32(&sh.a_full), a_empty = smem_u32(&sh.a_empty), b_full = smem_u32(&sh.b_full);
    const uint32_t acc_full[2] = {smem_u32(&sh.acc_full[0]), smem_u32(&sh.acc_full[1])};
    const uint32_t acc_empty[2] = {smem_u32(&sh.acc_empty[0]), smem_u32(&sh.acc_empty[1])};
    const uint32_t lbo = 128, sbo = (uint32_t)(kp >> 3) * 128;

    if (tid == 0) {
        mbar_init(a_full, kProdWarps * 32);
        mbar_init(a_empty, 1);
        mbar_init(b_full, 1);
        for (int b = 0; b < 2; ++b) {
            mbar_init(acc_full[b], 1);
            mbar_init(acc_empty[b], kScatWarps);
        }
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

    auto give_up = [&]() {
        atomicExch(err, 1);
        sh.abort = 1;
    };

    long long g0 = 0;      // tiles of this CTA before the current alpha string
    long long last_g = -1; // MMA thread: last tile whose MMAs were committed
    uint32_t b_phase = 0;   // thread 0: parity of the b_full phase of the last B copy issued
    bool b_pending = false; // thread 0: a B copy was issued and its completion not yet seen
    int nja = 0;            // alpha strings of this CTA so far
    for (int64_t Ja = blockIdx.x; Ja < N0a && !sh.abort; Ja += gridDim.x) {
        float* srow = sig + Ja * (int64_t)N0b;
        // ---- alpha string set-up (all warps): excitations k = pi * ma + qi, B, zero row
        if (tid < K) {
            const int pi = tid / ma, qi = tid % ma;
            const uint32_t ep = down_a[Ja * na + pi];
            const uint32_t eq = up_a[(int64_t)e_addr(ep) * ma + qi];
            sh.rowp[tid] = C + (int64_t)e_addr(eq) * N0b;
            sh.sfa[tid] = (e_neg(ep) ^ e_neg(eq)) ? -fa : fa; // the alpha sign is folded into A
            sh.pk[tid] = e_orb(ep);
            sh.qk[tid] = e_orb(eq);
        } else if (tid < kTcMaxK) { // padding columns of K: zero factors (never uninitialised memory)
            sh.rowp[tid] = C;
            sh.sfa[tid] = 0.0f;
            sh.pk[tid] = 0;
            sh.qk[tid] = 0;
        }
        for (int c = tid; c < N0b; c += kTcThreads)
            row_hi[c] = row_lo[c] = 0;
        if (tma_b) {
            // B of Ja from the prebuilt operands (k_build_bops): two boxes of kp rows x 256 halves,
            // copied by TMA while the producers gather the first A tile; the MMA thread waits for
            // them. The previous string's MMAs are complete (every tile was scattered).
            if (tid == 0) {
                const uint32_t bytes = 2u * kTcN * (uint32_t)kp * 2u;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b_full), "r"(bytes)
                             : "memory");
                const int y = (int)(Ja * 2 * kp);
                tma_load_2d(smem_u32(sh.b_hi), &bmap, 0, y, b_full);
                tma_load_2d(smem_u32(sh.b_lo), &bmap, 0, y + kp, b_full);
                b_phase = (uint32_t)(nja & 1);
                b_pending = true;
            }
            __syncthreads();
        } else {
            __syncthreads();
            // B = V'[(s, r)][k] 2^eb (zero outside the space); one 16-byte row of 8 k per task
            build_b(n, K, kp, fb, V, sh.pk, sh.qk, sh.b_hi, sh.b_lo, tid, kTcThreads);
            // make the generic-proxy shared-memory writes visible to the tensor cores
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
        }

        if (warp < kProdWarps) {
            // ---- producer: half h of row m of A (k in [40 h, 40 h + 40)) for every tile of Ja
            const int m = tid & (kTcM - 1), h = tid >> 7, kb = h * kProdHalf;
            float x[kProdHalf];
            auto request = [&](int ib0) {
                const int Ib = ib0 + m;
                const bool in = Ib < N0b;
#pragma unroll
                for (int i = 0; i < kProdHalf; ++i)
                    x[i] = (kb + i < K && in) ? __ldg(sh.rowp[kb + i] + Ib) : 0.0f;
            };
            request(0);
            for (int t = 0; t < ntile; ++t) {
                const long long g = g0 + t;
                if (sh.abort)
                    break;
                if (g > 0 && !mbar_wait(a_empty, (uint32_t)((g - 1) & 1), poll_limit, &sh.abort)) {
                    give_up();
                    break;
                }
#pragma unroll
                for (int j = 0; j < kProdHalf / 8; ++j) {
                    if (kb + 8 * j < kp) {
                        float v[8];
#pragma unroll
                        for (int c = 0; c < 8; ++c)
                            v[c] = x[8 * j + c] * sh.sfa[kb + 8 * j + c];
                        const uint32_t off = kmajor_off(m, kb + 8 * j, kp) >> 1;
                        split_store(v, sh.a_hi + off, sh.a_lo + off);
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(a_full);
                if (tid == 0) {
                    // ---- MMA issue: D[buf] = A B over kp / 16 steps of K = 16, three split products
                    const int buf = (int)(g & 1);
                    if (!mbar_wait(a_full, (uint32_t)(g & 1), poll_limit, &sh.abort) ||
                        (g >= 2 && !mbar_wait(acc_empty[buf], (uint32_t)(((g >> 1) - 1) & 1), poll_limit, &sh.abort))) {
                        give_up();
                        break;
                    }
                    if (b_pending) { // the B tiles of this alpha string have landed
                        if (!mbar_wait(b_full, b_phase, poll_limit, &sh.abort)) {
                            give_up();
                            break;
                        }
                        b_pending = false;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t ahi = smem_u32(sh.a_hi), alo = smem_u32(sh.a_lo);
                    const uint32_t bhi = smem_u32(sh.b_hi), blo = smem_u32(sh.b_lo);
                    const uint32_t acc = tmem + (uint32_t)buf * kTcN;
                    for (int kk = 0; kk < kp / 16; ++kk) {
                        const uint32_t adv = (uint32_t)kk * 2 * lbo; // 16 FP16 = two core matrices along K
                        mma_f16(acc, smem_desc(ahi + adv, lbo, sbo), smem_desc(bhi + adv, lbo, sbo), kk > 0);
                        mma_f16(acc, smem_desc(alo + adv, lbo, sbo), smem_desc(bhi + adv, lbo, sbo), 1);
                        mma_f16(acc, smem_desc(ahi + adv, lbo, sbo), smem_desc(blo + adv, lbo, sbo), 1);
                    }
                    mma_commit(a_empty);
                    mma_commit(acc_full[buf]);
                    last_g = g;
                }
                if (t + 1 < ntile)
                    request((t + 1) * kTcM);
            }
        } else {
            // ---- scatter: lanes 32 q .. +31 of the accumulator (q = warp mod 4, the quarter this warp
            // may read), every fourth s from grp on
            const int q = warp & 3, grp = (warp - kProdWarps) >> 2;
            const uint32_t nmask = (1u << n) - 1u;
            const uint32_t lane_base = (uint32_t)(q * 32) << 16;
            for (int t = 0; t < ntile; ++t) {
                const long long g = g0 + t;
                const int buf = (int)(g & 1);
                // lane 0 waits and decides for the whole warp (the warp-collective operations below
                // need every lane); __syncwarp orders the other lanes after its acquire
                int go = 0;
                if (lane == 0) {
                    go = !sh.abort;
                    if (go && !mbar_wait(acc_full[buf], (uint32_t)((g >> 1) & 1), poll_limit, &sh.abort)) {
                        give_up();
                        go = 0;
                    }
                }
                go = __shfl_sync(0xffffffffu, go, 0);
                __syncwarp();
                if (!go)
                    break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)buf * kTcN + lane_base;
                const int Ib = t * kTcM + q * 32 + lane;
                const bool valid = Ib < N0b;
                const uint64_t mI = valid ? str_b[Ib] : 0;
                // the excitation entries of the next s are requested before the current s is added
                uint4 en[4];
                auto request = [&](int s) {
                    if (valid && s < n && (mI >> s & 1)) {
                        const int si = popc64(mI & ((uint64_t(1) << s) - 1));
                        const uint4* src = reinterpret_cast<const uint4*>(exc_b + ((int64_t)Ib * nb + si) * 16);
#pragma unroll
                        for (int c = 0; c < 4; ++c)
                            en[c] = __ldg(src + c);
                    }
                };
                request(grp);
                for (int s = grp; s < n; s += kScatWarps / 4) {
                    const bool has = valid && (mI >> s & 1);
                    const uint32_t e[16] = {en[0].x, en[0].y, en[0].z, en[0].w, en[1].x, en[1].y, en[1].z, en[1].w,
                                            en[2].x, en[2].y, en[2].z, en[2].w, en[3].x, en[3].y, en[3].z, en[3].w};
                    request(s + kScatWarps / 4);
                    // r valid: r not in Ib - s (and r < n); the union over the warp decides which r
                    // slots the warp runs at all (uniform branches: the low orbitals of neighbouring
                    // strings mostly agree)
                    const uint32_t vm = has ? (~(uint32_t)(mI & ~(uint64_t(1) << s)) & nmask) : 0u;
                    const uint32_t U = __reduce_or_sync(0xffffffffu, vm);
                    if (!U)
                        continue;
                    uint32_t v[16];
                    tmem_ld16(acc + (uint32_t)(s * 16), v);
                    tmem_wait_ld();
#pragma unroll
                    for (int r = 0; r < 16; ++r) {
                        if (U >> r & 1) {
                            if (vm >> r & 1) // the sign bit of the entry flips the sign of the value
                                add_fixed(row_hi, row_lo, e[r] & 0x00FFFFFFu, v[r], e[r] >> 31);
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0)
                    mbar_arrive(acc_empty[buf]);
            }
        }
        __syncwarp();
        __syncthreads(); // every tile of Ja scattered (so every MMA of it complete), or an abort
        if (!sh.abort)
            for (int c = tid; c < N0b; c += kTcThreads) {
                const long long q = ((long long)row_hi[c] << 22) + row_lo[c]; // units of 2^-7
                const float x = __ll2float_rn(q) * unscale0 * unscale1 * unscale2;
                srow[c] += x;
            }
        g0 += ntile;
        ++nja;
        __syncthreads();
    }
    // a B copy still in flight after an abort lands before the CTA leaves (bounded wait)
    if (tid == 0 && b_pending)
        (void)mbar_wait(b_full, b_phase, (1ll << 26));
    // after an abort, MMAs may still be running: wait (bounded) for the last commit before the tensor
    // memory they write is released (a no-op when every tile was scattered)
    if (tid == 0 && last_g >= 0)
        (void)mbar_wait(acc_full[last_g & 1], (uint32_t)((last_g >> 1) & 1), (1ll << 26));
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
}

size_t opposite_tc_smem(int N0b) { return sizeof(TcShared) + (size_t)N0b * 2 * sizeof(int); }

// The prebuilt B operands of every alpha string and the tensor map the kernel's TMA copies read:
// a 2D FP16 tensor of rows of kTcN halves (512 B), 2 kp rows per alpha string (hi, then lo).
struct TcBOperands {
    CUtensorMap map{};
    DevBuf<uint16_t> buf;
    int kp = 0;
    int64_t N0a = 0;
};

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

// (Re)build the B operands for the integrals V (FP32) and their largest magnitude vmax, on st. The
// first call allocates them (N0a x 2 x kTcN x kp halves: 1.05 GB at CAS(16,16)) and encodes the
// tensor map; later calls (new integrals) refill the same buffer, so captured graphs stay valid.
void opposite_tc_build_b(const CIStrings* s, const float* V, const unsigned int* vmax,
                         std::shared_ptr<TcBOperands>& tb, cudaStream_t st) {
    const int na = s->na, ma = s->a.m1, K = na * ma, kp = (K + 15) & ~15;
    const int64_t N0a = s->a.N0;
    if (!tb) {
        PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
        if (!encode)
            throw Error(3, "tensor-core sigma: the driver offers no cuTensorMapEncodeTiled");
        auto t = std::make_shared<TcBOperands>();
        t->kp = kp;
        t->N0a = N0a;
        t->buf.reserve((size_t)N0a * 2 * kTcN * kp);
        const cuuint64_t dims[2] = {(cuuint64_t)kTcN, (cuuint64_t)N0a * 2 * kp};
        const cuuint64_t strides[1] = {(cuuint64_t)kTcN * sizeof(uint16_t)};
        const cuuint32_t box[2] = {(cuuint32_t)kTcN, (cuuint32_t)kp};
        const cuuint32_t estr[2] = {1, 1};
        const CUresult r = encode(&t->map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, t->buf.get(), dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            throw Error(3, "tensor-core sigma: cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
        tb = t;
    }
    if (tb->kp != kp || tb->N0a != N0a)
        throw Error(1, "tensor-core sigma: B operands of another space");
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(N0a, 1216));
    k_build_bops<<<grid, 256, 0, st>>>(s->norb, na, ma, N0a, s->a.down1.get(), s->a.up1.get(), V, vmax,
                                       reinterpret_cast<__half*>(tb->buf.get()));
    F2G_LAUNCH("k_build_bops");
}

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

// vmax <- the largest |V| of the n^4 FP32 integrals (as FP32 bits), ordered on st
void opposite_tc_vmax(const float* V, int64_t count, unsigned int* vmax, cudaStream_t st) {
    F2G_CUDA(cudaMemsetAsync(vmax, 0, sizeof(unsigned int), st));
    if (count == 0)
        return;
    k_absmax<<<dim3(64, 1), 256, 0, st>>>(count, V, vmax);
    F2G_LAUNCH("k_absmax V");
}

// vmax: the integrals' largest magnitude (opposite_tc_vmax); cmax: nvec words of scratch for the
// per-vector largest |C|, written here before the kernel runs.
// tb: the prebuilt B operands (TMA-fed B tiles), or nullptr (each CTA builds B itself; same sigma).
void launch_opposite_tc(const CIStrings* s, const uint32_t* exc, const float* V, const unsigned int* vmax,
                        const float* C, float* sig, unsigned int* cmax, int* err, long long poll_limit, int max_ctas,
                        cudaStream_t st, int nvec, const TcBOperands* tb) {
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
        V, vmax, cmax, C, sig, err, poll_limit > 0 ? poll_limit : (1ll << 26), tb ? tb->map : CUtensorMap{},
        tb ? 1 : 0);
    F2G_LAUNCH("k_opposite_tc");
}

} // namespace f2g
