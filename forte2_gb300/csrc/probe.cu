// Issue-rate probe of the FP64 fused multiply-add pipe, the roofline denominator of the FP64
// sigma kernels (whose work is DFMA on register and shared-memory operands, not a library GEMM).
//
// Every thread runs 16 independent DFMA chains for `iters` steps, so the pipe never waits on a
// result; blocks x threads x iters x 16 DFMA = 32 blocks threads iters FLOP per launch. The chains'
// final values are summed into out[block] so that none of the work can be removed.
#include "common.cuh"

namespace f2g {

constexpr int kChains = 16;

__global__ void k_probe_dfma(long long iters, double x, double y, double* __restrict__ out) {
    // x and y in registers (opaque to the optimiser), as the sigma kernels' operands are: a DFMA
    // with a constant-bank operand is not what the pipe runs there
    asm volatile("" : "+d"(x), "+d"(y));
    double a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        a[c] = threadIdx.x * 1e-3 + c;
    for (long long i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            a[c] = fma(a[c], x, y);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += a[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(out + blockIdx.x, s);
}

void probe_dfma(int blocks, int threads, long long iters, double* out, cudaStream_t st) {
    if (blocks <= 0 || threads <= 0 || threads > 1024 || (threads & 31) || iters <= 0)
        throw Error(2, "probe_dfma: blocks > 0, threads a multiple of 32 up to 1024, iters > 0");
    F2G_CUDA(cudaMemsetAsync(out, 0, (size_t)blocks * sizeof(double), st));
    // x slightly below 1 keeps the chains bounded: a -> a x + y converges to y / (1 - x)
    k_probe_dfma<<<blocks, threads, 0, st>>>(iters, 0.999999, 1e-6, out);
    F2G_LAUNCH("k_probe_dfma");
}

} // namespace f2g
