// Issue-rate probe of the FP64 fused multiply-add pipe, the roofline denominator of the FP64
// sigma kernels (whose work is DFMA on register and shared-memory operands, not a library GEMM).
//
// Every thread runs 8 independent DFMA chains for `iters` steps, so the pipe never waits on a
// result; blocks x threads x iters x 8 DFMA = 16 blocks threads iters FLOP per launch. The chains'
// final values are summed into out[block] so that none of the work can be removed.
#include "common.cuh"

namespace f2g {

__global__ void k_probe_dfma(long long iters, double x, double y, double* __restrict__ out) {
    double a0 = threadIdx.x * 1e-3, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0;
    double a4 = a0 + 4.0, a5 = a0 + 5.0, a6 = a0 + 6.0, a7 = a0 + 7.0;
    for (long long i = 0; i < iters; ++i) {
        a0 = fma(a0, x, y);
        a1 = fma(a1, x, y);
        a2 = fma(a2, x, y);
        a3 = fma(a3, x, y);
        a4 = fma(a4, x, y);
        a5 = fma(a5, x, y);
        a6 = fma(a6, x, y);
        a7 = fma(a7, x, y);
    }
    double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
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
