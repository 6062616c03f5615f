// fp64_rate.cu -- FP64 instruction-rate probe for the compute roof of the
// FP64 step kernels (measurement only; not part of the C-ABI of the solver).
//
// Every thread runs 8 independent dependency chains of one FP64 operation
// (fused multiply-add, add or multiply) for `iters` iterations; the grid is
// 8 blocks of 256 threads per SM, enough warps to cover the pipe's latency.
// The rate is (threads x iters x 8) instructions over the kernel's time,
// measured with CUDA events on the default stream (best of 3 launches after
// one warm-up launch).  Operands stay near 1, so no subnormal or overflow
// path is timed.
#include <cuda_runtime.h>

namespace {

constexpr int kThreads = 256;
constexpr int kChains = 8;

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_fp64_rate(double* out, int iters, double a, double b,
                                                        double one, double mzero) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = 1.0 + 1e-6 * (double)(t + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) {
            if (MODE == 0) x[k] = fma(x[k], a, b);
            else if (MODE == 1) x[k] = x[k] + b;
            else if (MODE == 2) x[k] = x[k] * a;
            else if (MODE == 3) x[k] = fma(x[k], one, b);  // an add issued as a fused multiply-add
            else x[k] = fma(x[k], a, mzero);                // a multiply issued as one
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++) s += x[k];
    out[t] = s;
}

template <int MODE>
cudaError_t launch(int blocks, double* out, int iters, double a, double b) {
    // one and -0 arrive as kernel arguments, so the compiler cannot fold them
    k_fp64_rate<MODE><<<blocks, kThreads>>>(out, iters, a, b, 1.0, -0.0);
    return cudaGetLastError();
}

}  // namespace

// mode 0: DFMA, 1: DADD, 2: DMUL, 3: add as DFMA (x * 1 + b), 4: multiply as
// DFMA (x * a + -0).  Writes FP64 instructions per second and the best kernel
// time.  Returns 0 or a CUDA error code.
extern "C" int mglc_roof_fp64(int mode, int iters, double* inst_per_s, double* best_ms) {
    if (mode < 0 || mode > 4 || iters < 1 || !inst_per_s) return (int)cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    const int blocks = sms * 8;
    double* out = nullptr;
    if ((e = cudaMalloc(&out, sizeof(double) * (size_t)blocks * kThreads)) != cudaSuccess) return (int)e;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // a = 1 - 2^-30, b = 2^-40: every chain stays within (0.99, 2) for any iters <= 2^24
    const double a = 1.0 - 0x1p-30, b = 0x1p-40;
    float best = 1e30f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(e0);
        e = mode == 0 ? launch<0>(blocks, out, iters, a, b)
          : mode == 1 ? launch<1>(blocks, out, iters, a, b)
          : mode == 2 ? launch<2>(blocks, out, iters, a, b)
          : mode == 3 ? launch<3>(blocks, out, iters, a, b)
                      : launch<4>(blocks, out, iters, a, b);
        cudaEventRecord(e1);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return (int)e;
    *inst_per_s = (double)blocks * kThreads * (double)iters * kChains / (best * 1e-3);
    if (best_ms) *best_ms = best;
    return 0;
}
