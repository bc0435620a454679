// Benchmark-side probe (not part of libpbd_gb300): FP32 FMA throughput of
// the current device, the denominator of the FP32 fraction bench.py reports
// beside the HBM one (the neighbour passes are instruction-bound, so the
// HBM fraction alone does not place them).  Built into its own library,
// libpbd_fp32_probe.so, which only bench.py loads.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 512;

// kChains independent FMA chains per thread, iters deep: 2 * kChains *
// iters flops per thread.  The result is stored only under a condition the
// inputs never meet, so nothing is eliminated.
__global__ void __launch_bounds__(kThreads) k_fma_peak(float *out, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (float)(threadIdx.x + c) * 1.0e-6f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == -12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

// GFLOP/s of a kernel of independent fused multiply-adds on every SM
// (best of three timed launches after a warm-up).  Returns 0 on success,
// else the CUDA error code.  Synchronous.
extern "C" int fp32_peak_gflops(double *gflops, void *stream) {
    if (!gflops) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    float *out = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 4;  // 2048 threads per SM
    const int iters = 1 << 14;
    if (e == cudaSuccess) e = cudaMalloc((void **)&out, (size_t)blocks * kThreads * sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    float best = 0.f;
    for (int rep = 0; e == cudaSuccess && rep < 4; ++rep) {  // the first is a warm-up
        cudaEventRecord(a, st);
        k_fma_peak<<<blocks, kThreads, 0, st>>>(out, iters, 0.9999999f, 1.0e-7f);
        cudaEventRecord(b, st);
        e = cudaEventSynchronize(b);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (out) cudaFree(out);
    if (e != cudaSuccess) return (int)e;
    if (best <= 0.f) return (int)cudaErrorUnknown;
    const double flops = 2.0 * kChains * (double)iters * blocks * kThreads;
    *gflops = flops / (best * 1e-3) / 1e9;
    return 0;
}
