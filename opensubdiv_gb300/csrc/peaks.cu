// Measured FP32 fused multiply-add rate of the current device: the compute denominator of the
// EvalPatches roofline (a patch point costs hundreds of FP32 operations against a few hundred
// bytes, so both the memory and the FP32 terms are reported).  No counterpart in the reference.
#include "common.cuh"

namespace gb300 {

constexpr int kFmaThreads = 256;
constexpr int kFmaChains = 8;    // independent accumulators per thread (hide the FMA latency)
constexpr int kFmaUnroll = 64;   // FMAs per chain per loop iteration

// Every thread runs kFmaChains independent chains x = x * a + b; the sum is stored only when
// it equals an impossible value, which keeps the chains live without memory traffic.
__global__ void __launch_bounds__(kFmaThreads) k_fma_rate(float *sink, int iters, float a,
                                                           float b) {
    float x[kFmaChains];
#pragma unroll
    for (int c = 0; c < kFmaChains; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < kFmaUnroll; ++u)
#pragma unroll
            for (int c = 0; c < kFmaChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kFmaChains; ++c) s += x[c];
    if (s == -1.0f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace gb300

extern "C" int GB300MeasureFp32Rate(double *tflops, void *stream) {
    using namespace gb300;
    static const char *who = "GB300MeasureFp32Rate";
    if (!tflops) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null output", who);
    cudaStream_t s = as_stream(stream);
    const int blocks = num_sms() * (2048 / kFmaThreads);  // full occupancy, one wave
    const int iters = 512;
    cudaEvent_t e0, e1;
    int st = check_cuda(cudaEventCreate(&e0), who);
    if (st != GB300_OK) return st;
    if ((st = check_cuda(cudaEventCreate(&e1), who)) != GB300_OK) {
        cudaEventDestroy(e0);
        return st;
    }
    // a = 1 - 2^-20, b = 2^-20: the chains stay in [0, 1) without denormals
    const float a = 1.0f - 9.5367431640625e-7f, b = 9.5367431640625e-7f;
    k_fma_rate<<<blocks, kFmaThreads, 0, s>>>(nullptr, iters, a, b);  // warm-up
    count_launch();
    const int reps = 5;
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps; ++r) {
        k_fma_rate<<<blocks, kFmaThreads, 0, s>>>(nullptr, iters, a, b);
        count_launch();
    }
    cudaEventRecord(e1, s);
    st = check_launch(who);
    float ms = 0.0f;
    if (st == GB300_OK) st = check_cuda(cudaEventSynchronize(e1), who);
    if (st == GB300_OK) st = check_cuda(cudaEventElapsedTime(&ms, e0, e1), who);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != GB300_OK) return st;
    const double fmas = (double)reps * blocks * kFmaThreads * iters * kFmaUnroll * kFmaChains;
    *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
    return ok();
}
