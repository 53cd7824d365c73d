// probe.cu - FP64 pipe throughput of the current device (roofline denominator).
//
// The engine's mixed and FP64 paths are bound by the FP64 pipe rather than by
// HBM on GB300, whose FP64 rate is a small fraction of its FP32 rate.  This
// kernel measures that rate directly: every thread runs eight independent
// chains of fused multiply-adds for a fixed count, the launch covers every SM
// many times over, and the result is 2 * FMAs / elapsed seconds.
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "../../include/xmd_gpu.h"

namespace xmdg {

constexpr int PROBE_CHAINS = 8;
constexpr int PROBE_ITERS = 2048;
constexpr int PROBE_THREADS = 256;

__global__ void __launch_bounds__(PROBE_THREADS) k_fp64_probe(double *sink, double seed) {
    double a[PROBE_CHAINS];
    const double m = 1.0 - 1e-12, c = 1e-13 * (threadIdx.x + 1);
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) a[k] = seed + k;
    for (int it = 0; it < PROBE_ITERS; ++it) {
#pragma unroll
        for (int k = 0; k < PROBE_CHAINS; ++k) a[k] = fma(a[k], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) s += a[k];
    if (s == 12345.678) sink[blockIdx.x] = s;   // never true; keeps the chains live
}

static void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e) + " at " + what);
}

double fp64_peak(int device) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    int sms = 0;
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attr");
    const int blocks = sms * 16;
    double *sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ck(cudaMalloc(&sink, sizeof(double) * blocks), "cudaMalloc");
    ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        ck(cudaEventRecord(e0, st), "record");
        k_fp64_probe<<<blocks, PROBE_THREADS, 0, st>>>(sink, 1.0 + rep);
        ck(cudaEventRecord(e1, st), "record");
        ck(cudaEventSynchronize(e1), "sync");
        float ms = 0.f;
        ck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
        if (rep > 0 && ms < best) best = ms;   // the first launch is warm-up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(sink);
    const double fmas = (double)blocks * PROBE_THREADS * PROBE_ITERS * PROBE_CHAINS;
    return 2.0 * fmas / (best * 1e-3) / 1e12;
}

}  // namespace xmdg
