// Checks the integer-pipe FP64 <-> FP32 conversions of the mixed path
// (narrow_f, widen_f in xmd_gb300/csrc/device.cuh) against the hardware
// conversions over random bit patterns and edge values; prints the number of
// mismatches and exits non-zero on any.  Built and run by tests/test_convert.py.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../xmd_gb300/csrc/device.cuh"

using namespace xmdg;

__global__ void k_check(unsigned long long seed, int n, unsigned long long *bad) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long s = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
    s ^= s >> 31; s *= 0xBF58476D1CE4E5B9ull; s ^= s >> 29;
    // doubles spread over the FP32 normal range (and a little beyond)
    const int e = 1023 - 130 + (int)(s % 262);
    const unsigned long long bits = (s & 0x800fffffffffffffull) | ((unsigned long long)e << 52);
    const double x = __longlong_as_double((long long)bits);
    const float hw = (float)x, sw = narrow_f(x);
    const bool normal = fabs(x) >= 1.1754943508222875e-38;   // at or above the smallest FP32 normal
    if (normal && __float_as_uint(hw) != __float_as_uint(sw) && !(hw == 0.0f && sw == 0.0f)) atomicAdd(&bad[0], 1ull);
    // widening of every normal float pattern reachable from s
    const unsigned u = (unsigned)(s >> 7);
    const float f = __uint_as_float(u);
    const unsigned ex = (u >> 23) & 0xff;
    if (ex != 0 && ex != 0xff) {
        const double a = (double)f, b = widen_f(f);
        if (__double_as_longlong(a) != __double_as_longlong(b)) atomicAdd(&bad[1], 1ull);
    }
}

int main() {
    unsigned long long *bad;
    if (cudaMalloc(&bad, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    cudaMemset(bad, 0, 2 * sizeof(unsigned long long));
    const int n = 1 << 24;
    for (int r = 0; r < 4; ++r) k_check<<<(n + 255) / 256, 256>>>(1234567ull * (r + 1), n, bad);
    unsigned long long h[2] = {0, 0};
    cudaMemcpy(h, bad, sizeof h, cudaMemcpyDeviceToHost);
    cudaError_t err = cudaGetLastError();
    printf("narrow mismatches %llu widen mismatches %llu status %s\n", h[0], h[1], cudaGetErrorString(err));
    return (h[0] || h[1] || err != cudaSuccess) ? 1 : 0;
}
