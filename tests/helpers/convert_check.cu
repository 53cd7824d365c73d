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

// Checks the float-float toolkit of the mixed path: split_d (h + l within
// 2^-46 |x|), ff_diff of split coordinates, ff_mul / ff_add and float-float
// accumulation against FP64 references.
__device__ unsigned long long mix(unsigned long long s) {
    s ^= s >> 31; s *= 0xBF58476D1CE4E5B9ull; s ^= s >> 29; s *= 0x94D049BB133111EBull; s ^= s >> 32;
    return s;
}
__device__ double rnd(unsigned long long s, int emin, int span) {   // random sign/mantissa, exponent in [emin, emin+span)
    const int e = 1023 + emin + (int)(s % (unsigned long long)span);
    const unsigned long long bits = (mix(s) & 0x800fffffffffffffull) | ((unsigned long long)e << 52);
    return __longlong_as_double((long long)bits);
}
__global__ void k_ff(unsigned long long seed, int n, unsigned long long *bad) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long s = mix(seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1));
    // split of coordinates of magnitude 2^-20 .. 2^20 (and exact zeros)
    const double x = (s & 1023u) == 0 ? 0.0 : rnd(s, -20, 40);
    const F2 q = split_d(x);
    const double back = (double)q.h + (double)q.l;
    if (fabs(x - back) > ldexp(fabs(x), -46) || fabs((double)q.h) > fabs(x)) atomicAdd(&bad[0], 1ull);
    // difference of two nearby coordinates
    const double u = rnd(mix(s + 1), -4, 10), w = u + rnd(mix(s + 2), -6, 8);
    const FF dd = ff_diff(split_d(u), split_d(w));
    const double ex = w - u;   // exact or within 1 ulp of |u|
    if (fabs(((double)dd.h + (double)dd.l) - ex) > ldexp(fmax(fabs(u), fabs(w)), -44)) atomicAdd(&bad[1], 1ull);
    // products and sums of float-float values
    const FF a = fast_two_sum((float)rnd(mix(s + 3), -8, 16), (float)rnd(mix(s + 4), -40, 8));
    const FF b = fast_two_sum((float)rnd(mix(s + 5), -8, 16), (float)rnd(mix(s + 6), -40, 8));
    const double ad = (double)a.h + (double)a.l, bd = (double)b.h + (double)b.l;
    const FF m = ff_mul(a, b), sm = ff_add(a, b);
    if (fabs(((double)m.h + (double)m.l) - ad * bd) > ldexp(fabs(ad * bd), -44)) atomicAdd(&bad[2], 1ull);
    if (fabs(((double)sm.h + (double)sm.l) - (ad + bd)) > ldexp(fabs(ad) + fabs(bd), -44)) atomicAdd(&bad[2], 1ull);
    // accumulation of 64 FP32 terms of mixed signs and magnitudes
    FF acc{0.0f, 0.0f};
    double ref = 0.0, mag = 0.0;
    for (int k = 0; k < 64; ++k) {
        const float v = (float)rnd(mix(s + 100 + k), -10, 20);
        ff_acc(acc, v);
        ref += (double)v;
        mag += fabs((double)v);
    }
    if (fabs(ff_to_d(acc) - ref) > ldexp(mag, -44)) atomicAdd(&bad[3], 1ull);
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
    unsigned long long *bf;
    if (cudaMalloc(&bf, 4 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    cudaMemset(bf, 0, 4 * sizeof(unsigned long long));
    const int m = 1 << 22;
    for (int r = 0; r < 2; ++r) k_ff<<<(m + 255) / 256, 256>>>(7654321ull * (r + 1), m, bf);
    unsigned long long g[4] = {0, 0, 0, 0};
    cudaMemcpy(g, bf, sizeof g, cudaMemcpyDeviceToHost);
    cudaError_t err2 = cudaGetLastError();
    printf("split mismatches %llu diff mismatches %llu ffop mismatches %llu acc mismatches %llu status %s\n", g[0], g[1],
           g[2], g[3], cudaGetErrorString(err2));
    return (h[0] || h[1] || g[0] || g[1] || g[2] || g[3] || err != cudaSuccess || err2 != cudaSuccess) ? 1 : 0;
}
