// noalloc.cu - a Verlet pair search that allocates no device memory.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// need a pair list: code that runs while a CUDA graph is being captured on its
// stream (an allocation there is not captured and may break the capture),
// hosts whose device memory is owned by a fixed pool or by a framework's
// caching allocator, and tight loops that cannot afford the implicit device
// synchronisation of cudaMalloc / cudaFree.  For them,
// xmd_gpu_verlet_pairs_noalloc() takes device buffers for all inputs and
// outputs and keeps the scratch of its cell list (bucket counts, starts and
// fills, bucket-sorted bead indices, per-bead row counts and offsets) in the
// file-scope array below: about 1.75 MiB that every GPU which loads the
// library holds until the process exits.
//
// The search itself is the one the engine runs at every Verlet rebuild:
// pairs i < j, not in the same chain with |seq_i - seq_j| < 3
// (legacy_update.cpp:24-26), whose minimum-image distance is below the
// cutoff (legacy_update.cpp:28-29), in (i, j) order.  Cells of the cutoff's
// edge are hashed into n buckets, which bounds the scratch by the bead count.
// One thread builds one bead's row and keeps it sorted by insertion, so a row
// of m partners costs O(m^2): cheap at Verlet-list densities (tens to a few
// hundred partners), slow when most beads are within the cutoff of most
// others (a periodic box under two cutoffs wide, a cluster much denser than
// a protein).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/xmd_gpu.h"
#include "engine.h"

namespace xmdg {
namespace {

constexpr int NA_MAX = XMD_NOALLOC_MAX_BEADS;   // beads, and buckets
constexpr int NA_BLOCK = 1024;

struct NaScratch {
    int bucket_cnt[NA_MAX];
    int bucket_start[NA_MAX];
    int bucket_fill[NA_MAX];
    int items[NA_MAX];
    int bead_bucket[NA_MAX];
    int row_cnt[NA_MAX];
    int row_off[NA_MAX];
    // grid of the current call
    int per[3], dims[3], nbuckets;
    double lo[3], inv_edge, cell[3], cell_inv[3];
};

// The scratch.  Every call reuses it and leaves its contents behind; each
// call clears what has to start at zero.  Calls that overlap on the GPU (two
// streams, or a second call before the first finishes on another stream)
// race on it.
static __device__ __align__(256) NaScratch g_na_scratch;

__device__ __forceinline__ int na_coord(const NaScratch &s, int a, double x) {
    if (s.per[a]) {
        double f = x * s.cell_inv[a];
        f -= floor(f);
        int k = (int)(f * s.dims[a]);
        return k < 0 ? 0 : (k >= s.dims[a] ? s.dims[a] - 1 : k);
    }
    int k = (int)floor((x - s.lo[a]) * s.inv_edge);
    return k < 0 ? 0 : k;
}
__device__ __forceinline__ int na_key(const NaScratch &s, int cx, int cy, int cz) {
    uint32_t h = (uint32_t)cx * 73856093u ^ (uint32_t)cy * 19349663u ^ (uint32_t)cz * 83492791u;
    return (int)(h % (uint32_t)s.nbuckets);
}
__device__ __forceinline__ double na_dist(const NaScratch &s, const double *r, int i, int j) {
    double d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double x = __dsub_rn(r[3 * j + a], r[3 * i + a]);
        d[a] = __dsub_rn(x, __dmul_rn(s.cell[a], rint(__dmul_rn(x, s.cell_inv[a]))));
    }
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2])));
}

// grid, bucket counts, scan, fill and in-bucket order: one block
__global__ void __launch_bounds__(NA_BLOCK) k_na_grid(NaScratch *s, const double *__restrict__ r, int n,
                                                      double c0, double c1, double c2, double cutoff) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    __shared__ double red[6][32];
    __shared__ int scan_s[NA_BLOCK];
    const double cellv[3] = {c0, c1, c2};
    double lo[3] = {1e300, 1e300, 1e300};
    for (int i = t; i < n; i += NA_BLOCK)
        for (int a = 0; a < 3; ++a) lo[a] = fmin(lo[a], r[3 * i + a]);
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o; o >>= 1) lo[a] = fmin(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
        if (lane == 0) red[a][w] = lo[a];
    }
    __syncthreads();
    if (t == 0) {
        const double edge = cutoff * (1.0 + 1e-9);
        for (int a = 0; a < 3; ++a) {
            double l = 1e300;
            for (int q = 0; q < NA_BLOCK / 32; ++q) l = fmin(l, red[a][q]);
            s->cell[a] = cellv[a];
            s->cell_inv[a] = cellv[a] != 0.0 ? 1.0 / cellv[a] : 0.0;
            s->per[a] = cellv[a] != 0.0;
            int dm = s->per[a] ? (int)floor(cellv[a] / edge) : 0;
            s->dims[a] = dm < 1 ? 1 : dm;
            s->lo[a] = l;
        }
        s->inv_edge = 1.0 / edge;
        s->nbuckets = n > 0 ? n : 1;
    }
    __syncthreads();
    const int nb = s->nbuckets;
    for (int c = t; c < nb; c += NA_BLOCK) {
        s->bucket_cnt[c] = 0;
        s->bucket_fill[c] = 0;
    }
    __syncthreads();
    for (int i = t; i < n; i += NA_BLOCK) {
        int k = na_key(*s, na_coord(*s, 0, r[3 * i]), na_coord(*s, 1, r[3 * i + 1]), na_coord(*s, 2, r[3 * i + 2]));
        s->bead_bucket[i] = k;
        atomicAdd(&s->bucket_cnt[k], 1);
    }
    __syncthreads();
    const int chunk = (nb + NA_BLOCK - 1) / NA_BLOCK;
    const int b0 = t * chunk, b1 = min(nb, b0 + chunk);
    int sum = 0;
    for (int c = b0; c < b1; ++c) sum += s->bucket_cnt[c];
    scan_s[t] = sum;
    __syncthreads();
    for (int o = 1; o < NA_BLOCK; o <<= 1) {
        int v = t >= o ? scan_s[t - o] : 0;
        __syncthreads();
        scan_s[t] += v;
        __syncthreads();
    }
    int run = scan_s[t] - sum;
    for (int c = b0; c < b1; ++c) {
        s->bucket_start[c] = run;
        run += s->bucket_cnt[c];
    }
    __syncthreads();
    // the order inside a bucket is free: each row is ordered by j below
    for (int i = t; i < n; i += NA_BLOCK) {
        int k = s->bead_bucket[i];
        s->items[s->bucket_start[k] + atomicAdd(&s->bucket_fill[k], 1)] = i;
    }
}

// partners j > i of bead i; pass 0 counts, pass 1 writes then orders by j
__global__ void __launch_bounds__(128) k_na_rows(NaScratch *s, const double *__restrict__ r,
                                                 const int32_t *__restrict__ chain, const int32_t *__restrict__ seq,
                                                 int n, double cutoff, int pass, int32_t *pairs, int cap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int cc[3];
    for (int a = 0; a < 3; ++a) cc[a] = na_coord(*s, a, r[3 * i + a]);
    int keys[27], nk = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int c[3] = {cc[0] + dx, cc[1] + dy, cc[2] + dz};
                bool skip = false;
                for (int a = 0; a < 3; ++a) {
                    if (s->per[a]) c[a] = ((c[a] % s->dims[a]) + s->dims[a]) % s->dims[a];
                    else if (c[a] < 0) skip = true;
                }
                if (skip) continue;
                int key = na_key(*s, c[0], c[1], c[2]);
                bool dup = false;
                for (int q = 0; q < nk; ++q) dup |= keys[q] == key;
                if (!dup) keys[nk++] = key;
            }
    const int ci = chain[i], si = seq[i];
    int cnt = 0;
    // pass 1: the row's m smallest partners (m = what fits below cap: all of
    // them, except in the row that straddles cap), kept sorted by j with
    // insertion as they are found, so the output is always the (i, j)-ordered
    // prefix of the full list
    const int base = pass ? s->row_off[i] : 0;
    const int m = pass ? min(s->row_cnt[i], max(0, cap - base)) : 0;
    int32_t *row = pairs + 2 * (size_t)base;
    int kept = 0;
    for (int kk = 0; kk < nk; ++kk) {
        const int q0 = s->bucket_start[keys[kk]], q1 = q0 + s->bucket_cnt[keys[kk]];
        for (int q = q0; q < q1; ++q) {
            int j = s->items[q];
            if (j <= i) continue;
            int sj = seq[j];
            int df = si > sj ? si - sj : sj - si;
            if (chain[j] == ci && df < 3) continue;
            if (!(na_dist(*s, r, i, j) < cutoff)) continue;
            ++cnt;
            if (m == 0 || (kept == m && j >= row[2 * (m - 1) + 1])) continue;
            int y = kept < m ? kept : m - 1;   // the slot that opens (the largest drops out when full)
            while (y > 0 && row[2 * (y - 1) + 1] > j) {
                row[2 * y + 1] = row[2 * (y - 1) + 1];
                --y;
            }
            row[2 * y + 1] = j;
            if (kept < m) ++kept;
        }
    }
    if (!pass) {
        s->row_cnt[i] = cnt;
        return;
    }
    for (int x = 0; x < m; ++x) row[2 * x] = i;
}

// exclusive scan of the row counts; total to the caller's counter
__global__ void __launch_bounds__(NA_BLOCK) k_na_scan(NaScratch *s, int n, int32_t *count) {
    const int t = threadIdx.x;
    __shared__ int scan_s[NA_BLOCK];
    const int chunk = (n + NA_BLOCK - 1) / NA_BLOCK;
    const int i0 = t * chunk, i1 = min(n, i0 + chunk);
    int sum = 0;
    for (int i = i0; i < i1; ++i) sum += s->row_cnt[i];
    scan_s[t] = sum;
    __syncthreads();
    for (int o = 1; o < NA_BLOCK; o <<= 1) {
        int v = t >= o ? scan_s[t - o] : 0;
        __syncthreads();
        scan_s[t] += v;
        __syncthreads();
    }
    int run = scan_s[t] - sum;
    for (int i = i0; i < i1; ++i) {
        s->row_off[i] = run;
        run += s->row_cnt[i];
    }
    if (t == NA_BLOCK - 1) *count = scan_s[t];
}

// Device address of the scratch, looked up once per device with that device
// current (in host code the symbol names a host-side stand-in, not device
// memory).
void *scratch_address() {
    static std::mutex mu;
    static void *addr[128] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 128) throw std::runtime_error("CUDA device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess)
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e) +
                                     " at cudaGetSymbolAddress(scratch)");
        addr[dev] = p;
    }
    return addr[dev];
}

}  // namespace

int verlet_pairs_noalloc(const double *d_r, const int32_t *d_chain, const int32_t *d_seq, int32_t n,
                         const double cell[3], double cutoff, int32_t *d_pairs, int32_t cap, int32_t *d_count,
                         void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    auto *s = (NaScratch *)scratch_address();
    if (n == 0) {
        cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(int32_t), st);
        if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e));
        return XMD_OK;
    }
    k_na_grid<<<1, NA_BLOCK, 0, st>>>(s, d_r, n, cell[0], cell[1], cell[2], cutoff);
    const int nb = (n + 127) / 128;
    k_na_rows<<<nb, 128, 0, st>>>(s, d_r, d_chain, d_seq, n, cutoff, 0, d_pairs, cap);
    k_na_scan<<<1, NA_BLOCK, 0, st>>>(s, n, d_count);
    k_na_rows<<<nb, 128, 0, st>>>(s, d_r, d_chain, d_seq, n, cutoff, 1, d_pairs, cap);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e));
    return XMD_OK;
}

}  // namespace xmdg
