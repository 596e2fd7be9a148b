// scan.cu -- device-wide exclusive prefix sum of uint32 counts, used by the
// grid builders (count -> offsets -> fill).  Three launches: per-block scan
// with block totals, one-block scan of the totals, offset add.
#include <algorithm>

#include "common.cuh"
#include "engine.h"

namespace dsim {

static constexpr int kScanThreads = 1024;
static constexpr int kScanItems = 4;
static constexpr int kScanTile = kScanThreads * kScanItems;

size_t scan_scratch_words(uint32_t n) { return (size_t)(n + kScanTile - 1) / kScanTile + 1; }

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot, uint32_t& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;  // inclusive warp prefix
    }
    __syncthreads();
    uint32_t warp_off = (w > 0) ? warp_tot[w - 1] : 0u;
    total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* out,
                                                             uint32_t n, uint32_t* tile_tot) {
    __shared__ uint32_t warp_tot[32];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t tot;
    uint32_t off = block_exclusive_scan(s, warp_tot, tot);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) tile_tot[blockIdx.x] = tot;
}

// one block: exclusive scan of the tile totals in place; writes the grand
// total to out[n]
__global__ void __launch_bounds__(kScanThreads) k_scan_totals(uint32_t* tile_tot, uint32_t ntiles,
                                                              uint32_t* out, uint32_t n) {
    __shared__ uint32_t warp_tot[32];
    uint32_t carry = 0;
    for (uint32_t b = 0; b < ntiles; b += kScanThreads) {
        uint32_t i = b + threadIdx.x;
        uint32_t v = (i < ntiles) ? tile_tot[i] : 0u;
        uint32_t tot;
        uint32_t off = block_exclusive_scan(v, warp_tot, tot);
        if (i < ntiles) tile_tot[i] = carry + off;
        carry += tot;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_scan_add(uint32_t* out, uint32_t n, const uint32_t* __restrict__ tile_tot) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_tot[i / kScanTile];
}

int launch_scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                          cudaStream_t st) {
    uint32_t ntiles = (uint32_t)((n + kScanTile - 1) / kScanTile);
    if (n == 0) {
        DSIM_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(uint32_t), st));
        return kOk;
    }
    k_scan_tiles<<<ntiles, kScanThreads, 0, st>>>(in, out, n, scratch);
    k_scan_totals<<<1, kScanThreads, 0, st>>>(scratch, ntiles, out, n);
    k_scan_add<<<(n + 255) / 256, 256, 0, st>>>(out, n, scratch);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

// ---- content hash of device arrays ------------------------------------------
// Sum over i of mix64(word_i ^ (i * golden) + salt), wrapping: one read of
// the array, order-sensitive through the index, deterministic.  The C-ABI
// drop-ins compare these per call to notice a caller that rewrote bound
// arrays in place, without copying them back.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) k_hash_words(const uint32_t* __restrict__ p, size_t n,
                                                    unsigned long long salt, unsigned long long* out) {
    unsigned long long acc = 0ull;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        acc += mix64(((unsigned long long)__ldg(p + i) ^ ((unsigned long long)i * 0x9E3779B97F4A7C15ull)) + salt);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

int hash_device_arrays(const void* const* ptrs, const size_t* nwords, int n, unsigned long long* dOut,
                       uint64_t* hostOut, cudaStream_t st) {
    if (n <= 0) return kOk;
    DSIM_CUDA_TRY(cudaMemsetAsync(dOut, 0, (size_t)n * 8, st));
    for (int k = 0; k < n; k++) {
        if (!ptrs[k] || nwords[k] == 0) continue;
        const size_t blocks = std::min<size_t>(608, (nwords[k] + 255) / 256);
        k_hash_words<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const uint32_t*>(ptrs[k]), nwords[k],
                                                        0x632BE59BD9B4E019ull * (unsigned long long)(k + 1), dOut + k);
    }
    DSIM_CUDA_TRY(cudaGetLastError());
    DSIM_CUDA_TRY(cudaMemcpyAsync(hostOut, dOut, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(st));
    return kOk;
}

}  // namespace dsim
