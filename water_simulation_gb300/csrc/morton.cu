// Morton-order variant of the neighbour sort (the reference's SpatialAccel,
// core/src/spatial_accel.cu:11-40,158-179): 30-bit Morton codes of positions
// normalised to the scene box, stably sorted. The sort is a least-significant-
// digit radix sort of four 8-bit passes; each pass histograms 1024-element
// tiles, scans the digit-major histogram and scatters with a rank that is
// stable inside the tile (warp match + per-warp digit counts), so equal codes
// keep ascending particle indices exactly as a stable sort of iota values.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/dfsph_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace dfsph {
namespace {

constexpr int RS_BLOCK = 256;
constexpr int RS_ROUNDS = 4;
constexpr int RS_TILE = RS_BLOCK * RS_ROUNDS;
constexpr int RS_BINS = 256;
constexpr int RS_WARPS = RS_BLOCK / 32;

// Spread the low 10 bits of v so that bit k lands on bit 3k.
__device__ __forceinline__ u32 spread10(u32 v) {
    v &= 0x3ffu;
    u32 out = 0;
#pragma unroll
    for (int k = 0; k < 10; ++k) out |= ((v >> k) & 1u) << (3 * k);
    return out;
}

// Quantise a normalised coordinate to [0, 1023] (spatial_accel.cu:21-23):
// clamp x * 1024 into [0, 1023], truncate.
__device__ __forceinline__ u32 quant10(float x) {
    const float q = fminf(fmaxf(x * 1024.0f, 0.0f), 1023.0f);
    return static_cast<u32>(q);
}

__global__ void __launch_bounds__(256) morton_code_kernel(int n, const float* __restrict__ xyz, float mx, float my,
                                                          float mz, float ix, float iy, float iz,
                                                          u32* __restrict__ codes, u32* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const u32 qx = quant10((xyz[3 * i] - mx) * ix);
    const u32 qy = quant10((xyz[3 * i + 1] - my) * iy);
    const u32 qz = quant10((xyz[3 * i + 2] - mz) * iz);
    codes[i] = (spread10(qx) << 2) | (spread10(qy) << 1) | spread10(qz);
    idx[i] = static_cast<u32>(i);
}

__global__ void __launch_bounds__(RS_BLOCK) radix_hist_kernel(const u32* __restrict__ keys, int n, int shift,
                                                              u32* __restrict__ hist, int n_tiles) {
    __shared__ u32 h[RS_BINS];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
#pragma unroll
    for (int k = 0; k < RS_ROUNDS; ++k) {
        const int e = base + k * RS_BLOCK + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    hist[size_t(threadIdx.x) * n_tiles + blockIdx.x] = h[threadIdx.x];  // digit-major
}

__global__ void __launch_bounds__(RS_BLOCK) radix_scatter_kernel(const u32* __restrict__ keys_in,
                                                                 const u32* __restrict__ vals_in, int n, int shift,
                                                                 const u32* __restrict__ offs, int n_tiles,
                                                                 u32* __restrict__ keys_out,
                                                                 u32* __restrict__ vals_out) {
    __shared__ u32 run[RS_BINS];
    __shared__ u32 wcnt[RS_WARPS][RS_BINS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    run[threadIdx.x] = offs[size_t(threadIdx.x) * n_tiles + blockIdx.x];
    const u32 lt_mask = (1u << lane) - 1u;
    const int base = blockIdx.x * RS_TILE;
    for (int k = 0; k < RS_ROUNDS; ++k) {
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) wcnt[w][threadIdx.x] = 0u;
        __syncthreads();
        const int e = base + k * RS_BLOCK + threadIdx.x;
        const bool valid = e < n;
        const u32 key = valid ? keys_in[e] : 0u;
        const u32 d = valid ? ((key >> shift) & 0xffu) : 0x100u;  // invalid lanes: their own group
        const u32 peers = __match_any_sync(0xffffffffu, d);
        const u32 rank_w = __popc(peers & lt_mask);
        if (valid && rank_w == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            u32 before = 0;
            for (int w = 0; w < warp; ++w) before += wcnt[w][d];
            const u32 dst = run[d] + before + rank_w;
            keys_out[dst] = key;
            vals_out[dst] = vals_in[e];
        }
        __syncthreads();
        u32 tot = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) tot += wcnt[w][threadIdx.x];
        run[threadIdx.x] += tot;
        __syncthreads();
    }
}

}  // namespace

void morton_sort(const float* xyz, u32 n, const float smin[3], const float smax[3], u32* sorted_codes,
                 u32* sorted_idx, cudaStream_t st) {
    if (n == 0) return;
    // extent reciprocals on the host, 0 for a flat axis (spatial_accel.cu:134-143)
    float inv[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = smax[a] - smin[a];
        inv[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    const int n_tiles = int((n + RS_TILE - 1) / RS_TILE);
    const size_t m = size_t(RS_BINS) * n_tiles;
    const u32 scan_tiles_n = u32((m + SCAN_TILE - 1) / SCAN_TILE);
    const size_t words = 4 * size_t(n) + m /*hist*/ + (m + 1) /*offsets*/ + scan_tiles_n + 1;
    u32* mem = nullptr;
    DFSPH_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&mem), words * sizeof(u32), st));
    u32* ka = mem;
    u32* va = ka + n;
    u32* kb = va + n;
    u32* vb = kb + n;
    u32* hist = vb + n;
    u32* offs = hist + m;
    u32* tsum = offs + m + 1;
    const int nb = int((n + 255) / 256);
    morton_code_kernel<<<nb, 256, 0, st>>>(int(n), xyz, smin[0], smin[1], smin[2], inv[0], inv[1], inv[2], ka, va);
    DFSPH_LAUNCHED();
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 8 * pass;
        radix_hist_kernel<<<n_tiles, RS_BLOCK, 0, st>>>(ka, int(n), shift, hist, n_tiles);
        DFSPH_LAUNCHED();
        // exclusive scan of the digit-major histogram (it is cleared on the way)
        scan_tile_sums<<<scan_tiles_n, SCAN_BLOCK, 0, st>>>(hist, u32(m), tsum);
        DFSPH_LAUNCHED();
        scan_tile_offsets<<<1, 1024, 0, st>>>(tsum, scan_tiles_n, offs + m, nullptr, 0, nullptr, 0);
        DFSPH_LAUNCHED();
        scan_tiles<<<scan_tiles_n, SCAN_BLOCK, 0, st>>>(hist, u32(m), tsum, offs);
        DFSPH_LAUNCHED();
        radix_scatter_kernel<<<n_tiles, RS_BLOCK, 0, st>>>(ka, va, int(n), shift, offs, n_tiles, kb, vb);
        DFSPH_LAUNCHED();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (sorted_codes) DFSPH_CUDA(cudaMemcpyAsync(sorted_codes, ka, size_t(n) * sizeof(u32), cudaMemcpyDeviceToDevice, st));
    if (sorted_idx) DFSPH_CUDA(cudaMemcpyAsync(sorted_idx, va, size_t(n) * sizeof(u32), cudaMemcpyDeviceToDevice, st));
    DFSPH_CUDA(cudaFreeAsync(mem, st));
}

}  // namespace dfsph
