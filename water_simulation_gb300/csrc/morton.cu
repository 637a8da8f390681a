// Morton-order variant of the neighbour sort (the reference's SpatialAccel,
// core/src/spatial_accel.cu:11-40,158-179): 30-bit Morton codes of positions
// normalised to the scene box, stably sorted.
//
// The sort is a least-significant-digit radix sort of three 10-bit passes over
// tiles of 4096 keys, in seven launches:
//   codes   Morton codes + iota indices, the first pass's per-tile digit
//           counts (digit-major) and its digit totals;
//   offsets one warp per digit: digit base from the totals, prefix of the
//           digit's counts over the tiles -> each tile's scatter offsets;
//   scatter a rank that is stable inside the tile (each warp ranks its own
//           slice, then one block-wide pass over the per-warp digit counts)
//           places the tile's keys in shared memory in digit order;
//           each digit's run then leaves as consecutive stores, and the next
//           pass's per-tile counts and totals are gathered on the way (the
//           tile of a key in the next pass is its destination slot / 4096).
// Equal codes keep ascending particle indices exactly as a stable sort of iota
// values does. The last pass writes the caller's arrays directly.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/dfsph_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace dfsph {
namespace {

constexpr int RS_BLOCK = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_BLOCK * RS_ROUNDS;
constexpr int RS_BITS = 10;
constexpr int RS_BINS = 1 << RS_BITS;
constexpr u32 RS_MASK = RS_BINS - 1;
constexpr int RS_WARPS = RS_BLOCK / 32;
constexpr int RS_PASSES = 3;
constexpr int RS_DPT = RS_BINS / RS_BLOCK;  // digits per thread in the block-wide digit passes
static_assert(RS_BINS % RS_BLOCK == 0 && RS_BITS * RS_PASSES >= 30, "radix layout");
constexpr u32 NO_DIGIT = 0xFFFFFFFFu;

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

// counter_base[value] += 1 for every valid lane, one atomic per distinct
// value in the warp (coherent inputs put most of a warp on one counter).
__device__ __forceinline__ void warp_count(u32* counter_base, u32 value, bool valid) {
    const u32 v = valid ? value : NO_DIGIT;
    const u32 peers = __match_any_sync(0xffffffffu, v);
    const u32 lt = (1u << (threadIdx.x & 31)) - 1u;
    if (valid && (peers & lt) == 0u) atomicAdd(counter_base + value, static_cast<u32>(__popc(peers)));
}

// Per-block digit counts -> the tile's column of the digit-major histogram
// and the pass's digit totals.
__device__ __forceinline__ void flush_tile_counts(const u32* h, u32* hist, int n_tiles, int tile, u32* totals) {
#pragma unroll
    for (int j = 0; j < RS_BINS / RS_BLOCK; ++j) {
        const int d = threadIdx.x + RS_BLOCK * j;
        const u32 c = h[d];
        hist[size_t(d) * n_tiles + tile] = c;
        if (c) atomicAdd(totals + d, c);
    }
}

__global__ void __launch_bounds__(RS_BLOCK) morton_codes_kernel(int n, const float* __restrict__ xyz, float mx,
                                                                float my, float mz, float ix, float iy, float iz,
                                                                u32* __restrict__ codes, u32* __restrict__ idx,
                                                                u32* __restrict__ hist, int n_tiles,
                                                                u32* __restrict__ totals) {
    pdl_wait();
    __shared__ u32 h[RS_BINS];
#pragma unroll
    for (int j = 0; j < RS_BINS / RS_BLOCK; ++j) h[threadIdx.x + RS_BLOCK * j] = 0u;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
#pragma unroll
    for (int k = 0; k < RS_ROUNDS; ++k) {
        const int i = base + k * RS_BLOCK + threadIdx.x;
        const bool valid = i < n;
        u32 code = 0;
        if (valid) {
            const u32 qx = quant10((xyz[3 * i] - mx) * ix);
            const u32 qy = quant10((xyz[3 * i + 1] - my) * iy);
            const u32 qz = quant10((xyz[3 * i + 2] - mz) * iz);
            code = (spread10(qx) << 2) | (spread10(qy) << 1) | spread10(qz);
            codes[i] = code;
            idx[i] = static_cast<u32>(i);
        }
        warp_count(h, code & RS_MASK, valid);
    }
    __syncthreads();
    flush_tile_counts(h, hist, n_tiles, blockIdx.x, totals);
}

// hist[d][t] (the pass's counts) becomes the slot of the first key of digit d
// in tile t: the keys of smaller digits plus those of digit d in earlier
// tiles. One warp per digit; it also clears the digit's row of the other
// histogram, which the next scatter fills.
__global__ void __launch_bounds__(256) radix_offsets_kernel(u32* __restrict__ hist, int n_tiles,
                                                            const u32* __restrict__ totals,
                                                            u32* __restrict__ next_hist) {
    pdl_wait();
    __shared__ u32 tot[RS_BINS];
#pragma unroll
    for (int j = 0; j < RS_BINS / 256; ++j) tot[threadIdx.x + 256 * j] = totals[threadIdx.x + 256 * j];
    __syncthreads();
    const int d = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    u32 base = 0;
#pragma unroll
    for (int j = 0; j < RS_BINS / 32; ++j) {
        const int k = lane + 32 * j;
        base += k < d ? tot[k] : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) base += __shfl_xor_sync(0xffffffffu, base, o);
    // each lane a contiguous segment of the row: independent loads, then a
    // warp scan of the segment sums
    u32* row = hist + size_t(d) * n_tiles;
    const int per = (n_tiles + 31) / 32;
    const int t0 = min(lane * per, n_tiles), t1 = min(t0 + per, n_tiles);
    u32 sum = 0;
#pragma unroll 8
    for (int t = t0; t < t1; ++t) sum += row[t];
    u32 x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    u32 run = base + x - sum;
#pragma unroll 8
    for (int t = t0; t < t1; ++t) {
        const u32 v = row[t];
        row[t] = run;
        run += v;
    }
    if (next_hist) {
        u32* nrow = next_hist + size_t(d) * n_tiles;
        for (int t = lane; t < n_tiles; t += 32) nrow[t] = 0u;  // stores only: nothing waits
    }
}

// Each warp ranks its own contiguous 512-key slice of the tile (warp match,
// a per-warp digit count in shared memory, no block barrier per round); one
// block-wide pass then turns the per-warp counts into tile-local slots in
// digit order (digit by digit, warp by warp), so the rank is stable.
constexpr int RS_SLICE = RS_TILE / RS_WARPS;
constexpr int RS_SLICE_ROUNDS = RS_SLICE / 32;

// Shared memory of the scatter (dynamic: above the static limit at 10-bit
// digits): start, dst0, ncount [RS_BINS] each, wcnt [RS_WARPS][RS_BINS],
// skey, sval [RS_TILE] each.
constexpr size_t RS_SCATTER_SMEM = sizeof(u32) * (3 * RS_BINS + RS_WARPS * RS_BINS + 2 * RS_TILE);

__global__ void __launch_bounds__(RS_BLOCK) radix_scatter_kernel(
    const u32* __restrict__ keys_in, const u32* __restrict__ vals_in, int n, int shift,
    const u32* __restrict__ offs, int n_tiles, u32* __restrict__ keys_out, u32* __restrict__ vals_out,
    u32* __restrict__ next_hist, u32* __restrict__ next_totals) {
    pdl_wait();
    extern __shared__ u32 rs_smem[];
    u32* start = rs_smem;             // tile-local slot of the digit's first key
    u32* dst0 = start + RS_BINS;      // global slot of the digit's first key of this tile
    u32* ncount = dst0 + RS_BINS;     // next pass's digit counts of this tile's keys
    u32* wcnt = ncount + RS_BINS;     // [warp][digit]: counts, then first slots
    u32* skey = wcnt + RS_WARPS * RS_BINS;
    u32* sval = skey + RS_TILE;
    __shared__ u32 wsum[RS_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int base = blockIdx.x * RS_TILE;
    const int count = min(RS_TILE, n - base);
    const int slice = warp * RS_SLICE;
    // this lane's keys of the warp's slice, all loads in flight at once
    u32 keys[RS_SLICE_ROUNDS], vals[RS_SLICE_ROUNDS];
#pragma unroll
    for (int k = 0; k < RS_SLICE_ROUNDS; ++k) {
        const int p = slice + k * 32 + lane;
        keys[k] = p < count ? keys_in[base + p] : 0u;
        vals[k] = p < count ? vals_in[base + p] : 0u;
    }
#pragma unroll
    for (int j = 0; j < RS_DPT; ++j) {
        const int d = threadIdx.x + RS_BLOCK * j;
        ncount[d] = 0u;
        dst0[d] = offs[size_t(d) * n_tiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) wcnt[w * RS_BINS + d] = 0u;
    }
    __syncthreads();
    const u32 lt_mask = (1u << lane) - 1u;
    u32 rank[RS_SLICE_ROUNDS];
#pragma unroll
    for (int k = 0; k < RS_SLICE_ROUNDS; ++k) {
        const bool valid = slice + k * 32 + lane < count;
        const u32 d = valid ? ((keys[k] >> shift) & RS_MASK) : NO_DIGIT;  // invalid lanes: their own group
        const u32 peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        u32 old = 0;
        if (valid && lane == leader) {
            old = wcnt[warp * RS_BINS + d];
            wcnt[warp * RS_BINS + d] = old + __popc(peers);
        }
        rank[k] = __shfl_sync(0xffffffffu, old, leader) + __popc(peers & lt_mask);
        __syncwarp();
    }
    __syncthreads();
    // digits [RS_DPT t, RS_DPT (t + 1)) (thread t): their tile counts,
    // exclusive prefix over digits, then each warp's first slot of the digit
    {
        u32 cd[RS_DPT];
        u32 c = 0;
#pragma unroll
        for (int j = 0; j < RS_DPT; ++j) {
            const int d = RS_DPT * threadIdx.x + j;
            cd[j] = 0;
#pragma unroll
            for (int w = 0; w < RS_WARPS; ++w) cd[j] += wcnt[w * RS_BINS + d];
            c += cd[j];
        }
        u32 x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        u32 run = x - c;
        for (int w = 0; w < warp; ++w) run += wsum[w];
#pragma unroll
        for (int j = 0; j < RS_DPT; ++j) {
            const int d = RS_DPT * threadIdx.x + j;
            start[d] = run;
#pragma unroll
            for (int w = 0; w < RS_WARPS; ++w) {
                const u32 cw = wcnt[w * RS_BINS + d];
                wcnt[w * RS_BINS + d] = run;
                run += cw;
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RS_SLICE_ROUNDS; ++k) {
        if (slice + k * 32 + lane < count) {
            const u32 p = wcnt[warp * RS_BINS + ((keys[k] >> shift) & RS_MASK)] + rank[k];
            skey[p] = keys[k];
            sval[p] = vals[k];
        }
    }
    __syncthreads();
    // runs leave in digit order, consecutive threads to consecutive slots
#pragma unroll 4
    for (int k = 0; k < RS_ROUNDS; ++k) {
        const int p = k * RS_BLOCK + threadIdx.x;
        const bool valid = p < count;
        const u32 key = valid ? skey[p] : 0u;
        u32 dst = 0;
        if (valid) {
            const u32 d = (key >> shift) & RS_MASK;
            dst = dst0[d] + (static_cast<u32>(p) - start[d]);
            keys_out[dst] = key;
            vals_out[dst] = sval[p];
        }
        if (next_hist) {
            // the next pass's digit and tile of this key
            const u32 d2 = (key >> (shift + RS_BITS)) & RS_MASK;
            const u32 t2 = dst / RS_TILE;
            const u32 cell = (t2 << RS_BITS) | d2;
            const u32 p2 = __match_any_sync(0xffffffffu, valid ? cell : NO_DIGIT);
            if (valid && (p2 & lt_mask) == 0u)
                atomicAdd(next_hist + size_t(d2) * n_tiles + t2, static_cast<u32>(__popc(p2)));
            warp_count(ncount, d2, valid);
        }
    }
    if (next_hist) {
        __syncthreads();
#pragma unroll
        for (int j = 0; j < RS_DPT; ++j) {
            const int d = threadIdx.x + RS_BLOCK * j;
            if (ncount[d]) atomicAdd(next_totals + d, ncount[d]);
        }
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
    {
        // the scatter's shared memory is above the static limit: opt in once per device
        static bool opted[64] = {};
        int dev = 0;
        DFSPH_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= 64 || !opted[dev]) {
            DFSPH_CUDA(cudaFuncSetAttribute(radix_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            int(RS_SCATTER_SMEM)));
            if (dev >= 0 && dev < 64) opted[dev] = true;
        }
    }
    const int n_tiles = int((n + RS_TILE - 1) / RS_TILE);
    const size_t m = size_t(RS_BINS) * n_tiles;
    const size_t words = 4 * size_t(n) + 2 * m /*histograms*/ + RS_PASSES * RS_BINS /*digit totals*/;
    u32* mem = nullptr;
    DFSPH_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&mem), words * sizeof(u32), st));
    u32* ka = mem;
    u32* va = ka + n;
    u32* kb = va + n;
    u32* vb = kb + n;
    u32* hist[2] = {vb + n, vb + n + m};
    u32* totals = vb + n + 2 * m;
    DFSPH_CUDA(cudaMemsetAsync(totals, 0, RS_PASSES * RS_BINS * sizeof(u32), st));
    launch_pdl(morton_codes_kernel, n_tiles, RS_BLOCK, 0, st, int(n), xyz, smin[0], smin[1], smin[2], inv[0], inv[1],
               inv[2], ka, va, hist[0], n_tiles, totals);
    DFSPH_LAUNCHED();
    for (int pass = 0; pass < RS_PASSES; ++pass) {
        const bool last = pass == RS_PASSES - 1;
        u32* cur = hist[pass & 1];
        u32* nxt = last ? nullptr : hist[(pass + 1) & 1];
        launch_pdl(radix_offsets_kernel, RS_BINS / 8, 256, 0, st, cur, n_tiles, (const u32*)(totals + pass * RS_BINS),
                   nxt);
        DFSPH_LAUNCHED();
        // the last pass writes the caller's arrays where given
        u32* ko = (last && sorted_codes) ? sorted_codes : kb;
        u32* vo = (last && sorted_idx) ? sorted_idx : vb;
        launch_pdl(radix_scatter_kernel, n_tiles, RS_BLOCK, RS_SCATTER_SMEM, st, (const u32*)ka, (const u32*)va,
                   int(n), RS_BITS * pass, (const u32*)cur, n_tiles, ko, vo, nxt,
                   last ? nullptr : totals + (pass + 1) * RS_BINS);
        DFSPH_LAUNCHED();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    DFSPH_CUDA(cudaFreeAsync(mem, st));
}

}  // namespace dfsph
