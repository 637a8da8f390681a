// Linear BVH over particles (the reference's SpatialAccel,
// core/src/spatial_accel.cu:42-179) and the Akinci cohesion kernel
// (core/include/water/core/sph_kernels.cuh:43-51). Neither is on the DFSPH
// step; both exist for the reference's later ray-tracing and surface-tension
// work.
//
// Build: Morton order of the positions in the scene box (dfsph_morton_sort),
// internal nodes by Karras' construction (T. Karras, "Maximizing Parallelism
// in the Construction of BVHs, Octrees, and k-d Trees", HPG 2012) with equal
// codes ordered by sorted slot as in the reference, leaf boxes p +- radius, and
// the bottom-up pass over internal boxes that the reference leaves for later.
// Node numbering as in the reference: internal nodes 0..n-2 (root 0), leaf k
// (sorted slot k) is node n-1+k.
//
// Refit: new leaf boxes from moved positions and internal boxes bottom-up on
// the same topology. Every leaf walks towards the root carrying its box in
// registers; at each internal node the first of its two children to arrive
// stops (acquire-release arrival count) and the second merges its box with
// the sibling's and goes on. Nothing waits on another thread.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/dfsph_gb300.h"
#include "common.cuh"
#include "solver_api.h"

namespace dfsph {
namespace {

// Length of the common prefix of the sorted codes i and j (Karras' delta);
// equal codes are ordered by slot index, so every pair of slots differs.
__device__ __forceinline__ int common_prefix(const u32* __restrict__ codes, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const u32 a = codes[i], b = codes[j];
    return a != b ? __clz(a ^ b) : 32 + __clz(static_cast<u32>(i) ^ static_cast<u32>(j));
}

// empty_slots, when given, is the box array viewed as 8-byte words: node i's
// box slot (3 words) is set to the all-ones pattern the box pass starts from.
__global__ void __launch_bounds__(256) lbvh_internal_kernel(const u32* __restrict__ codes, int n,
                                                            u32* __restrict__ left, u32* __restrict__ right,
                                                            u32* __restrict__ parent,
                                                            unsigned long long* __restrict__ empty_slots) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    if (empty_slots) {
        empty_slots[3 * size_t(i)] = ~0ull;
        empty_slots[3 * size_t(i) + 1] = ~0ull;
        empty_slots[3 * size_t(i) + 2] = ~0ull;
    }
    if (i == 0) parent[0] = 0xFFFFFFFFu;  // the root
    // the node's range extends towards the neighbour sharing the longer prefix
    const int d = common_prefix(codes, n, i, i + 1) > common_prefix(codes, n, i, i - 1) ? 1 : -1;
    const int dmin = common_prefix(codes, n, i, i - d);
    // other end of the range: doubling, then bisection (the prefix is
    // non-increasing along the range and -1 beyond the array, so both end)
    int lmax = 2;
    while (common_prefix(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int len = 0;
    for (int t = lmax >> 1; t > 0; t >>= 1)
        if (common_prefix(codes, n, i, i + (len + t) * d) > dmin) len += t;
    const int j = i + len * d;
    // split: the last position s in [0, len) whose prefix with i is longer
    // than the node's own prefix
    const int dnode = common_prefix(codes, n, i, j);
    int lo = 0, hi = len;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (common_prefix(codes, n, i, i + mid * d) > dnode) lo = mid;
        else hi = mid;
    }
    const int gamma = i + lo * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    const u32 nl = static_cast<u32>(n - 1);
    const u32 l = first == gamma ? nl + static_cast<u32>(gamma) : static_cast<u32>(gamma);
    const u32 r = last == gamma + 1 ? nl + static_cast<u32>(gamma + 1) : static_cast<u32>(gamma + 1);
    left[i] = l;
    right[i] = r;
    parent[l] = static_cast<u32>(i);
    parent[r] = static_cast<u32>(i);
}

// Arrival count with acquire-release semantics at device scope: the stores
// made before it (the arriving child's box) are visible to the thread whose
// add returns after it, and that thread sees the earlier arrival's stores.
__device__ __forceinline__ u32 arrive(u32* p) {
    u32 old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

__global__ void __launch_bounds__(256) lbvh_refit_kernel(const float* __restrict__ xyz, int n, float radius,
                                                         const u32* __restrict__ sorted, const u32* __restrict__ left,
                                                         const u32* __restrict__ right, const u32* __restrict__ parent,
                                                         float* boxes, u32* arrivals) {
    pdl_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const u32 p = sorted[k];
    const float x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
    // the box this thread carries up, kept in registers
    float b0 = x - radius, b1 = y - radius, b2 = z - radius;
    float b3 = x + radius, b4 = y + radius, b5 = z + radius;
    u32 child = static_cast<u32>(n - 1 + k);
    float* o = boxes + 6 * size_t(child);
    o[0] = b0; o[1] = b1; o[2] = b2; o[3] = b3; o[4] = b4; o[5] = b5;
    u32 node = parent[child];
    while (node != 0xFFFFFFFFu) {
        // topology loads issued before the arrival (nothing writes them), so
        // their latency overlaps the atomic's
        const u32 l = left[node], r = right[node], up = parent[node];
        // the first child to arrive stops; the second merges the two boxes
        if (arrive(arrivals + node) == 0u) return;
        const u32 sib = l == child ? r : l;
        const float* q = boxes + 6 * size_t(sib);
        // from L2, where the sibling's box was stored before its arrival
        b0 = fminf(b0, __ldcg(q + 0)); b1 = fminf(b1, __ldcg(q + 1)); b2 = fminf(b2, __ldcg(q + 2));
        b3 = fmaxf(b3, __ldcg(q + 3)); b4 = fmaxf(b4, __ldcg(q + 4)); b5 = fmaxf(b5, __ldcg(q + 5));
        o = boxes + 6 * size_t(node);
        o[0] = b0; o[1] = b1; o[2] = b2; o[3] = b3; o[4] = b4; o[5] = b5;
        child = node;
        node = up;
    }
}

// Refit without fences, in two phases per block of REFIT_BLOCK consecutive
// leaves.
//  1. In the block: every lane starts at its leaf; lanes whose current nodes
//     share a parent meet in shared memory, one merges and climbs on, until
//     no two lanes meet (the subtrees of the block's leaves are complete).
//  2. The lanes left (roots of the block's complete subtrees, and lanes whose
//     partner lies in another block) walk on with three independent exchange
//     walks, one per 8-byte pair of box words ((min x, min y), (min z, max x),
//     (max y, max z)): a walk swaps its pair into the parent's slot with one
//     64-bit atomicExch; getting back the empty pattern means it arrived first
//     and stops, otherwise it got the sibling's pair, merges, stores and goes
//     on. The data travels inside the atomic, so no ordering of other memory
//     operations is needed. Internal slots start as all-ones words, a NaN
//     pattern that float arithmetic never produces (its results are canonical
//     NaNs).
constexpr unsigned long long EMPTY_PAIR = ~0ull;
constexpr int REFIT_BLOCK = 128;  // leaves merged in shared memory before the global walks

__device__ __forceinline__ unsigned long long pack_pair(float a, float b) {
    return static_cast<unsigned long long>(__float_as_uint(a)) |
           (static_cast<unsigned long long>(__float_as_uint(b)) << 32);
}

__device__ __forceinline__ unsigned long long* pair_slot(float* boxes, u32 node, int w) {
    return reinterpret_cast<unsigned long long*>(boxes + 6 * size_t(node) + 2 * w);
}

__global__ void __launch_bounds__(REFIT_BLOCK) lbvh_refit_pairs_kernel(const float* __restrict__ xyz, int n, float radius,
                                                               const u32* __restrict__ sorted,
                                                               const u32* __restrict__ parent, float* boxes) {
    pdl_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    bool active = k < n;
    float b[6] = {0, 0, 0, 0, 0, 0};
    u32 node = 0, up = 0xFFFFFFFFu;
    if (active) {
        const u32 p = sorted[k];
        const float x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
        b[0] = x - radius; b[1] = y - radius; b[2] = z - radius;
        b[3] = x + radius; b[4] = y + radius; b[5] = z + radius;
        node = static_cast<u32>(n - 1 + k);
#pragma unroll
        for (int w = 0; w < 3; ++w) *pair_slot(boxes, node, w) = pack_pair(b[2 * w], b[2 * w + 1]);
        up = parent[node];
    }
    // 1. merges inside the block. A parent P whose both children hold leaves
    //    of this block has its whole range among them, so P, an endpoint of
    //    its range, lies in [L, L + REFIT_BLOCK); a parent outside has a child
    //    outside.
    //    Per round: lanes at such a parent count their arrival in shared
    //    memory; the first leaves its box there and waits, the second merges
    //    it (after a barrier) and climbs on. Rounds stop when nothing merged
    //    (or after 64 levels); lanes still waiting then climb globally.
    __shared__ u32 arrivals[REFIT_BLOCK];
    __shared__ float waiting[REFIT_BLOCK][6];
    __shared__ int merged;
    const u32 L = blockIdx.x * static_cast<u32>(REFIT_BLOCK);
    arrivals[threadIdx.x] = 0u;
    bool parked = false;
    for (int round = 0; round < 64; ++round) {
        if (threadIdx.x == 0) merged = 0;
        __syncthreads();
        const bool meet = active && !parked && up != 0xFFFFFFFFu && up >= L && up - L < static_cast<u32>(REFIT_BLOCK);
        u32 rank = 2u;
        if (meet) {
            rank = atomicAdd(&arrivals[up - L], 1u);
            if (rank == 0u) {
#pragma unroll
                for (int c = 0; c < 6; ++c) waiting[up - L][c] = b[c];
                parked = true;
            }
        }
        __syncthreads();
        if (meet && rank == 1u) {
            const float* o = waiting[up - L];
            b[0] = fminf(b[0], o[0]); b[1] = fminf(b[1], o[1]); b[2] = fminf(b[2], o[2]);
            b[3] = fmaxf(b[3], o[3]); b[4] = fmaxf(b[4], o[4]); b[5] = fmaxf(b[5], o[5]);
            node = up;
#pragma unroll
            for (int w = 0; w < 3; ++w) *pair_slot(boxes, node, w) = pack_pair(b[2 * w], b[2 * w + 1]);
            up = parent[node];
            merged = 1;
        } else if (parked && arrivals[up - L] == 2u) {
            active = false;  // the partner took this box up
            parked = false;
        }
        __syncthreads();
        if (!merged) break;
    }
    if (!active || up == 0xFFFFFFFFu) return;
    // 2. three exchange walks from the parent of this subtree's root
    u32 cur[3] = {up, up, up};
    float pa[3] = {b[0], b[2], b[4]}, pb[3] = {b[1], b[3], b[5]};
    bool go[3] = {true, true, true};
    while (go[0] || go[1] || go[2]) {
        u32 nxt[3];
        unsigned long long old[3];
#pragma unroll
        for (int w = 0; w < 3; ++w) {
            nxt[w] = go[w] ? parent[cur[w]] : 0xFFFFFFFFu;
            old[w] = go[w] ? atomicExch(pair_slot(boxes, cur[w], w), pack_pair(pa[w], pb[w])) : EMPTY_PAIR;
        }
#pragma unroll
        for (int w = 0; w < 3; ++w) {
            if (!go[w]) continue;
            if (old[w] == EMPTY_PAIR) {  // the sibling's walk finishes this node
                go[w] = false;
                continue;
            }
            const float oa = __uint_as_float(static_cast<u32>(old[w]));
            const float ob = __uint_as_float(static_cast<u32>(old[w] >> 32));
            pa[w] = w <= 1 ? fminf(pa[w], oa) : fmaxf(pa[w], oa);
            pb[w] = w == 0 ? fminf(pb[w], ob) : fmaxf(pb[w], ob);
            *pair_slot(boxes, cur[w], w) = pack_pair(pa[w], pb[w]);
            cur[w] = nxt[w];
            go[w] = nxt[w] != 0xFFFFFFFFu;
        }
    }
}

// Akinci 2013 cohesion kernel: 32 / (pi l^9) times (l - r)^3 r^3 for
// l/2 < r <= l, 2 (l - r)^3 r^3 - l^6 / 64 for 0 < r <= l/2, else 0.
__global__ void __launch_bounds__(256) cohesion_kernel(const float* __restrict__ r, int n, float l,
                                                       float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ri = r[i];
    float c = 0.0f;
    if (ri > 0.0f && ri <= l) {
        const float l3 = l * l * l;
        const float sigma = 32.0f / (3.14159265358979323846f * (l3 * l3 * l3));
        const float lm = l - ri;
        const float t = lm * lm * lm * ri * ri * ri;
        c = 2.0f * ri > l ? sigma * t : sigma * (2.0f * t - (l3 * l3) / 64.0f);
    }
    out[i] = c;
}

}  // namespace

namespace {
bool pair_aligned(const float* boxes) { return (reinterpret_cast<uintptr_t>(boxes) & 7u) == 0; }

void refit_boxes(const float* xyz, u32 n, float radius, const u32* sorted, const u32* left, const u32* right,
                 const u32* parent, float* boxes, u32* scratch, bool slots_empty, cudaStream_t st) {
    if (n == 0) return;
    if (pair_aligned(boxes)) {
        // 8-byte aligned boxes: the exchange walks (internal slots emptied first)
        if (n > 1 && !slots_empty)
            DFSPH_CUDA(cudaMemsetAsync(boxes, 0xFF, size_t(n - 1) * 6 * sizeof(float), st));
        launch_pdl(lbvh_refit_pairs_kernel, (n + REFIT_BLOCK - 1) / REFIT_BLOCK, REFIT_BLOCK, 0, st, xyz, int(n),
                   radius, sorted, parent, boxes);
        DFSPH_LAUNCHED();
        return;
    }
    if (n > 1) DFSPH_CUDA(cudaMemsetAsync(scratch, 0, size_t(n - 1) * sizeof(u32), st));
    launch_pdl(lbvh_refit_kernel, (n + 255) / 256, 256, 0, st, xyz, int(n), radius, sorted, left, right, parent, boxes,
               scratch);
    DFSPH_LAUNCHED();
}
}  // namespace

void lbvh_build(const float* xyz, u32 n, const float smin[3], const float smax[3], float radius, u32* codes,
                u32* sorted, u32* left, u32* right, u32* parent, float* boxes, u32* scratch, cudaStream_t st) {
    if (n == 0) return;
    morton_sort(xyz, n, smin, smax, codes, sorted, st);
    // the internal-node pass also empties the internal box slots for the box pass
    const bool fill = pair_aligned(boxes);
    if (n > 1) {
        launch_pdl(lbvh_internal_kernel, (n - 1 + 255) / 256, 256, 0, st, (const u32*)codes, int(n), left, right, parent,
                   fill ? reinterpret_cast<unsigned long long*>(boxes) : nullptr);
        DFSPH_LAUNCHED();
    } else {
        DFSPH_CUDA(cudaMemsetAsync(parent, 0xFF, sizeof(u32), st));  // the single leaf is the root
    }
    refit_boxes(xyz, n, radius, sorted, left, right, parent, boxes, scratch, fill, st);
}

void lbvh_refit(const float* xyz, u32 n, float radius, const u32* sorted, const u32* left, const u32* right,
                const u32* parent, float* boxes, u32* scratch, cudaStream_t st) {
    refit_boxes(xyz, n, radius, sorted, left, right, parent, boxes, scratch, false, st);
}

void cohesion(const float* r, u32 n, float l, float* out, cudaStream_t st) {
    if (n == 0) return;
    cohesion_kernel<<<(n + 255) / 256, 256, 0, st>>>(r, int(n), l, out);
    DFSPH_LAUNCHED();
}

}  // namespace dfsph
