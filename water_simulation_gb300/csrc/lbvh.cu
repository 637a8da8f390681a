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
// the same topology. Every leaf walks towards the root; at each internal node
// the first of its two children to arrive stops (atomic arrival count) and the
// second merges both boxes and goes on. Nothing waits on another thread.
#include <cstdint>

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

__global__ void __launch_bounds__(256) lbvh_internal_kernel(const u32* __restrict__ codes, int n,
                                                            u32* __restrict__ left, u32* __restrict__ right,
                                                            u32* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
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

__global__ void __launch_bounds__(256) lbvh_refit_kernel(const float* __restrict__ xyz, int n, float radius,
                                                         const u32* __restrict__ sorted, const u32* __restrict__ left,
                                                         const u32* __restrict__ right, const u32* __restrict__ parent,
                                                         float* boxes, u32* arrivals) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const u32 p = sorted[k];
    const float x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
    u32 node = static_cast<u32>(n - 1 + k);
    float* b = boxes + 6 * size_t(node);
    b[0] = x - radius; b[1] = y - radius; b[2] = z - radius;
    b[3] = x + radius; b[4] = y + radius; b[5] = z + radius;
    __threadfence();
    node = parent[node];
    while (node != 0xFFFFFFFFu) {
        if (atomicAdd(arrivals + node, 1u) == 0u) return;  // the other child finishes this node
        __threadfence();
        const volatile float* a = boxes + 6 * size_t(left[node]);
        const volatile float* c = boxes + 6 * size_t(right[node]);
        float* o = boxes + 6 * size_t(node);
        o[0] = fminf(a[0], c[0]); o[1] = fminf(a[1], c[1]); o[2] = fminf(a[2], c[2]);
        o[3] = fmaxf(a[3], c[3]); o[4] = fmaxf(a[4], c[4]); o[5] = fmaxf(a[5], c[5]);
        __threadfence();
        node = parent[node];
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

void lbvh_build(const float* xyz, u32 n, const float smin[3], const float smax[3], float radius, u32* codes,
                u32* sorted, u32* left, u32* right, u32* parent, float* boxes, u32* scratch, cudaStream_t st) {
    if (n == 0) return;
    morton_sort(xyz, n, smin, smax, codes, sorted, st);
    if (n > 1) {
        lbvh_internal_kernel<<<(n - 1 + 255) / 256, 256, 0, st>>>(codes, int(n), left, right, parent);
        DFSPH_LAUNCHED();
    } else {
        DFSPH_CUDA(cudaMemsetAsync(parent, 0xFF, sizeof(u32), st));  // the single leaf is the root
    }
    lbvh_refit(xyz, n, radius, sorted, left, right, parent, boxes, scratch, st);
}

void lbvh_refit(const float* xyz, u32 n, float radius, const u32* sorted, const u32* left, const u32* right,
                const u32* parent, float* boxes, u32* scratch, cudaStream_t st) {
    if (n == 0) return;
    if (n > 1) DFSPH_CUDA(cudaMemsetAsync(scratch, 0, size_t(n - 1) * sizeof(u32), st));
    lbvh_refit_kernel<<<(n + 255) / 256, 256, 0, st>>>(xyz, int(n), radius, sorted, left, right, parent, boxes,
                                                        scratch);
    DFSPH_LAUNCHED();
}

void cohesion(const float* r, u32 n, float l, float* out, cudaStream_t st) {
    if (n == 0) return;
    cohesion_kernel<<<(n + 255) / 256, 256, 0, st>>>(r, int(n), l, out);
    DFSPH_LAUNCHED();
}

}  // namespace dfsph
