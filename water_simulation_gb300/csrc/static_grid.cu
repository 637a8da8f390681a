// dfsph_build_cell_grid_static: the cell-grid build (same result as
// dfsph_build_cell_grid) for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc / cudaMallocAsync is not
// available or not allowed — inside a host callback or a CUDA-graph node that
// must not touch the allocator, under a memory budget that forbids growth
// after start-up, or in a plugin whose host application owns every device
// allocation. Such callers pass their inputs and outputs and this entry point
// uses a fixed scratch area that is part of the library image instead.
//
// The scratch is one file-scope __device__ array (DFSPH_STATIC_GRID_SCRATCH_BYTES,
// sized for DFSPH_STATIC_GRID_MAX_PARTICLES particles and
// DFSPH_STATIC_GRID_MAX_CELLS cells). Every GPU that loads the library holds
// it until the process exits. Larger inputs are rejected with
// DFSPH_ERR_OUT_OF_RANGE. All calls share the one array: calls that overlap on
// the GPU (different streams, or different host threads, without ordering
// between them) race on it and give wrong results. Each call clears the
// per-cell counters it needs before use, so a call never depends on what an
// earlier call left behind.
//
// The device address of the array is looked up with cudaGetSymbolAddress the
// first time the entry point runs on a device (with that device current); that
// first call therefore performs a runtime query and should come before any
// stream capture. Nothing here calls cudaMalloc, cudaFree or any allocating
// library routine.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/dfsph_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace dfsph {
namespace {

constexpr u32 kMaxParticles = DFSPH_STATIC_GRID_MAX_PARTICLES;
constexpr u32 kMaxCells = DFSPH_STATIC_GRID_MAX_CELLS;
constexpr u32 kMaxTiles = (kMaxCells + 1 + SCAN_TILE - 1) / SCAN_TILE;

// scratch layout (u32 words): count[cells+1] | tiles[n_tiles+1] | key | rank |
// ids | tmp_src | tmp_id  (key .. tmp_id: max particles each)
constexpr size_t kWords = size_t(kMaxCells) + 1 + kMaxTiles + 1 + 5 * size_t(kMaxParticles);
static_assert(kWords * 4 <= DFSPH_STATIC_GRID_SCRATCH_BYTES, "scratch size constant too small");

__device__ __align__(256) unsigned char g_static_grid_scratch[DFSPH_STATIC_GRID_SCRATCH_BYTES];

std::mutex g_mutex;
void* g_scratch_addr[64] = {};

// Keys and per-cell counts straight from the caller's AoS positions.
__global__ void __launch_bounds__(256) static_count_kernel(int n, const float* __restrict__ xyz, GridDev<float> g,
                                                           u32* __restrict__ key, u32* __restrict__ rank,
                                                           u32* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const u32 k = cell_key(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], g);
    key[i] = k;
    rank[i] = atomicAdd(count + k, 1u);
}

// Canonical (key, index) order within each cell; writes the outputs directly.
__global__ void __launch_bounds__(256) static_order_kernel(int n, const u32* __restrict__ tmp_src,
                                                           const u32* __restrict__ tmp_id,
                                                           const u32* __restrict__ key,
                                                           const u32* __restrict__ cell_start, u32 total,
                                                           u32* __restrict__ sorted_keys,
                                                           u32* __restrict__ sorted_idx) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const u32 my = tmp_id[t];
    const u32 c = key[tmp_src[t]];
    const u32 b = cell_start[c];
    const u32 e = (c == total) ? static_cast<u32>(n) : cell_start[c + 1];
    u32 r = 0;
    for (u32 u = b; u < e; ++u) r += (tmp_id[u] < my) ? 1u : 0u;
    const u32 dst = b + r;
    if (sorted_idx) sorted_idx[dst] = my;
    if (sorted_keys) sorted_keys[dst] = c;
}

__global__ void iota_kernel(int n, u32* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = static_cast<u32>(i);
}

}  // namespace
}  // namespace dfsph

extern "C" int dfsph_build_cell_grid_static(const float* xyz_dev, uint32_t n, const float origin[3],
                                            const int dims[3], float cell_length, uint32_t* sorted_keys_dev,
                                            uint32_t* sorted_indices_dev, uint32_t* cell_start_dev,
                                            void* stream) {
    using namespace dfsph;
    if ((n > 0 && !xyz_dev) || !origin || !dims || !cell_start_dev || !(cell_length > 0.0f))
        return DFSPH_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < 3; ++a)
        if (dims[a] <= 0) return DFSPH_ERR_INVALID_ARGUMENT;
    const double cells_d = double(dims[0]) * double(dims[1]) * double(dims[2]);
    if (cells_d > double(kMaxCells) || n > kMaxParticles) return DFSPH_ERR_OUT_OF_RANGE;
    if (n == 0) return DFSPH_OK;  // CellGrid::build leaves the grid untouched (cell_grid.cu:74-77)

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DFSPH_ERR_CUDA;
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_static_grid_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return DFSPH_ERR_CUDA;
            }
            g_scratch_addr[dev] = p;
        }
        base = g_scratch_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GridGeom geo;
    for (int a = 0; a < 3; ++a) { geo.origin[a] = origin[a]; geo.dims[a] = dims[a]; }
    geo.cell_length = cell_length;
    geo.total = u32(dims[0]) * u32(dims[1]) * u32(dims[2]);
    geo.inv_bin = 1.0f / cell_length;
    geo.inv_stencil = geo.inv_bin;
    const GridDev<float> g = to_dev<float>(geo);
    const u32 m = geo.total + 1;
    const u32 n_tiles = (m + SCAN_TILE - 1) / SCAN_TILE;

    u32* w = static_cast<u32*>(base);
    u32* count = w;
    u32* tiles = count + m;
    u32* key = tiles + n_tiles + 1;
    u32* rank = key + n;
    u32* ids = rank + n;
    u32* tsrc = ids + n;
    u32* tid = tsrc + n;

    const int nb = int((n + 255) / 256);
    if (cudaMemsetAsync(count, 0, size_t(m) * sizeof(u32), st) != cudaSuccess) return DFSPH_ERR_CUDA;
    static_count_kernel<<<nb, 256, 0, st>>>(int(n), xyz_dev, g, key, rank, count);
    iota_kernel<<<nb, 256, 0, st>>>(int(n), ids);  // the input order is the original order
    scan_tile_sums<<<n_tiles, SCAN_BLOCK, 0, st>>>(count, m, tiles, nullptr, 0u);
    scan_tile_offsets<<<1, 1024, 0, st>>>(tiles, n_tiles, nullptr, nullptr, 0, nullptr, 0, nullptr, m, 0u, nullptr);
    scan_tiles<<<n_tiles, SCAN_BLOCK, 0, st>>>(count, m, tiles, cell_start_dev, nullptr);
    scatter_kernel<<<nb, 256, 0, st>>>(int(n), key, rank, cell_start_dev, ids, tsrc, tid);
    static_order_kernel<<<nb, 256, 0, st>>>(int(n), tsrc, tid, key, cell_start_dev, geo.total, sorted_keys_dev,
                                            sorted_indices_dev);
    if (cudaGetLastError() != cudaSuccess) return DFSPH_ERR_CUDA;
    return DFSPH_OK;
}
