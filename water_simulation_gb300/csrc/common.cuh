// Shared device/host definitions of the GB300 DFSPH step.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <utility>
#include <stdexcept>
#include <string>

namespace dfsph {

using u32 = std::uint32_t;
using u64 = std::uint64_t;

// A 4-lane vector of the working real type; 16 B for float (one LDG.128),
// 32 B for double.
template <class R> struct alignas(4 * sizeof(R)) R4 { R x, y, z, w; };

// Status carrying exception used inside the library; converted to a status
// code at the C ABI and never thrown across it.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] void throw_cuda(cudaError_t e, const char* expr, const char* file, int line);

#define DFSPH_CUDA(expr)                                                      \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) ::dfsph::throw_cuda(_e, #expr, __FILE__, __LINE__); \
    } while (0)

#define DFSPH_LAUNCHED()                                                      \
    do {                                                                      \
        cudaError_t _e = cudaGetLastError();                                  \
        if (_e != cudaSuccess) ::dfsph::throw_cuda(_e, "kernel launch", __FILE__, __LINE__); \
    } while (0)

// Uniform grid of the reference's make_grid (solvers/dfsph/src/dfsph.cu:55-65).
struct GridGeom {
    float origin[3];
    int dims[3];
    float cell_length;
    u32 total;          // dims.x*dims.y*dims.z; the key of out-of-grid particles
    float inv_bin;      // host IEEE 1.0f/cell_length: bins particles (cell_grid.cu:81)
    float inv_stencil;  // device 1.0f/cell_length under the reference's fast math:
                        // centres the 27-cell stencil (dfsph_kernels.cu:52,89,...)
};

GridGeom make_grid_geom(const float dmin[3], const float dmax[3], float smoothing_length);

// Device-side copy of the grid. The cell arithmetic is FP32 in every build:
// positions are rounded to float and binned and centred with the float
// origin and the two float reciprocals, exactly as the reference's FP32
// kernels do, so the FP64 build (the GPU oracle) visits the neighbour sets
// the FP32 build visits for the same positions instead of switching a
// particle's cell wherever the exact reciprocal 1/l differs from the float one.
template <class R> struct GridDev {
    float ox, oy, oz;
    int nx, ny, nz;
    u32 total;
    float inv_bin;
    float inv_stencil;
    // Scenes stepped together share the geometry; scene s owns the keys
    // [s * cells1, (s + 1) * cells1), cells1 = total + 1 (its out-of-grid key
    // last). slot_scene[s] is the scene of sorted slot s (null: one scene).
    u32 cells1;
    const unsigned short* slot_scene;
    // Morton slot order: rank[c] is the sort key of x-major cell c (its rank
    // in the Morton order of the grid's cells; rank[total] = total); null for
    // the reference's x-major order, where the sort key is c itself.
    const u32* rank;
};

template <class R> inline GridDev<R> to_dev(const GridGeom& g) {
    GridDev<R> d;
    d.ox = g.origin[0]; d.oy = g.origin[1]; d.oz = g.origin[2];
    d.nx = g.dims[0]; d.ny = g.dims[1]; d.nz = g.dims[2];
    d.total = g.total;
    d.cells1 = g.total + 1;
    d.slot_scene = nullptr;
    d.inv_bin = g.inv_bin;
    d.inv_stencil = g.inv_stencil;
    d.rank = nullptr;
    return d;
}

#ifdef __CUDACC__
// floor + float->int with the GPU's saturating conversion (NaN -> 0), as the
// reference's static_cast<int>(floorf(...)) compiles on the device.
__device__ __forceinline__ int floor_to_int(float v) { return static_cast<int>(floorf(v)); }

template <class R> __device__ __forceinline__ u32 scene_of(const GridDev<R>& g, int slot) {
    return g.slot_scene ? static_cast<u32>(g.slot_scene[slot]) : 0u;
}

// hash_cell (core/src/cell_grid.cu:10-22): x-major id, out of grid -> total.
template <class R>
__device__ __forceinline__ u32 cell_key(R px, R py, R pz, const GridDev<R>& g) {
    const int cx = floor_to_int(__fmul_rn(__fsub_rn(float(px), g.ox), g.inv_bin));
    const int cy = floor_to_int(__fmul_rn(__fsub_rn(float(py), g.oy), g.inv_bin));
    const int cz = floor_to_int(__fmul_rn(__fsub_rn(float(pz), g.oz), g.inv_bin));
    if (cx < 0 || cx >= g.nx || cy < 0 || cy >= g.ny || cz < 0 || cz >= g.nz) return g.total;
    return (static_cast<u32>(cx) * static_cast<u32>(g.ny) + static_cast<u32>(cy)) *
               static_cast<u32>(g.nz) + static_cast<u32>(cz);
}

// The sort key of x-major cell c: c itself, or in Morton slot order its
// Morton rank (rank[total] = total keeps the out-of-grid key last).
template <bool MORTON, class R> __device__ __forceinline__ u32 sort_key(const GridDev<R>& g, u32 c) {
    if constexpr (MORTON) {
        return __ldg(g.rank + c);
    } else {
        return c;
    }
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while the kernel before it on the stream drains;
// this waits until that kernel has completed and its memory is visible
// (griddepcontrol.wait; without the launch attribute it returns at once).
// Every kernel of the step calls it before touching global memory.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// A launch with programmatic stream serialization; the kernel must begin with
// pdl_wait().
template <class... P, class... A>
inline void launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = grid;
    lc.blockDim = block;
    lc.dynamicSmemBytes = smem;
    lc.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    DFSPH_CUDA(cudaLaunchKernelEx(&lc, kernel, std::forward<A>(args)...));
}

// Stencil-centre cell (dfsph_kernels.cu:15-17) clamped to [-2, dims+1]: any
// value outside that range selects no cell on that axis, exactly as the
// unclamped coordinate would, and the clamp keeps the +-1 arithmetic in range.
struct Centre { int x, y, z; };

template <class R>
__device__ __forceinline__ Centre stencil_centre(R px, R py, R pz, const GridDev<R>& g) {
    Centre c;
    c.x = min(max(floor_to_int(__fmul_rn(__fsub_rn(float(px), g.ox), g.inv_stencil)), -2), g.nx + 1);
    c.y = min(max(floor_to_int(__fmul_rn(__fsub_rn(float(py), g.oy), g.inv_stencil)), -2), g.ny + 1);
    c.z = min(max(floor_to_int(__fmul_rn(__fsub_rn(float(pz), g.oz), g.inv_stencil)), -2), g.nz + 1);
    return c;
}

// The reference's 27-cell stencil (ITER_NEIGHBORS, dfsph_kernels.cu:13-35)
// visited as 9 runs: for each valid (dx, dy) the cells z-1..z+1 are adjacent
// keys, so their particles form one contiguous range of sorted slots
// [cs[first], cs[last+1]). Same candidate set, fewer range lookups. The x, y
// and z ranges are clamped to the grid once per particle, and the runs are
// stepped through by adding the column and slab strides to one cell index, so
// a run costs its two cell_start loads and the loop step (2 % of the step
// against per-run bounds checks, same candidates in the same order).
#ifdef DFSPH_BOUNDS_CHECK
// Checked build: every run is validated against the closing entry of its
// cell_start array (the first slot beyond the grid's particles); a run out of
// range or reversed is skipped and counted here instead of being read.
static __device__ u32 g_bounds_violations;
#endif

// The grid of the wall particles: the fluid grid's geometry in the x-major
// order, whatever the fluid's slot order (walls are always sorted by x-major
// key, and their cell_start is indexed by it). for_each_run ignores rank; the
// copy keeps the wall walks free of the fluid's rank table all the same.
template <class R> __device__ __forceinline__ GridDev<R> wall_grid(const GridDev<R>& g) {
    GridDev<R> w = g;
    w.rank = nullptr;
    return w;
}

template <class R, class F>
__device__ __forceinline__ void for_each_run(const Centre& c, const GridDev<R>& g,
                                             const u32* __restrict__ cs, F&& f) {
    const int x0 = max(c.x - 1, 0), x1 = min(c.x + 1, g.nx - 1);
    const int y0 = max(c.y - 1, 0), y1 = min(c.y + 1, g.ny - 1);
    const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, g.nz - 1);
    if (x0 > x1 || y0 > y1 || z0 > z1) return;
#ifdef DFSPH_BOUNDS_CHECK
    const u32 limit = __ldg(cs + g.cells1);
#endif
    const u32 span = static_cast<u32>(z1 - z0 + 1);
    const int ny_runs = y1 - y0;
    u32 row = (static_cast<u32>(x0) * static_cast<u32>(g.ny) + static_cast<u32>(y0)) * static_cast<u32>(g.nz) +
              static_cast<u32>(z0);
    // not unrolled: one copy of the pair loop keeps the instruction cache warm
#pragma unroll 1
    for (int kx = x1 - x0; kx >= 0; --kx, row += static_cast<u32>(g.ny) * static_cast<u32>(g.nz)) {
        u32 at = row;
#pragma unroll 1
        for (int ky = ny_runs; ky >= 0; --ky, at += static_cast<u32>(g.nz)) {
            const u32 b = __ldg(cs + at);
            const u32 e = __ldg(cs + at + span);
#ifdef DFSPH_BOUNDS_CHECK
            if (b > e || e > limit) {
                atomicAdd(&g_bounds_violations, 1u);
                continue;
            }
#endif
            f(b, e);
        }
    }
}

// The same 27 cells in the same sequence in Morton slot order (g.rank set):
// a column's cells are not adjacent in slot order, so each cell is one run,
// looked up through the rank table.
template <class R, class F>
__device__ __forceinline__ void for_each_run_ranked(const Centre& c, const GridDev<R>& g,
                                                    const u32* __restrict__ cs, F&& f) {
    const int z0 = max(c.z - 1, 0);
    const int z1 = min(c.z + 1, g.nz - 1);
    if (z0 > z1) return;
#ifdef DFSPH_BOUNDS_CHECK
    const u32 limit = __ldg(cs + g.cells1);
#endif
#pragma unroll 1
    for (int dx = -1; dx <= 1; ++dx) {
        const int nx = c.x + dx;
        if (nx < 0 || nx >= g.nx) continue;
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const int ny = c.y + dy;
            if (ny < 0 || ny >= g.ny) continue;
            const u32 base = (static_cast<u32>(nx) * static_cast<u32>(g.ny) + static_cast<u32>(ny)) *
                             static_cast<u32>(g.nz);
#pragma unroll 1
            for (int z = z0; z <= z1; ++z) {
                const u32 r = __ldg(g.rank + base + static_cast<u32>(z));
                const u32 b = __ldg(cs + r);
                const u32 e = __ldg(cs + r + 1);
#ifdef DFSPH_BOUNDS_CHECK
                if (b > e || e > limit) {
                    atomicAdd(&g_bounds_violations, 1u);
                    continue;
                }
#endif
                f(b, e);
            }
        }
    }
}

// The fluid stencil walk of a kernel instantiated for the x-major slot order
// (MORTON = false, the reference's) or the Morton one.
template <bool MORTON, class R, class F>
__device__ __forceinline__ void for_each_fluid_run(const Centre& c, const GridDev<R>& g, const u32* __restrict__ cs,
                                                   F&& f) {
    if constexpr (MORTON) {
        for_each_run_ranked(c, g, cs, f);
    } else {
        for_each_run(c, g, cs, f);
    }
}

#endif  // __CUDACC__

}  // namespace dfsph
