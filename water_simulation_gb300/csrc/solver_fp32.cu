// FP32 instantiation of the solver, plus the stand-alone cell-grid build.
#include "solver.cuh"

namespace dfsph {

std::unique_ptr<SolverBase> make_solver_fp32(const dfsph_config& cfg, int device, cudaStream_t s) {
    return std::unique_ptr<SolverBase>(new Solver<float>(cfg, device, s));
}

// CellGrid::build (core/src/cell_grid.cu:73-138) for an arbitrary grid, with
// stream-ordered temporaries (or none, when the caller passes every array).
void build_cell_grid(const float* xyz, u32 n, const float origin[3], const int dims[3], float cell_length,
                     u32* sorted_keys, u32* sorted_idx, u32* cell_start, cudaStream_t st) {
    GridGeom geo;
    for (int a = 0; a < 3; ++a) { geo.origin[a] = origin[a]; geo.dims[a] = dims[a]; }
    geo.cell_length = cell_length;
    geo.total = u32(dims[0]) * u32(dims[1]) * u32(dims[2]);
    geo.inv_bin = 1.0f / cell_length;
    geo.inv_stencil = geo.inv_bin;
    const GridDev<float> g = to_dev<float>(geo);
    const size_t cells = size_t(geo.total) + 1;
    if (n == 0) {
        // count == 0 leaves the grid untouched (cell_grid.cu:74-77)
        return;
    }
    const u32 n_tiles = u32((cells + SCAN_TILE - 1) / SCAN_TILE);
    // one allocation for every temporary
    const size_t words = cells /*count*/ + (cells + 1) /*starts*/ + (n_tiles + 1) + 7 * size_t(n);
    const size_t vbytes = 4 * size_t(n) * sizeof(R4<float>);
    unsigned char* mem = nullptr;
    DFSPH_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&mem), vbytes + words * sizeof(u32), st));
    R4<float>* x_in = reinterpret_cast<R4<float>*>(mem);
    R4<float>* x_out = x_in + n;
    R4<float>* v_in = x_out + n;
    R4<float>* v_out = v_in + n;
    u32* w = reinterpret_cast<u32*>(mem + vbytes);
    u32* count = w; w += cells;
    u32* starts = w; w += cells + 1;  // cell_start with its closing entry
    u32* tiles = w; w += n_tiles + 1;
    u32* key = w; w += n;
    u32* rank = w; w += n;
    u32* id0 = w; w += n;
    u32* tsrc = w; w += n;
    u32* tid = w; w += n;
    u32* idn = w; w += n;
    u32* ks = w; w += n;
    DFSPH_CUDA(cudaMemsetAsync(count, 0, cells * sizeof(u32), st));
    DFSPH_CUDA(cudaMemsetAsync(v_in, 0, size_t(n) * sizeof(R4<float>), st));
    IterCtl* ctl = nullptr;
    DFSPH_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&ctl), sizeof(IterCtl), st));
    DFSPH_CUDA(cudaMemsetAsync(ctl, 0, sizeof(IterCtl), st));
    import_kernel<float><<<blocks_for(n, 256), 256, 0, st>>>(int(n), xyz, nullptr, x_in, v_in, id0);
    DFSPH_LAUNCHED();
    count_kernel<float><<<blocks_for(n, 256), 256, 0, st>>>(int(n), x_in, g, key, rank, count, nullptr);
    DFSPH_LAUNCHED();
    const u32 m = geo.total + 1;
    scan_tile_sums<<<n_tiles, SCAN_BLOCK, 0, st>>>(count, m, tiles, nullptr, 0u);
    DFSPH_LAUNCHED();
    scan_tile_offsets<<<1, 1024, 0, st>>>(tiles, n_tiles, starts + m, nullptr, 0, nullptr, 0, nullptr, m, 0u, nullptr);
    DFSPH_LAUNCHED();
    scan_tiles<<<n_tiles, SCAN_BLOCK, 0, st>>>(count, m, tiles, starts, nullptr);
    DFSPH_LAUNCHED();
    scatter_kernel<<<blocks_for(n, 256), 256, 0, st>>>(int(n), key, rank, starts, id0, tsrc, tid);
    DFSPH_LAUNCHED();
    reorder_kernel<float><<<blocks_for(n, 256), 256, 0, st>>>(int(n), tsrc, tid, key, starts, m, ~0u, x_in, v_in,
                                                              x_out, v_out, idn, ks, ctl);
    DFSPH_LAUNCHED();
    DFSPH_CUDA(cudaMemcpyAsync(cell_start, starts, size_t(m) * sizeof(u32), cudaMemcpyDeviceToDevice, st));
    if (sorted_keys) DFSPH_CUDA(cudaMemcpyAsync(sorted_keys, ks, size_t(n) * sizeof(u32), cudaMemcpyDeviceToDevice, st));
    if (sorted_idx) DFSPH_CUDA(cudaMemcpyAsync(sorted_idx, idn, size_t(n) * sizeof(u32), cudaMemcpyDeviceToDevice, st));
    DFSPH_CUDA(cudaFreeAsync(ctl, st));
    DFSPH_CUDA(cudaFreeAsync(mem, st));
}

}  // namespace dfsph
