// Host-side pieces shared by every solver instantiation: grid geometry, error
// formatting and the boundary sampler.
#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/dfsph_gb300.h"
#include "common.cuh"

namespace dfsph {

[[noreturn]] void throw_cuda(cudaError_t e, const char* expr, const char* file, int line) {
    // reset the runtime's last-error slot, so that a recoverable error does not
    // resurface at the next launch check
    cudaGetLastError();
    std::string m = "CUDA error at ";
    m += file; m += ":"; m += std::to_string(line);
    m += " (";  m += expr; m += "): ";
    m += cudaGetErrorString(e);
    throw Error(DFSPH_ERR_CUDA, m);
}

// make_grid (solvers/dfsph/src/dfsph.cu:55-65): dims = ceil(extent / l) + 2
// evaluated in float, origin one cell below domain_min, cell length l.
GridGeom make_grid_geom(const float dmin[3], const float dmax[3], float l) {
    GridGeom g;
    for (int a = 0; a < 3; ++a) {
        const float ext = dmax[a] - dmin[a];
        g.dims[a] = static_cast<int>(std::ceil(ext / l)) + 2;
        g.origin[a] = dmin[a] - l;
    }
    g.cell_length = l;
    g.total = static_cast<u32>(g.dims[0]) * static_cast<u32>(g.dims[1]) * static_cast<u32>(g.dims[2]);
    g.inv_bin = 1.0f / l;
    g.inv_stencil = g.inv_bin;
    return g;
}

}  // namespace dfsph

// water::solvers::sample_aabb_boundary (solvers/dfsph/src/boundary_sampler.cpp:6-32):
// for each of the six faces, n_layers inward layers, u/v walked with float
// accumulation up to hi + spacing/2, so edges and corners are emitted by every
// face that touches them. Built with -ffp-contract=off so that the float
// arithmetic is the same on every host architecture.
extern "C" int64_t dfsph_sample_aabb_boundary(const float lo[3], const float hi[3], float spacing,
                                              int n_layers, float* out, int64_t cap) {
    if (!lo || !hi || !(spacing > 0.0f) || n_layers < 0) return -DFSPH_ERR_INVALID_ARGUMENT;
    int64_t count = 0;
    const int axes[6] = {0, 0, 1, 1, 2, 2};
    for (int f = 0; f < 6; ++f) {
        const int axis = axes[f];
        const bool low_face = (f % 2) == 0;
        const float face = low_face ? lo[axis] : hi[axis];
        const float step = low_face ? spacing : -spacing;
        const int ua = (axis + 1) % 3, va = (axis + 2) % 3;
        for (int layer = 0; layer < n_layers; ++layer) {
            const float pos = face + static_cast<float>(layer) * step;
            for (float u = lo[ua]; u <= hi[ua] + 0.5f * spacing; u += spacing)
                for (float w = lo[va]; w <= hi[va] + 0.5f * spacing; w += spacing) {
                    if (out && count < cap) {
                        float* p = out + 3 * count;
                        p[axis] = pos;
                        p[ua] = u;
                        p[va] = w;
                    }
                    ++count;
                }
        }
    }
    return count;
}
