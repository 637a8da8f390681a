// sample_aabb_boundary: static wall particles on the six inner faces of a box,
// n_layers inward layers at `spacing` (edges and corners emitted by every face
// that touches them). Same signature and points as the reference
// (solvers/dfsph/include/water/solvers/boundary_sampler.h:24-25); computed by
// dfsph_sample_aabb_boundary in the GB300 library.
#pragma once

#include <stdexcept>
#include <vector>

#include "dfsph_gb300.h"
#include "water/core/types.h"

namespace water::solvers {

inline std::vector<Vec3f> sample_aabb_boundary(Vec3f lo, Vec3f hi, f32 spacing, int n_layers = 3) {
    const float l[3] = {lo.x, lo.y, lo.z};
    const float h[3] = {hi.x, hi.y, hi.z};
    const int64_t n = dfsph_sample_aabb_boundary(l, h, spacing, n_layers, nullptr, 0);
    if (n < 0) throw std::invalid_argument("sample_aabb_boundary: spacing must be > 0 and n_layers >= 0");
    std::vector<Vec3f> pts(static_cast<std::size_t>(n));
    dfsph_sample_aabb_boundary(l, h, spacing, n_layers, reinterpret_cast<float*>(pts.data()), n);
    return pts;
}

}  // namespace water::solvers
