// CellGrid: uniform grid for fixed-radius neighbour queries, rebuilt with
// build(positions, count). Same interface as the reference
// (core/include/water/core/cell_grid.h:16-50); the build runs the GB300
// library's counting sort (dfsph_build_cell_grid) and yields the same arrays:
// sorted keys, the stable (key, index) permutation and cell_start[C+1] with
// empty cells pointing at the next start and cell_start[C] = in-grid count.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "dfsph_gb300.h"
#include "water/core/device_buffer.h"
#include "water/core/types.h"

namespace water {

class CellGrid {
public:
    CellGrid(Vec3f origin, Vec3i cells_per_axis, f32 cell_length, cudaStream_t stream = 0)
        : origin_(origin), cells_per_axis_(cells_per_axis), cell_length_(cell_length), stream_(stream),
          cell_start_(static_cast<std::size_t>(total_cells()) + 1, stream) {
        cell_start_.fill_zero();
    }

    void reserve(std::size_t capacity) {
        if (capacity <= capacity_) return;
        capacity_ = capacity;
        cell_ids_ = DeviceBuffer<u32>(capacity, stream_);
        sorted_indices_ = DeviceBuffer<u32>(capacity, stream_);
    }

    void build(const Vec3f* positions, std::size_t count) {
        if (count == 0) {  // core/src/cell_grid.cu:74-77
            count_ = 0;
            return;
        }
        if (count > capacity_) reserve(count);
        count_ = count;
        const float o[3] = {origin_.x, origin_.y, origin_.z};
        const int d[3] = {cells_per_axis_.x, cells_per_axis_.y, cells_per_axis_.z};
        const int st = dfsph_build_cell_grid(reinterpret_cast<const float*>(positions), static_cast<uint32_t>(count),
                                             o, d, cell_length_, cell_ids_.data(), sorted_indices_.data(),
                                             cell_start_.data(), stream_);
        if (st != DFSPH_OK)
            throw std::runtime_error(std::string("CellGrid::build: ") + dfsph_status_string(st) + ": " +
                                     dfsph_last_error(nullptr));
    }

    // a grid whose arrays are filled by the owner (the solver façade)
    u32* mutable_cell_start() noexcept { return cell_start_.data(); }
    u32* mutable_sorted_indices() noexcept { return sorted_indices_.data(); }

    const u32* cell_start() const noexcept { return cell_start_.data(); }
    const u32* sorted_indices() const noexcept { return sorted_indices_.data(); }
    Vec3f origin() const noexcept { return origin_; }
    Vec3i cells_per_axis() const noexcept { return cells_per_axis_; }
    f32 cell_length() const noexcept { return cell_length_; }
    u32 total_cells() const noexcept {
        return static_cast<u32>(cells_per_axis_.x) * static_cast<u32>(cells_per_axis_.y) *
               static_cast<u32>(cells_per_axis_.z);
    }
    cudaStream_t stream() const noexcept { return stream_; }
    std::size_t count() const noexcept { return count_; }

private:
    Vec3f origin_;
    Vec3i cells_per_axis_;
    f32 cell_length_;
    cudaStream_t stream_;
    std::size_t capacity_ = 0;
    std::size_t count_ = 0;
    DeviceBuffer<u32> cell_ids_;
    DeviceBuffer<u32> sorted_indices_;
    DeviceBuffer<u32> cell_start_;
};

}  // namespace water
