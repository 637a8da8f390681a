// Interface between the C ABI layer and the per-precision solvers.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <memory>

#include "../../include/dfsph_gb300.h"

namespace dfsph {

// The device reciprocal 1.0f / l as the reference's stencil code evaluates it
// (compiled with the reference's -use_fast_math in its own translation unit).
float device_stencil_reciprocal(float cell_length, cudaStream_t stream);

// Polymorphic face of the per-precision solvers.
struct SolverBase {
    virtual ~SolverBase() = default;
    virtual void set_stream(cudaStream_t s) = 0;
    virtual void set_boundary(const float* xyz, std::uint32_t n, int mem) = 0;
    virtual void set_fluid(const float* xyz, const float* vel, std::uint32_t n, int mem) = 0;
    virtual void set_fluid_batch(std::uint32_t n_scenes, const std::uint32_t* counts, const float* xyz,
                                 const float* vel, int mem) = 0;
    virtual void set_scene_viscosity(const float* eps, std::uint32_t n_scenes) = 0;
    virtual void get_scene_max_velocity(float* out, std::uint32_t n_scenes) = 0;
    virtual void step(float dt, std::uint32_t n_steps) = 0;
    virtual void step_store(float* pos, float* vel, std::uint32_t n, float dt, float* density, float* alpha,
                            float* kappa, float* density_adv) = 0;
    virtual void get_field(int field, void* dst, std::size_t bytes, int mem) = 0;
    virtual void get_state(float* pos, float* vel, int mem) = 0;
    virtual double get_scalar(int which) = 0;
    virtual void synchronize() = 0;
    // Throws DFSPH_ERR_DEVICE_TIMEOUT (and clears the word) when a bounded
    // device wait gave up since the last check; call after the stream synced.
    virtual void check_device_status() = 0;
    virtual void set_wait_limit(unsigned long long limit_ns, std::uint32_t missing_blocks) = 0;
    virtual void profile_enable(std::uint32_t mask) = 0;
    virtual void profile_read(int kclass, double* total_ms, unsigned long long* count) = 0;
    virtual void step_frames(const dfsph_frame_config& fc, std::uint32_t n_frames, std::uint32_t* substeps) = 0;
    virtual void autotune(float dt, std::uint32_t steps, int* chosen) = 0;
    virtual void save_state(const char* path) = 0;
    virtual void load_state(const char* path) = 0;
    virtual void block_sizes(int* out) const = 0;
    // differentiable rollout; arrays hold the working type (float or double)
    virtual void adjoint_set_state(const void* pos, const void* vel, std::uint32_t n, int mem) = 0;
    virtual void adjoint_get_state(void* pos, void* vel, int mem) = 0;
    virtual void adjoint_forward(float dt, std::uint32_t n_steps, std::uint32_t checkpoint_every) = 0;
    virtual void adjoint_backward(const void* pos_bar, const void* vel_bar, void* pos0_bar, void* vel0_bar,
                                  double* xsph_bar, int mem) = 0;
};

std::unique_ptr<SolverBase> make_solver_fp32(const dfsph_config& cfg, int device, cudaStream_t s);
std::unique_ptr<SolverBase> make_solver_fp64(const dfsph_config& cfg, int device, cudaStream_t s);

// CellGrid::build (core/src/cell_grid.cu:73-138) on an arbitrary grid.
void build_cell_grid(const float* xyz, std::uint32_t n, const float origin[3], const int dims[3],
                     float cell_length, std::uint32_t* sorted_keys, std::uint32_t* sorted_idx,
                     std::uint32_t* cell_start, cudaStream_t st);

// SpatialAccel's Morton order (core/src/spatial_accel.cu:11-40,158-179).
void morton_sort(const float* xyz, std::uint32_t n, const float smin[3], const float smax[3],
                 std::uint32_t* sorted_codes, std::uint32_t* sorted_idx, cudaStream_t st);

// SpatialAccel::build (core/src/spatial_accel.cu:110-179) with the bottom-up
// box pass, and its refit on moved positions.
void lbvh_build(const float* xyz, std::uint32_t n, const float smin[3], const float smax[3], float radius,
                std::uint32_t* codes, std::uint32_t* sorted, std::uint32_t* left, std::uint32_t* right,
                std::uint32_t* parent, float* boxes, std::uint32_t* scratch, cudaStream_t st);
void lbvh_refit(const float* xyz, std::uint32_t n, float radius, const std::uint32_t* sorted,
                const std::uint32_t* left, const std::uint32_t* right, const std::uint32_t* parent, float* boxes,
                std::uint32_t* scratch, cudaStream_t st);

// Akinci cohesion kernel C(r, l) (core/include/water/core/sph_kernels.cuh:43-51).
void cohesion(const float* r, std::uint32_t n, float l, float* out, cudaStream_t st);

}  // namespace dfsph
