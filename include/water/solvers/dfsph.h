// DFSPHSolver: the reference's solver class (solvers/dfsph/include/water/solvers/
// dfsph.h:17-84) as a header-only façade over the GB300 C ABI. It keeps the
// reference's construction contract (registers dfsph_density, dfsph_alpha,
// dfsph_kappa, dfsph_density_adv on the caller's fluid store and
// dfsph_boundary_mass on the boundary store, builds the boundary grid once,
// calibrates the Akinci masses) and its step(dt) semantics on the caller's
// ParticleStore buffers; the step itself runs in libdfsph_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <stdexcept>
#include <string>

#include "dfsph_gb300.h"
#include "water/core/cell_grid.h"
#include "water/core/particle_store.h"
#include "water/core/timestep.h"
#include "water/core/types.h"

namespace water::solvers {

namespace detail {
[[noreturn]] inline void throw_status(int status, const dfsph_ctx* ctx, const char* where) {
    const std::string msg = std::string(where) + ": " + dfsph_status_string(status) + ": " + dfsph_last_error(ctx);
    if (status == DFSPH_ERR_OUT_OF_RANGE) throw std::out_of_range(msg);
    if (status == DFSPH_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}
inline void check(int status, const dfsph_ctx* ctx, const char* where) {
    if (status != DFSPH_OK) throw_status(status, ctx, where);
}
}  // namespace detail

class DFSPHSolver {
public:
    struct Config {
        f32 rest_density = 1000.0f;
        f32 particle_radius = 0.0015f;
        f32 smoothing_length = 0.003f;
        f32 viscosity = 1e-3f;
        f32 damping = 0.5f;
        f32 surface_tension = 0.0f;
        Vec3f gravity{0.0f, -9.81f, 0.0f};
        u32 max_density_iters = 100;
        u32 max_divergence_iters = 100;
        f32 eta_density = 1e-3f;
        f32 eta_divergence = 1e-3f;
        Vec3f domain_min{0.0f, 0.0f, 0.0f};
        Vec3f domain_max{1.0f, 1.0f, 1.0f};
        // GB300 extensions. The reference declares the divergence fields but
        // never runs a divergence solve; it runs here only when enabled.
        bool enable_divergence_solver = false;
        u32 precision = DFSPH_PRECISION_FP32;
        // step_frame runs a whole frame as one CUDA graph launch, with the
        // substep size chosen on the device, when the iteration counts are
        // fixed (eta = 0); otherwise it runs the host loop.
        bool device_frames = true;
    };

    DFSPHSolver(ParticleStore& fluid, ParticleStore* boundary, Config cfg, cudaStream_t stream = 0)
        : fluid_(fluid), boundary_(boundary), cfg_(cfg), stream_(stream) {
        dfsph_config c;
        dfsph_config_init(&c);
        c.rest_density = cfg.rest_density;
        c.particle_radius = cfg.particle_radius;
        c.smoothing_length = cfg.smoothing_length;
        c.viscosity = cfg.viscosity;
        c.damping = cfg.damping;
        c.surface_tension = cfg.surface_tension;
        c.gravity[0] = cfg.gravity.x; c.gravity[1] = cfg.gravity.y; c.gravity[2] = cfg.gravity.z;
        c.max_density_iters = cfg.max_density_iters;
        c.max_divergence_iters = cfg.enable_divergence_solver ? cfg.max_divergence_iters : 0u;
        c.eta_density = cfg.eta_density;
        c.eta_divergence = cfg.eta_divergence;
        c.domain_min[0] = cfg.domain_min.x; c.domain_min[1] = cfg.domain_min.y; c.domain_min[2] = cfg.domain_min.z;
        c.domain_max[0] = cfg.domain_max.x; c.domain_max[1] = cfg.domain_max.y; c.domain_max[2] = cfg.domain_max.z;
        c.precision = cfg.precision;
        c.use_cuda_graph = cfg.device_frames ? 1u : 0u;
        c.capacity = static_cast<uint32_t>(fluid.capacity());
        c.boundary_capacity = boundary ? static_cast<uint32_t>(boundary->capacity()) : 0u;
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
        dfsph_ctx* ctx = nullptr;
        detail::check(dfsph_create(&c, dev, stream, &ctx), nullptr, "DFSPHSolver");
        ctx_.reset(ctx);
        float origin[3];
        int dims[3];
        dfsph_grid_geometry(&c, origin, dims);
        fluid_grid_ = std::make_unique<CellGrid>(Vec3f{origin[0], origin[1], origin[2]}, Vec3i{dims[0], dims[1], dims[2]},
                                                 cfg.smoothing_length, stream);
        fluid_grid_->reserve(fluid.capacity());
        const float spacing = 2.0f * cfg.particle_radius;
        mass_ = cfg.rest_density * (spacing * spacing * spacing);

        density_ = fluid_.register_attribute<f32>("dfsph_density", AttribType::F32);
        alpha_ = fluid_.register_attribute<f32>("dfsph_alpha", AttribType::F32);
        kappa_ = fluid_.register_attribute<f32>("dfsph_kappa", AttribType::F32);
        density_adv_ = fluid_.register_attribute<f32>("dfsph_density_adv", AttribType::F32);

        if (boundary_) {
            boundary_mass_ = boundary_->register_attribute<f32>("dfsph_boundary_mass", AttribType::F32);
            boundary_grid_ = std::make_unique<CellGrid>(Vec3f{origin[0], origin[1], origin[2]},
                                                        Vec3i{dims[0], dims[1], dims[2]}, cfg.smoothing_length, stream);
            boundary_grid_->reserve(boundary_->capacity());
            const uint32_t nb = static_cast<uint32_t>(boundary_->count());
            detail::check(dfsph_set_boundary(ctx_.get(), reinterpret_cast<const float*>(boundary_->positions()), nb,
                                             DFSPH_MEM_DEVICE),
                          ctx_.get(), "DFSPHSolver: boundary");
            if (nb) {
                detail::check(dfsph_get_field(ctx_.get(), DFSPH_FIELD_BOUNDARY_MASS,
                                              boundary_->attribute_data(boundary_mass_), nb * sizeof(float),
                                              DFSPH_MEM_DEVICE),
                              ctx_.get(), "DFSPHSolver: boundary mass");
                const std::size_t cs = (static_cast<std::size_t>(boundary_grid_->total_cells()) + 1) * sizeof(u32);
                detail::check(dfsph_get_field(ctx_.get(), DFSPH_FIELD_BOUNDARY_CELL_START,
                                              boundary_grid_->mutable_cell_start(), cs, DFSPH_MEM_DEVICE),
                              ctx_.get(), "DFSPHSolver: boundary grid");
                detail::check(dfsph_get_field(ctx_.get(), DFSPH_FIELD_BOUNDARY_SORTED_INDEX,
                                              boundary_grid_->mutable_sorted_indices(), nb * sizeof(u32),
                                              DFSPH_MEM_DEVICE),
                              ctx_.get(), "DFSPHSolver: boundary grid");
            }
        }
    }

    DFSPHSolver(const DFSPHSolver&) = delete;
    DFSPHSolver& operator=(const DFSPHSolver&) = delete;

    // DFSPHSolver::step (solvers/dfsph/src/dfsph.cu:120-133) on the caller's store.
    void step(f32 dt) {
        const std::size_t n = fluid_.count();
        if (n == 0) return;
        detail::check(dfsph_step_store(ctx_.get(), reinterpret_cast<float*>(fluid_.positions()),
                                       reinterpret_cast<float*>(fluid_.velocities()), static_cast<uint32_t>(n), dt,
                                       fluid_.attribute_data(density_), fluid_.attribute_data(alpha_),
                                       fluid_.attribute_data(kappa_), fluid_.attribute_data(density_adv_)),
                      ctx_.get(), "DFSPHSolver::step");
        grid_dirty_ = true;
        stats_dirty_ = true;
    }

    // One frame of CFL substeps on the caller's store: sim_cli's loop
    // (apps/sim_cli/main.cpp:171-181) with TimeStepper::next_dt, each dt from
    // max(max |v|, min_velocity); no counterpart in the reference's library.
    // Returns the number of substeps taken. Each frame imports the store as
    // new state, so with compensated position updates the carries span one
    // frame's substeps (consecutive step() calls keep them across steps).
    u32 step_frame(const TimeStepper& ts, f32 frame_dt, f32 min_velocity = 0.5f, u32 max_substeps_per_frame = 64) {
        const std::size_t n = fluid_.count();
        const TimeStepper::Config tc = ts.config();
        dfsph_frame_config fc;
        dfsph_frame_config_init(&fc);
        fc.frame_dt = frame_dt;
        fc.stepper_frame_dt = tc.frame_dt;
        fc.dt_max = tc.dt_max;
        fc.cfl_lambda = tc.cfl_lambda;
        fc.max_substeps = tc.max_substeps;
        fc.min_velocity = min_velocity;
        fc.max_substeps_per_frame = max_substeps_per_frame;
        detail::check(dfsph_set_fluid(ctx_.get(), reinterpret_cast<const float*>(fluid_.positions()),
                                      reinterpret_cast<const float*>(fluid_.velocities()), static_cast<uint32_t>(n),
                                      DFSPH_MEM_DEVICE),
                      ctx_.get(), "DFSPHSolver::step_frame");
        uint32_t sub = 0;
        detail::check(dfsph_step_frames(ctx_.get(), &fc, 1, &sub), ctx_.get(), "DFSPHSolver::step_frame");
        if (n) {
            const std::size_t v3 = n * sizeof(Vec3f), s1 = n * sizeof(f32);
            const struct { int field; void* dst; std::size_t bytes; } outs[] = {
                {DFSPH_FIELD_POSITION, fluid_.positions(), v3},
                {DFSPH_FIELD_VELOCITY, fluid_.velocities(), v3},
                {DFSPH_FIELD_DENSITY, fluid_.attribute_data(density_), s1},
                {DFSPH_FIELD_ALPHA, fluid_.attribute_data(alpha_), s1},
                {DFSPH_FIELD_KAPPA, fluid_.attribute_data(kappa_), s1},
                {DFSPH_FIELD_DENSITY_ADV, fluid_.attribute_data(density_adv_), s1},
            };
            for (const auto& o : outs)
                detail::check(dfsph_get_field(ctx_.get(), o.field, o.dst, o.bytes, DFSPH_MEM_DEVICE), ctx_.get(),
                              "DFSPHSolver::step_frame");
        }
        grid_dirty_ = true;
        stats_dirty_ = true;
        return sub;
    }

    // State file of the run (dfsph_save_state): the store's fluid and the
    // walls. No counterpart in the reference, which cannot resume.
    void save_state(const std::string& path) {
        const std::size_t n = fluid_.count();
        detail::check(dfsph_set_fluid(ctx_.get(), reinterpret_cast<const float*>(fluid_.positions()),
                                      reinterpret_cast<const float*>(fluid_.velocities()), static_cast<uint32_t>(n),
                                      DFSPH_MEM_DEVICE),
                      ctx_.get(), "DFSPHSolver::save_state");
        detail::check(dfsph_save_state(ctx_.get(), path.c_str()), ctx_.get(), "DFSPHSolver::save_state");
    }
    // Resumes a saved run: the store is resized to the saved count (within its
    // capacity) and takes the saved positions and velocities.
    void load_state(const std::string& path) {
        detail::check(dfsph_load_state(ctx_.get(), path.c_str()), ctx_.get(), "DFSPHSolver::load_state");
        double count = 0.0;
        detail::check(dfsph_get_scalar(ctx_.get(), DFSPH_SCALAR_FLUID_COUNT, &count), ctx_.get(),
                      "DFSPHSolver::load_state");
        const std::size_t n = static_cast<std::size_t>(count);
        fluid_.resize(n);
        if (n) {
            detail::check(dfsph_get_field(ctx_.get(), DFSPH_FIELD_POSITION, fluid_.positions(), n * sizeof(Vec3f),
                                          DFSPH_MEM_DEVICE),
                          ctx_.get(), "DFSPHSolver::load_state");
            detail::check(dfsph_get_field(ctx_.get(), DFSPH_FIELD_VELOCITY, fluid_.velocities(), n * sizeof(Vec3f),
                                          DFSPH_MEM_DEVICE),
                          ctx_.get(), "DFSPHSolver::load_state");
        }
        grid_dirty_ = true;
        stats_dirty_ = true;
    }

    // Largest particle speed after the last step (0 before the first step).
    f32 max_velocity() const noexcept {
        refresh_stats();
        return max_velocity_;
    }
    u32 last_density_iters() const noexcept {
        refresh_stats();
        return last_density_iters_;
    }

    const CellGrid& fluid_grid() const {
        if (grid_dirty_) {
            const std::size_t n = fluid_.count();
            const std::size_t cs = (static_cast<std::size_t>(fluid_grid_->total_cells()) + 1) * sizeof(u32);
            detail::check(dfsph_get_field(ctx_.get(), DFSPH_FIELD_CELL_START, fluid_grid_->mutable_cell_start(), cs,
                                          DFSPH_MEM_DEVICE),
                          ctx_.get(), "DFSPHSolver::fluid_grid");
            if (n)
                detail::check(dfsph_get_field(ctx_.get(), DFSPH_FIELD_SORTED_INDEX, fluid_grid_->mutable_sorted_indices(),
                                              n * sizeof(u32), DFSPH_MEM_DEVICE),
                              ctx_.get(), "DFSPHSolver::fluid_grid");
            grid_dirty_ = false;
        }
        return *fluid_grid_;
    }
    const CellGrid* boundary_grid() const noexcept { return boundary_grid_.get(); }
    f32 particle_mass() const noexcept { return mass_; }

    // synchronous device -> host reads (dfsph.cu:330-353)
    f32 density_at(std::size_t i) const { return read_one(fluid_.attribute_data(density_), i); }
    f32 alpha_at(std::size_t i) const { return read_one(fluid_.attribute_data(alpha_), i); }
    f32 boundary_mass_at(std::size_t i) const {
        if (!boundary_) return 0.0f;
        return read_one(boundary_->attribute_data(boundary_mass_), i);
    }

    dfsph_ctx* native() const noexcept { return ctx_.get(); }

private:
    struct CtxDeleter {
        void operator()(dfsph_ctx* c) const { dfsph_destroy(c); }
    };

    f32 read_one(const f32* dev, std::size_t i) const {
        f32 v = 0.0f;
        WATER_CUDA_CHECK(cudaStreamSynchronize(stream_));
        WATER_CUDA_CHECK(cudaMemcpy(&v, dev + i, sizeof(f32), cudaMemcpyDeviceToHost));
        return v;
    }

    void refresh_stats() const noexcept {
        if (!stats_dirty_) return;
        double v = 0.0, it = 0.0;
        if (dfsph_get_scalar(ctx_.get(), DFSPH_SCALAR_MAX_VELOCITY, &v) == DFSPH_OK &&
            dfsph_get_scalar(ctx_.get(), DFSPH_SCALAR_LAST_DENSITY_ITERS, &it) == DFSPH_OK) {
            max_velocity_ = static_cast<f32>(v);
            last_density_iters_ = static_cast<u32>(it);
            stats_dirty_ = false;
        }
    }

    ParticleStore& fluid_;
    ParticleStore* boundary_;
    Config cfg_;
    cudaStream_t stream_;
    std::unique_ptr<dfsph_ctx, CtxDeleter> ctx_;
    std::unique_ptr<CellGrid> fluid_grid_;
    std::unique_ptr<CellGrid> boundary_grid_;
    f32 mass_ = 0.0f;
    mutable f32 max_velocity_ = 0.0f;
    mutable u32 last_density_iters_ = 0;
    mutable bool grid_dirty_ = false;
    mutable bool stats_dirty_ = false;
    AttribHandle<f32> density_, alpha_, kappa_, density_adv_, boundary_mass_;
};

}  // namespace water::solvers
