// The C ABI (include/dfsph_gb300.h): argument checks, dispatch to the solver
// of the configured precision, and exception -> status translation. Nothing
// throws across this boundary.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/dfsph_gb300.h"
#include "common.cuh"
#include "solver_api.h"

struct dfsph_ctx {
    std::unique_ptr<dfsph::SolverBase> solver;
    dfsph_config cfg;
    int device = 0;
    std::string last_error;
    unsigned long long wait_ns = 1000000000ull;  // bounded device waits (dfsph_set_wait_limit)
    uint32_t wait_missing = 0;                   // dfsph_test_stall_waits
};

namespace {

thread_local std::string g_create_error;

template <class F> int guarded(dfsph_ctx* ctx, F&& f) {
    try {
        f();
        return DFSPH_OK;
    } catch (const dfsph::Error& e) {
        if (ctx) ctx->last_error = e.what();
        else g_create_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->last_error = "host allocation failed";
        else g_create_error = "host allocation failed";
        return DFSPH_ERR_CUDA;
    } catch (const std::exception& e) {
        if (ctx) ctx->last_error = e.what();
        else g_create_error = e.what();
        return DFSPH_ERR_INVALID_ARGUMENT;
    }
}

bool finite3(const float v[3]) {
    for (int a = 0; a < 3; ++a)
        if (!(v[a] == v[a]) || v[a] > 3.0e38f || v[a] < -3.0e38f) return false;
    return true;
}

}  // namespace

extern "C" {

int dfsph_config_init(dfsph_config* c) {
    if (!c) return DFSPH_ERR_INVALID_ARGUMENT;
    std::memset(c, 0, sizeof(*c));
    // DFSPHSolver::Config defaults (solvers/dfsph/include/water/solvers/dfsph.h:19-33)
    c->rest_density = 1000.0f;
    c->particle_radius = 0.0015f;
    c->smoothing_length = 0.003f;
    c->viscosity = 1e-3f;
    c->damping = 0.5f;
    c->surface_tension = 0.0f;
    c->gravity[0] = 0.0f; c->gravity[1] = -9.81f; c->gravity[2] = 0.0f;
    c->max_density_iters = 100;
    c->max_divergence_iters = 100;
    c->eta_density = 1e-3f;
    c->eta_divergence = 1e-3f;
    c->domain_min[0] = c->domain_min[1] = c->domain_min[2] = 0.0f;
    c->domain_max[0] = c->domain_max[1] = c->domain_max[2] = 1.0f;
    c->precision = DFSPH_PRECISION_FP32;
    c->capacity = 0;
    c->boundary_capacity = 0;
    c->record_diagnostics = 0;
    c->n_scenes = 1;
    c->use_cuda_graph = 0;
    return DFSPH_OK;
}

int dfsph_grid_geometry(const dfsph_config* cfg, float origin[3], int dims[3]) {
    if (!cfg || !origin || !dims) return DFSPH_ERR_INVALID_ARGUMENT;
    const dfsph::GridGeom g = dfsph::make_grid_geom(cfg->domain_min, cfg->domain_max, cfg->smoothing_length);
    for (int a = 0; a < 3; ++a) { origin[a] = g.origin[a]; dims[a] = g.dims[a]; }
    return DFSPH_OK;
}

int dfsph_create(const dfsph_config* cfg, int device, void* stream, dfsph_ctx** out) {
    if (!cfg || !out) return DFSPH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!(cfg->smoothing_length > 0.0f) || !(cfg->particle_radius > 0.0f) || !(cfg->rest_density > 0.0f) ||
        !finite3(cfg->domain_min) || !finite3(cfg->domain_max)) {
        g_create_error = "dfsph_create: smoothing_length, particle_radius and rest_density must be > 0 and the domain finite";
        return DFSPH_ERR_INVALID_ARGUMENT;
    }
    for (int a = 0; a < 3; ++a)
        if (!(cfg->domain_max[a] > cfg->domain_min[a])) {
            g_create_error = "dfsph_create: domain_max must exceed domain_min on every axis";
            return DFSPH_ERR_INVALID_ARGUMENT;
        }
    if (cfg->precision > DFSPH_PRECISION_FP32_COMPENSATED) {
        g_create_error = "dfsph_create: unknown precision";
        return DFSPH_ERR_INVALID_ARGUMENT;
    }
    if (cfg->slot_order > DFSPH_ORDER_MORTON) {
        g_create_error = "dfsph_create: unknown slot order";
        return DFSPH_ERR_INVALID_ARGUMENT;
    }
    {
        const dfsph::GridGeom g = dfsph::make_grid_geom(cfg->domain_min, cfg->domain_max, cfg->smoothing_length);
        const double cells = double(g.dims[0]) * double(g.dims[1]) * double(g.dims[2]);
        if (g.dims[0] <= 0 || g.dims[1] <= 0 || g.dims[2] <= 0 || cells >= 4294967295.0) {
            g_create_error = "dfsph_create: the uniform grid needs fewer than 2^32 cells";
            return DFSPH_ERR_INVALID_ARGUMENT;
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        g_create_error = "dfsph_create: no CUDA device";
        return DFSPH_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) {
        g_create_error = "dfsph_create: device index out of range";
        return DFSPH_ERR_INVALID_ARGUMENT;
    }
    dfsph_ctx* ctx = new (std::nothrow) dfsph_ctx;
    if (!ctx) return DFSPH_ERR_CUDA;
    ctx->cfg = *cfg;
    ctx->device = device;
    const int st = guarded(nullptr, [&] {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (cfg->precision == DFSPH_PRECISION_FP64)
            ctx->solver = dfsph::make_solver_fp64(*cfg, device, s);
        else
            ctx->solver = dfsph::make_solver_fp32(*cfg, device, s);
    });
    if (st != DFSPH_OK) {
        delete ctx;
        return st;
    }
    *out = ctx;
    return DFSPH_OK;
}

void dfsph_destroy(dfsph_ctx* ctx) {
    if (!ctx) return;
    if (ctx->solver) {
        cudaSetDevice(ctx->device);
        try { ctx->solver->synchronize(); } catch (...) {}
    }
    delete ctx;
}

int dfsph_set_stream(dfsph_ctx* ctx, void* stream) {
    if (!ctx) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] { ctx->solver->set_stream(static_cast<cudaStream_t>(stream)); });
}

int dfsph_set_boundary(dfsph_ctx* ctx, const float* xyz, uint32_t n, int mem) {
    if (!ctx || (n > 0 && !xyz) || (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE))
        return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->set_boundary(xyz, n, mem);
    });
}

int dfsph_set_fluid(dfsph_ctx* ctx, const float* xyz, const float* vel, uint32_t n, int mem) {
    if (!ctx || (n > 0 && !xyz) || (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE))
        return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->set_fluid(xyz, vel, n, mem);
    });
}

int dfsph_set_fluid_batch(dfsph_ctx* ctx, uint32_t n_scenes, const uint32_t* counts, const float* xyz,
                          const float* vel, int mem) {
    if (!ctx || !counts || n_scenes == 0 || (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE))
        return DFSPH_ERR_INVALID_ARGUMENT;
    unsigned long long total = 0;
    for (uint32_t s = 0; s < n_scenes; ++s) total += counts[s];
    if (total > 0 && !xyz) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->set_fluid_batch(n_scenes, counts, xyz, vel, mem);
    });
}

int dfsph_set_scene_viscosity(dfsph_ctx* ctx, const float* viscosity, uint32_t n_scenes) {
    if (!ctx || !viscosity || n_scenes == 0) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->set_scene_viscosity(viscosity, n_scenes);
    });
}

int dfsph_get_scene_max_velocity(dfsph_ctx* ctx, float* out, uint32_t n_scenes) {
    if (!ctx || !out || n_scenes == 0) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->get_scene_max_velocity(out, n_scenes);
    });
}

int dfsph_step(dfsph_ctx* ctx, float dt, uint32_t n_steps) {
    if (!ctx) return DFSPH_ERR_INVALID_ARGUMENT;
    if (!(dt > 0.0f) || dt > 1.0e30f) {
        ctx->last_error = "dfsph_step: dt must be a positive finite number";
        return DFSPH_ERR_INVALID_ARGUMENT;
    }
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->step(dt, n_steps);
    });
}

int dfsph_step_store(dfsph_ctx* ctx, float* pos, float* vel, uint32_t n, float dt, float* density,
                     float* alpha, float* kappa, float* density_adv) {
    if (!ctx || (n > 0 && (!pos || !vel))) return DFSPH_ERR_INVALID_ARGUMENT;
    if (!(dt > 0.0f) || dt > 1.0e30f) {
        ctx->last_error = "dfsph_step_store: dt must be a positive finite number";
        return DFSPH_ERR_INVALID_ARGUMENT;
    }
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->step_store(pos, vel, n, dt, density, alpha, kappa, density_adv);
    });
}

int dfsph_get_state(dfsph_ctx* ctx, float* pos, float* vel, int mem) {
    if (!ctx || (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE)) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->get_state(pos, vel, mem);
        ctx->solver->check_device_status();
    });
}

int dfsph_get_field(dfsph_ctx* ctx, int field, void* dst, size_t dst_bytes, int mem) {
    if (!ctx || !dst || (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE)) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->get_field(field, dst, dst_bytes, mem);
        ctx->solver->check_device_status();
    });
}

int dfsph_get_scalar(dfsph_ctx* ctx, int which, double* out) {
    if (!ctx || !out) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        *out = ctx->solver->get_scalar(which);
    });
}

int dfsph_profile_enable(dfsph_ctx* ctx, uint32_t mask) {
    if (!ctx) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] { ctx->solver->profile_enable(mask); });
}

int dfsph_profile_read(dfsph_ctx* ctx, int kernel_class, double* total_ms, uint64_t* launches) {
    if (!ctx || !total_ms || !launches || kernel_class < 0 || kernel_class >= DFSPH_KERNEL_CLASSES)
        return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        unsigned long long c = 0;
        ctx->solver->profile_read(kernel_class, total_ms, &c);
        *launches = c;
    });
}

int dfsph_set_wait_limit(dfsph_ctx* ctx, uint64_t limit_ns) {
    if (!ctx || limit_ns == 0) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] { ctx->solver->set_wait_limit(limit_ns, ctx->wait_missing); ctx->wait_ns = limit_ns; });
}

int dfsph_test_stall_waits(dfsph_ctx* ctx, uint32_t missing_blocks) {
    if (!ctx) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        ctx->solver->set_wait_limit(ctx->wait_ns, missing_blocks);
        ctx->wait_missing = missing_blocks;
    });
}

int dfsph_synchronize(dfsph_ctx* ctx) {
    if (!ctx) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->synchronize();
    });
}

int dfsph_save_state(dfsph_ctx* ctx, const char* path) {
    if (!ctx || !path) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->save_state(path);
    });
}

int dfsph_load_state(dfsph_ctx* ctx, const char* path) {
    if (!ctx || !path) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->load_state(path);
    });
}

int dfsph_autotune(dfsph_ctx* ctx, float dt, uint32_t steps, int32_t* block_sizes) {
    if (!ctx || !(dt > 0.0f) || dt > 1.0e30f || steps == 0 || steps > 1000) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        int b[DFSPH_KERNEL_CLASSES];
        ctx->solver->autotune(dt, steps, b);
        if (block_sizes)
            for (int k = 0; k < DFSPH_KERNEL_CLASSES; ++k) block_sizes[k] = b[k];
    });
}

int dfsph_get_block_sizes(dfsph_ctx* ctx, int32_t* block_sizes) {
    if (!ctx || !block_sizes) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        int b[DFSPH_KERNEL_CLASSES];
        ctx->solver->block_sizes(b);
        for (int k = 0; k < DFSPH_KERNEL_CLASSES; ++k) block_sizes[k] = b[k];
    });
}

int dfsph_frame_config_init(dfsph_frame_config* fc) {
    if (!fc) return DFSPH_ERR_INVALID_ARGUMENT;
    // TimeStepper::Config (core/include/water/core/timestep.h:10-15) and
    // sim_cli's floor and cap (apps/sim_cli/main.cpp:172,175)
    fc->frame_dt = 1.0f / 24.0f;
    fc->stepper_frame_dt = 1.0f / 24.0f;
    fc->dt_max = 1.0f / 24.0f;
    fc->cfl_lambda = 0.4f;
    fc->max_substeps = 16;
    fc->min_velocity = 0.5f;
    fc->max_substeps_per_frame = 64;
    return DFSPH_OK;
}

int dfsph_step_frames(dfsph_ctx* ctx, const dfsph_frame_config* fc, uint32_t n_frames, uint32_t* substeps) {
    if (!ctx || !fc) return DFSPH_ERR_INVALID_ARGUMENT;
    if (!(fc->frame_dt > 0.0f) || fc->frame_dt > 1.0e30f || !(fc->stepper_frame_dt > 0.0f) ||
        !(fc->dt_max > 0.0f) || !(fc->cfl_lambda > 0.0f) ||
        fc->max_substeps == 0 || fc->max_substeps_per_frame == 0 || !(fc->min_velocity >= 0.0f))
        return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->step_frames(*fc, n_frames, substeps);
        ctx->solver->check_device_status();
    });
}

int dfsph_adjoint_set_state(dfsph_ctx* ctx, const void* pos, const void* vel, uint32_t n, int mem) {
    if (!ctx || (n > 0 && !pos)) return DFSPH_ERR_INVALID_ARGUMENT;
    if (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->adjoint_set_state(pos, vel, n, mem);
    });
}

int dfsph_adjoint_get_state(dfsph_ctx* ctx, void* pos, void* vel, int mem) {
    if (!ctx) return DFSPH_ERR_INVALID_ARGUMENT;
    if (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->adjoint_get_state(pos, vel, mem);
    });
}

int dfsph_adjoint_forward(dfsph_ctx* ctx, float dt, uint32_t n_steps, uint32_t checkpoint_every) {
    if (!ctx || !(dt > 0.0f) || dt > 1.0e30f || n_steps == 0 || checkpoint_every == 0)
        return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->adjoint_forward(dt, n_steps, checkpoint_every);
    });
}

int dfsph_adjoint_backward(dfsph_ctx* ctx, const void* pos_bar, const void* vel_bar, void* pos0_bar,
                           void* vel0_bar, double* xsph_bar, int mem) {
    if (!ctx) return DFSPH_ERR_INVALID_ARGUMENT;
    if (mem != DFSPH_MEM_HOST && mem != DFSPH_MEM_DEVICE) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(ctx, [&] {
        cudaSetDevice(ctx->device);
        ctx->solver->adjoint_backward(pos_bar, vel_bar, pos0_bar, vel0_bar, xsph_bar, mem);
    });
}

const char* dfsph_last_error(const dfsph_ctx* ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->last_error.c_str();
}

const char* dfsph_status_string(int s) {
    switch (s) {
        case DFSPH_OK: return "ok";
        case DFSPH_ERR_INVALID_ARGUMENT: return "invalid argument";
        case DFSPH_ERR_CUDA: return "CUDA error";
        case DFSPH_ERR_OUT_OF_RANGE: return "out of range";
        case DFSPH_ERR_STATE: return "invalid state";
        case DFSPH_ERR_DEVICE_TIMEOUT: return "device wait timed out";
        case DFSPH_ERR_NONFINITE: return "non-finite value";
        case DFSPH_ERR_NO_DEVICE: return "no CUDA device";
        case DFSPH_ERR_IO: return "state file error";
        default: return "unknown status";
    }
}

int dfsph_morton_sort(const float* xyz_dev, uint32_t n, const float scene_min[3], const float scene_max[3],
                      uint32_t* sorted_codes_dev, uint32_t* sorted_indices_dev, void* stream) {
    if ((n > 0 && !xyz_dev) || !scene_min || !scene_max) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(nullptr, [&] {
        dfsph::morton_sort(xyz_dev, n, scene_min, scene_max, sorted_codes_dev, sorted_indices_dev,
                           static_cast<cudaStream_t>(stream));
    });
}

int dfsph_lbvh_build(const float* xyz_dev, uint32_t n, const float scene_min[3], const float scene_max[3],
                     float leaf_radius, uint32_t* codes_dev, uint32_t* sorted_indices_dev, uint32_t* left_dev,
                     uint32_t* right_dev, uint32_t* parent_dev, float* boxes_dev, uint32_t* scratch_dev,
                     void* stream) {
    if (!scene_min || !scene_max || n >= (1u << 30)) return DFSPH_ERR_INVALID_ARGUMENT;
    if (n > 0 && (!xyz_dev || !codes_dev || !sorted_indices_dev || !parent_dev || !boxes_dev))
        return DFSPH_ERR_INVALID_ARGUMENT;
    if (n > 1 && (!left_dev || !right_dev || !scratch_dev)) return DFSPH_ERR_INVALID_ARGUMENT;
    if (!(leaf_radius >= 0.0f) || leaf_radius > 1.0e30f) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(nullptr, [&] {
        dfsph::lbvh_build(xyz_dev, n, scene_min, scene_max, leaf_radius, codes_dev, sorted_indices_dev, left_dev,
                          right_dev, parent_dev, boxes_dev, scratch_dev, static_cast<cudaStream_t>(stream));
    });
}

int dfsph_lbvh_refit(const float* xyz_dev, uint32_t n, float leaf_radius, const uint32_t* sorted_indices_dev,
                     const uint32_t* left_dev, const uint32_t* right_dev, const uint32_t* parent_dev,
                     float* boxes_dev, uint32_t* scratch_dev, void* stream) {
    if (n >= (1u << 30)) return DFSPH_ERR_INVALID_ARGUMENT;
    if (n > 0 && (!xyz_dev || !sorted_indices_dev || !parent_dev || !boxes_dev)) return DFSPH_ERR_INVALID_ARGUMENT;
    if (n > 1 && (!left_dev || !right_dev || !scratch_dev)) return DFSPH_ERR_INVALID_ARGUMENT;
    if (!(leaf_radius >= 0.0f) || leaf_radius > 1.0e30f) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(nullptr, [&] {
        dfsph::lbvh_refit(xyz_dev, n, leaf_radius, sorted_indices_dev, left_dev, right_dev, parent_dev, boxes_dev,
                          scratch_dev, static_cast<cudaStream_t>(stream));
    });
}

int dfsph_cohesion_kernel(const float* r_dev, uint32_t n, float support, float* out_dev, void* stream) {
    if ((n > 0 && (!r_dev || !out_dev)) || !(support > 0.0f)) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(nullptr, [&] { dfsph::cohesion(r_dev, n, support, out_dev, static_cast<cudaStream_t>(stream)); });
}

int dfsph_build_cell_grid(const float* xyz_dev, uint32_t n, const float origin[3], const int dims[3],
                          float cell_length, uint32_t* sorted_keys_dev, uint32_t* sorted_indices_dev,
                          uint32_t* cell_start_dev, void* stream) {
    if ((n > 0 && !xyz_dev) || !origin || !dims || !cell_start_dev || !(cell_length > 0.0f))
        return DFSPH_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < 3; ++a)
        if (dims[a] <= 0) return DFSPH_ERR_INVALID_ARGUMENT;
    if (double(dims[0]) * double(dims[1]) * double(dims[2]) >= 4294967295.0) return DFSPH_ERR_INVALID_ARGUMENT;
    return guarded(nullptr, [&] {
        dfsph::build_cell_grid(xyz_dev, n, origin, dims, cell_length, sorted_keys_dev, sorted_indices_dev,
                               cell_start_dev, static_cast<cudaStream_t>(stream));
    });
}

}  // extern "C"
