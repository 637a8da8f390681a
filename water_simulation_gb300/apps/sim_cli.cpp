// sim_cli: the reference's offline simulation driver (apps/sim_cli/main.cpp)
// on the GB300 library: scene JSON -> lattice block -> DFSPHSolver substeps
// per frame (CFL TimeStepper) -> optional binary frame files.
//
//   sim_cli --scene PATH [--frames START:END] [--record] [--out DIR]
//           [--no-vulkan] [--damping F] [--viscosity F] [--fixed-iters N]
//           [--host-substeps] [--load-state PATH] [--save-state PATH]
//           [--solver-params]
//
// By default each frame is one DFSPHSolver::step_frame: with fixed iteration
// counts (--fixed-iters N: N density iterations, eta = 0) the whole frame is
// one CUDA graph launch whose substep size is chosen on the device;
// --host-substeps runs the reference's host loop of next_dt + step instead.
// --load-state resumes from a state file (positions, velocities, walls)
// written by --save-state after the last frame. --solver-params applies the
// scene's solver_params block (iteration caps, tolerances, divergence solve,
// CFL factor), which the reference parses nowhere.
//
// Frame file format (read by the reference's tools/*.py): little-endian u32 N
// followed by N x 3 float32 positions. --no-vulkan is accepted for
// compatibility; no graphics device is ever created.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "water/core/cuda_check.h"
#include "water/core/particle_store.h"
#include "water/core/timestep.h"
#include "water/scene/scene.h"
#include "water/solvers/boundary_sampler.h"
#include "water/solvers/dfsph.h"

namespace {

struct Args {
    std::string scene_path;
    int frames_start = -1;
    int frames_end = -1;
    bool record = false;
    std::string out_dir = "out";
    float damping = -1.0f;
    float viscosity = -1.0f;
    int fixed_iters = -1;
    bool host_substeps = false;
    std::string load_state;
    std::string save_state;
    bool solver_params = false;
};

[[noreturn]] void usage_exit(int code) {
    std::puts("Usage: sim_cli --scene PATH [--frames START:END] [--record] "
              "[--out DIR] [--no-vulkan] [--damping F] [--viscosity F] [--fixed-iters N] [--host-substeps] "
              "[--load-state PATH] [--save-state PATH] [--solver-params]");
    std::exit(code);
}

// The command line as a table of options: a flag, whether it takes a value,
// and what it sets. Unknown flags, a missing value, a malformed --frames range
// and a missing --scene end the program with status 2; --help with status 0.
struct Option {
    const char* flag;
    bool takes_value;
    void (*apply)(Args&, const char* value);
};

[[noreturn]] void fail(const std::string& msg) {
    std::fprintf(stderr, "%s\n", msg.c_str());
    std::exit(2);
}

void set_frames(Args& a, const char* v) {
    const std::string r = v;
    const auto colon = r.find(':');
    if (colon == std::string::npos) fail("--frames expects START:END");
    a.frames_start = std::stoi(r.substr(0, colon));
    a.frames_end = std::stoi(r.substr(colon + 1));
}

const Option kOptions[] = {
    {"--scene", true, [](Args& a, const char* v) { a.scene_path = v; }},
    {"--frames", true, set_frames},
    {"--record", false, [](Args& a, const char*) { a.record = true; }},
    {"--out", true, [](Args& a, const char* v) { a.out_dir = v; }},
    {"--no-vulkan", false, [](Args&, const char*) {}},  // no graphics path exists
    {"--damping", true, [](Args& a, const char* v) { a.damping = std::stof(v); }},
    {"--viscosity", true, [](Args& a, const char* v) { a.viscosity = std::stof(v); }},
    {"--fixed-iters", true, [](Args& a, const char* v) { a.fixed_iters = std::stoi(v); }},
    {"--host-substeps", false, [](Args& a, const char*) { a.host_substeps = true; }},
    {"--load-state", true, [](Args& a, const char* v) { a.load_state = v; }},
    {"--save-state", true, [](Args& a, const char* v) { a.save_state = v; }},
    {"--solver-params", false, [](Args& a, const char*) { a.solver_params = true; }},
};

Args parse(int argc, char** argv) {
    Args a;
    int i = 1;
    while (i < argc) {
        const std::string flag = argv[i++];
        if (flag == "-h" || flag == "--help") usage_exit(0);
        const Option* opt = nullptr;
        for (const Option& o : kOptions)
            if (flag == o.flag) opt = &o;
        if (!opt) fail("Unknown arg: " + flag);
        if (opt->takes_value && i >= argc) fail("Unknown arg: " + flag);  // a flag without its value
        opt->apply(a, opt->takes_value ? argv[i++] : nullptr);
    }
    if (a.scene_path.empty()) fail("Error: --scene required");
    return a;
}

// Lattice of the initial block: float loops x outer, z inner, at spacing 2r
// (apps/sim_cli/main.cpp:65-74).
std::vector<water::Vec3f> initial_block(const water::scene::FluidCfg& f) {
    std::vector<water::Vec3f> pts;
    const float spacing = 2.0f * f.particle_radius;
    for (float x = f.initial_block_min.x; x <= f.initial_block_max.x; x += spacing)
        for (float y = f.initial_block_min.y; y <= f.initial_block_max.y; y += spacing)
            for (float z = f.initial_block_min.z; z <= f.initial_block_max.z; z += spacing) pts.push_back({x, y, z});
    return pts;
}

void write_frame(const std::string& path, const water::Vec3f* p, std::size_t n) {
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("cannot open " + path + " for writing");
    const std::uint32_t count = static_cast<std::uint32_t>(n);
    out.write(reinterpret_cast<const char*>(&count), sizeof(count));
    out.write(reinterpret_cast<const char*>(p), static_cast<std::streamsize>(sizeof(water::Vec3f) * n));
    if (!out) throw std::runtime_error("short write to " + path);
}

void make_dirs(const std::string& dir) {
    std::string cur;
    for (std::size_t i = 0; i <= dir.size(); ++i) {
        if (i == dir.size() || dir[i] == '/') {
            if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
                throw std::runtime_error("cannot create directory " + cur);
        }
        if (i < dir.size()) cur += dir[i];
    }
}

}  // namespace

int main(int argc, char** argv) try {
    Args args = parse(argc, argv);
    const water::scene::Scene scene = water::scene::load_scene(args.scene_path);
    if (args.frames_start < 0) args.frames_start = scene.output.frame_start;
    if (args.frames_end < 0) args.frames_end = scene.output.frame_end;

    std::printf("=== water_sim sim_cli (GB300) ===\n");
    std::printf("scene:        %s\n", scene.name.c_str());
    std::printf("frames:       %d..%d (%d total)\n", args.frames_start, args.frames_end,
                args.frames_end - args.frames_start);
    std::printf("solver:       %s\n", scene.fluid.solver.c_str());
    std::printf("record:       %s%s\n", args.record ? "yes -> " : "no", args.record ? args.out_dir.c_str() : "");

    const std::vector<water::Vec3f> initial = initial_block(scene.fluid);
    if (initial.empty()) {
        std::fprintf(stderr, "no particles\n");
        return 1;
    }
    std::printf("particles:    %zu\n", initial.size());

    water::ParticleStore store(initial.size());
    store.resize(initial.size());
    WATER_CUDA_CHECK(cudaMemcpy(store.positions(), initial.data(), sizeof(water::Vec3f) * initial.size(),
                                cudaMemcpyHostToDevice));

    water::solvers::DFSPHSolver::Config cfg;
    cfg.rest_density = scene.fluid.rest_density;
    cfg.particle_radius = scene.fluid.particle_radius;
    cfg.smoothing_length = 2.0f * scene.fluid.particle_radius;
    cfg.viscosity = (args.viscosity > 0.0f) ? args.viscosity : std::max(scene.fluid.viscosity, 1e-2f);
    cfg.surface_tension = scene.fluid.surface_tension;
    cfg.gravity = scene.fluid.gravity;
    cfg.domain_min = {0.0f, 0.0f, 0.0f};
    cfg.domain_max = {1.0f, 1.0f, 1.0f};
    if (args.damping >= 0.0f) cfg.damping = args.damping;
    water::TimeStepper::Config tsc;
    if (args.solver_params && scene.fluid.solver_params.present) {
        const water::scene::SolverParams& sp = scene.fluid.solver_params;
        cfg.max_density_iters = sp.max_density_iters;
        cfg.max_divergence_iters = sp.max_divergence_iters;
        cfg.eta_density = sp.eta_density;
        cfg.eta_divergence = sp.eta_divergence;
        cfg.enable_divergence_solver = sp.max_divergence_iters > 0;
        tsc.cfl_lambda = sp.cfl_lambda;
        std::printf("solver_params: density %u iters eta %.2g, divergence %u iters eta %.2g, cfl %.2f\n",
                    sp.max_density_iters, double(sp.eta_density), sp.max_divergence_iters,
                    double(sp.eta_divergence), double(sp.cfl_lambda));
    }
    if (args.fixed_iters >= 0) {
        cfg.max_density_iters = static_cast<water::u32>(args.fixed_iters);
        cfg.eta_density = 0.0f;
    }
    std::printf("solver cfg:   damping=%.3f viscosity=%.4f\n", cfg.damping, cfg.viscosity);

    const float spacing = 2.0f * cfg.particle_radius;
    const std::vector<water::Vec3f> bpts =
        water::solvers::sample_aabb_boundary(cfg.domain_min, cfg.domain_max, spacing, 3);
    std::printf("boundary:     %zu particles (Akinci 2012, 3 layers)\n", bpts.size());
    auto boundary = std::make_unique<water::ParticleStore>(bpts.size());
    boundary->resize(bpts.size());
    WATER_CUDA_CHECK(cudaMemcpy(boundary->positions(), bpts.data(), sizeof(water::Vec3f) * bpts.size(),
                                cudaMemcpyHostToDevice));

    water::solvers::DFSPHSolver solver(store, boundary.get(), cfg);
    water::TimeStepper ts(tsc);
    std::vector<water::Vec3f> start = initial;
    if (!args.load_state.empty()) {
        solver.load_state(args.load_state);
        start.resize(store.count());
        WATER_CUDA_CHECK(cudaMemcpy(start.data(), store.positions(), sizeof(water::Vec3f) * store.count(),
                                    cudaMemcpyDeviceToHost));
        std::printf("resumed:      %s (%zu particles)\n", args.load_state.c_str(), store.count());
    }

    if (args.record) {
        make_dirs(args.out_dir);
        char fname[512];
        std::snprintf(fname, sizeof(fname), "%s/frame_%04d.bin", args.out_dir.c_str(), args.frames_start);
        write_frame(fname, start.data(), start.size());
    }

    const float frame_dt = 1.0f / scene.output.fps;
    std::vector<water::Vec3f> host(store.count());
    for (int f = args.frames_start; f < args.frames_end; ++f) {
        int sub = 0;
        if (args.host_substeps) {
            float remaining = frame_dt;
            while (remaining > 1e-6f && sub < 64) {
                const float dt = ts.next_dt(std::max(solver.max_velocity(), 0.5f), cfg.particle_radius, remaining);
                solver.step(dt);
                remaining -= dt;
                ++sub;
            }
        } else {
            sub = static_cast<int>(solver.step_frame(ts, frame_dt));
        }
        WATER_CUDA_CHECK(cudaDeviceSynchronize());
        std::printf("frame %4d: substeps=%2d, max_v=%.4f m/s\n", f + 1, sub, solver.max_velocity());
        if (args.record) {
            WATER_CUDA_CHECK(cudaMemcpy(host.data(), store.positions(), sizeof(water::Vec3f) * store.count(),
                                        cudaMemcpyDeviceToHost));
            char fname[512];
            std::snprintf(fname, sizeof(fname), "%s/frame_%04d.bin", args.out_dir.c_str(), f + 1);
            write_frame(fname, host.data(), host.size());
        }
    }
    if (!args.save_state.empty()) {
        solver.save_state(args.save_state);
        std::printf("saved:        %s\n", args.save_state.c_str());
    }
    std::printf("=== sim_cli OK ===\n");
    return 0;
} catch (const std::exception& e) {
    std::fprintf(stderr, "sim_cli error: %s\n", e.what());
    return 1;
}
