// Scene description and its JSON loader: the reference's water::scene API
// (scene/include/water/scene/scene.h:9-45, scene/src/loader.cpp:12-83) with
// the same structs, defaults, schema check ("schema_version" must be "1.0")
// and errors (std::runtime_error for a missing file, a parse error, a missing
// or unsupported schema). Parsing uses the project's own reader (json.h).
#pragma once

#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>

#include "water/core/types.h"
#include "water/scene/json.h"

namespace water::scene {

struct Camera {
    Vec3f position{0.0f, 0.0f, 1.0f};
    Vec3f look_at{0.0f, 0.0f, 0.0f};
    Vec3f up{0.0f, 1.0f, 0.0f};
    f32 fov_y_deg = 30.0f;
};

struct OutputCfg {
    i32 width = 1920;
    i32 height = 1080;
    f32 fps = 24.0f;
    i32 frame_start = 0;
    i32 frame_end = 120;
    std::string format = "exr";
    std::string video = "mp4";
};

// The design spec's solver_params block (docs/superpowers/specs/
// 2026-04-23-water-simulation-rebuild-design.md:485-491). The reference's
// loader does not read it; here it is parsed and `present` tells whether the
// scene had one. sim_cli applies it only when asked (--solver-params).
struct SolverParams {
    bool present = false;
    u32 max_density_iters = 100;
    u32 max_divergence_iters = 100;
    f32 eta_density = 1e-3f;
    f32 eta_divergence = 1e-3f;
    f32 cfl_lambda = 0.4f;
};

struct FluidCfg {
    std::string solver = "dfsph";
    f32 particle_radius = 0.0015f;
    f32 rest_density = 1000.0f;
    f32 viscosity = 1e-3f;
    f32 surface_tension = 0.0728f;
    Vec3f gravity{0.0f, -9.81f, 0.0f};
    Vec3f initial_block_min{0.4f, 0.05f, 0.4f};
    Vec3f initial_block_max{0.6f, 0.25f, 0.6f};
    SolverParams solver_params;
};

struct Scene {
    std::string name;
    OutputCfg output;
    Camera camera;
    FluidCfg fluid;
};

namespace detail {

inline Vec3f read_vec3(const Json& j, const char* key, Vec3f fallback) {
    if (!j.contains(key)) return fallback;
    const Json& a = j.at(key);
    return {a[0].as_float(), a[1].as_float(), a[2].as_float()};
}

inline void parse_camera(const Json& j, Camera& c) {
    if (!j.contains("camera")) return;
    const Json& cam = j["camera"];
    c.position = read_vec3(cam, "position", c.position);
    c.look_at = read_vec3(cam, "look_at", c.look_at);
    c.up = read_vec3(cam, "up", c.up);
    if (cam.contains("fov_y_deg")) c.fov_y_deg = cam["fov_y_deg"].as_float();
}

inline void parse_output(const Json& j, OutputCfg& o) {
    if (!j.contains("output")) return;
    const Json& out = j["output"];
    if (out.contains("resolution")) {
        o.width = out["resolution"][0].as_int();
        o.height = out["resolution"][1].as_int();
    }
    if (out.contains("fps")) o.fps = out["fps"].as_float();
    if (out.contains("frame_range")) {
        o.frame_start = out["frame_range"][0].as_int();
        o.frame_end = out["frame_range"][1].as_int();
    }
    if (out.contains("format")) o.format = out["format"].as_string();
    if (out.contains("video")) o.video = out["video"].as_string();
}

inline void parse_fluid(const Json& j, FluidCfg& f) {
    if (!j.contains("scene") || !j["scene"].contains("fluid")) return;
    const Json& fl = j["scene"]["fluid"];
    if (fl.contains("solver")) f.solver = fl["solver"].as_string();
    if (fl.contains("particle_radius")) f.particle_radius = fl["particle_radius"].as_float();
    if (fl.contains("rest_density")) f.rest_density = fl["rest_density"].as_float();
    if (fl.contains("viscosity")) f.viscosity = fl["viscosity"].as_float();
    if (fl.contains("surface_tension")) f.surface_tension = fl["surface_tension"].as_float();
    f.gravity = read_vec3(fl, "gravity", f.gravity);
    f.initial_block_min = read_vec3(fl, "initial_block_min", f.initial_block_min);
    f.initial_block_max = read_vec3(fl, "initial_block_max", f.initial_block_max);
    if (fl.contains("solver_params")) {
        const Json& sp = fl["solver_params"];
        SolverParams& p = f.solver_params;
        p.present = true;
        if (sp.contains("max_density_iters")) p.max_density_iters = static_cast<u32>(sp["max_density_iters"].as_int());
        if (sp.contains("max_divergence_iters"))
            p.max_divergence_iters = static_cast<u32>(sp["max_divergence_iters"].as_int());
        if (sp.contains("eta_density")) p.eta_density = sp["eta_density"].as_float();
        if (sp.contains("eta_divergence")) p.eta_divergence = sp["eta_divergence"].as_float();
        if (sp.contains("cfl_lambda")) p.cfl_lambda = sp["cfl_lambda"].as_float();
    }
}

}  // namespace detail

// Parse a scene from JSON text; `origin` names the source in error messages.
inline Scene parse_scene(const std::string& text, const std::string& origin = "<string>") {
    Json j;
    try {
        j = Json::parse(text);
    } catch (const JsonError& e) {
        throw std::runtime_error("scene::load_scene: JSON parse failed in " + origin + ": " + e.what());
    }
    if (!j.contains("schema_version"))
        throw std::runtime_error("scene::load_scene: missing schema_version in " + origin);
    const std::string sv = j["schema_version"].as_string();
    if (sv != "1.0") throw std::runtime_error("scene::load_scene: unsupported schema_version: " + sv);
    Scene s;
    try {
        if (j.contains("name")) s.name = j["name"].as_string();
        detail::parse_output(j, s.output);
        detail::parse_camera(j, s.camera);
        detail::parse_fluid(j, s.fluid);
    } catch (const JsonError& e) {
        throw std::runtime_error("scene::load_scene: bad value in " + origin + ": " + e.what());
    }
    return s;
}

// Throws std::runtime_error on a missing file, a parse error or a missing /
// unsupported schema_version.
inline Scene load_scene(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("scene::load_scene: cannot open " + path);
    std::ostringstream ss;
    ss << in.rdbuf();
    return parse_scene(ss.str(), path);
}

}  // namespace water::scene
