// The scene loader cases of the reference (tests/unit/test_scene_loader.cpp:17-79)
// against water/scene/scene.h, plus JSON edge cases. Host only.
#include <cstdio>
#include <fstream>
#include <string>

#include "check.h"
#include "water/scene/scene.h"

using namespace water::scene;

namespace {
std::string tmp_path(const char* name) { return std::string("/tmp/water_gb300_") + name; }
void write_file(const std::string& p, const std::string& s) { std::ofstream(p) << s; }
}  // namespace

TEST_CASE("minimal valid scene parses with defaults") {
    const std::string p = tmp_path("minimal.json");
    write_file(p, R"({"schema_version": "1.0", "name": "test"})");
    const Scene s = load_scene(p);
    CHECK(s.name == "test");
    CHECK(s.output.width == 1920);
    CHECK(s.fluid.solver == "dfsph");
    CHECK(s.fluid.particle_radius == 0.0015f);
    CHECK(s.fluid.initial_block_max.y == 0.25f);
    std::remove(p.c_str());
}

TEST_CASE("missing schema_version throws") {
    const std::string p = tmp_path("noschema.json");
    write_file(p, R"({"name": "broken"})");
    CHECK_THROWS_AS(load_scene(p), std::runtime_error);
    std::remove(p.c_str());
}

TEST_CASE("unsupported schema version throws") {
    const std::string p = tmp_path("badschema.json");
    write_file(p, R"({"schema_version": "99.0"})");
    CHECK_THROWS_AS(load_scene(p), std::runtime_error);
    std::remove(p.c_str());
}

TEST_CASE("file not found throws") { CHECK_THROWS_AS(load_scene("/nonexistent/path.json"), std::runtime_error); }

TEST_CASE("full scene fields populate") {
    const std::string p = tmp_path("full.json");
    write_file(p, R"({
        "schema_version": "1.0", "name": "full_test",
        "output": {"resolution": [800, 600], "fps": 30, "frame_range": [10, 20], "format": "bin", "video": "none"},
        "camera": {"position": [1.0, 2.0, 3.0], "look_at": [0.0, 0.0, 0.0], "fov_y_deg": 45.0},
        "scene": {"fluid": {"particle_radius": 0.005, "gravity": [0.0, -9.81, 0.0], "rest_density": 998.5,
                            "viscosity": 0.002, "surface_tension": 0.0, "solver": "dfsph",
                            "initial_block_min": [0.1, 0.2, 0.3], "initial_block_max": [0.4, 0.5, 0.6]}}
    })");
    const Scene s = load_scene(p);
    CHECK(s.name == "full_test");
    CHECK(s.output.width == 800 && s.output.height == 600);
    CHECK(check::approx(s.output.fps, 30.0, 1e-7));
    CHECK(s.output.frame_start == 10 && s.output.frame_end == 20);
    CHECK(s.output.format == "bin" && s.output.video == "none");
    CHECK(check::approx(s.camera.position.x, 1.0, 1e-7));
    CHECK(check::approx(s.camera.fov_y_deg, 45.0, 1e-7));
    CHECK(s.camera.up.y == 1.0f);  // default kept
    CHECK(check::approx(s.fluid.particle_radius, 0.005, 1e-7));
    CHECK(check::approx(s.fluid.gravity.y, -9.81, 1e-7));
    CHECK(check::approx(s.fluid.rest_density, 998.5, 1e-7));
    CHECK(s.fluid.initial_block_min.z == 0.3f && s.fluid.initial_block_max.x == 0.4f);
    std::remove(p.c_str());
}

TEST_CASE("malformed JSON throws runtime_error") {
    const char* bad[] = {R"({"schema_version": "1.0",})", R"({"schema_version": "1.0")", R"([1, 2)",
                         R"({"schema_version": 1.0e})", R"({"a": "unterminated)", R"({"a": tru})", "",
                         R"({"schema_version": "1.0"} trailing)"};
    for (const char* t : bad) CHECK_THROWS_AS(parse_scene(t), std::runtime_error);
}

TEST_CASE("wrong value types throw runtime_error") {
    CHECK_THROWS_AS(parse_scene(R"({"schema_version": 1})"), std::runtime_error);
    CHECK_THROWS_AS(parse_scene(R"({"schema_version": "1.0", "output": {"fps": "fast"}})"), std::runtime_error);
    CHECK_THROWS_AS(parse_scene(R"({"schema_version": "1.0", "output": {"resolution": [800]}})"),
                    std::runtime_error);
}

TEST_CASE("JSON escapes, nesting and numbers") {
    const Scene s = parse_scene(R"({"schema_version":"1.0","name":"a\"b\\cé😀\n",
                                    "extra":{"x":[[],{},null,true,false,-0.5e-3,12]},
                                    "output":{"fps":2.5E1}})");
    CHECK(s.name == "a\"b\\c\xc3\xa9\xf0\x9f\x98\x80\n");
    CHECK(check::approx(s.output.fps, 25.0, 1e-7));
}

TEST_CASE("solver_params block (read here, ignored by the reference's loader)") {
    const Scene none = parse_scene(R"({"schema_version": "1.0"})");
    CHECK(!none.fluid.solver_params.present);
    CHECK(none.fluid.solver_params.max_density_iters == 100u);
    const Scene s = parse_scene(R"({"schema_version": "1.0", "scene": {"fluid": {"solver_params": {
        "max_density_iters": 12, "max_divergence_iters": 3, "eta_density": 1e-4,
        "eta_divergence": 2e-3, "cfl_lambda": 0.25}}}})");
    CHECK(s.fluid.solver_params.present);
    CHECK(s.fluid.solver_params.max_density_iters == 12u && s.fluid.solver_params.max_divergence_iters == 3u);
    CHECK(check::approx(s.fluid.solver_params.eta_density, 1e-4, 1e-6));
    CHECK(check::approx(s.fluid.solver_params.eta_divergence, 2e-3, 1e-6));
    CHECK(check::approx(s.fluid.solver_params.cfl_lambda, 0.25, 1e-7));
    CHECK_THROWS_AS(parse_scene(R"({"schema_version": "1.0", "scene": {"fluid": {"solver_params":
        {"cfl_lambda": "big"}}}})"), std::runtime_error);
}

int main() { return check::run_all(); }
