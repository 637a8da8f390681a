// The C++ façade (include/water) on a GPU: the reference's unit tests of
// ParticleStore (tests/unit/test_particle_store.cu:8-83), CellGrid
// (tests/unit/test_cell_grid.cu:9-74), the boundary sampler
// (tests/unit/test_boundary_sampler.cu:7-31) and DFSPHSolver
// (tests/unit/test_dfsph_density.cu:16-109, tests/regression/
// test_settled_puddle.cu:66-117), written against the same API.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <vector>

#include "check.h"
#include "water/core/cell_grid.h"
#include "water/core/cuda_check.h"
#include "water/core/particle_store.h"
#include "water/solvers/boundary_sampler.h"
#include "water/solvers/dfsph.h"

using namespace water;
using namespace water::solvers;

TEST_CASE("ParticleStore: construction registers position+velocity") {
    ParticleStore store(100);
    CHECK(store.capacity() == 100);
    CHECK(store.count() == 0);
    CHECK(store.has_attribute("position"));
    CHECK(store.has_attribute("velocity"));
    CHECK(!store.has_attribute("density"));
}

TEST_CASE("ParticleStore: resize within capacity, beyond throws out_of_range") {
    ParticleStore store(50);
    store.resize(10);
    CHECK(store.count() == 10);
    store.resize(50);
    CHECK(store.count() == 50);
    CHECK_THROWS_AS(store.resize(51), std::out_of_range);
}

TEST_CASE("ParticleStore: custom attribute, duplicate throws runtime_error") {
    ParticleStore store(64);
    auto h = store.register_attribute<float>("density", AttribType::F32);
    CHECK(h.valid());
    CHECK(store.has_attribute("density"));
    CHECK_THROWS_AS(store.register_attribute<float>("density", AttribType::F32), std::runtime_error);
}

TEST_CASE("ParticleStore: host round trips") {
    ParticleStore store(8);
    store.resize(8);
    std::vector<Vec3f> p = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 1}};
    WATER_CUDA_CHECK(cudaMemcpy(store.positions(), p.data(), sizeof(Vec3f) * 8, cudaMemcpyHostToDevice));
    std::vector<Vec3f> back(8);
    WATER_CUDA_CHECK(cudaMemcpy(back.data(), store.positions(), sizeof(Vec3f) * 8, cudaMemcpyDeviceToHost));
    for (int i = 0; i < 8; ++i) CHECK(back[i].x == p[i].x && back[i].y == p[i].y && back[i].z == p[i].z);
    auto h = store.register_attribute<float>("temperature", AttribType::F32);
    std::vector<float> t = {1, 2, 3, 4, 5, 6, 7, 8}, tb(8);
    WATER_CUDA_CHECK(cudaMemcpy(store.attribute_data(h), t.data(), 32, cudaMemcpyHostToDevice));
    WATER_CUDA_CHECK(cudaMemcpy(tb.data(), store.attribute_data(h), 32, cudaMemcpyDeviceToHost));
    CHECK(t == tb);
}

TEST_CASE("ParticleStore: attributes are zero-filled, disjoint and keep their address") {
    ParticleStore store(1000);
    Vec3f* pos = store.positions();
    std::vector<AttribHandle<float>> hs;
    const char* names[] = {"a", "b", "c", "d", "e", "f", "g"};  // more than the first arena block holds
    for (const char* n : names) hs.push_back(store.register_attribute<float>(n, AttribType::F32));
    auto u = store.register_attribute<unsigned>("flags", AttribType::U32);
    CHECK(store.positions() == pos);  // no attribute moved
    std::vector<const unsigned char*> lo, hi;
    for (auto h : hs) {
        lo.push_back(reinterpret_cast<const unsigned char*>(store.attribute_data(h)));
        hi.push_back(lo.back() + 1000 * sizeof(float));
        CHECK(reinterpret_cast<std::uintptr_t>(lo.back()) % 256 == 0);
    }
    lo.push_back(reinterpret_cast<const unsigned char*>(store.positions()));
    hi.push_back(lo.back() + 1000 * sizeof(Vec3f));
    lo.push_back(reinterpret_cast<const unsigned char*>(store.velocities()));
    hi.push_back(lo.back() + 1000 * sizeof(Vec3f));
    lo.push_back(reinterpret_cast<const unsigned char*>(store.attribute_data(u)));
    hi.push_back(lo.back() + 1000 * sizeof(unsigned));
    for (std::size_t a = 0; a < lo.size(); ++a)
        for (std::size_t b = a + 1; b < lo.size(); ++b) CHECK(hi[a] <= lo[b] || hi[b] <= lo[a]);
    WATER_CUDA_CHECK(cudaStreamSynchronize(store.stream()));
    std::vector<float> back(1000, 1.0f);
    WATER_CUDA_CHECK(cudaMemcpy(back.data(), store.attribute_data(hs.back()), 4000, cudaMemcpyDeviceToHost));
    CHECK(std::all_of(back.begin(), back.end(), [](float v) { return v == 0.0f; }));
}

TEST_CASE("ParticleStore: a handle that names no attribute throws out_of_range") {
    ParticleStore store(16);
    AttribHandle<float> none;
    CHECK(!none.valid());
    CHECK_THROWS_AS(store.attribute_data(none), std::out_of_range);
    CHECK_THROWS_AS(store.attribute_data(AttribHandle<float>(99)), std::out_of_range);
}

TEST_CASE("DeviceBuffer: move leaves the source empty; copies round trip") {
    DeviceBuffer<int> a(64);
    std::vector<int> in(64), out(64, -1);
    for (int i = 0; i < 64; ++i) in[i] = i * 3;
    a.copy_from_host(in.data(), 64);
    DeviceBuffer<int> b(std::move(a));
    CHECK(a.empty() && a.data() == nullptr && b.size() == 64);
    DeviceBuffer<int> c;
    c = std::move(b);
    CHECK(b.empty() && c.size() == 64);
    c.copy_to_host(out.data(), 64);
    WATER_CUDA_CHECK(cudaStreamSynchronize(c.stream()));
    CHECK(in == out);
    c.fill_zero();
    c.copy_to_host(out.data(), 64);
    WATER_CUDA_CHECK(cudaStreamSynchronize(c.stream()));
    CHECK(std::all_of(out.begin(), out.end(), [](int v) { return v == 0; }));
}

TEST_CASE("CellGrid: 8 grid-aligned points map to 8 distinct cells") {
    CellGrid grid({0.f, 0.f, 0.f}, {4, 4, 4}, 0.5f);
    grid.reserve(8);
    std::vector<Vec3f> pts = {{0.25f, 0.25f, 0.25f}, {0.75f, 0.25f, 0.25f}, {0.25f, 0.75f, 0.25f},
                              {0.75f, 0.75f, 0.25f}, {0.25f, 0.25f, 0.75f}, {0.75f, 0.25f, 0.75f},
                              {0.25f, 0.75f, 0.75f}, {0.75f, 0.75f, 0.75f}};
    Vec3f* d = nullptr;
    WATER_CUDA_CHECK(cudaMalloc(&d, sizeof(Vec3f) * pts.size()));
    WATER_CUDA_CHECK(cudaMemcpy(d, pts.data(), sizeof(Vec3f) * pts.size(), cudaMemcpyHostToDevice));
    grid.build(d, pts.size());
    WATER_CUDA_CHECK(cudaDeviceSynchronize());
    std::vector<u32> sorted(8);
    WATER_CUDA_CHECK(cudaMemcpy(sorted.data(), grid.sorted_indices(), 32, cudaMemcpyDeviceToHost));
    std::vector<u32> copy = sorted;
    std::sort(copy.begin(), copy.end());
    for (u32 i = 0; i < 8; ++i) CHECK(copy[i] == i);
    std::vector<u32> cs(grid.total_cells() + 1);
    WATER_CUDA_CHECK(cudaMemcpy(cs.data(), grid.cell_start(), sizeof(u32) * cs.size(), cudaMemcpyDeviceToHost));
    for (std::size_t i = 1; i < cs.size(); ++i) CHECK(cs[i] >= cs[i - 1]);
    cudaFree(d);
}

TEST_CASE("CellGrid: out-of-bounds particle goes to the sentinel cell") {
    CellGrid grid({0.f, 0.f, 0.f}, {2, 2, 2}, 0.5f);
    grid.reserve(2);
    std::vector<Vec3f> pts = {{0.25f, 0.25f, 0.25f}, {99.0f, 99.0f, 99.0f}};
    Vec3f* d = nullptr;
    WATER_CUDA_CHECK(cudaMalloc(&d, sizeof(Vec3f) * 2));
    WATER_CUDA_CHECK(cudaMemcpy(d, pts.data(), sizeof(Vec3f) * 2, cudaMemcpyHostToDevice));
    grid.build(d, 2);
    WATER_CUDA_CHECK(cudaDeviceSynchronize());
    std::vector<u32> cs(grid.total_cells() + 1);
    WATER_CUDA_CHECK(cudaMemcpy(cs.data(), grid.cell_start(), sizeof(u32) * cs.size(), cudaMemcpyDeviceToHost));
    CHECK(cs.back() == 1);
    CHECK(cs[0] == 0);
    cudaFree(d);
}

TEST_CASE("boundary sampler counts and layers") {
    auto p1 = sample_aabb_boundary({0.f, 0.f, 0.f}, {1.f, 1.f, 1.f}, 0.05f, 1);
    CHECK(p1.size() > 2000 && p1.size() < 4000);
    auto p2 = sample_aabb_boundary({0.f, 0.f, 0.f}, {1.f, 1.f, 1.f}, 0.05f, 2);
    CHECK(p2.size() > p1.size() * 1.5 && p2.size() < p1.size() * 2.5);
    CHECK(sample_aabb_boundary({0.f, 0.f, 0.f}, {1.f, 1.f, 1.f}, 0.02f, 3).size() == 46818);
}

static f32 host_W0(f32 l) { return 1.0f / (3.14159265358979323846f * l * l * l); }

TEST_CASE("DFSPHSolver: isolated particle density = mass * W(0)") {
    ParticleStore store(1);
    store.resize(1);
    Vec3f p{0.5f, 0.5f, 0.5f};
    WATER_CUDA_CHECK(cudaMemcpy(store.positions(), &p, sizeof(Vec3f), cudaMemcpyHostToDevice));
    DFSPHSolver::Config cfg;
    cfg.particle_radius = 0.01f;
    cfg.smoothing_length = 0.04f;
    DFSPHSolver solver(store, nullptr, cfg);
    solver.step(0.001f);
    WATER_CUDA_CHECK(cudaDeviceSynchronize());
    CHECK(check::approx(solver.density_at(0), solver.particle_mass() * host_W0(0.04f), 1e-4));
    CHECK(store.has_attribute("dfsph_density") && store.has_attribute("dfsph_alpha") &&
          store.has_attribute("dfsph_kappa") && store.has_attribute("dfsph_density_adv"));
}

TEST_CASE("DFSPHSolver: dense pack centre density near rest, alpha finite") {
    const f32 r = 0.01f, s = 2 * r;
    std::vector<Vec3f> pts;
    for (int z = 0; z < 10; ++z)
        for (int y = 0; y < 10; ++y)
            for (int x = 0; x < 10; ++x) pts.push_back({0.1f + x * s, 0.1f + y * s, 0.1f + z * s});
    ParticleStore store(pts.size());
    store.resize(pts.size());
    WATER_CUDA_CHECK(cudaMemcpy(store.positions(), pts.data(), sizeof(Vec3f) * pts.size(), cudaMemcpyHostToDevice));
    DFSPHSolver::Config cfg;
    cfg.particle_radius = r;
    cfg.smoothing_length = 4 * r;
    DFSPHSolver solver(store, nullptr, cfg);
    solver.step(0.001f);
    const f32 d = solver.density_at(555);
    CHECK(check::approx(d, 1000.0, 0.30));
    CHECK(d > 500.0f && d < 1500.0f);
    const f32 a = solver.alpha_at(555);
    CHECK(a >= 0.0f && std::isfinite(a));
}

TEST_CASE("DFSPHSolver: single particle falls under gravity") {
    ParticleStore store(1);
    store.resize(1);
    Vec3f p{0.5f, 0.5f, 0.5f}, v{0, 0, 0};
    WATER_CUDA_CHECK(cudaMemcpy(store.positions(), &p, sizeof(Vec3f), cudaMemcpyHostToDevice));
    WATER_CUDA_CHECK(cudaMemcpy(store.velocities(), &v, sizeof(Vec3f), cudaMemcpyHostToDevice));
    DFSPHSolver::Config cfg;
    cfg.particle_radius = 0.01f;
    cfg.smoothing_length = 0.04f;
    cfg.viscosity = 0.0f;
    DFSPHSolver solver(store, nullptr, cfg);
    for (int k = 0; k < 5; ++k) solver.step(0.01f);
    CHECK(solver.max_velocity() > 0.0f);  // falling, not yet at the floor clamp
    for (int k = 5; k < 50; ++k) solver.step(0.01f);
    WATER_CUDA_CHECK(cudaDeviceSynchronize());
    Vec3f pf{};
    WATER_CUDA_CHECK(cudaMemcpy(&pf, store.positions(), sizeof(Vec3f), cudaMemcpyDeviceToHost));
    CHECK(pf.y < 0.5f);
    CHECK(check::approx(pf.x, 0.5, 0.01) && check::approx(pf.z, 0.5, 0.01));
}

TEST_CASE("DFSPHSolver: boundary masses, grids and a short drop") {
    const f32 r = 0.012f;
    DFSPHSolver::Config cfg;
    cfg.particle_radius = r;
    cfg.smoothing_length = 2 * r;
    cfg.viscosity = 0.0f;
    ParticleStore fluid(1);
    fluid.resize(1);
    Vec3f p{0.5f, 0.05f, 0.5f};
    WATER_CUDA_CHECK(cudaMemcpy(fluid.positions(), &p, sizeof(Vec3f), cudaMemcpyHostToDevice));
    auto bpts = sample_aabb_boundary(cfg.domain_min, cfg.domain_max, 2 * r, 3);
    auto boundary = std::make_unique<ParticleStore>(bpts.size());
    boundary->resize(bpts.size());
    WATER_CUDA_CHECK(
        cudaMemcpy(boundary->positions(), bpts.data(), sizeof(Vec3f) * bpts.size(), cudaMemcpyHostToDevice));
    DFSPHSolver solver(fluid, boundary.get(), cfg);
    CHECK(solver.particle_mass() > 0);
    CHECK(solver.boundary_mass_at(0) > 0 && solver.boundary_mass_at(100) > 0 && solver.boundary_mass_at(1000) > 0);
    CHECK(boundary->has_attribute("dfsph_boundary_mass"));
    CHECK(solver.boundary_grid() != nullptr);
    for (int k = 0; k < 5; ++k) solver.step(0.001f);
    const CellGrid& g = solver.fluid_grid();
    std::vector<u32> cs(g.total_cells() + 1);
    WATER_CUDA_CHECK(cudaMemcpy(cs.data(), g.cell_start(), sizeof(u32) * cs.size(), cudaMemcpyDeviceToHost));
    CHECK(cs.back() == 1);
    CHECK(solver.last_density_iters() >= 1);
    // a second solver on the same store re-registers the attributes: throws like the reference
    CHECK_THROWS_AS(DFSPHSolver(fluid, boundary.get(), cfg), std::runtime_error);
}

int main() { return check::run_all(); }
