// Host sanitizer run of the CPU oracle (test infrastructure): the oracle's
// source compiled with AddressSanitizer and UndefinedBehaviorSanitizer and
// driven through every entry point on a small case: FP32 and FP64 steps with
// walls and both solvers, the forward-mode instance, the grid build, Morton
// order, the LBVH restatement and the spline / cohesion evaluations. Any
// finding aborts with a non-zero exit.
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../oracle/dfsph_oracle.cpp"

int main() {
    Config c{};
    c.rest_density = 1000.0f;
    c.particle_radius = 0.02f;
    c.smoothing_length = 0.04f;
    c.viscosity = 0.01f;
    c.damping = 0.5f;
    c.gravity[1] = -9.81f;
    c.max_density_iters = 4;
    c.max_divergence_iters = 2;
    c.eta_density = 1e-4f;
    c.eta_divergence = 1e-3f;
    for (int a = 0; a < 3; ++a) { c.domain_min[a] = 0.0f; c.domain_max[a] = 1.0f; }
    // wall particles
    const float lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    const long long nb = oracle_sample_aabb_boundary(lo, hi, 0.04f, 3, nullptr, 0);
    std::vector<float> wall(3 * nb);
    oracle_sample_aabb_boundary(lo, hi, 0.04f, 3, wall.data(), nb);
    // a 6 x 6 x 6 block with one particle outside the domain
    std::vector<float> x, v;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j)
            for (int k = 0; k < 6; ++k) {
                x.insert(x.end(), {0.3f + 0.04f * i, 0.4f + 0.04f * j, 0.3f + 0.04f * k});
                v.insert(v.end(), {0.1f * (i - 3), 0.0f, -0.05f * k});
            }
    x.insert(x.end(), {2.0f, 2.0f, 2.0f});
    v.insert(v.end(), {0.0f, 0.0f, 0.0f});
    const u32 n = static_cast<u32>(x.size() / 3);
    std::vector<double> out(3 * n);
    for (int prec : {32, 64}) {
        void* h = oracle_create(&c, prec, x.data(), v.data(), n, wall.data(), static_cast<u32>(nb));
        oracle_step(h, 1e-3f, 5);
        oracle_get(h, 0, out.data());
        for (double d : out)
            if (!std::isfinite(d) && d != 2.0) return 2;
        (void)oracle_scalar(h, 0);
        oracle_destroy(h);
    }
    std::vector<double> dv(3 * n, 1.0), dx(3 * n, 0.01);
    void* d = oracle_dual_create(&c, x.data(), v.data(), n, wall.data(), static_cast<u32>(nb), dx.data(), dv.data(),
                                 1.0);
    oracle_dual_step(d, 1e-3f, 3);
    std::vector<double> a(3 * n), b(3 * n), e(3 * n), f(3 * n);
    oracle_dual_get(d, a.data(), b.data(), e.data(), f.data());
    oracle_dual_destroy(d);
    const float smin[3] = {0, 0, 0}, smax[3] = {1, 1, 1};
    std::vector<u32> codes(n), idx(n), left(n - 1), right(n - 1), parent(2 * n - 1);
    std::vector<float> boxes(6 * (2 * n - 1));
    oracle_morton_sort(x.data(), n, smin, smax, codes.data(), idx.data());
    oracle_lbvh_build(x.data(), n, codes.data(), idx.data(), 0.01f, left.data(), right.data(), parent.data(),
                      boxes.data());
    const int dims[3] = {27, 27, 27};
    const float origin[3] = {-0.04f, -0.04f, -0.04f};
    std::vector<u32> keys(n), sorted(n), cs(27 * 27 * 27 + 1);
    oracle_build_grid_f32(x.data(), n, origin, dims, 0.04f, keys.data(), sorted.data(), cs.data());
    double sum = oracle_W_f64(0.01, 0.04) + oracle_cohesion_C(0.01, 0.04) + oracle_W_f32(0.03f, 0.04f);
    float g[3];
    const float rij[3] = {0.01f, 0.0f, 0.0f};
    oracle_gradW_f32(rij, 0.04f, g);
    std::printf("oracle sanitizer run ok %.6g %.6g\n", sum, double(g[0]));
    return 0;
}
