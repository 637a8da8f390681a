// oracle/dfsph_oracle.cpp
//
// TEST INFRASTRUCTURE ONLY — the CPU oracle for the DFSPH step.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg and
// reference arm load this library, and only as the parity reference (or as the timed
// CPU baseline). The product path (water_simulation_gb300/csrc) never links,
// loads or calls it.
//
// This is a plain C++/OpenMP restatement of the reference DFSPH step of
// Qervas/water_simulation, templated on the real type:
//   * Real = float  : the FP32 instance (the timed CPU baseline, and the
//                     reference for bit-exact grid/neighbour structure);
//   * Real = double : the FP64 oracle that field errors are reported against.
// Each function cites the reference file:line it restates. It follows the
// reference's data layout (particles kept in their ORIGINAL order, neighbours
// gathered through the sorted permutation) and its arithmetic order, without
// the reference's -use_fast_math approximations.
//
// Deliberate deviations:
//   * XSPH is Jacobi (every particle reads the pre-XSPH velocities). The
//     reference updates velocities in place while neighbours read them
//     (solvers/dfsph/src/dfsph_kernels.cu:327,338-340), a data race whose result
//     depends on thread scheduling.
//   * The divergence solver (absent from the reference; specified in its plan
//     docs/superpowers/plans/2026-04-24-water-simulation-v2-phase2-dfsph-solver.md
//     :1856-1987) runs right after alpha, before external forces. With
//     max_divergence_iters = 0 (the reference's behaviour) it does nothing.
//   * Convergence sums are accumulated in double.
//
// Parity pins: the reference's unit tests re-expressed in tests/test_oracle.py,
// and golden vectors produced by the reference's own compiled kernels
// (tests/golden/).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

using u32 = std::uint32_t;

// Mirrors DFSPHSolver::Config (solvers/dfsph/include/water/solvers/dfsph.h:19-33)
// plus the two knobs the oracle needs from the device side.
struct Config {
    float rest_density;
    float particle_radius;
    float smoothing_length;
    float viscosity;
    float damping;
    float surface_tension;
    float gravity[3];
    u32   max_density_iters;
    u32   max_divergence_iters;
    float eta_density;
    float eta_divergence;
    float domain_min[3];
    float domain_max[3];
    // 1/cell_length as evaluated by the device code that centres the 27-cell
    // stencil (the reference computes it on the device under -use_fast_math,
    // dfsph_kernels.cu:52,89,...). 0 => use the IEEE float reciprocal.
    float stencil_inv_cell;
};

template <class R> struct V3 { R x, y, z; };

// Forward-mode dual number: a value and its derivative along one direction.
// Solver<Dual> runs the FP64 step on the values (every branch, max(0, .),
// clamp and neighbour set decided by them) and carries the exact directional
// derivative of the step along, against which the GPU adjoint is tested
// (dfsph_adjoint_backward): <gradient, direction> must equal it.
struct Dual {
    double v = 0.0, d = 0.0;
    Dual() = default;
    Dual(double a) : v(a), d(0.0) {}  // NOLINT: constants promote implicitly
    Dual(double a, double b) : v(a), d(b) {}
    explicit operator double() const { return v; }
    Dual operator-() const { return {-v, -d}; }
    Dual& operator+=(const Dual& o) { v += o.v; d += o.d; return *this; }
    Dual& operator-=(const Dual& o) { v -= o.v; d -= o.d; return *this; }
    Dual& operator*=(const Dual& o) { d = d * o.v + v * o.d; v *= o.v; return *this; }
};
inline Dual operator+(const Dual& a, const Dual& b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(const Dual& a, const Dual& b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator*(const Dual& a, const Dual& b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(const Dual& a, const Dual& b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline Dual operator+(const Dual& a, double b) { return {a.v + b, a.d}; }
inline Dual operator+(double a, const Dual& b) { return {a + b.v, b.d}; }
inline Dual operator-(const Dual& a, double b) { return {a.v - b, a.d}; }
inline Dual operator-(double a, const Dual& b) { return {a - b.v, -b.d}; }
inline Dual operator*(const Dual& a, double b) { return {a.v * b, a.d * b}; }
inline Dual operator*(double a, const Dual& b) { return {a * b.v, a * b.d}; }
inline Dual operator/(const Dual& a, double b) { return {a.v / b, a.d / b}; }
inline Dual operator/(double a, const Dual& b) { return {a / b.v, -a * b.d / (b.v * b.v)}; }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
inline bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
inline bool operator<(const Dual& a, double b) { return a.v < b; }
inline bool operator>(const Dual& a, double b) { return a.v > b; }
// sqrt(0) carries a zero derivative: only a self pair has r^2 = 0, and its
// r^2 is identically zero.
inline Dual sqrt(const Dual& a) {
    const double r = std::sqrt(a.v);
    return {r, r > 0.0 ? a.d / (2.0 * r) : 0.0};
}
inline Dual exp(const Dual& a) {
    const double e = std::exp(a.v);
    return {e, e * a.d};
}
inline double floor(const Dual& a) { return std::floor(a.v); }
// A coordinate as the cell arithmetic sees it: rounded to float in every
// instance (the FP64 and dual instances keep the FP32 instance's neighbour
// structure for the same positions; a dual's derivative plays no part).
inline float cell_coord(float p) { return p; }
inline float cell_coord(double p) { return static_cast<float>(p); }
inline float cell_coord(const Dual& p) { return static_cast<float>(p.v); }
using std::exp;
using std::floor;
using std::sqrt;

// Float -> int conversion with the GPU's cvt.rzi.s32.f32 semantics
// (NaN -> 0, saturating). The reference casts floorf(...) results to int
// (core/src/cell_grid.cu:11-13, dfsph_kernels.cu:15-17); on the GPU that cast
// saturates, which this reproduces on the CPU where the cast would be UB.
static inline long long f2i_sat(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return 2147483647LL;
    if (v <= -2147483648.0) return -2147483648LL;
    return static_cast<long long>(v);
}

struct Grid {
    float origin[3];
    int   dims[3];
    float cell_length;
    u32   total;        // dims.x*dims.y*dims.z (the sentinel key)
};

// make_grid (solvers/dfsph/src/dfsph.cu:55-65): dims = ceil(extent/l)+2 in f32,
// origin = domain_min - l, cell = l.
static Grid make_grid(const Config& c) {
    Grid g;
    for (int a = 0; a < 3; ++a) {
        const float ext = c.domain_max[a] - c.domain_min[a];
        g.dims[a] = static_cast<int>(std::ceil(ext / c.smoothing_length)) + 2;
        g.origin[a] = c.domain_min[a] - c.smoothing_length;
    }
    g.cell_length = c.smoothing_length;
    g.total = static_cast<u32>(g.dims[0]) * static_cast<u32>(g.dims[1]) *
              static_cast<u32>(g.dims[2]);
    return g;
}

// x-major linear cell id (core/src/cell_grid.cu:20-21, dfsph_kernels.cu:24-26).
static inline u32 linear_cell(long long cx, long long cy, long long cz, const Grid& g) {
    return (static_cast<u32>(cx) * static_cast<u32>(g.dims[1]) + static_cast<u32>(cy)) *
               static_cast<u32>(g.dims[2]) + static_cast<u32>(cz);
}

// hash_cell (core/src/cell_grid.cu:10-22); `inv` is the host reciprocal
// 1.0f / cell_length computed in CellGrid::build (core/src/cell_grid.cu:81).
// The arithmetic is float in every instance (cell_coord).
template <class R>
static inline u32 hash_cell(const V3<R>& p, const Grid& g, float inv) {
    const long long cx = f2i_sat(std::floor((cell_coord(p.x) - g.origin[0]) * inv));
    const long long cy = f2i_sat(std::floor((cell_coord(p.y) - g.origin[1]) * inv));
    const long long cz = f2i_sat(std::floor((cell_coord(p.z) - g.origin[2]) * inv));
    if (cx < 0 || cx >= g.dims[0] || cy < 0 || cy >= g.dims[1] || cz < 0 || cz >= g.dims[2])
        return g.total;
    return linear_cell(cx, cy, cz, g);
}

// The neighbour structure of one CellGrid::build (core/src/cell_grid.cu:73-138).
struct GridArrays {
    std::vector<u32> keys;        // per particle, original order
    std::vector<u32> sorted;      // sorted slot -> original index
    std::vector<u32> cell_start;  // total + 1 entries
};

// CellGrid::build: keys, stable (key, index) sort (CUB radix sort is stable and
// the values start as iota, cell_grid.cu:24-30,98-110), then cell_start filled
// with the sentinel `count`, starts scattered at key boundaries and the serial
// right-to-left min pass (cell_grid.cu:119-137), restated literally.
template <class R>
static void build_grid(const V3<R>* pos, std::size_t n, const Grid& g, GridArrays& out) {
    if (n == 0) {
        // count == 0 returns before touching anything (cell_grid.cu:74-77); the
        // arrays stay as constructed (cell_start zero-filled, cell_grid.cu:62-63).
        out.keys.clear();
        out.sorted.clear();
        if (out.cell_start.size() != std::size_t(g.total) + 1) out.cell_start.assign(std::size_t(g.total) + 1, 0u);
        return;
    }
    const float inv = 1.0f / g.cell_length;
    out.keys.resize(n);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) out.keys[i] = hash_cell(pos[i], g, inv);
    out.sorted.resize(n);
    std::iota(out.sorted.begin(), out.sorted.end(), 0u);
    std::stable_sort(out.sorted.begin(), out.sorted.end(),
                     [&](u32 a, u32 b) { return out.keys[a] < out.keys[b]; });
    const std::size_t cs = std::size_t(g.total) + 1;
    out.cell_start.assign(cs, static_cast<u32>(n));
    for (std::size_t s = 0; s < n; ++s) {
        const u32 c = out.keys[out.sorted[s]];
        if (s == 0 || out.keys[out.sorted[s - 1]] != c) out.cell_start[c] = static_cast<u32>(s);
    }
    for (long long i = (long long)cs - 2; i >= 0; --i)
        if (out.cell_start[i] > out.cell_start[i + 1]) out.cell_start[i] = out.cell_start[i + 1];
}

// ITER_NEIGHBORS (solvers/dfsph/src/dfsph_kernels.cu:13-35): 27 cells around the
// cell of p (centred with the device reciprocal), dz outer, dx inner, bounds-
// checked, iterating sorted slots [cell_start[c], cell_start[c+1]).
template <class R, class F>
static inline void for_neighbors(const V3<R>& p, const Grid& g, float inv_stencil,
                                 const GridArrays& ga, F&& f) {
    const long long cx = f2i_sat(std::floor((cell_coord(p.x) - g.origin[0]) * inv_stencil));
    const long long cy = f2i_sat(std::floor((cell_coord(p.y) - g.origin[1]) * inv_stencil));
    const long long cz = f2i_sat(std::floor((cell_coord(p.z) - g.origin[2]) * inv_stencil));
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const long long nx = cx + dx, ny = cy + dy, nz = cz + dz;
                if (nx < 0 || nx >= g.dims[0] || ny < 0 || ny >= g.dims[1] || nz < 0 ||
                    nz >= g.dims[2])
                    continue;
                const u32 c = linear_cell(nx, ny, nz, g);
                if (c >= g.total) continue;
                const u32 b = ga.cell_start[c], e = ga.cell_start[c + 1];
                for (u32 s = b; s < e; ++s) f(ga.sorted[s]);
            }
}

// Cubic spline W (core/include/water/core/sph_kernels.cuh:12-22).
template <class R> static inline R kernel_W(R r, R l) {
    const R q = r / l;
    if (q >= R(2)) return R(0);
    const R sigma = R(1) / (R(3.14159265358979323846) * l * l * l);
    if (q < R(1)) return sigma * (R(1) - R(1.5) * q * q + R(0.75) * q * q * q);
    const R t = R(2) - q;
    return sigma * R(0.25) * t * t * t;
}

// Cubic spline gradient (core/include/water/core/sph_kernels.cuh:25-41).
template <class R> static inline V3<R> kernel_gradW(const V3<R>& rij, R l) {
    const R r2 = rij.x * rij.x + rij.y * rij.y + rij.z * rij.z;
    const R r = sqrt(r2);
    if (r < R(1e-12)) return {R(0), R(0), R(0)};
    const R q = r / l;
    if (q >= R(2)) return {R(0), R(0), R(0)};
    const R sigma = R(1) / (R(3.14159265358979323846) * l * l * l);
    R dWdq;
    if (q < R(1)) {
        dWdq = sigma * (R(-3) * q + R(2.25) * q * q);
    } else {
        const R t = R(2) - q;
        dWdq = sigma * R(-0.75) * t * t;
    }
    const R c = dWdq / (l * r);
    return {rij.x * c, rij.y * c, rij.z * c};
}

template <class R> static inline V3<R> sub(const V3<R>& a, const V3<R>& b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}

template <class R>
struct Solver {
    Config cfg;
    Grid grid;
    float inv_stencil;
    R mass;
    R l;
    std::vector<V3<R>> x, v, xb;
    std::vector<R> rho, alpha, kappa, rho_adv, mb, kappa_v, rho_dot;
    std::vector<u32> nbr_f, nbr_b;
    GridArrays fg, bg;
    u32 last_density_iters = 0, last_divergence_iters = 0;
    R max_v = 0;
    R last_density_err = 0, last_divergence_err = 0;
    R xsph = 0;  // XSPH coefficient (Config::viscosity; a Dual carries its seed)

    void init(const Config& c, const float* fx, const float* fv, std::size_t n,
              const float* bx, std::size_t nb) {
        cfg = c;
        grid = make_grid(c);
        xsph = R(c.viscosity);
        l = R(c.smoothing_length);
        // The stencil reciprocal: the device value when given (every instance
        // centres its stencil with the device's float arithmetic), else the
        // IEEE float reciprocal.
        inv_stencil = c.stencil_inv_cell != 0.0f ? c.stencil_inv_cell : 1.0f / c.smoothing_length;
        // mass = rho0 * (2r)^3 (dfsph.cu:76-78), evaluated in float as there.
        const float spacing = 2.0f * c.particle_radius;
        const float v0 = spacing * spacing * spacing;
        // Both instances use this float value, so the FP64 oracle solves the
        // same problem as the FP32 runs.
        mass = R(c.rest_density * v0);
        x.resize(n); v.resize(n);
        for (std::size_t i = 0; i < n; ++i) {
            x[i] = {R(fx[3 * i]), R(fx[3 * i + 1]), R(fx[3 * i + 2])};
            v[i] = fv ? V3<R>{R(fv[3 * i]), R(fv[3 * i + 1]), R(fv[3 * i + 2])}
                      : V3<R>{R(0), R(0), R(0)};
        }
        rho.assign(n, R(0)); alpha.assign(n, R(0)); kappa.assign(n, R(0));
        rho_adv.assign(n, R(0)); kappa_v.assign(n, R(0)); rho_dot.assign(n, R(0));
        nbr_f.assign(n, 0); nbr_b.assign(n, 0);
        xb.resize(nb);
        for (std::size_t i = 0; i < nb; ++i) xb[i] = {R(bx[3 * i]), R(bx[3 * i + 1]), R(bx[3 * i + 2])};
        mb.assign(nb, R(0));
        fg.cell_start.assign(std::size_t(grid.total) + 1, 0u);
        bg.cell_start.assign(std::size_t(grid.total) + 1, 0u);
        if (nb > 0) {
            // Boundary grid built once (dfsph.cu:90-99) + Akinci mass.
            build_grid(xb.data(), nb, grid, bg);
            compute_boundary_mass();
        }
    }

    bool has_boundary() const { return !xb.empty(); }

    // compute_boundary_mass_kernel (dfsph_kernels.cu:40-65):
    // m_b = rho0 / max(sum_b' W, 1e-9), self included.
    void compute_boundary_mass() {
        const long long nb = (long long)xb.size();
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < nb; ++i) {
            R sum_w = 0;
            const V3<R> pi = xb[i];
            for_neighbors(pi, grid, inv_stencil, bg, [&](u32 j) {
                const V3<R> r = sub(pi, xb[j]);
                const R d = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
                sum_w += kernel_W(d, l);
            });
            mb[i] = R(cfg.rest_density) / std::max(sum_w, R(1e-9));
        }
    }

    // density_kernel (dfsph_kernels.cu:68-112) fused with neighbour counting:
    // rho = sum_fluid m W (self included) + sum_boundary m_b W.
    void compute_density() {
        const long long n = (long long)x.size();
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < n; ++i) {
            const V3<R> pi = x[i];
            R r_acc = 0;
            u32 cf = 0, cb = 0;
            for_neighbors(pi, grid, inv_stencil, fg, [&](u32 j) {
                const V3<R> r = sub(pi, x[j]);
                const R d = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
                r_acc += mass * kernel_W(d, l);
                ++cf;
            });
            if (has_boundary()) {
                for_neighbors(pi, grid, inv_stencil, bg, [&](u32 j) {
                    const V3<R> r = sub(pi, xb[j]);
                    const R d = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
                    r_acc += mb[j] * kernel_W(d, l);
                    ++cb;
                });
            }
            rho[i] = r_acc;
            nbr_f[i] = cf;
            nbr_b[i] = cb;
        }
    }

    // alpha_kernel (dfsph_kernels.cu:117-169).
    void compute_alpha() {
        const long long n = (long long)x.size();
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < n; ++i) {
            const V3<R> pi = x[i];
            V3<R> sg{0, 0, 0};
            R sq = 0;
            for_neighbors(pi, grid, inv_stencil, fg, [&](u32 j) {
                if ((long long)j == i) return;
                const V3<R> gW = kernel_gradW(sub(pi, x[j]), l);
                const V3<R> m{mass * gW.x, mass * gW.y, mass * gW.z};
                sg.x += m.x; sg.y += m.y; sg.z += m.z;
                sq += m.x * m.x + m.y * m.y + m.z * m.z;
            });
            if (has_boundary()) {
                for_neighbors(pi, grid, inv_stencil, bg, [&](u32 j) {
                    const V3<R> gW = kernel_gradW(sub(pi, xb[j]), l);
                    const V3<R> m{mb[j] * gW.x, mb[j] * gW.y, mb[j] * gW.z};
                    sg.x += m.x; sg.y += m.y; sg.z += m.z;
                    sq += m.x * m.x + m.y * m.y + m.z * m.z;
                });
            }
            const R denom = sg.x * sg.x + sg.y * sg.y + sg.z * sg.z + sq;
            alpha[i] = (denom > R(1e-9)) ? (rho[i] / denom) : R(0);
        }
    }

    // apply_gravity_kernel (dfsph_kernels.cu:347-355): v <- v e^{-d dt} + g dt.
    void apply_external_forces(R dt) {
        const R decay = exp(-R(cfg.damping) * dt);
        const R g[3] = {R(cfg.gravity[0]), R(cfg.gravity[1]), R(cfg.gravity[2])};
        const long long n = (long long)x.size();
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; ++i) {
            v[i].x = v[i].x * decay + g[0] * dt;
            v[i].y = v[i].y * decay + g[1] * dt;
            v[i].z = v[i].z * decay + g[2] * dt;
        }
    }

    // xsph_viscosity_kernel (dfsph_kernels.cu:305-341), Jacobi form: every
    // particle reads the velocities as they were before this pass.
    void apply_xsph() {
        if (!(cfg.viscosity > 0.0f)) return;  // dfsph.cu:198
        const R eps = xsph;
        const std::vector<V3<R>> v0 = v;
        const long long n = (long long)x.size();
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < n; ++i) {
            const V3<R> pi = x[i];
            const V3<R> vi = v0[i];
            const R rho_i = rho[i];
            V3<R> d{0, 0, 0};
            for_neighbors(pi, grid, inv_stencil, fg, [&](u32 j) {
                if ((long long)j == i) return;
                const V3<R> r = sub(pi, x[j]);
                const R dist = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
                const R W = kernel_W(dist, l);
                const R rho_avg = R(0.5) * (rho_i + rho[j]);
                const R c = eps * (mass / std::max(rho_avg, R(1e-9))) * W;
                d.x += c * (v0[j].x - vi.x);
                d.y += c * (v0[j].y - vi.y);
                d.z += c * (v0[j].z - vi.z);
            });
            v[i].x = vi.x + d.x;
            v[i].y = vi.y + d.y;
            v[i].z = vi.z + d.z;
        }
    }

    // sum_j m (v_i - v_j).gradW_ij over fluid (self skipped) + sum_b m_b v_i.gradW
    // (the rho_dot of density_change_kernel, dfsph_kernels.cu:196-224).
    R density_rate(long long i) const {
        const V3<R> pi = x[i];
        const V3<R> vi = v[i];
        R rd = 0;
        for_neighbors(pi, grid, inv_stencil, fg, [&](u32 j) {
            if ((long long)j == i) return;
            const V3<R> gW = kernel_gradW(sub(pi, x[j]), l);
            const V3<R> dv = sub(vi, v[j]);
            rd += mass * (dv.x * gW.x + dv.y * gW.y + dv.z * gW.z);
        });
        if (has_boundary()) {
            for_neighbors(pi, grid, inv_stencil, bg, [&](u32 j) {
                const V3<R> gW = kernel_gradW(sub(pi, xb[j]), l);
                rd += mb[j] * (vi.x * gW.x + vi.y * gW.y + vi.z * gW.z);
            });
        }
        return rd;
    }

    // apply_kappa_kernel (dfsph_kernels.cu:237-301):
    // v_i += -dt sum_j m (k_i/max(rho_i^2,1e-9) + k_j/max(rho_j^2,1e-9)) gradW,
    // boundary with k_j = k_i and rho_j = rho0 (mirror).
    void apply_kappa(const std::vector<R>& k, R dt) {
        const long long n = (long long)x.size();
        const R rho0 = R(cfg.rest_density);
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < n; ++i) {
            const V3<R> pi = x[i];
            const R rho_i = rho[i];
            const R k_i = k[i];
            const R kif = k_i / std::max(rho_i * rho_i, R(1e-9));
            V3<R> dv{0, 0, 0};
            for_neighbors(pi, grid, inv_stencil, fg, [&](u32 j) {
                if ((long long)j == i) return;
                const R rho_j = rho[j];
                const V3<R> gW = kernel_gradW(sub(pi, x[j]), l);
                const R kjf = k[j] / std::max(rho_j * rho_j, R(1e-9));
                const R c2 = mass * (kif + kjf);
                dv.x -= dt * c2 * gW.x;
                dv.y -= dt * c2 * gW.y;
                dv.z -= dt * c2 * gW.z;
            });
            if (has_boundary()) {
                const R bf = k_i / std::max(rho0 * rho0, R(1e-9));
                for_neighbors(pi, grid, inv_stencil, bg, [&](u32 j) {
                    const V3<R> gW = kernel_gradW(sub(pi, xb[j]), l);
                    const R c2 = mb[j] * (kif + bf);
                    dv.x -= dt * c2 * gW.x;
                    dv.y -= dt * c2 * gW.y;
                    dv.z -= dt * c2 * gW.z;
                });
            }
            v[i].x += dv.x;
            v[i].y += dv.y;
            v[i].z += dv.z;
        }
    }

    // density_solve (dfsph.cu:215-260) with density_change_kernel
    // (dfsph_kernels.cu:176-232) and the error of reduce_density_error_
    // (dfsph.cu:277-301): mean over all n of max(0, rho* - rho0), checked from
    // the second iteration on.
    void density_solve(R dt) {
        const long long n = (long long)x.size();
        const R rho0 = R(cfg.rest_density);
        last_density_iters = 0;
        for (u32 it = 0; it < cfg.max_density_iters; ++it) {
#pragma omp parallel for schedule(dynamic, 256)
            for (long long i = 0; i < n; ++i) {
                const R rd = density_rate(i);
                const R rp = rho[i] + dt * rd;
                rho_adv[i] = rp;
                const R over = std::max(R(0), rp - rho0);
                kappa[i] = over * alpha[i] / (dt * dt);
            }
            apply_kappa(kappa, dt);
            last_density_iters = it + 1;
            if (it >= 1) {
                double s = 0;
                for (long long i = 0; i < n; ++i) s += double(std::max(R(0), rho_adv[i] - rho0));
                const R err = R(s / double(n));
                last_density_err = err;
                if (err < R(cfg.eta_density) * rho0) break;
            }
        }
    }

    // Divergence solver as specified in the reference's plan
    // (docs/superpowers/plans/2026-04-24-water-simulation-v2-phase2-dfsph-solver.md
    // :1856-1910,1958-1987): s = max(0, rho_dot), kappa_v = s alpha / dt, the
    // apply_kappa velocity update, stop when mean(max(0, rho_dot)) < eta_div rho0
    // (checked every iteration).
    void divergence_solve(R dt) {
        const long long n = (long long)x.size();
        last_divergence_iters = 0;
        for (u32 it = 0; it < cfg.max_divergence_iters; ++it) {
#pragma omp parallel for schedule(dynamic, 256)
            for (long long i = 0; i < n; ++i) {
                const R rd = density_rate(i);
                rho_dot[i] = rd;
                kappa_v[i] = std::max(R(0), rd) * alpha[i] / dt;
            }
            apply_kappa(kappa_v, dt);
            last_divergence_iters = it + 1;
            double s = 0;
            for (long long i = 0; i < n; ++i) s += double(std::max(R(0), rho_dot[i]));
            const R err = R(s / double(n));
            last_divergence_err = err;
            if (err < R(cfg.eta_divergence) * R(cfg.rest_density)) break;
        }
    }

    // advect_kernel (dfsph_kernels.cu:363-386), MAX_VELOCITY_CLAMP = 5
    // (dfsph.cu:268), then the max-|v| reduction (dfsph.cu:303-326).
    void advect(R dt) {
        const R max_vc = R(5);
        const R eps = R(1e-3);
        const R lo[3] = {R(cfg.domain_min[0]), R(cfg.domain_min[1]), R(cfg.domain_min[2])};
        const R hi[3] = {R(cfg.domain_max[0]), R(cfg.domain_max[1]), R(cfg.domain_max[2])};
        const long long n = (long long)x.size();
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; ++i) {
            V3<R> vv = v[i];
            const R sp = sqrt(vv.x * vv.x + vv.y * vv.y + vv.z * vv.z);
            if (sp > max_vc) {
                const R s = max_vc / sp;
                vv.x *= s; vv.y *= s; vv.z *= s;
            }
            V3<R> p{x[i].x + vv.x * dt, x[i].y + vv.y * dt, x[i].z + vv.z * dt};
            if (p.x < lo[0] + eps) { p.x = lo[0] + eps; if (vv.x < 0) vv.x = 0; }
            if (p.y < lo[1] + eps) { p.y = lo[1] + eps; if (vv.y < 0) vv.y = 0; }
            if (p.z < lo[2] + eps) { p.z = lo[2] + eps; if (vv.z < 0) vv.z = 0; }
            if (p.x > hi[0] - eps) { p.x = hi[0] - eps; if (vv.x > 0) vv.x = 0; }
            if (p.y > hi[1] - eps) { p.y = hi[1] - eps; if (vv.y > 0) vv.y = 0; }
            if (p.z > hi[2] - eps) { p.z = hi[2] - eps; if (vv.z > 0) vv.z = 0; }
            v[i] = vv;
            x[i] = p;
        }
        R m = 0;
        bool nan = false;
        for (long long i = 0; i < n; ++i) {
            const R s = sqrt(v[i].x * v[i].x + v[i].y * v[i].y + v[i].z * v[i].z);
            if (s != s) nan = true;
            m = std::max(m, s);
        }
        max_v = nan ? std::numeric_limits<R>::quiet_NaN() : m;
    }

    // DFSPHSolver::step (dfsph.cu:120-133), with the divergence solve after alpha.
    void step(R dt) {
        if (x.empty()) return;  // dfsph.cu:121-122
        build_grid(x.data(), x.size(), grid, fg);
        compute_density();
        compute_alpha();
        if (cfg.max_divergence_iters > 0) divergence_solve(dt);
        apply_external_forces(dt);
        apply_xsph();
        density_solve(dt);
        advect(dt);
    }
};

}  // namespace oracle

// ----------------------------------------------------------------------------
// C interface for the Python tests (ctypes).
// ----------------------------------------------------------------------------
using oracle::Config;
using oracle::Solver;
using oracle::u32;

namespace {
struct Handle {
    int precision;  // 32 or 64
    Solver<float>* s32 = nullptr;
    Solver<double>* s64 = nullptr;
};

enum Field : int {
    F_POSITION = 0, F_VELOCITY = 1, F_DENSITY = 2, F_ALPHA = 3, F_KAPPA = 4,
    F_DENSITY_ADV = 5, F_CELL_KEY = 6, F_SORTED_INDEX = 7, F_CELL_START = 8,
    F_NBR_FLUID = 9, F_NBR_BOUNDARY = 10, F_BOUNDARY_MASS = 11, F_KAPPA_V = 12,
    F_BOUNDARY_CELL_START = 13, F_BOUNDARY_SORTED_INDEX = 14,
};

template <class R>
int get_field(Solver<R>& s, int field, void* out) {
    const std::size_t n = s.x.size();
    auto put_real = [&](const std::vector<R>& a) {
        double* o = static_cast<double*>(out);
        for (std::size_t i = 0; i < a.size(); ++i) o[i] = double(a[i]);
        return 0;
    };
    auto put_v3 = [&](const std::vector<oracle::V3<R>>& a) {
        double* o = static_cast<double*>(out);
        for (std::size_t i = 0; i < a.size(); ++i) {
            o[3 * i] = double(a[i].x); o[3 * i + 1] = double(a[i].y); o[3 * i + 2] = double(a[i].z);
        }
        return 0;
    };
    auto put_u32 = [&](const std::vector<u32>& a) {
        if (!a.empty()) std::memcpy(out, a.data(), a.size() * sizeof(u32));
        return 0;
    };
    (void)n;
    switch (field) {
        case F_POSITION: return put_v3(s.x);
        case F_VELOCITY: return put_v3(s.v);
        case F_DENSITY: return put_real(s.rho);
        case F_ALPHA: return put_real(s.alpha);
        case F_KAPPA: return put_real(s.kappa);
        case F_DENSITY_ADV: return put_real(s.rho_adv);
        case F_CELL_KEY: return put_u32(s.fg.keys);
        case F_SORTED_INDEX: return put_u32(s.fg.sorted);
        case F_CELL_START: return put_u32(s.fg.cell_start);
        case F_NBR_FLUID: return put_u32(s.nbr_f);
        case F_NBR_BOUNDARY: return put_u32(s.nbr_b);
        case F_BOUNDARY_MASS: return put_real(s.mb);
        case F_KAPPA_V: return put_real(s.kappa_v);
        case F_BOUNDARY_CELL_START: return put_u32(s.bg.cell_start);
        case F_BOUNDARY_SORTED_INDEX: return put_u32(s.bg.sorted);
        default: return -1;
    }
}
}  // namespace

extern "C" {

// sample_aabb_boundary (solvers/dfsph/src/boundary_sampler.cpp:6-32): six faces,
// n_layers inward layers each, float-accumulated u/v loops, edges duplicated.
// Writes up to `cap` points (xyz) to `out` and returns the total count.
long long oracle_sample_aabb_boundary(const float lo[3], const float hi[3], float spacing,
                                      int n_layers, float* out, long long cap) {
    long long count = 0;
    auto emit_face = [&](int axis, float face_coord, float inward_step) {
        const int ua = (axis + 1) % 3, va = (axis + 2) % 3;
        for (int layer = 0; layer < n_layers; ++layer) {
            const float axis_pos = face_coord + static_cast<float>(layer) * inward_step;
            for (float u = lo[ua]; u <= hi[ua] + 0.5f * spacing; u += spacing)
                for (float w = lo[va]; w <= hi[va] + 0.5f * spacing; w += spacing) {
                    if (out && count < cap) {
                        float* p = out + 3 * count;
                        p[axis] = axis_pos; p[ua] = u; p[va] = w;
                    }
                    ++count;
                }
        }
    };
    emit_face(0, lo[0], spacing);
    emit_face(0, hi[0], -spacing);
    emit_face(1, lo[1], spacing);
    emit_face(1, hi[1], -spacing);
    emit_face(2, lo[2], spacing);
    emit_face(2, hi[2], -spacing);
    return count;
}

// SpatialAccel's Morton order (core/src/spatial_accel.cu:11-40,110-179): each
// coordinate normalised by the host reciprocal of the scene extent (0 for a
// flat axis), clamped to [0, 1023] after * 1024 and truncated; 10 bits per axis
// interleaved x, y, z (x highest); stable sort of (code, index).
int oracle_morton_sort(const float* xyz, u32 n, const float smin[3], const float smax[3], u32* codes_out,
                       u32* idx_out) {
    float inv[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = smax[a] - smin[a];
        inv[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    auto spread = [](u32 v) {
        u32 o = 0;
        for (int k = 0; k < 10; ++k) o |= ((v >> k) & 1u) << (3 * k);
        return o;
    };
    std::vector<u32> code(n), idx(n);
    for (u32 i = 0; i < n; ++i) {
        u32 q[3];
        for (int a = 0; a < 3; ++a) {
            const float t = (xyz[3 * i + a] - smin[a]) * inv[a];
            const float c = std::fmin(std::fmax(t * 1024.0f, 0.0f), 1023.0f);
            q[a] = static_cast<u32>(c);
        }
        code[i] = (spread(q[0]) << 2) | (spread(q[1]) << 1) | spread(q[2]);
        idx[i] = i;
    }
    std::stable_sort(idx.begin(), idx.end(), [&](u32 a, u32 b) { return code[a] < code[b]; });
    for (u32 s = 0; s < n; ++s) {
        codes_out[s] = code[idx[s]];
        idx_out[s] = idx[s];
    }
    return 0;
}

// SpatialAccel's internal nodes (core/src/spatial_accel.cu:42-97): for each
// internal node, the reference's delta with the index tie-break, its range
// direction, doubling + bisection for the range end and its split search,
// restated loop for loop; leaf boxes p +- radius (init_leaf_aabbs,
// spatial_accel.cu:99-107); internal boxes as the union of their subtree's
// leaf boxes (the pass the reference leaves for later). Inputs: the sorted
// codes and permutation of oracle_morton_sort. Outputs as dfsph_lbvh_build.
static int clz32(u32 v) {
    int c = 0;
    for (u32 m = 0x80000000u; m && !(v & m); m >>= 1) ++c;
    return c;
}

static int lbvh_delta(int i, int j, const u32* codes, int n) {
    if (j < 0 || j >= n) return -1;
    const u32 ci = codes[i], cj = codes[j];
    if (ci == cj) return 32 + clz32(static_cast<u32>(i ^ j));
    return clz32(ci ^ cj);
}

int oracle_lbvh_build(const float* xyz, u32 n, const u32* codes, const u32* sorted, float radius, u32* left,
                      u32* right, u32* parent, float* boxes) {
    if (n == 0) return 0;
    const int nl = static_cast<int>(n);
    const int n_internal = nl - 1;
    parent[0] = 0xFFFFFFFFu;
    for (int i = 0; i < n_internal; ++i) {
        const int d = (lbvh_delta(i, i + 1, codes, nl) - lbvh_delta(i, i - 1, codes, nl)) > 0 ? 1 : -1;
        const int delta_min = lbvh_delta(i, i - d, codes, nl);
        int l_max = 2;
        while (lbvh_delta(i, i + l_max * d, codes, nl) > delta_min) l_max *= 2;
        int l = 0;
        for (int t = l_max / 2; t > 0; t /= 2)
            if (lbvh_delta(i, i + (l + t) * d, codes, nl) > delta_min) l += t;
        const int j = i + l * d;
        const int delta_node = lbvh_delta(i, j, codes, nl);
        int s = 0;
        int t = (l + 1) / 2;
        while (t > 0) {
            if (lbvh_delta(i, i + (s + t) * d, codes, nl) > delta_node) s += t;
            t = (t == 1) ? 0 : (t + 1) / 2;
        }
        const int gamma = i + s * d + std::min(d, 0);
        const int lc = (std::min(i, j) == gamma) ? (n_internal + gamma) : gamma;
        const int rc = (std::max(i, j) == gamma + 1) ? (n_internal + gamma + 1) : (gamma + 1);
        left[i] = static_cast<u32>(lc);
        right[i] = static_cast<u32>(rc);
        parent[lc] = static_cast<u32>(i);
        parent[rc] = static_cast<u32>(i);
    }
    for (int k = 0; k < nl; ++k) {
        const float* p = xyz + 3 * std::size_t(sorted[k]);
        float* b = boxes + 6 * std::size_t(n_internal + k);
        for (int a = 0; a < 3; ++a) {
            b[a] = p[a] - radius;
            b[3 + a] = p[a] + radius;
        }
    }
    // children before parents: post-order over an explicit stack
    if (n_internal > 0) {
        std::vector<std::pair<u32, bool>> stack{{0u, false}};
        while (!stack.empty()) {
            const auto [node, expanded] = stack.back();
            stack.pop_back();
            if (node >= static_cast<u32>(n_internal)) continue;
            if (!expanded) {
                stack.push_back({node, true});
                stack.push_back({left[node], false});
                stack.push_back({right[node], false});
                continue;
            }
            const float* a = boxes + 6 * std::size_t(left[node]);
            const float* c = boxes + 6 * std::size_t(right[node]);
            float* o = boxes + 6 * std::size_t(node);
            for (int k = 0; k < 3; ++k) {
                o[k] = std::min(a[k], c[k]);
                o[3 + k] = std::max(a[3 + k], c[3 + k]);
            }
        }
    }
    return 0;
}

// cohesion_C (core/include/water/core/sph_kernels.cuh:44-51), in double.
double oracle_cohesion_C(double r, double l) {
    if (r <= 0.0 || r > l) return 0.0;
    const double sigma = 32.0 / (3.14159265358979323846 * std::pow(l, 9.0));
    const double lm = l - r;
    const double t = lm * lm * lm * r * r * r;
    if (2.0 * r > l) return sigma * t;
    return sigma * (2.0 * t - std::pow(l, 6.0) / 64.0);
}

// make_grid geometry (dfsph.cu:55-65).
void oracle_grid_geometry(const Config* cfg, float origin[3], int dims[3]) {
    const oracle::Grid g = oracle::make_grid(*cfg);
    for (int a = 0; a < 3; ++a) { origin[a] = g.origin[a]; dims[a] = g.dims[a]; }
}

// One CellGrid::build on an arbitrary grid (core/src/cell_grid.cu:73-138), FP32.
// cell_start must hold dims.x*dims.y*dims.z + 1 entries.
int oracle_build_grid_f32(const float* xyz, u32 n, const float origin[3], const int dims[3],
                          float cell_length, u32* keys, u32* sorted, u32* cell_start) {
    oracle::Grid g;
    for (int a = 0; a < 3; ++a) { g.origin[a] = origin[a]; g.dims[a] = dims[a]; }
    g.cell_length = cell_length;
    g.total = u32(dims[0]) * u32(dims[1]) * u32(dims[2]);
    std::vector<oracle::V3<float>> p(n);
    for (u32 i = 0; i < n; ++i) p[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    oracle::GridArrays ga;
    ga.cell_start.assign(std::size_t(g.total) + 1, 0u);
    oracle::build_grid(p.data(), n, g, ga);
    if (n) {
        std::memcpy(keys, ga.keys.data(), n * sizeof(u32));
        std::memcpy(sorted, ga.sorted.data(), n * sizeof(u32));
    }
    std::memcpy(cell_start, ga.cell_start.data(), ga.cell_start.size() * sizeof(u32));
    return 0;
}

// Single cubic-spline evaluations (sph_kernels.cuh:12-41), FP32 and FP64.
float oracle_W_f32(float r, float l) { return oracle::kernel_W<float>(r, l); }
double oracle_W_f64(double r, double l) { return oracle::kernel_W<double>(r, l); }
void oracle_gradW_f32(const float rij[3], float l, float out[3]) {
    const auto g = oracle::kernel_gradW<float>({rij[0], rij[1], rij[2]}, l);
    out[0] = g.x; out[1] = g.y; out[2] = g.z;
}

void* oracle_create(const Config* cfg, int precision, const float* fluid_xyz,
                    const float* fluid_v, u32 n, const float* boundary_xyz, u32 nb) {
    Handle* h = new Handle;
    h->precision = precision;
    if (precision == 64) {
        h->s64 = new Solver<double>;
        h->s64->init(*cfg, fluid_xyz, fluid_v, n, boundary_xyz, nb);
    } else {
        h->precision = 32;
        h->s32 = new Solver<float>;
        h->s32->init(*cfg, fluid_xyz, fluid_v, n, boundary_xyz, nb);
    }
    return h;
}

void oracle_destroy(void* p) {
    Handle* h = static_cast<Handle*>(p);
    if (!h) return;
    delete h->s32;
    delete h->s64;
    delete h;
}

int oracle_step(void* p, float dt, u32 n_steps) {
    Handle* h = static_cast<Handle*>(p);
    for (u32 k = 0; k < n_steps; ++k) {
        if (h->s32) h->s32->step(dt);
        else h->s64->step(double(dt));
    }
    return 0;
}

int oracle_get(void* p, int field, void* out) {
    Handle* h = static_cast<Handle*>(p);
    return h->s32 ? get_field(*h->s32, field, out) : get_field(*h->s64, field, out);
}

// scalars: 0 max_velocity, 1 particle_mass, 2 last_density_iters,
// 3 last_divergence_iters, 4 last density error, 5 last divergence error,
// 6 total cells, 7 stencil reciprocal in use
double oracle_scalar(void* p, int which) {
    Handle* h = static_cast<Handle*>(p);
    auto f = [&](auto& s) -> double {
        switch (which) {
            case 0: return double(s.max_v);
            case 1: return double(s.mass);
            case 2: return double(s.last_density_iters);
            case 3: return double(s.last_divergence_iters);
            case 4: return double(s.last_density_err);
            case 5: return double(s.last_divergence_err);
            case 6: return double(s.grid.total);
            case 7: return double(s.inv_stencil);
            default: return 0.0;
        }
    };
    return h->s32 ? f(*h->s32) : f(*h->s64);
}

// Forward-mode (dual number) instance: the same FP64 step carrying the
// derivative along the direction (dx, dv, d_xsph) of the initial positions,
// velocities and XSPH coefficient. Used to test the GPU adjoint only.
void* oracle_dual_create(const Config* cfg, const float* fluid_xyz, const float* fluid_v, u32 n,
                         const float* boundary_xyz, u32 nb, const double* dx, const double* dv, double d_xsph) {
    auto* s = new Solver<oracle::Dual>;
    s->init(*cfg, fluid_xyz, fluid_v, n, boundary_xyz, nb);
    for (u32 i = 0; i < n; ++i) {
        if (dx) { s->x[i].x.d = dx[3 * i]; s->x[i].y.d = dx[3 * i + 1]; s->x[i].z.d = dx[3 * i + 2]; }
        if (dv) { s->v[i].x.d = dv[3 * i]; s->v[i].y.d = dv[3 * i + 1]; s->v[i].z.d = dv[3 * i + 2]; }
    }
    s->xsph.d = d_xsph;
    return s;
}

int oracle_dual_step(void* p, float dt, u32 n_steps) {
    auto* s = static_cast<Solver<oracle::Dual>*>(p);
    for (u32 k = 0; k < n_steps; ++k) s->step(oracle::Dual(double(dt)));
    return 0;
}

// Values and derivatives of positions and velocities (double[3n] each; any may be NULL).
int oracle_dual_get(void* p, double* x, double* v, double* dx, double* dv) {
    auto* s = static_cast<Solver<oracle::Dual>*>(p);
    for (std::size_t i = 0; i < s->x.size(); ++i) {
        const oracle::V3<oracle::Dual>& a = s->x[i];
        const oracle::V3<oracle::Dual>& b = s->v[i];
        if (x) { x[3 * i] = a.x.v; x[3 * i + 1] = a.y.v; x[3 * i + 2] = a.z.v; }
        if (dx) { dx[3 * i] = a.x.d; dx[3 * i + 1] = a.y.d; dx[3 * i + 2] = a.z.d; }
        if (v) { v[3 * i] = b.x.v; v[3 * i + 1] = b.y.v; v[3 * i + 2] = b.z.v; }
        if (dv) { dv[3 * i] = b.x.d; dv[3 * i + 1] = b.y.d; dv[3 * i + 2] = b.z.d; }
    }
    return 0;
}

void oracle_dual_destroy(void* p) { delete static_cast<Solver<oracle::Dual>*>(p); }

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
