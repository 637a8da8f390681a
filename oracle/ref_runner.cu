// oracle/ref_runner.cu — TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own compiled DFSPH kernels on the GPU: the kernels of
// solvers/dfsph/src/dfsph_kernels.cu and core/src/cell_grid.cu, compiled from
// the reference sources by oracle/build.py into oracle/_ref/*.fatbin, are loaded
// with the driver API and launched by this host code, which restates the
// reference's host orchestration:
//   * CellGrid::build            (core/src/cell_grid.cu:73-138)
//   * DFSPHSolver ctor / step    (solvers/dfsph/src/dfsph.cu:71-133)
//   * density_solve / advect     (dfsph.cu:215-273)
//   * the CUB reductions         (dfsph.cu:277-326)
// with the same launch shapes (256-thread grid kernels, 128-thread solver
// kernels, the serial 1x1 cell_start pass), the same per-build stream-ordered
// allocations and the same host synchronisations. CUB comes from the CUDA
// toolkit and is called exactly as the reference calls it.
//
// Used for golden vectors (tests/golden/) and for timing the reference CUDA
// step next to this project's step. Never part of the product.

#include <cuda.h>
#include <cuda_runtime.h>
#include <cxxabi.h>

#include <cub/cub.cuh>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

// Same layout as oracle::Config (dfsph_oracle.cpp); stencil_inv_cell unused.
// Declared outside the anonymous namespace: the extern "C" entry points take it.
struct RefConfig {
    float rest_density, particle_radius, smoothing_length, viscosity, damping, surface_tension;
    float gravity[3];
    std::uint32_t max_density_iters, max_divergence_iters;
    float eta_density, eta_divergence;
    float domain_min[3], domain_max[3];
    float stencil_inv_cell;
};

namespace {

using u32 = std::uint32_t;
struct Vec3f { float x, y, z; };
struct Vec3i { int x, y, z; };

struct Fail : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define RT(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) throw Fail(std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define DRV(x)                                                                         \
    do {                                                                               \
        CUresult r_ = (x);                                                             \
        if (r_ != CUDA_SUCCESS) {                                                      \
            const char* s_ = nullptr;                                                  \
            cuGetErrorString(r_, &s_);                                                 \
            throw Fail(std::string(#x) + ": " + (s_ ? s_ : "?"));                      \
        }                                                                              \
    } while (0)

std::string demangle(const char* m) {
    int st = 0;
    char* d = abi::__cxa_demangle(m, nullptr, nullptr, &st);
    std::string s = (st == 0 && d) ? d : m;
    std::free(d);
    return s;
}

struct Module {
    CUmodule mod = nullptr;
    std::vector<std::pair<std::string, CUfunction>> fns;
    void load(const std::string& path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw Fail("cannot open " + path);
        std::vector<char> buf((std::istreambuf_iterator<char>(f)), {});
        DRV(cuModuleLoadData(&mod, buf.data()));
        unsigned int n = 0;
        DRV(cuModuleGetFunctionCount(&n, mod));
        std::vector<CUfunction> v(n);
        DRV(cuModuleEnumerateFunctions(v.data(), n, mod));
        for (CUfunction fn : v) {
            const char* nm = nullptr;
            DRV(cuFuncGetName(&nm, fn));
            fns.emplace_back(demangle(nm), fn);
        }
    }
    // kernel whose demangled name starts with `qualified` followed by '('
    CUfunction get(const std::string& qualified) const {
        for (auto& p : fns)
            if (p.first.compare(0, qualified.size() + 1, qualified + "(") == 0) return p.second;
        throw Fail("kernel not found in fatbin: " + qualified);
    }
};

struct Kernels {
    CUfunction cell_ids, fill, scatter, propagate;
    CUfunction bmass, density, alpha, dchange, kappa, xsph, gravity, advect, derr, vmag;
};

void launch(CUfunction f, unsigned grid, unsigned block, void** args) {
    if (grid == 0) return;
    DRV(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, /*stream 0*/ nullptr, args, nullptr));
}

template <class T> struct Buf {
    T* p = nullptr;
    size_t n = 0;
    Buf() = default;
    explicit Buf(size_t count) { reset(count); }
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    Buf(Buf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    Buf& operator=(Buf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~Buf() { release(); }
    void release() { if (p) cudaFreeAsync(p, 0); p = nullptr; n = 0; }
    void reset(size_t count) {
        release();
        if (count) RT(cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(T), 0));
        n = count;
    }
};

// CellGrid (core/include/water/core/cell_grid.h:16-50, core/src/cell_grid.cu).
struct Grid {
    Vec3f origin;
    Vec3i dims;
    float cell;
    size_t capacity = 0, count = 0;
    Buf<u32> cell_ids, sorted, cell_start;
    Buf<unsigned char> cub_temp;
    const Kernels* k;
    Grid(Vec3f o, Vec3i d, float c, const Kernels* kk) : origin(o), dims(d), cell(c), k(kk) {
        cell_start.reset(size_t(total()) + 1);
        RT(cudaMemsetAsync(cell_start.p, 0, cell_start.n * sizeof(u32), 0));
    }
    u32 total() const { return u32(dims.x) * u32(dims.y) * u32(dims.z); }
    void reserve(size_t cap) {
        if (cap <= capacity) return;
        capacity = cap;
        cell_ids.reset(cap);
        sorted.reset(cap);
    }
    void build(const Vec3f* pos, size_t n) {
        if (n == 0) { count = 0; return; }
        if (n > capacity) reserve(n);
        count = n;
        float inv = 1.0f / cell;
        {
            void* a[] = {(void*)&pos, &cell_ids.p, &sorted.p, &n, &origin, &inv, &dims};
            launch(k->cell_ids, unsigned((n + 255) / 256), 256, a);
        }
        Buf<u32> sk(n), sv(n);
        size_t bytes = 0;
        RT(cub::DeviceRadixSort::SortPairs(nullptr, bytes, cell_ids.p, sk.p, sorted.p, sv.p, int(n), 0, 32, 0));
        if (bytes > cub_temp.n) cub_temp.reset(bytes);
        RT(cub::DeviceRadixSort::SortPairs(cub_temp.p, bytes, cell_ids.p, sk.p, sorted.p, sv.p, int(n), 0, 32, 0));
        RT(cudaMemcpyAsync(cell_ids.p, sk.p, n * sizeof(u32), cudaMemcpyDeviceToDevice, 0));
        RT(cudaMemcpyAsync(sorted.p, sv.p, n * sizeof(u32), cudaMemcpyDeviceToDevice, 0));
        u32 sentinel = u32(n);
        size_t cs = size_t(total()) + 1;
        {
            void* a[] = {&cell_start.p, &sentinel, &cs};
            launch(k->fill, unsigned((cs + 255) / 256), 256, a);
        }
        {
            void* a[] = {&cell_ids.p, &cell_start.p, &n};
            launch(k->scatter, unsigned((n + 255) / 256), 256, a);
        }
        {
            void* a[] = {&cell_start.p, &cs};
            launch(k->propagate, 1, 1, a);
        }
    }
};

Grid make_grid(const RefConfig& c, const Kernels* k) {
    Vec3i d;
    d.x = int(std::ceil((c.domain_max[0] - c.domain_min[0]) / c.smoothing_length)) + 2;
    d.y = int(std::ceil((c.domain_max[1] - c.domain_min[1]) / c.smoothing_length)) + 2;
    d.z = int(std::ceil((c.domain_max[2] - c.domain_min[2]) / c.smoothing_length)) + 2;
    Vec3f o{c.domain_min[0] - c.smoothing_length, c.domain_min[1] - c.smoothing_length,
            c.domain_min[2] - c.smoothing_length};
    return Grid(o, d, c.smoothing_length, k);
}

struct Runner {
    Module grid_mod, dfsph_mod;
    Kernels k;
    RefConfig cfg;
    size_t n = 0, nb = 0;
    float mass = 0, max_v = 0;
    u32 last_iters = 0;
    Buf<Vec3f> pos, vel, bpos;
    Buf<float> density, alpha, kappa, density_adv, bmass, reduce_in, reduce_out;
    Buf<unsigned char> reduce_temp;
    std::unique_ptr<Grid> fg, bg;

    Runner(const std::string& dir, const RefConfig& c, const float* x, const float* v, size_t n_, const float* bx,
           size_t nb_)
        : cfg(c), n(n_), nb(nb_) {
        RT(cudaFree(nullptr));  // primary context
        grid_mod.load(dir + "/cell_grid.fatbin");
        dfsph_mod.load(dir + "/dfsph_kernels.fatbin");
        const std::string g = "water::(anonymous namespace)::";
        k.cell_ids = grid_mod.get(g + "compute_cell_ids");
        k.fill = grid_mod.get(g + "fill_u32");
        k.scatter = grid_mod.get(g + "scatter_starts");
        k.propagate = grid_mod.get(g + "propagate_starts_right_to_left");
        const std::string s = "water::solvers::detail::";
        k.bmass = dfsph_mod.get(s + "compute_boundary_mass_kernel");
        k.density = dfsph_mod.get(s + "density_kernel");
        k.alpha = dfsph_mod.get(s + "alpha_kernel");
        k.dchange = dfsph_mod.get(s + "density_change_kernel");
        k.kappa = dfsph_mod.get(s + "apply_kappa_kernel");
        k.xsph = dfsph_mod.get(s + "xsph_viscosity_kernel");
        k.gravity = dfsph_mod.get(s + "apply_gravity_kernel");
        k.advect = dfsph_mod.get(s + "advect_kernel");
        k.derr = dfsph_mod.get(s + "density_error_kernel");
        k.vmag = dfsph_mod.get(s + "velocity_magnitude_kernel");

        // ParticleStore: zero-filled attributes (particle_store.h:109-127)
        auto zf = [&](auto& b, size_t count) {
            b.reset(std::max<size_t>(count, 1));
            RT(cudaMemsetAsync(b.p, 0, b.n * sizeof(*b.p), 0));
        };
        zf(pos, n); zf(vel, n);
        if (n) RT(cudaMemcpy(pos.p, x, n * sizeof(Vec3f), cudaMemcpyHostToDevice));
        if (n && v) RT(cudaMemcpy(vel.p, v, n * sizeof(Vec3f), cudaMemcpyHostToDevice));
        // DFSPHSolver ctor (dfsph.cu:71-100)
        fg.reset(new Grid(make_grid(cfg, &k)));
        const float spacing = 2.0f * cfg.particle_radius;
        const float v0 = spacing * spacing * spacing;
        mass = cfg.rest_density * v0;
        zf(density, n); zf(alpha, n); zf(kappa, n); zf(density_adv, n);
        fg->reserve(n);
        reduce_in.reset(std::max<size_t>(n, 1));
        reduce_out.reset(1);
        if (bx && nb) {
            zf(bpos, nb);
            RT(cudaMemcpy(bpos.p, bx, nb * sizeof(Vec3f), cudaMemcpyHostToDevice));
            zf(bmass, nb);
            bg.reset(new Grid(make_grid(cfg, &k)));
            bg->reserve(nb);
            bg->build(bpos.p, nb);
            compute_boundary_mass();
        }
        RT(cudaDeviceSynchronize());
    }

    void compute_boundary_mass() {
        Vec3f o = bg->origin;
        Vec3i d = bg->dims;
        float cl = bg->cell, rho0 = cfg.rest_density, l = cfg.smoothing_length;
        void* a[] = {&bpos.p, &bg->sorted.p, &bg->cell_start.p, &bmass.p, &nb, &o, &d, &cl, &rho0, &l};
        launch(k.bmass, unsigned((nb + 127) / 128), 128, a);
    }

    // the boundary tail of the solver kernels' argument lists
    struct BArgs {
        const Vec3f* pb; const u32* sb; const u32* cb; const float* mb;
        Vec3f ob; Vec3i db; float lb; size_t nb;
    };
    BArgs bargs() const {
        BArgs b{};
        if (bg) {
            b.pb = bpos.p; b.sb = bg->sorted.p; b.cb = bg->cell_start.p; b.mb = bmass.p;
            b.ob = bg->origin; b.db = bg->dims; b.lb = bg->cell; b.nb = nb;
        } else {
            b.pb = nullptr; b.sb = nullptr; b.cb = nullptr; b.mb = nullptr;
            b.ob = {0, 0, 0}; b.db = {0, 0, 0}; b.lb = 0.0f; b.nb = 0;
        }
        return b;
    }

    void step(float dt) {
        if (n == 0) return;
        fg->build(pos.p, n);
        const unsigned grid = unsigned((n + 127) / 128);
        BArgs b = bargs();
        Vec3f of = fg->origin;
        Vec3i df = fg->dims;
        float lf = fg->cell, l = cfg.smoothing_length, rho0 = cfg.rest_density;
        {   // compute_density (dfsph.cu:137-160)
            void* a[] = {&pos.p, &fg->sorted.p, &fg->cell_start.p, &density.p, &n, &of, &df, &lf, &mass, &l,
                         &b.pb, &b.sb, &b.cb, &b.mb, &b.ob, &b.db, &b.lb, &b.nb};
            launch(k.density, grid, 128, a);
        }
        {   // compute_alpha (dfsph.cu:162-186)
            void* a[] = {&pos.p, &density.p, &fg->sorted.p, &fg->cell_start.p, &alpha.p, &n, &of, &df, &lf,
                         &mass, &l, &b.pb, &b.sb, &b.cb, &b.mb, &b.ob, &b.db, &b.lb, &b.nb};
            launch(k.alpha, grid, 128, a);
        }
        {   // apply_external_forces (dfsph.cu:188-195)
            Vec3f g{cfg.gravity[0], cfg.gravity[1], cfg.gravity[2]};
            float damp = cfg.damping;
            void* a[] = {&vel.p, &n, &g, &dt, &damp};
            launch(k.gravity, grid, 128, a);
        }
        if (cfg.viscosity > 0.0f) {  // apply_xsph_viscosity (dfsph.cu:197-213)
            float eps = cfg.viscosity;
            void* a[] = {&pos.p, &vel.p, &density.p, &fg->sorted.p, &fg->cell_start.p, &n, &of, &df, &lf, &mass,
                         &l, &eps};
            launch(k.xsph, grid, 128, a);
        }
        // density_solve (dfsph.cu:215-260)
        last_iters = 0;
        for (u32 it = 0; it < cfg.max_density_iters; ++it) {
            {
                void* a[] = {&pos.p, &vel.p, &density.p, &fg->sorted.p, &fg->cell_start.p, &density_adv.p,
                             &kappa.p, &alpha.p, &rho0, &n, &of, &df, &lf, &mass, &l, &dt,
                             &b.pb, &b.sb, &b.cb, &b.mb, &b.ob, &b.db, &b.lb, &b.nb};
                launch(k.dchange, grid, 128, a);
            }
            {
                void* a[] = {&pos.p, &vel.p, &density.p, &kappa.p, &fg->sorted.p, &fg->cell_start.p, &n, &of,
                             &df, &lf, &mass, &l, &dt, &rho0, &b.pb, &b.sb, &b.cb, &b.mb, &b.ob, &b.db, &b.lb,
                             &b.nb};
                launch(k.kappa, grid, 128, a);
            }
            last_iters = it + 1;
            if (it >= 1) {
                const float err = reduce_density_error();
                if (err < cfg.eta_density * cfg.rest_density) break;
            }
        }
        {   // advect (dfsph.cu:262-273)
            float maxv = 5.0f;
            Vec3f lo{cfg.domain_min[0], cfg.domain_min[1], cfg.domain_min[2]};
            Vec3f hi{cfg.domain_max[0], cfg.domain_max[1], cfg.domain_max[2]};
            void* a[] = {&pos.p, &vel.p, &n, &dt, &maxv, &lo, &hi};
            launch(k.advect, grid, 128, a);
        }
        max_v = reduce_max_velocity();
    }

    float reduce_density_error() {  // dfsph.cu:277-301
        const unsigned grid = unsigned((n + 127) / 128);
        float rho0 = cfg.rest_density;
        void* a[] = {&density_adv.p, &rho0, &reduce_in.p, &n};
        launch(k.derr, grid, 128, a);
        size_t bytes = 0;
        RT(cub::DeviceReduce::Sum(nullptr, bytes, reduce_in.p, reduce_out.p, int(n), 0));
        if (bytes > reduce_temp.n) reduce_temp.reset(bytes);
        RT(cub::DeviceReduce::Sum(reduce_temp.p, bytes, reduce_in.p, reduce_out.p, int(n), 0));
        float s = 0.0f;
        RT(cudaMemcpyAsync(&s, reduce_out.p, sizeof(float), cudaMemcpyDeviceToHost, 0));
        RT(cudaStreamSynchronize(0));
        return s / float(n);
    }

    float reduce_max_velocity() {  // dfsph.cu:303-326
        const unsigned grid = unsigned((n + 127) / 128);
        void* a[] = {&vel.p, &reduce_in.p, &n};
        launch(k.vmag, grid, 128, a);
        size_t bytes = 0;
        RT(cub::DeviceReduce::Max(nullptr, bytes, reduce_in.p, reduce_out.p, int(n), 0));
        if (bytes > reduce_temp.n) reduce_temp.reset(bytes);
        RT(cub::DeviceReduce::Max(reduce_temp.p, bytes, reduce_in.p, reduce_out.p, int(n), 0));
        float m = 0.0f;
        RT(cudaMemcpyAsync(&m, reduce_out.p, sizeof(float), cudaMemcpyDeviceToHost, 0));
        RT(cudaStreamSynchronize(0));
        return m;
    }
};

thread_local std::string g_err;

// SpatialAccel (core/include/water/core/spatial_accel.h:19-53) around the
// reference's own kernels from core/src/spatial_accel.cu. build() restates
// SpatialAccel::build (spatial_accel.cu:110-179): the member buffers are
// replaced by fresh stream-ordered allocations on every build, the Morton
// codes of the positions normalised by the scene box, a CUB radix sort of
// (code, index) over bits [0, 30) into two temporary buffers, two device
// copies back, the internal nodes (Karras 2012) and the leaf boxes with
// radius 0. Internal boxes and the root's parent are left unwritten there.
struct AccelBox { Vec3f min, max; };

struct Lbvh {
    Module mod;
    CUfunction morton = nullptr, internal = nullptr, leaves = nullptr;
    Buf<u32> codes, idx, left, right, parent;
    Buf<AccelBox> boxes;
    size_t leaf_count = 0;

    // DeviceBuffer<T>(count, stream) move-assigned over the member: the new
    // allocation is made before the old one is released
    template <class T> static void renew(Buf<T>& b, size_t n) {
        Buf<T> t(n);
        b = std::move(t);
    }

    Lbvh(const Lbvh&) = delete;
    Lbvh& operator=(const Lbvh&) = delete;
    ~Lbvh() {
        cudaDeviceSynchronize();
        if (mod.mod) cuModuleUnload(mod.mod);
    }

    explicit Lbvh(const std::string& dir) {
        RT(cudaFree(nullptr));  // primary context
        mod.load(dir + "/spatial_accel.fatbin");
        const std::string a = "water::(anonymous namespace)::";
        morton = mod.get(a + "compute_morton");
        internal = mod.get(a + "build_internal_nodes");
        leaves = mod.get(a + "init_leaf_aabbs");
    }

    void build(const Vec3f* pos, size_t count, Vec3f smin, Vec3f smax) {
        if (count < 2) {  // spatial_accel.cu:112-125
            leaf_count = count;
            if (count == 1) {
                renew(idx, 1);
                renew(boxes, 1);
                const u32 zero = 0;
                RT(cudaMemcpyAsync(idx.p, &zero, sizeof(u32), cudaMemcpyHostToDevice, 0));
            }
            return;
        }
        leaf_count = count;
        int n_internal = int(count) - 1;
        renew(codes, count);
        renew(idx, count);
        renew(left, size_t(n_internal));
        renew(right, size_t(n_internal));
        renew(parent, count + size_t(n_internal));
        renew(boxes, count + size_t(n_internal));
        const Vec3f ext{smax.x - smin.x, smax.y - smin.y, smax.z - smin.z};
        Vec3f inv{ext.x > 0 ? 1.0f / ext.x : 0.0f, ext.y > 0 ? 1.0f / ext.y : 0.0f,
                  ext.z > 0 ? 1.0f / ext.z : 0.0f};
        {
            void* a[] = {(void*)&pos, &codes.p, &idx.p, &count, &smin, &inv};
            launch(morton, unsigned((count + 255) / 256), 256, a);
        }
        Buf<u32> sk(count), sv(count);
        size_t bytes = 0;
        RT(cub::DeviceRadixSort::SortPairs(nullptr, bytes, codes.p, sk.p, idx.p, sv.p, int(count), 0, 30, 0));
        Buf<unsigned char> temp(bytes);
        RT(cub::DeviceRadixSort::SortPairs(temp.p, bytes, codes.p, sk.p, idx.p, sv.p, int(count), 0, 30, 0));
        RT(cudaMemcpyAsync(codes.p, sk.p, count * sizeof(u32), cudaMemcpyDeviceToDevice, 0));
        RT(cudaMemcpyAsync(idx.p, sv.p, count * sizeof(u32), cudaMemcpyDeviceToDevice, 0));
        int n_leaves = int(count);
        {
            void* a[] = {&codes.p, &left.p, &right.p, &parent.p, &n_leaves};
            launch(internal, unsigned((n_internal + 255) / 256), 256, a);
        }
        float radius = 0.0f;
        {
            void* a[] = {(void*)&pos, &idx.p, &boxes.p, &n_internal, &n_leaves, &radius};
            launch(leaves, unsigned((n_leaves + 255) / 256), 256, a);
        }
    }
};

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

void* ref_create(const char* fatbin_dir, const RefConfig* cfg, const float* xyz, const float* vel, u32 n,
                 const float* bxyz, u32 nb) {
    try {
        return new Runner(fatbin_dir, *cfg, xyz, vel, n, bxyz, nb);
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void ref_destroy(void* h) {
    try {
        cudaDeviceSynchronize();
        delete static_cast<Runner*>(h);
        cudaDeviceSynchronize();
    } catch (...) {
    }
}

int ref_step(void* h, float dt, u32 steps) {
    try {
        Runner* r = static_cast<Runner*>(h);
        for (u32 s = 0; s < steps; ++s) r->step(dt);
        RT(cudaDeviceSynchronize());
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// Milliseconds of `steps` reference steps between CUDA events on stream 0.
double ref_time_steps(void* h, float dt, u32 steps) {
    try {
        Runner* r = static_cast<Runner*>(h);
        cudaEvent_t a, b;
        RT(cudaEventCreate(&a));
        RT(cudaEventCreate(&b));
        RT(cudaDeviceSynchronize());
        RT(cudaEventRecord(a, 0));
        for (u32 s = 0; s < steps; ++s) r->step(dt);
        RT(cudaEventRecord(b, 0));
        RT(cudaEventSynchronize(b));
        float ms = 0;
        RT(cudaEventElapsedTime(&ms, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return double(ms);
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1.0;
    }
}

// Fields in original particle order; ids as in oracle/dfsph_oracle.cpp.
int ref_get(void* h, int field, void* out) {
    try {
        Runner* r = static_cast<Runner*>(h);
        RT(cudaDeviceSynchronize());
        auto cp = [&](const void* src, size_t bytes) {
            if (bytes) RT(cudaMemcpy(out, src, bytes, cudaMemcpyDeviceToHost));
        };
        const size_t n = r->n;
        switch (field) {
            case 0: cp(r->pos.p, n * sizeof(Vec3f)); return 0;
            case 1: cp(r->vel.p, n * sizeof(Vec3f)); return 0;
            case 2: cp(r->density.p, n * 4); return 0;
            case 3: cp(r->alpha.p, n * 4); return 0;
            case 4: cp(r->kappa.p, n * 4); return 0;
            case 5: cp(r->density_adv.p, n * 4); return 0;
            case 6: {  // per-particle key = sorted keys scattered back by sorted index
                std::vector<u32> sk(n), si(n);
                if (n) {
                    RT(cudaMemcpy(sk.data(), r->fg->cell_ids.p, n * 4, cudaMemcpyDeviceToHost));
                    RT(cudaMemcpy(si.data(), r->fg->sorted.p, n * 4, cudaMemcpyDeviceToHost));
                }
                u32* o = static_cast<u32*>(out);
                for (size_t s = 0; s < n; ++s) o[si[s]] = sk[s];
                return 0;
            }
            case 7: cp(r->fg->sorted.p, n * 4); return 0;
            case 8: cp(r->fg->cell_start.p, r->fg->cell_start.n * 4); return 0;
            case 11: if (r->bg) cp(r->bmass.p, r->nb * 4); return 0;
            case 13: if (r->bg) cp(r->bg->cell_start.p, r->bg->cell_start.n * 4); return 0;
            case 14: if (r->bg) cp(r->bg->sorted.p, r->nb * 4); return 0;
            default: g_err = "unsupported field"; return 2;
        }
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// SpatialAccel::build on n host positions (xyz[n][3]) and the scene box.
// Host outputs, each may be NULL: codes[n], sorted index[n], left/right[n-1],
// parent[2n-1] (the root's entry is whatever the allocation held) and the
// leaf boxes leaf_boxes[n][6] (min xyz, max xyz). Then `reps` further builds
// of the same input between CUDA events on stream 0: *ms = their mean.
int ref_lbvh(const char* fatbin_dir, const float* xyz, u32 n, const float* smin, const float* smax, u32* codes,
             u32* idx, u32* left, u32* right, u32* parent, float* leaf_boxes, u32 reps, double* ms) {
    try {
        Lbvh b(fatbin_dir);
        Buf<Vec3f> pos(std::max<size_t>(n, 1));
        if (n) RT(cudaMemcpy(pos.p, xyz, size_t(n) * sizeof(Vec3f), cudaMemcpyHostToDevice));
        const Vec3f lo{smin[0], smin[1], smin[2]}, hi{smax[0], smax[1], smax[2]};
        b.build(pos.p, n, lo, hi);
        RT(cudaDeviceSynchronize());
        auto cp = [](void* dst, const void* src, size_t bytes) {
            if (dst && bytes) RT(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
        };
        if (n >= 2) {
            cp(codes, b.codes.p, size_t(n) * 4);
            cp(idx, b.idx.p, size_t(n) * 4);
            cp(left, b.left.p, size_t(n - 1) * 4);
            cp(right, b.right.p, size_t(n - 1) * 4);
            cp(parent, b.parent.p, size_t(2 * n - 1) * 4);
            cp(leaf_boxes, b.boxes.p + (n - 1), size_t(n) * sizeof(AccelBox));
        } else if (n == 1) {
            cp(idx, b.idx.p, 4);
        }
        if (ms) {
            *ms = 0.0;
            if (reps) {
                cudaEvent_t e0, e1;
                RT(cudaEventCreate(&e0));
                RT(cudaEventCreate(&e1));
                RT(cudaEventRecord(e0, 0));
                for (u32 r = 0; r < reps; ++r) b.build(pos.p, n, lo, hi);
                RT(cudaEventRecord(e1, 0));
                RT(cudaEventSynchronize(e1));
                float t = 0;
                RT(cudaEventElapsedTime(&t, e0, e1));
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                *ms = double(t) / reps;
            }
        }
        RT(cudaDeviceSynchronize());
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// 0 max_velocity, 1 particle_mass, 2 last_density_iters, 6 total cells
double ref_scalar(void* h, int which) {
    Runner* r = static_cast<Runner*>(h);
    switch (which) {
        case 0: return r->max_v;
        case 1: return r->mass;
        case 2: return r->last_iters;
        case 6: return r->fg->total();
        default: return 0.0;
    }
}

}  // extern "C"
