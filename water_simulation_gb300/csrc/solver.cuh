// Host orchestration of the GB300 DFSPH step (one instantiation per working
// real type). The stage order is DFSPHSolver::step (solvers/dfsph/src/dfsph.cu
// :120-133): grid build, density + alpha, [divergence solve], external forces +
// XSPH, density solve, advect + max |v|.
//
// Scenes: a context steps S >= 1 independent scenes that share the grid
// geometry, the wall particles and dt. Scene s owns the cell keys
// [s (C+1), (s+1)(C+1)) (its out-of-grid key last), so one counting sort orders
// all of them, scene after scene, and one launch per kernel steps all of them.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "adjoint.cuh"
#include "frames.cuh"
#include "kernels.cuh"
#include "solver_api.h"

namespace dfsph {

template <class T> struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { if (p) cudaFree(p); }
    void alloc(size_t count) {
        if (p) { cudaFree(p); p = nullptr; n = 0; }
        if (count == 0) return;
        DFSPH_CUDA(cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T)));
        n = count;
    }
};

inline int blocks_for(long long n, int block) { return static_cast<int>((n + block - 1) / block); }

// NVTX range for profilers (Nsight Systems / Compute timelines); a few
// nanoseconds when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// The rank of every cell of a dims[0] x dims[1] x dims[2] grid in the Morton
// order of its cell coordinates (bits interleaved x highest, as SpatialAccel's
// morton3D, core/src/spatial_accel.cu:11-28), indexed by x-major cell id, with
// the out-of-grid key (the cell count) ranked last.
inline std::vector<u32> morton_cell_ranks(const int dims[3]) {
    auto spread = [](u64 v) {  // bit k of v to bit 3k
        v &= 0x1FFFFFull;
        v = (v | (v << 32)) & 0x1F00000000FFFFull;
        v = (v | (v << 16)) & 0x1F0000FF0000FFull;
        v = (v | (v << 8)) & 0x100F00F00F00F00Full;
        v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
        v = (v | (v << 2)) & 0x1249249249249249ull;
        return v;
    };
    auto gather = [](u64 v) {  // inverse of spread
        v &= 0x1249249249249249ull;
        v = (v ^ (v >> 2)) & 0x10C30C30C30C30C3ull;
        v = (v ^ (v >> 4)) & 0x100F00F00F00F00Full;
        v = (v ^ (v >> 8)) & 0x1F0000FF0000FFull;
        v = (v ^ (v >> 16)) & 0x1F00000000FFFFull;
        v = (v ^ (v >> 32)) & 0x1FFFFFull;
        return v;
    };
    const u64 nx = u64(dims[0]), ny = u64(dims[1]), nz = u64(dims[2]);
    const u64 total = nx * ny * nz;
    std::vector<u64> codes;
    codes.reserve(total);
    for (u64 x = 0; x < nx; ++x)
        for (u64 y = 0; y < ny; ++y)
            for (u64 z = 0; z < nz; ++z) codes.push_back((spread(x) << 2) | (spread(y) << 1) | spread(z));
    std::sort(codes.begin(), codes.end());
    std::vector<u32> rank(total + 1);
    for (u64 k = 0; k < total; ++k) {
        const u64 c = codes[k];
        const u64 x = gather(c >> 2), y = gather(c >> 1), z = gather(c);
        rank[(x * ny + y) * nz + z] = static_cast<u32>(k);
    }
    rank[total] = static_cast<u32>(total);
    return rank;
}

template <class R>
class Solver final : public SolverBase {
public:
    using V4 = R4<R>;

    Solver(const dfsph_config& cfg, int device, cudaStream_t stream)
        : cfg_(cfg), device_(device), stream_(stream) {
        DFSPH_CUDA(cudaSetDevice(device_));
        geom_ = make_grid_geom(cfg_.domain_min, cfg_.domain_max, cfg_.smoothing_length);
        geom_.inv_stencil = device_stencil_reciprocal(cfg_.smoothing_length, stream_);
        g_ = to_dev<R>(geom_);
        gb_ = g_;  // the wall grid: one "scene"
        scenes_ = cfg_.n_scenes > 1 ? cfg_.n_scenes : 1u;
        if (scenes_ > 65535u) throw Error(DFSPH_ERR_INVALID_ARGUMENT, "at most 65535 scenes");
        cells1_ = geom_.total + 1;
        if (double(scenes_) * double(cells1_) >= 4294967295.0)
            throw Error(DFSPH_ERR_INVALID_ARGUMENT, "scenes x cells must stay below 2^32");
        // particle mass rho0 * (2r)^3 evaluated in float (dfsph.cu:76-78)
        const float spacing = 2.0f * cfg_.particle_radius;
        const float v0 = spacing * spacing * spacing;
        mass_f_ = cfg_.rest_density * v0;
        const R l = R(cfg_.smoothing_length);
        phys_.l = l;
        phys_.inv_l = R(1) / l;
        phys_.support2 = R(4) * l * l;
        phys_.grad_c = R(1) / (R(3.14159265358979323846) * l * l * l) / l;
        phys_.mass = R(mass_f_);
        phys_.rho0 = R(cfg_.rest_density);
        // the cubic spline per branch in terms of r (kernels.cuh, "Pair terms")
        {
            const double ld = double(cfg_.smoothing_length);
            const double sg = 1.0 / (3.14159265358979323846 * ld * ld * ld);
            phys_.sigma = R(sg);
            phys_.two_l = R(2.0 * ld);
            phys_.wA2 = R(-1.5 * sg / (ld * ld));
            phys_.wA3 = R(0.75 * sg / (ld * ld * ld));
            phys_.wB = R(0.25 * sg / (ld * ld * ld));
            phys_.gA = R(2.25 * sg / (ld * ld * ld));
            phys_.gB = R(-3.0 * sg / (ld * ld));
            phys_.gC = R(-0.75 * sg / (ld * ld * ld));
        }

        cap_ = cfg_.capacity;
        bcap_ = cfg_.boundary_capacity;
        keys_ = size_t(scenes_) * cells1_;  // fluid keys of all scenes
        for (int k = 0; k < 2; ++k) {
            xk_[k].alloc(cap_);
            vr_[k].alloc(cap_);
            id_[k].alloc(cap_);
        }
        alpha_.alloc(cap_); rho_adv_.alloc(cap_); kap_.alloc(cap_); kap_v_.alloc(cap_);
        rho_dot_.alloc(cap_);
        key_.alloc(cap_); rank_.alloc(cap_); tmp_src_.alloc(cap_); tmp_id_.alloc(cap_);
        key_sorted_.alloc(cap_);
        if (cfg_.record_diagnostics) { nbr_f_.alloc(cap_); nbr_b_.alloc(cap_); nbr_sig_.alloc(cap_); }
        count_.alloc(keys_);
        cell_start_.alloc(keys_ + 1);  // closing entry = n
        n_tiles_ = static_cast<u32>((keys_ + SCAN_TILE - 1) / SCAN_TILE);
        tile_sums_.alloc(n_tiles_ + 1);
        // block partials of the per-pass reductions (blocks of >= 64 threads)
        // and the per-warp sums of the cooperative solve, behind the
        // reductions' arrival counters (REDUCE_GROUP_WORDS words)
        partials_.alloc(REDUCE_GROUP_WORDS / 2 + std::max<size_t>(1, (std::max(cap_, 1u) + 31) / 32));
        ctl_.alloc(3);
        dev_err_.alloc(1);
        staging_.alloc(std::max<size_t>(size_t(std::max(cap_, bcap_)) * 6, 6));
        if (bcap_) {
            for (int k = 0; k < 2; ++k) { xb_[k].alloc(bcap_); bid_[k].alloc(bcap_); }
            bkey_.alloc(bcap_); brank_.alloc(bcap_); bkey_sorted_.alloc(bcap_);
            btmp_src_.alloc(bcap_); btmp_id_.alloc(bcap_);
        }
        bcs_.alloc(size_t(cells1_) + 1);
        bmask_.alloc(std::max<size_t>(geom_.total, 1));
        krange_.alloc(2 * KRANGE_SLOTS);
        cs_range_.alloc(2);
        reset_key_range();
        DFSPH_CUDA(cudaMemsetAsync(cs_range_.p, 0, 2 * sizeof(u32), stream_));
        {
            // a stencil centred up to one cell off a particle's key cell reads
            // cells up to two cells away on every axis, and cell_start[c + 1]
            const u32 ny = u32(geom_.dims[1]), nz = u32(geom_.dims[2]);
            margin_ = 2u * (ny * nz + nz + 1u) + 2u;
        }
        if (comp_) {
            xc_.alloc(std::max(cap_, 1u));
            DFSPH_CUDA(cudaMemsetAsync(xc_.p, 0, size_t(std::max(cap_, 1u)) * sizeof(V4), stream_));
        }
        if (cfg_.slot_order == DFSPH_ORDER_MORTON) {
            // the fluid slots follow the Morton order of the cells; the wall
            // grid (gb_) keeps the x-major order
            const std::vector<u32> rank = morton_cell_ranks(geom_.dims);
            morton_rank_.alloc(rank.size());
            DFSPH_CUDA(cudaMemcpyAsync(morton_rank_.p, rank.data(), rank.size() * sizeof(u32),
                                       cudaMemcpyHostToDevice, stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));  // the host vector goes out of scope
            g_.rank = morton_rank_.p;
        }
        if (scenes_ > 1) {
            slot_scene_.alloc(std::max(cap_, 1u));
            eps_scene_.alloc(scenes_);
            maxv_scene_.alloc(scenes_);
            g_.slot_scene = slot_scene_.p;
            std::vector<R> eps(scenes_, R(cfg_.viscosity));
            DFSPH_CUDA(cudaMemcpyAsync(eps_scene_.p, eps.data(), scenes_ * sizeof(R), cudaMemcpyHostToDevice, stream_));
            DFSPH_CUDA(cudaMemsetAsync(maxv_scene_.p, 0, scenes_ * sizeof(u32), stream_));
            DFSPH_CUDA(cudaMemsetAsync(slot_scene_.p, 0, std::max(cap_, 1u) * sizeof(unsigned short), stream_));
        }
        DFSPH_CUDA(cudaMemsetAsync(count_.p, 0, keys_ * sizeof(u32), stream_));
        DFSPH_CUDA(cudaMemsetAsync(cell_start_.p, 0, (keys_ + 1) * sizeof(u32), stream_));
        DFSPH_CUDA(cudaMemsetAsync(bcs_.p, 0, (size_t(cells1_) + 1) * sizeof(u32), stream_));
        DFSPH_CUDA(cudaMemsetAsync(ctl_.p, 0, 3 * sizeof(IterCtl), stream_));
        DFSPH_CUDA(cudaMemsetAsync(partials_.p, 0, REDUCE_GROUP_WORDS * sizeof(u32), stream_));
        DFSPH_CUDA(cudaMemsetAsync(dev_err_.p, 0, sizeof(u32), stream_));
        DFSPH_CUDA(cudaMemsetAsync(alpha_.p, 0, size_t(cap_) * sizeof(R), stream_));
        DFSPH_CUDA(cudaMemsetAsync(rho_adv_.p, 0, size_t(cap_) * sizeof(R), stream_));
        DFSPH_CUDA(cudaMemsetAsync(kap_.p, 0, size_t(cap_) * sizeof(R), stream_));
        DFSPH_CUDA(cudaMemsetAsync(kap_v_.p, 0, size_t(cap_) * sizeof(R), stream_));
        if (cfg_.record_diagnostics) {
            DFSPH_CUDA(cudaMemsetAsync(nbr_f_.p, 0, size_t(cap_) * sizeof(u32), stream_));
            DFSPH_CUDA(cudaMemsetAsync(nbr_b_.p, 0, size_t(cap_) * sizeof(u32), stream_));
            DFSPH_CUDA(cudaMemsetAsync(nbr_sig_.p, 0, size_t(cap_) * sizeof(u32), stream_));
        }
        DFSPH_CUDA(cudaMallocHost(reinterpret_cast<void**>(&host_ctl_), 3 * sizeof(IterCtl)));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
    }

    ~Solver() override {
        drop_graph();
        drop_adjoint_graph();
        if (replay_stream_) {
            cudaStreamSynchronize(replay_stream_);
            cudaStreamDestroy(replay_stream_);
            for (cudaEvent_t e : {ev_start_, ev_replayed_[0], ev_replayed_[1], ev_reversed_[0], ev_reversed_[1]})
                if (e) cudaEventDestroy(e);
        }
        if (capture_stream_) cudaStreamDestroy(capture_stream_);
        if (loop_stream_) cudaStreamDestroy(loop_stream_);
        if (host_ctl_) cudaFreeHost(host_ctl_);
        if (eps_host_) cudaFreeHost(eps_host_);
        if (host_fctl_) cudaFreeHost(host_fctl_);
        for (const Record& r : records_) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
        for (cudaEvent_t e : free_events_) cudaEventDestroy(e);
    }

    // Calls f with std::true_type when the fluid slots are in Morton order
    // (the kernels' MORTON instantiation) and std::false_type otherwise.
    template <class F> void with_slot_order(F&& f) {
        if (g_.rank) f(std::true_type{});
        else f(std::false_type{});
    }
    // the integrator's instantiations: compensated position update or not
    template <class F> void with_compensation(bool on, F&& f) {
        if (on) f(std::true_type{});
        else f(std::false_type{});
    }

    void set_stream(cudaStream_t s) override {
        stream_ = s;
        drop_graph();
    }

    // ------------------------------------------------------------------ setup
    void set_boundary(const float* xyz, u32 n, int mem) override {
        if (n > bcap_) throw Error(DFSPH_ERR_OUT_OF_RANGE, "boundary count exceeds boundary_capacity");
        nb_ = n;
        drop_pending_counts();
        drop_graph();
        drop_adjoint_graph();  // it baked in the wall count
        ad_valid_ = false;  // a recorded rollout ran against the old walls
        if (n == 0) {
            DFSPH_CUDA(cudaMemsetAsync(bcs_.p, 0, (size_t(cells1_) + 1) * sizeof(u32), stream_));
            return;
        }
        const float* src = upload(xyz, nullptr, n, mem);
        launch_import(n, src, nullptr, xb_[0].p, vr_scratch(), bid_[0].p);
        // sort by cell (the boundary CellGrid built once, dfsph.cu:93-97)
        launch(DFSPH_KERNEL_GRID_COUNT, count_kernel<R>, blocks_for(n, 256), 256, int(n), xb_[0].p, gb_, bkey_.p,
               brank_.p, count_.p, (u32*)nullptr);
        scan(bcs_.p, cells1_, /*step start*/ false);
        launch(DFSPH_KERNEL_GRID_SCATTER, scatter_kernel, blocks_for(n, 256), 256, int(n), bkey_.p, brank_.p, bcs_.p,
               bid_[0].p, btmp_src_.p, btmp_id_.p);
        launch(DFSPH_KERNEL_GRID_REORDER, reorder_kernel<R>, blocks_for(n, 256), 256, int(n), btmp_src_.p,
               btmp_id_.p, bkey_.p, bcs_.p, cells1_, kSentinelCap, xb_[0].p, vr_scratch(), xb_[1].p,
               vr_scratch2(), bid_[1].p, bkey_sorted_.p, ctl_.p);
        // Akinci mass into the w lane (dfsph_kernels.cu:40-65)
        launch(DFSPH_KERNEL_OTHER, boundary_mass_kernel<R>, blocks_for(n, 128), 128, int(n), xb_[1].p, xb_[0].p,
               bcs_.p, gb_, phys_);
        std::swap(bid_[0].p, bid_[1].p);  // bid_[0] holds the sorted order now
        launch(DFSPH_KERNEL_OTHER, boundary_mask_kernel<R>, blocks_for(geom_.total, 256), 256, geom_.total, bcs_.p,
               gb_, bmask_.p);
    }

    void set_fluid(const float* xyz, const float* vel, u32 n, int mem) override {
        const u32 counts = n;
        set_fluid_batch(1, &counts, xyz, vel, mem);
    }

    void set_fluid_batch(u32 n_scenes, const u32* counts, const float* xyz, const float* vel, int mem) override {
        store_run_ = false;
        const u32 n = check_counts(n_scenes, counts);
        // page-locked host arrays are read in place by the import kernel;
        // other host memory goes through the staging buffer
        const float* mp = nullptr;
        const float* mv = nullptr;
        if (mem == DFSPH_MEM_HOST && n) {
            mp = mapped_host(xyz);
            mv = vel ? mapped_host(vel) : nullptr;
            if (vel && !mv) mp = nullptr;
        }
        const float* pos = mp ? nullptr : upload(xyz, vel, n, mem);
        const float* v = vel && pos ? pos + 3 * size_t(n) : nullptr;
        if (mem == DFSPH_MEM_DEVICE) { pos = xyz; v = vel; }
        install_counts(n_scenes, counts, n);
        if (n == 0) {
            // an empty fluid is a state like any other: steps return at once
            // (dfsph.cu:121-122), as for an empty ParticleStore
            counts_valid_ = false;
            have_state_ = true;
            return;
        }
        if (mp) {
            launch(DFSPH_KERNEL_IO, import_mapped_kernel<R>, blocks_for(n, 256), 256, int(n), mp, mv, xk_[cx_].p,
                   vr_[cv_].p, id_[ci_].p);
            // the caller may free its arrays after return
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
        } else {
            launch_import(n, pos, v, xk_[cx_].p, vr_[cv_].p, id_[ci_].p);
        }
        counts_valid_ = false;
        reset_compensation();
        have_state_ = true;
    }

    // The device address of caller memory passed as host memory when the GPU
    // can use it in place: page-locked (registered or cudaHostAlloc) and
    // 16-byte aligned. Null for pageable or unaligned memory.
    static const float* mapped_host(const void* p) {
        if (!p || (reinterpret_cast<uintptr_t>(p) & 15u)) return nullptr;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer ||
            (reinterpret_cast<uintptr_t>(a.devicePointer) & 15u))
            return nullptr;
        return static_cast<const float*>(a.devicePointer);
    }

    u32 check_counts(u32 n_scenes, const u32* counts) const {
        if (n_scenes != scenes_)
            throw Error(DFSPH_ERR_INVALID_ARGUMENT, "scene count differs from the context's n_scenes (" +
                                                        std::to_string(scenes_) + ")");
        unsigned long long total = 0;
        for (u32 s = 0; s < n_scenes; ++s) total += counts[s];
        if (total > cap_)
            throw Error(DFSPH_ERR_OUT_OF_RANGE, "ParticleStore::resize: count " + std::to_string(total) +
                                                    " exceeds capacity " + std::to_string(cap_));
        return static_cast<u32>(total);
    }

    // New fluid counts: the slot -> scene map, and the captured graphs when
    // the counts changed.
    void install_counts(u32 n_scenes, const u32* counts, u32 n) {
        // captured graphs bake the particle counts in; new values of the same
        // counts keep them valid
        const bool same = n == n_ && scene_counts_.size() == n_scenes &&
                          std::equal(counts, counts + n_scenes, scene_counts_.begin());
        n_ = n;
        drop_pending_counts();
        if (!same) drop_graph();
        scene_counts_.assign(counts, counts + n_scenes);
        if (scenes_ > 1 && n) {
            // sorted order is scene-major, so slot -> scene never changes
            std::vector<unsigned short> ss(n);
            size_t o = 0;
            for (u32 s = 0; s < n_scenes; ++s)
                for (u32 k = 0; k < counts[s]; ++k) ss[o++] = static_cast<unsigned short>(s);
            DFSPH_CUDA(cudaMemcpyAsync(slot_scene_.p, ss.data(), n * sizeof(unsigned short), cudaMemcpyHostToDevice,
                                       stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
        }
    }

    void set_scene_viscosity(const float* eps, u32 n_scenes) override {
        if (n_scenes != scenes_) throw Error(DFSPH_ERR_INVALID_ARGUMENT, "scene count mismatch");
        if (scenes_ == 1) {
            cfg_.viscosity = eps[0];
            drop_graph();
            return;
        }
        std::vector<R> e(eps, eps + n_scenes);
        DFSPH_CUDA(cudaMemcpyAsync(eps_scene_.p, e.data(), n_scenes * sizeof(R), cudaMemcpyHostToDevice, stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        any_xsph_ = false;
        for (u32 s = 0; s < n_scenes; ++s) any_xsph_ = any_xsph_ || eps[s] > 0.0f;
        explicit_eps_ = true;
        drop_graph();
    }

    void get_scene_max_velocity(float* out, u32 n_scenes) override {
        if (n_scenes != scenes_) throw Error(DFSPH_ERR_INVALID_ARGUMENT, "scene count mismatch");
        if (scenes_ == 1) {
            out[0] = float(get_scalar(DFSPH_SCALAR_MAX_VELOCITY));
            return;
        }
        std::vector<u32> bits(scenes_);
        DFSPH_CUDA(cudaMemcpyAsync(bits.data(), maxv_scene_.p, scenes_ * sizeof(u32), cudaMemcpyDeviceToHost, stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        for (u32 s = 0; s < scenes_; ++s) std::memcpy(out + s, &bits[s], sizeof(float));
        if (!stepped_)
            for (u32 s = 0; s < scenes_; ++s) out[s] = 0.0f;
    }

    // ------------------------------------------------------------------- step
    void step(float dt, u32 n_steps) override {
        store_run_ = false;
        u32 k = 0;
        if (graph_ok()) {
            if (!counts_valid_ && k < n_steps) {  // the first step after new input counts itself
                step_once(R(dt), true);
                ++k;
            }
            if (n_steps - k >= 2) {
                ensure_graph(dt);
                for (; k + 2 <= n_steps; k += 2) {
                    DFSPH_CUDA(cudaGraphLaunch(graph_exec_, stream_));
                    launches_ += graph_kernels_;
                }
                iters_on_device_ = adaptive();
            }
        }
        for (; k < n_steps; ++k) step_once(R(dt), /*count_next=*/true);
    }

    void step_store(float* pos, float* vel, u32 n, float dt, float* density, float* alpha, float* kappa,
                    float* density_adv) override {
        if (scenes_ != 1) throw Error(DFSPH_ERR_STATE, "dfsph_step_store steps one scene");
        if (n > cap_) throw Error(DFSPH_ERR_OUT_OF_RANGE, "store count exceeds capacity");
        // a store stepped by consecutive calls holds the positions the
        // previous call wrote back: a compensated run keeps its carries
        const bool continuing = store_run_ && n == n_;
        store_run_ = false;
        n_ = n;
        drop_pending_counts();
        drop_graph();
        if (n == 0) return;  // dfsph.cu:121-122
        launch_import(n, pos, vel, xk_[cx_].p, vr_[cv_].p, id_[ci_].p);
        counts_valid_ = false;
        if (!continuing) reset_compensation();
        have_state_ = true;
        step_once(R(dt), /*count_next=*/false);
        launch(DFSPH_KERNEL_IO, export_kernel<R>, blocks_for(n, 256), 256, int(n), id_[ci_].p, xk_[cx_].p,
               vr_[cv_].p, alpha_.p, kap_.p, rho_adv_.p, pos, vel, density, alpha, kappa, density_adv);
        store_run_ = true;
    }

    // -------------------------------------------------------------- readback
    void get_field(int field, void* dst, size_t bytes, int mem) override {
        size_t need = 0;
        const size_t n = n_;
        switch (field) {
            case DFSPH_FIELD_POSITION: case DFSPH_FIELD_VELOCITY: need = 3 * n * sizeof(float); break;
            case DFSPH_FIELD_DENSITY: case DFSPH_FIELD_ALPHA: case DFSPH_FIELD_KAPPA:
            case DFSPH_FIELD_DENSITY_ADV: case DFSPH_FIELD_KAPPA_V: need = n * sizeof(float); break;
            case DFSPH_FIELD_CELL_KEY: case DFSPH_FIELD_SORTED_INDEX: case DFSPH_FIELD_NBR_FLUID:
            case DFSPH_FIELD_NBR_BOUNDARY: case DFSPH_FIELD_NBR_SIGNATURE: need = n * sizeof(u32); break;
            case DFSPH_FIELD_CELL_START: need = keys_ * sizeof(u32); break;
            case DFSPH_FIELD_BOUNDARY_CELL_START: need = size_t(cells1_) * sizeof(u32); break;
            case DFSPH_FIELD_BOUNDARY_MASS: need = size_t(nb_) * sizeof(float); break;
            case DFSPH_FIELD_BOUNDARY_SORTED_INDEX: need = size_t(nb_) * sizeof(u32); break;
            default: throw Error(DFSPH_ERR_INVALID_ARGUMENT, "unknown field " + std::to_string(field));
        }
        if (bytes < need) throw Error(DFSPH_ERR_INVALID_ARGUMENT, "destination too small for field");
        if ((field == DFSPH_FIELD_NBR_FLUID || field == DFSPH_FIELD_NBR_BOUNDARY ||
             field == DFSPH_FIELD_NBR_SIGNATURE) && !cfg_.record_diagnostics)
            throw Error(DFSPH_ERR_STATE, "neighbour counts need record_diagnostics = 1");
        if (need == 0) return;
        if (mem == DFSPH_MEM_HOST && export_mapped(field, dst)) return;
        // Produce the field in device scratch (original order), then copy out.
        void* out = (mem == DFSPH_MEM_DEVICE) ? dst : scratch_bytes(need);
        const int nb = blocks_for(std::max<size_t>(n, 1), 256);
        const u32* id = id_[ci_].p;
        switch (field) {
            case DFSPH_FIELD_POSITION:
                launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, float>, nb, 256, int(n), id, xk_[cx_].p, -1, (float*)out);
                break;
            case DFSPH_FIELD_VELOCITY:
                launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, float>, nb, 256, int(n), id, vr_[cv_].p, -1, (float*)out);
                break;
            case DFSPH_FIELD_DENSITY:
                launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, float>, nb, 256, int(n), id, vr_[cv_].p, 3, (float*)out);
                break;
            case DFSPH_FIELD_ALPHA:
                launch(DFSPH_KERNEL_IO, unsort_kernel<R, float>, nb, 256, int(n), id, alpha_.p, (float*)out); break;
            case DFSPH_FIELD_KAPPA:
                launch(DFSPH_KERNEL_IO, unsort_kernel<R, float>, nb, 256, int(n), id, kap_.p, (float*)out); break;
            case DFSPH_FIELD_DENSITY_ADV:
                launch(DFSPH_KERNEL_IO, unsort_kernel<R, float>, nb, 256, int(n), id, rho_adv_.p, (float*)out); break;
            case DFSPH_FIELD_KAPPA_V:
                launch(DFSPH_KERNEL_IO, unsort_kernel<R, float>, nb, 256, int(n), id, kap_v_.p, (float*)out); break;
            case DFSPH_FIELD_CELL_KEY:
                launch(DFSPH_KERNEL_IO, unsort_kernel<u32, u32>, nb, 256, int(n), id, key_sorted_.p, (u32*)out); break;
            case DFSPH_FIELD_SORTED_INDEX:
                DFSPH_CUDA(cudaMemcpyAsync(out, id, need, cudaMemcpyDeviceToDevice, stream_)); break;
            case DFSPH_FIELD_CELL_START:
                complete_cell_start();
                DFSPH_CUDA(cudaMemcpyAsync(out, cell_start_.p, need, cudaMemcpyDeviceToDevice, stream_)); break;
            case DFSPH_FIELD_BOUNDARY_CELL_START:
                DFSPH_CUDA(cudaMemcpyAsync(out, bcs_.p, need, cudaMemcpyDeviceToDevice, stream_)); break;
            case DFSPH_FIELD_NBR_FLUID:
                launch(DFSPH_KERNEL_IO, unsort_kernel<u32, u32>, nb, 256, int(n), id, nbr_f_.p, (u32*)out); break;
            case DFSPH_FIELD_NBR_BOUNDARY:
                launch(DFSPH_KERNEL_IO, unsort_kernel<u32, u32>, nb, 256, int(n), id, nbr_b_.p, (u32*)out); break;
            case DFSPH_FIELD_NBR_SIGNATURE:
                launch(DFSPH_KERNEL_IO, unsort_kernel<u32, u32>, nb, 256, int(n), id, nbr_sig_.p, (u32*)out); break;
            case DFSPH_FIELD_BOUNDARY_MASS:
                launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, float>, blocks_for(nb_, 256), 256, int(nb_), bid_[0].p,
                       xb_[0].p, 3, (float*)out);
                break;
            case DFSPH_FIELD_BOUNDARY_SORTED_INDEX:
                DFSPH_CUDA(cudaMemcpyAsync(out, bid_[0].p, need, cudaMemcpyDeviceToDevice, stream_)); break;
        }
        if (mem != DFSPH_MEM_DEVICE) {
            DFSPH_CUDA(cudaMemcpyAsync(dst, out, need, cudaMemcpyDeviceToHost, stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
        }
    }

    // Positions and velocities (original order, float3 each; either may be
    // null): one inverse permutation, one export pass and one
    // synchronisation when both destinations are page-locked host memory;
    // otherwise the two fields one after the other.
    void get_state(float* pos, float* vel, int mem) override {
        const size_t n = n_;
        if (n == 0 || (!pos && !vel)) return;
        float* mp = pos && mem == DFSPH_MEM_HOST ? const_cast<float*>(mapped_host(pos)) : nullptr;
        float* mv = vel && mem == DFSPH_MEM_HOST ? const_cast<float*>(mapped_host(vel)) : nullptr;
        if ((!pos || mp) && (!vel || mv)) {
            u32* inv = static_cast<u32*>(scratch_bytes(n * sizeof(u32)));
            launch(DFSPH_KERNEL_IO, invert_kernel, blocks_for(n, 256), 256, int(n), (const u32*)id_[ci_].p, inv);
            launch(DFSPH_KERNEL_IO, export_state_mapped_kernel<R>, blocks_for(n, 256), 256, int(n), (const u32*)inv,
                   (const V4*)xk_[cx_].p, (const V4*)vr_[cv_].p, mp, mv);
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
            return;
        }
        if (pos) get_field(DFSPH_FIELD_POSITION, pos, 3 * n * sizeof(float), mem);
        if (vel) get_field(DFSPH_FIELD_VELOCITY, vel, 3 * n * sizeof(float), mem);
    }

    // The float particle fields written in place to page-locked host memory
    // (export_mapped_kernel, in original order); false for other fields or
    // memory, which take the staging copy.
    bool export_mapped(int field, void* dst) {
        const V4* in = nullptr;
        const R* sc = nullptr;
        int lane = -1;
        switch (field) {
            case DFSPH_FIELD_POSITION: in = xk_[cx_].p; break;
            case DFSPH_FIELD_VELOCITY: in = vr_[cv_].p; break;
            case DFSPH_FIELD_DENSITY: in = vr_[cv_].p; lane = 3; break;
            case DFSPH_FIELD_ALPHA: sc = alpha_.p; break;
            case DFSPH_FIELD_KAPPA: sc = kap_.p; break;
            case DFSPH_FIELD_DENSITY_ADV: sc = rho_adv_.p; break;
            case DFSPH_FIELD_KAPPA_V: sc = kap_v_.p; break;
            default: return false;
        }
        float* out = const_cast<float*>(mapped_host(dst));
        if (!out) return false;
        const size_t n = n_;
        u32* inv = static_cast<u32*>(scratch_bytes(n * sizeof(u32)));
        launch(DFSPH_KERNEL_IO, invert_kernel, blocks_for(n, 256), 256, int(n), (const u32*)id_[ci_].p, inv);
        launch(DFSPH_KERNEL_IO, export_mapped_kernel<R>, blocks_for(n, 256), 256, int(n), (const u32*)inv, in, lane,
               sc, out);
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        return true;
    }

    double get_scalar(int which) override {
        switch (which) {
            case DFSPH_SCALAR_PARTICLE_MASS: return double(mass_f_);
            case DFSPH_SCALAR_TOTAL_CELLS: return double(geom_.total);
            case DFSPH_SCALAR_STENCIL_INV_CELL: return double(geom_.inv_stencil);
            case DFSPH_SCALAR_FLUID_COUNT: return double(n_);
            case DFSPH_SCALAR_BOUNDARY_COUNT: return double(nb_);
            case DFSPH_SCALAR_KERNEL_LAUNCHES: return double(launches_);
            case DFSPH_SCALAR_ACTIVE_BOUNDARY: return double(active_boundary());
            case DFSPH_SCALAR_FRAME_GRAPH: return double(last_frame_graph_);
            case DFSPH_SCALAR_COOP_SOLVES: return double(coop_launches_);
            case DFSPH_SCALAR_BOUNDS_VIOLATIONS: {
#ifdef DFSPH_BOUNDS_CHECK
                u32 v = 0;
                DFSPH_CUDA(cudaStreamSynchronize(stream_));
                DFSPH_CUDA(cudaMemcpyFromSymbol(&v, g_bounds_violations, sizeof(u32)));
                return double(v);
#else
                return -1.0;
#endif
            }
            default: break;
        }
        read_ctl();
        switch (which) {
            case DFSPH_SCALAR_MAX_VELOCITY: {
                u32 bits = 0;
                for (int w = 0; w < MAXV_SLOTS; ++w) bits = std::max(bits, host_ctl_[0].maxv_slot[w]);
                float f;
                std::memcpy(&f, &bits, sizeof(f));
                return stepped_ ? double(f) : 0.0;
            }
            case DFSPH_SCALAR_LAST_DENSITY_ITERS:
                if (iters_on_device_) return double(host_ctl_[2].iters);
                return double(iters_done(host_ctl_[2], last_density_launched_));
            case DFSPH_SCALAR_LAST_DIVERGENCE_ITERS:
                if (iters_on_device_) return double(host_ctl_[1].iters);
                return double(iters_done(host_ctl_[1], last_divergence_launched_));
            case DFSPH_SCALAR_DENSITY_ERROR: return n_ ? host_ctl_[2].err_sum / double(n_) : 0.0;
            case DFSPH_SCALAR_DIVERGENCE_ERROR: return n_ ? host_ctl_[1].err_sum / double(n_) : 0.0;
            case DFSPH_SCALAR_FLAGS: return double(host_ctl_[0].flags | host_ctl_[1].flags | host_ctl_[2].flags);
            default: throw Error(DFSPH_ERR_INVALID_ARGUMENT, "unknown scalar " + std::to_string(which));
        }
    }

    void synchronize() override {
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        check_device_status();
    }

    // The device error word is written only by the cooperative solve (its
    // bounded grid barrier); until one was launched or captured there is
    // nothing to read.
    void check_device_status() override {
        if (!coop_used_) return;
        u32 w = 0;
        DFSPH_CUDA(cudaMemcpyAsync(&w, dev_err_.p, sizeof(u32), cudaMemcpyDeviceToHost, stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        if (w == 0) return;
        DFSPH_CUDA(cudaMemsetAsync(dev_err_.p, 0, sizeof(u32), stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        throw Error(DFSPH_ERR_DEVICE_TIMEOUT,
                    "a grid barrier of the cooperative Jacobi solve gave up after " +
                        std::to_string(double(wait_limit_ns_) * 1e-6) +
                        " ms; the state of that step is not valid (set it again to continue)");
    }

    void set_wait_limit(unsigned long long limit_ns, u32 missing_blocks) override {
        wait_limit_ns_ = limit_ns;
        wait_missing_ = missing_blocks;
        drop_graph();  // captured launches carry the old limit
    }

    void profile_enable(u32 mask) override {
        profile_mask_ = mask;
        if (mask) drop_graph();
    }

    void profile_read(int kclass, double* total_ms, unsigned long long* count) override {
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        double t = 0.0;
        unsigned long long c = 0;
        std::vector<Record> keep;
        for (const Record& r : records_) {
            if (r.kclass != kclass) { keep.push_back(r); continue; }
            float ms = 0.0f;
            DFSPH_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
            t += ms;
            ++c;
            free_events_.push_back(r.a);
            free_events_.push_back(r.b);
        }
        records_.swap(keep);
        *total_ms = t;
        *count = c;
    }

    // ------------------------------------------------------------ state file
    // Header, per-scene counts, positions and velocities in the working type
    // (original order), wall positions in their input order. Little-endian
    // fixed-width fields; read back by load_state on either build machine.
    struct StateHeader {
        char magic[8];        // "DFSPHST1"
        u32 version;          // 1
        u32 real_bytes;       // 4 (float) or 8 (double)
        u32 n_scenes;
        u32 n;
        u32 nb;
        u32 stepped;          // 1: max_velocity holds the last step's value
        u32 maxv_bits;        // max |v| after the last step (float bits)
        u32 flags;            // bit 0: the position carries of a compensated run follow the walls
    };
    static constexpr u32 kStateCarries = 1u;

    void save_state(const char* path) override {
        const size_t n = n_;
        StateHeader h{};
        std::memcpy(h.magic, "DFSPHST1", 8);
        h.version = 1;
        h.real_bytes = sizeof(R);
        h.n_scenes = scenes_;
        h.n = have_state_ ? n_ : 0;
        h.nb = nb_;
        if (stepped_) {
            const float mv = float(get_scalar(DFSPH_SCALAR_MAX_VELOCITY));
            h.stepped = 1u;
            std::memcpy(&h.maxv_bits, &mv, sizeof(mv));
        }
        std::vector<u32> counts(scenes_, 0u);
        if (h.n) {
            if (scene_counts_.size() == scenes_) counts = scene_counts_;
            else counts[0] = n_;
        }
        std::vector<R> xv(6 * size_t(h.n));
        std::vector<float> xb(3 * size_t(nb_));
        // a compensated run continues exactly only with its position carries
        // (original order, x y z per particle)
        std::vector<V4> carries;
        if (comp_ && h.n) {
            h.flags |= kStateCarries;
            carries.resize(n);
            DFSPH_CUDA(cudaMemcpyAsync(carries.data(), xc_.p, n * sizeof(V4), cudaMemcpyDeviceToHost, stream_));
        }
        if (h.n) {
            R* d = static_cast<R*>(scratch_bytes(6 * n * sizeof(R)));
            launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, R>, blocks_for(n, 256), 256, int(n), id_[ci_].p,
                   (const V4*)xk_[cx_].p, -1, d);
            launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, R>, blocks_for(n, 256), 256, int(n), id_[ci_].p,
                   (const V4*)vr_[cv_].p, -1, d + 3 * n);
            DFSPH_CUDA(cudaMemcpyAsync(xv.data(), d, 6 * n * sizeof(R), cudaMemcpyDeviceToHost, stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
        }
        if (nb_) {
            float* d = static_cast<float*>(scratch_bytes(3 * size_t(nb_) * sizeof(float)));
            launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, float>, blocks_for(nb_, 256), 256, int(nb_), bid_[0].p,
                   (const V4*)xb_[0].p, -1, d);
            DFSPH_CUDA(cudaMemcpyAsync(xb.data(), d, 3 * size_t(nb_) * sizeof(float), cudaMemcpyDeviceToHost,
                                       stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
        }
        std::FILE* f = std::fopen(path, "wb");
        if (!f) throw Error(DFSPH_ERR_IO, std::string("cannot open ") + path + " for writing");
        bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
                  std::fwrite(counts.data(), sizeof(u32), counts.size(), f) == counts.size() &&
                  std::fwrite(xv.data(), sizeof(R), xv.size(), f) == xv.size() &&
                  std::fwrite(xb.data(), sizeof(float), xb.size(), f) == xb.size();
        for (size_t i = 0; ok && i < carries.size(); ++i) {
            const R c3[3] = {carries[i].x, carries[i].y, carries[i].z};
            ok = std::fwrite(c3, sizeof(R), 3, f) == 3;
        }
        ok = (std::fclose(f) == 0) && ok;
        if (!ok) throw Error(DFSPH_ERR_IO, std::string("short write to ") + path);
    }

    void load_state(const char* path) override {
        store_run_ = false;
        std::FILE* f = std::fopen(path, "rb");
        if (!f) throw Error(DFSPH_ERR_IO, std::string("cannot open ") + path);
        struct Closer { std::FILE* f; ~Closer() { std::fclose(f); } } closer{f};
        StateHeader h{};
        if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, "DFSPHST1", 8) != 0 || h.version != 1)
            throw Error(DFSPH_ERR_IO, std::string(path) + " is not a DFSPH state file");
        if (h.real_bytes != 4 && h.real_bytes != 8) throw Error(DFSPH_ERR_IO, "bad real width in state file");
        if (h.n_scenes != scenes_)
            throw Error(DFSPH_ERR_INVALID_ARGUMENT, "state file holds " + std::to_string(h.n_scenes) +
                                                        " scenes, the context " + std::to_string(scenes_));
        std::vector<u32> counts(h.n_scenes);
        if (std::fread(counts.data(), sizeof(u32), counts.size(), f) != counts.size())
            throw Error(DFSPH_ERR_IO, "truncated state file");
        unsigned long long total = 0;
        for (u32 c : counts) total += c;
        if (total != h.n) throw Error(DFSPH_ERR_IO, "inconsistent counts in state file");
        if (h.nb > bcap_) throw Error(DFSPH_ERR_OUT_OF_RANGE, "state file walls exceed boundary_capacity");
        const size_t n = h.n;
        std::vector<R> xv(6 * n);
        if (h.real_bytes == sizeof(R)) {
            if (std::fread(xv.data(), sizeof(R), xv.size(), f) != xv.size())
                throw Error(DFSPH_ERR_IO, "truncated state file");
        } else if (h.real_bytes == 4) {
            std::vector<float> t(6 * n);
            if (std::fread(t.data(), sizeof(float), t.size(), f) != t.size())
                throw Error(DFSPH_ERR_IO, "truncated state file");
            for (size_t k = 0; k < t.size(); ++k) xv[k] = R(t[k]);
        } else {
            std::vector<double> t(6 * n);
            if (std::fread(t.data(), sizeof(double), t.size(), f) != t.size())
                throw Error(DFSPH_ERR_IO, "truncated state file");
            for (size_t k = 0; k < t.size(); ++k) xv[k] = R(t[k]);
        }
        std::vector<float> xb(3 * size_t(h.nb));
        if (std::fread(xb.data(), sizeof(float), xb.size(), f) != xb.size())
            throw Error(DFSPH_ERR_IO, "truncated state file");
        // the carries of a compensated run: kept by a compensated context,
        // skipped by the others (which round every position update)
        std::vector<V4> carries;
        if ((h.flags & kStateCarries) && n) {
            if (h.real_bytes != 4) throw Error(DFSPH_ERR_IO, "position carries of a non-float state file");
            std::vector<float> t(3 * n);
            if (std::fread(t.data(), sizeof(float), t.size(), f) != t.size())
                throw Error(DFSPH_ERR_IO, "truncated state file");
            if (comp_) {
                carries.resize(n);
                for (size_t i = 0; i < n; ++i) carries[i] = {R(t[3 * i]), R(t[3 * i + 1]), R(t[3 * i + 2]), R(0)};
            }
        }
        check_counts(h.n_scenes, counts.data());
        set_boundary(xb.data(), h.nb, DFSPH_MEM_HOST);
        install_counts(h.n_scenes, counts.data(), h.n);
        ad_valid_ = false;
        if (n == 0) return;
        ensure_adjoint_buffers();
        R* st = static_cast<R*>(ad_staging(6 * n * sizeof(R)));
        DFSPH_CUDA(cudaMemcpyAsync(st, xv.data(), 6 * n * sizeof(R), cudaMemcpyHostToDevice, stream_));
        const int nbk = blocks_for(n, 256);
        launch(DFSPH_KERNEL_IO, pack3_kernel<R>, nbk, 256, int(n), (const R*)st, xg_.p);
        launch(DFSPH_KERNEL_IO, pack3_kernel<R>, nbk, 256, int(n), (const R*)(st + 3 * n), vg_.p);
        launch(DFSPH_KERNEL_IO, load_state_kernel<R>, nbk, 256, int(n), (const V4*)xg_.p, (const V4*)vg_.p,
               xk_[cx_].p, vr_[cv_].p, id_[ci_].p);
        // the saved run's max |v|, which sizes the next CFL substep
        DFSPH_CUDA(cudaMemsetAsync(ctl_.p->maxv_slot, 0, sizeof(ctl_.p->maxv_slot), stream_));
        if (h.stepped)
            DFSPH_CUDA(cudaMemcpyAsync(ctl_.p->maxv_slot, &h.maxv_bits, sizeof(u32), cudaMemcpyHostToDevice, stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        stepped_ = h.stepped != 0;
        counts_valid_ = false;
        reset_compensation();
        if (!carries.empty()) {
            DFSPH_CUDA(cudaMemcpyAsync(xc_.p, carries.data(), n * sizeof(V4), cudaMemcpyHostToDevice, stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
        }
        have_state_ = true;
    }

    // ------------------------------------------------------------ tuning
    // Threads per block of the four neighbour passes, measured on the
    // context's own state: each candidate runs `steps` steps from the same
    // snapshot with per-class CUDA-event timing, every class keeps its fastest
    // candidate, and the state (and the iteration controls) are put back.
    void autotune(float dt, u32 steps, int* chosen) override {
        if (!have_state_ || n_ == 0) throw Error(DFSPH_ERR_STATE, "no fluid state: call dfsph_set_fluid first");
        static const int kClasses[4] = {DFSPH_KERNEL_DENSITY_ALPHA, DFSPH_KERNEL_PRESSURE_RATE,
                                        DFSPH_KERNEL_PRESSURE_APPLY, DFSPH_KERNEL_FORCES_XSPH};
        static const int kCandidates[3] = {64, 128, 256};
        const size_t n = n_;
        if (tune_ck_.n < 2 * n) tune_ck_.alloc(2 * n);
        if (tune_ctl_.n < 3) tune_ctl_.alloc(3);
        drop_pending_counts();
        launch(DFSPH_KERNEL_IO, save_state_kernel<R>, blocks_for(n, 256), 256, int(n), id_[ci_].p, xk_[cx_].p,
               vr_[cv_].p, tune_ck_.p, tune_ck_.p + n);
        DFSPH_CUDA(cudaMemcpyAsync(tune_ctl_.p, ctl_.p, 3 * sizeof(IterCtl), cudaMemcpyDeviceToDevice, stream_));
        if (comp_) {
            if (tune_xc_.n < n) tune_xc_.alloc(n);
            DFSPH_CUDA(cudaMemcpyAsync(tune_xc_.p, xc_.p, n * sizeof(V4), cudaMemcpyDeviceToDevice, stream_));
        }
        const u32 saved_mask = profile_mask_;
        const bool saved_stepped = stepped_;
        profile_mask_ = 0;  // whole steps, unprofiled: passes keep their launch overlap
        // Every trial step starts from a cold L2, as a step of a large scene
        // does: a temporary buffer larger than the L2 is written before it.
        size_t l2 = 0;
        {
            int bytes = 0;
            DFSPH_CUDA(cudaDeviceGetAttribute(&bytes, cudaDevAttrL2CacheSize, device_));
            l2 = size_t(bytes);
        }
        DevBuf<unsigned char> flush;
        flush.alloc(2 * l2 + (1u << 20));
        cudaEvent_t ea = take_event(), eb = take_event();
        // median time of `trials` steps from the snapshot with the current shapes
        const u32 trials = std::max(steps, 5u);
        auto time_config = [&]() {
            restore_tuning_state();
            step_once(R(dt), true);  // untimed: first touch of this configuration
            std::vector<float> t(trials);
            for (u32 s = 0; s < trials; ++s) {
                DFSPH_CUDA(cudaMemsetAsync(flush.p, 0, flush.n, stream_));
                DFSPH_CUDA(cudaEventRecord(ea, stream_));
                step_once(R(dt), true);
                DFSPH_CUDA(cudaEventRecord(eb, stream_));
                DFSPH_CUDA(cudaEventSynchronize(eb));
                DFSPH_CUDA(cudaEventElapsedTime(&t[s], ea, eb));
            }
            std::sort(t.begin(), t.end());
            return double(t[trials / 2]);
        };
        // coordinate descent: each pass in turn takes the launch shape that
        // gives the shortest whole step with the other passes' shapes fixed;
        // a shape replaces the current one only when it saves more than 1 %
        // of the step, more than run-to-run noise
        int pick[4] = {bs_[kClasses[0]], bs_[kClasses[1]], bs_[kClasses[2]], bs_[kClasses[3]]};
        double best_ms = time_config();
        for (int k = 0; k < 4; ++k) {
            for (int c = 0; c < 3; ++c) {
                if (kCandidates[c] == pick[k]) continue;
                bs_[kClasses[k]] = kCandidates[c];
                const double ms = time_config();
                if (ms < 0.99 * best_ms) {
                    best_ms = ms;
                    pick[k] = kCandidates[c];
                }
                bs_[kClasses[k]] = pick[k];
            }
        }
        free_events_.push_back(ea);
        free_events_.push_back(eb);
        for (int k = 0; k < 4; ++k) bs_[kClasses[k]] = pick[k];
        restore_tuning_state();
        DFSPH_CUDA(cudaMemcpyAsync(ctl_.p, tune_ctl_.p, 3 * sizeof(IterCtl), cudaMemcpyDeviceToDevice, stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        profile_mask_ = saved_mask;
        stepped_ = saved_stepped;
        drop_graph();  // captured launches carry the old block sizes
        drop_adjoint_graph();
        if (chosen)
            for (int k = 0; k < DFSPH_KERNEL_CLASSES; ++k) chosen[k] = bs_[k];
    }

    void block_sizes(int* out) const override {
        for (int k = 0; k < DFSPH_KERNEL_CLASSES; ++k) out[k] = bs_[k];
    }

    // ------------------------------------------------------------ frames
    // n_frames frames of CFL substeps (sim_cli's loop, apps/sim_cli/main.cpp
    // :171-181). With graphs enabled and fixed iteration counts each frame is
    // one launch of a graph whose WHILE node repeats a captured substep and
    // whose dt is chosen on the device; otherwise the host runs the
    // reference's loop, reading max |v| back before every substep.
    void step_frames(const dfsph_frame_config& fc, u32 n_frames, u32* substeps) override {
        store_run_ = false;
        const NvtxRange range("dfsph frames");
        if (!have_state_) throw Error(DFSPH_ERR_STATE, "no fluid state: call dfsph_set_fluid first");
        if (n_frames == 0) return;
        std::vector<u32> subs(n_frames, 0u);
        if (graph_ok()) {
            if (!fctl_.p) {
                fctl_.alloc(1);
                DFSPH_CUDA(cudaMallocHost(reinterpret_cast<void**>(&host_fctl_), sizeof(FrameCtl)));
            }
            if (frame_sub_.n < n_frames) frame_sub_.alloc(n_frames);
            FrameCtl& h = *host_fctl_;
            std::memset(&h, 0, sizeof(h));
            h.frame_dt = fc.frame_dt;
            h.dt_max = fc.dt_max;
            h.cfl_lambda = fc.cfl_lambda;
            h.radius = cfg_.particle_radius;
            h.dt_min = fc.stepper_frame_dt / static_cast<float>(fc.max_substeps);
            h.v_floor = fc.min_velocity;
            h.damping = cfg_.damping;
            h.max_per_frame = fc.max_substeps_per_frame;
            h.fresh = stepped_ ? 0u : 1u;
            h.max_frames = n_frames;
            h.substeps_out = frame_sub_.p;
            DFSPH_CUDA(cudaMemcpyAsync(fctl_.p, &h, sizeof(FrameCtl), cudaMemcpyHostToDevice, stream_));
            if (!counts_valid_) {
                launch(DFSPH_KERNEL_GRID_COUNT, count_kernel<R>, blocks_for(n_, 256), 256, int(n_), xk_[cx_].p, g_,
                       key_.p, rank_.p, count_.p, fluid_krange());
                counts_valid_ = true;
            }
            ensure_frame_graph();
            for (u32 f = 0; f < n_frames; ++f) DFSPH_CUDA(cudaGraphLaunch(frame_exec_, stream_));
            DFSPH_CUDA(cudaMemcpyAsync(subs.data(), frame_sub_.p, n_frames * sizeof(u32), cudaMemcpyDeviceToHost,
                                       stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
            unsigned long long total = 0;
            for (u32 v : subs) total += v;
            launches_ += total * frame_body_kernels_ + 2ull * n_frames;
            stepped_ = true;
            iters_on_device_ = adaptive();
            last_frame_graph_ = 1;
        } else {
            for (u32 f = 0; f < n_frames; ++f) {
                float remaining = fc.frame_dt;
                u32 sub = 0;
                while (remaining > 1e-6f && sub < fc.max_substeps_per_frame) {
                    const float maxv = float(get_scalar(DFSPH_SCALAR_MAX_VELOCITY));
                    const float dt = host_next_dt(fc, std::max(maxv, fc.min_velocity), remaining);
                    step(dt, 1);
                    remaining -= dt;
                    ++sub;
                }
                subs[f] = sub;
            }
            last_frame_graph_ = 0;
        }
        if (substeps) std::memcpy(substeps, subs.data(), n_frames * sizeof(u32));
    }

    // ------------------------------------------------------------- adjoint
    void adjoint_set_state(const void* pos, const void* vel, u32 n, int mem) override {
        store_run_ = false;
        if (scenes_ != 1) throw Error(DFSPH_ERR_STATE, "the adjoint steps one scene");
        if (n > cap_) throw Error(DFSPH_ERR_OUT_OF_RANGE, "count " + std::to_string(n) + " exceeds capacity");
        const R* p = static_cast<const R*>(pos);
        const R* v = static_cast<const R*>(vel);
        if (mem == DFSPH_MEM_HOST && n) {
            R* st = static_cast<R*>(ad_staging(size_t(n) * 6 * sizeof(R)));
            DFSPH_CUDA(cudaMemcpyAsync(st, p, size_t(n) * 3 * sizeof(R), cudaMemcpyHostToDevice, stream_));
            if (v)
                DFSPH_CUDA(cudaMemcpyAsync(st + 3 * size_t(n), v, size_t(n) * 3 * sizeof(R), cudaMemcpyHostToDevice,
                                           stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
            p = st;
            v = v ? st + 3 * size_t(n) : nullptr;
        }
        n_ = n;
        drop_pending_counts();
        drop_graph();
        ad_valid_ = false;
        if (n == 0) return;
        ensure_adjoint_buffers();
        const int nb = blocks_for(n, 256);
        launch(DFSPH_KERNEL_IO, pack3_kernel<R>, nb, 256, int(n), p, xg_.p);
        launch(DFSPH_KERNEL_IO, pack3_kernel<R>, nb, 256, int(n), v, vg_.p);
        launch(DFSPH_KERNEL_IO, load_state_kernel<R>, nb, 256, int(n), (const V4*)xg_.p, (const V4*)vg_.p,
               xk_[cx_].p, vr_[cv_].p, id_[ci_].p);
        counts_valid_ = false;
        reset_compensation();
        have_state_ = true;
    }

    void adjoint_get_state(void* pos, void* vel, int mem) override {
        const size_t n = n_;
        if (n == 0) return;
        const size_t bytes = 3 * n * sizeof(R);
        void* outs[2] = {pos, vel};
        for (int k = 0; k < 2; ++k) {
            if (!outs[k]) continue;
            void* out = mem == DFSPH_MEM_DEVICE ? outs[k] : scratch_bytes(bytes);
            launch(DFSPH_KERNEL_IO, unsort_vec_kernel<R, R>, blocks_for(n, 256), 256, int(n), id_[ci_].p,
                   k == 0 ? (const V4*)xk_[cx_].p : (const V4*)vr_[cv_].p, -1, (R*)out);
            if (mem != DFSPH_MEM_DEVICE) {
                DFSPH_CUDA(cudaMemcpyAsync(outs[k], out, bytes, cudaMemcpyDeviceToHost, stream_));
                DFSPH_CUDA(cudaStreamSynchronize(stream_));
            }
        }
    }

    void adjoint_forward(float dt, u32 n_steps, u32 every) override {
        check_adjoint_config();
        if (!have_state_ || n_ == 0) throw Error(DFSPH_ERR_STATE, "no fluid state: set one first");
        ad_valid_ = false;
        const u32 segs = (n_steps + every - 1) / every;
        const size_t need = (size_t(segs) + 1) * 2 * size_t(n_);
        if (ck_.n < need) ck_.alloc(need);
        for (u32 s = 0; s < segs; ++s) {
            save_checkpoint(s);
            step(dt, std::min(every, n_steps - s * every));
        }
        save_checkpoint(segs);
        ad_n_ = n_;
        ad_steps_ = n_steps;
        ad_every_ = every;
        ad_dt_ = dt;
        ad_eps_ = cfg_.viscosity;
        ad_valid_ = true;
    }

    void adjoint_backward(const void* xbar, const void* vbar, void* x0bar, void* v0bar, double* eps_bar,
                          int mem) override {
        const NvtxRange range("dfsph adjoint backward");
        if (!ad_valid_ || n_ != ad_n_) throw Error(DFSPH_ERR_STATE, "no recorded rollout: call dfsph_adjoint_forward");
        if (cfg_.viscosity != ad_eps_) throw Error(DFSPH_ERR_STATE, "the XSPH coefficient changed since the rollout");
        check_adjoint_config();
        if (!xbar) throw Error(DFSPH_ERR_INVALID_ARGUMENT, "pos_bar is required");
        const u32 n = n_;
        ensure_adjoint_buffers();
        const R* xb = static_cast<const R*>(xbar);
        const R* vb = static_cast<const R*>(vbar);
        if (mem == DFSPH_MEM_HOST) {
            R* st = static_cast<R*>(ad_staging(size_t(n) * 6 * sizeof(R)));
            DFSPH_CUDA(cudaMemcpyAsync(st, xb, size_t(n) * 3 * sizeof(R), cudaMemcpyHostToDevice, stream_));
            if (vb)
                DFSPH_CUDA(cudaMemcpyAsync(st + 3 * size_t(n), vb, size_t(n) * 3 * sizeof(R), cudaMemcpyHostToDevice,
                                           stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
            xb = st;
            vb = vb ? st + 3 * size_t(n) : nullptr;
        }
        const int nb = blocks_for(n, 256);
        launch(DFSPH_KERNEL_IO, pack3_kernel<R>, nb, 256, int(n), xb, xg_.p);
        launch(DFSPH_KERNEL_IO, pack3_kernel<R>, nb, 256, int(n), vb, vg_.p);
        DFSPH_CUDA(cudaMemsetAsync(eps_acc_.p, 0, sizeof(double), stream_));
        DFSPH_CUDA(cudaMemsetAsync(eps_ctr_.p, 0, sizeof(u32), stream_));
        const u32 segs = (ad_steps_ + ad_every_ - 1) / ad_every_;
        const u32 full = ad_steps_ / ad_every_;  // segments 0 .. full-1 have ad_every_ steps
        const bool pipelined = full > 0 && profile_mask_ == 0;
        ensure_tape(pipelined ? 2 * ad_every_ : std::min(ad_every_, ad_steps_));
        // the segments run from the last; a shorter last segment, and every
        // segment while the passes are profiled, run plainly
        for (u32 s = segs; s-- > (pipelined ? full : 0u);) {
            const u32 cnt = std::min(ad_every_, ad_steps_ - s * ad_every_);
            restore_checkpoint(s);
            {
                const NvtxRange replay("adjoint segment replay");
                for (u32 k = 0; k < cnt; ++k) {
                    const StepTape<R> t = tape_at(k);
                    step_once(R(ad_dt_), true, &t);
                }
            }
            const NvtxRange reverse("adjoint segment reverse");
            for (u32 k = cnt; k-- > 0;) backward_step(tape_at(k));
        }
        if (pipelined) {
            // Full segments: the replay of segment s - 1 (side stream, record
            // buffer (s - 1) & 1) runs while the reverse of segment s (this
            // stream, buffer s & 1) does; a buffer is rewritten only after
            // the reverse that read it. The reverse kernels read only the
            // records and the adjoint arrays, the replays write only the state
            // and their records.
            const NvtxRange pipe("adjoint segments, replay and reverse overlapped");
            ensure_adjoint_graphs(ad_every_);
            if (!replay_stream_) {
                DFSPH_CUDA(cudaStreamCreateWithFlags(&replay_stream_, cudaStreamNonBlocking));
                for (cudaEvent_t* e : {&ev_start_, &ev_replayed_[0], &ev_replayed_[1], &ev_reversed_[0],
                                       &ev_reversed_[1]})
                    DFSPH_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
            }
            const cudaStream_t rev = stream_, side = replay_stream_;
            DFSPH_CUDA(cudaEventRecord(ev_start_, rev));
            DFSPH_CUDA(cudaStreamWaitEvent(side, ev_start_, 0));
            auto replay = [&](u32 s) {
                const u32 b = s & 1u;
                stream_ = side;
                try {
                    restore_checkpoint(s);
                } catch (...) {
                    stream_ = rev;
                    throw;
                }
                stream_ = rev;
                DFSPH_CUDA(cudaGraphLaunch(adj_replay_[b].e, side));
                launches_ += adj_replay_[b].kernels;
                counts_valid_ = true;  // the last replayed step counted the next one's cells
                DFSPH_CUDA(cudaEventRecord(ev_replayed_[b], side));
            };
            replay(full - 1);
            for (u32 s = full; s-- > 0;) {
                const u32 b = s & 1u;
                DFSPH_CUDA(cudaStreamWaitEvent(rev, ev_replayed_[b], 0));
                DFSPH_CUDA(cudaGraphLaunch(adj_reverse_[b].e, rev));
                launches_ += adj_reverse_[b].kernels;
                DFSPH_CUDA(cudaEventRecord(ev_reversed_[b], rev));
                if (s > 0) {
                    // buffer (s - 1) & 1 was last read by the reverse of segment s + 1
                    if (s + 1 < full) DFSPH_CUDA(cudaStreamWaitEvent(side, ev_reversed_[(s - 1) & 1u], 0));
                    replay(s - 1);
                }
            }
        }
        const size_t bytes = 3 * size_t(n) * sizeof(R);
        void* outs[2] = {x0bar, v0bar};
        for (int k = 0; k < 2; ++k) {
            if (!outs[k]) continue;
            void* out = mem == DFSPH_MEM_DEVICE ? outs[k] : scratch_bytes(bytes);
            launch(DFSPH_KERNEL_IO, unpack3_kernel<R>, nb, 256, int(n), k == 0 ? (const V4*)xg_.p : (const V4*)vg_.p,
                   (R*)out);
            if (mem != DFSPH_MEM_DEVICE) {
                DFSPH_CUDA(cudaMemcpyAsync(outs[k], out, bytes, cudaMemcpyDeviceToHost, stream_));
                DFSPH_CUDA(cudaStreamSynchronize(stream_));
            }
        }
        if (eps_bar) {
            DFSPH_CUDA(cudaMemcpyAsync(eps_host_, eps_acc_.p, sizeof(double), cudaMemcpyDeviceToHost, stream_));
            DFSPH_CUDA(cudaStreamSynchronize(stream_));
            *eps_bar = *eps_host_;
        }
        restore_checkpoint(segs);
    }

private:
    void restore_tuning_state() {
        const size_t n = n_;
        drop_pending_counts();
        launch(DFSPH_KERNEL_IO, load_state_kernel<R>, blocks_for(n, 256), 256, int(n), (const V4*)tune_ck_.p,
               (const V4*)(tune_ck_.p + n), xk_[cx_].p, vr_[cv_].p, id_[ci_].p);
        if (comp_)
            DFSPH_CUDA(cudaMemcpyAsync(xc_.p, tune_xc_.p, n * sizeof(V4), cudaMemcpyDeviceToDevice, stream_));
        counts_valid_ = false;
    }

    void check_adjoint_config() const {
        if (scenes_ != 1) throw Error(DFSPH_ERR_STATE, "the adjoint steps one scene");
        if (comp_)
            throw Error(DFSPH_ERR_STATE, "the adjoint differentiates the FP32, FP32_KAHAN or FP64 step, not the "
                                         "compensated position update of FP32_COMPENSATED");
        if (g_.rank) throw Error(DFSPH_ERR_STATE, "the adjoint needs the x-major slot order");
        if ((cfg_.max_density_iters > 0 && cfg_.eta_density > 0.0f) ||
            (cfg_.max_divergence_iters > 0 && cfg_.eta_divergence > 0.0f))
            throw Error(DFSPH_ERR_STATE, "the adjoint needs fixed iteration counts (eta_density = eta_divergence = 0)");
    }

    void* ad_staging(size_t bytes) {
        if (ad_staging_.n < bytes) ad_staging_.alloc(bytes);
        return ad_staging_.p;
    }

    // the partials (or warp sums) of the error reductions, past their counters
    double* red_partials() const { return partials_.p + REDUCE_GROUP_WORDS / 2; }

    int sm_count() {
        if (sm_count_ == 0) DFSPH_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_));
        return sm_count_;
    }

    void ensure_adjoint_buffers() {
        if (xg_.n >= cap_ && cap_) return;
        const size_t c = std::max(cap_, 1u);
        xg_.alloc(c); vg_.alloc(c); xbar_.alloc(c); vbar_[0].alloc(c); vbar_[1].alloc(c);
        xr_.alloc(c); xq_.alloc(c); gq_.alloc(c);
        rhobar_.alloc(c); alphabar_.alloc(c);
        eps_part_.alloc((c + 127) / 128);
        eps_ctr_.alloc(1);
        eps_acc_.alloc(1);
        if (!eps_host_) DFSPH_CUDA(cudaMallocHost(reinterpret_cast<void**>(&eps_host_), sizeof(double)));
    }

    void save_checkpoint(u32 slot) {
        const size_t n = n_;
        V4* base = ck_.p + size_t(slot) * 2 * n;
        launch(DFSPH_KERNEL_IO, save_state_kernel<R>, blocks_for(n, 256), 256, int(n), id_[ci_].p, xk_[cx_].p,
               vr_[cv_].p, base, base + n);
    }

    void restore_checkpoint(u32 slot) {
        const size_t n = n_;
        const V4* base = ck_.p + size_t(slot) * 2 * n;
        drop_pending_counts();
        launch(DFSPH_KERNEL_IO, load_state_kernel<R>, blocks_for(n, 256), 256, int(n), base, base + n, xk_[cx_].p,
               vr_[cv_].p, id_[ci_].p);
        counts_valid_ = false;
    }

    // Per-step record layout: 256-byte aligned arrays of stride np slots.
    static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
    size_t tape_stride() const { return (size_t(n_) + 63) & ~size_t(63); }
    size_t tape_step_bytes() const {
        const size_t np = tape_stride();
        const size_t kd = cfg_.max_divergence_iters, kr = cfg_.max_density_iters;
        return align256(np * sizeof(V4)) * (4 + 2 * (kd + kr)) + align256(np * sizeof(R)) * 2 * (kd + kr) +
               align256(np * sizeof(u32)) + align256(np) + align256((keys_ + 1) * sizeof(u32));
    }
    void ensure_tape(u32 steps) {
        const size_t need = tape_step_bytes() * steps;
        if (tape_.n < need) {
            drop_adjoint_graph();  // its replays write the old records
            tape_.alloc(need);
        }
    }

    // Graphs of the backward pass, per record buffer b (0, 1): the replay of
    // a full segment (its k steps from the restored checkpoint, writing the
    // records of buffer b) and its reverse (the k reverse steps reading them).
    // Steps leave the buffer parity unchanged and the records sit at fixed
    // addresses, so one capture serves every full segment (and every backward
    // pass with the same k, n, dt and XSPH coefficient). Checkpoint restores
    // run outside.
    struct SegmentGraph {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t e = nullptr;
        unsigned long long kernels = 0;
    };

    template <class Body> void capture_segment_graph(SegmentGraph& sg, Body&& body) {
        if (!capture_stream_) DFSPH_CUDA(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
        const cudaStream_t caller = stream_;
        const unsigned long long k0 = graph_kernels_;
        const bool counted = counts_valid_;
        const int cx = cx_, cv = cv_, ci = ci_;
        DFSPH_CUDA(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal));
        stream_ = capture_stream_;
        capturing_ = true;
        counts_valid_ = false;  // a replay starts from a restored checkpoint
        try {
            body();
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(capture_stream_, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            capturing_ = false;
            stream_ = caller;
            counts_valid_ = counted;
            graph_kernels_ = k0;
            cx_ = cx; cv_ = cv; ci_ = ci;
            throw;
        }
        capturing_ = false;
        stream_ = caller;
        counts_valid_ = counted;
        DFSPH_CUDA(cudaStreamEndCapture(capture_stream_, &sg.g));
        if (cx_ != cx || cv_ != cv || ci_ != ci) throw Error(DFSPH_ERR_STATE, "a step changed buffer parity");
        DFSPH_CUDA(cudaGraphInstantiate(&sg.e, sg.g, 0));
        sg.kernels = graph_kernels_ - k0;
        graph_kernels_ = k0;
    }

    void ensure_adjoint_graphs(u32 cnt) {
        if (adj_replay_[0].e && adj_len_ == cnt && adj_n_ == n_ && adj_dt_ == ad_dt_ && adj_eps_ == ad_eps_ &&
            cx_ == adj_cx_ && cv_ == adj_cv_ && ci_ == adj_ci_)
            return;
        drop_adjoint_graph();
        for (u32 b = 0; b < 2; ++b) {
            capture_segment_graph(adj_replay_[b], [&] {
                for (u32 k = 0; k < cnt; ++k) {
                    const StepTape<R> t = tape_at(k, b);
                    step_once(R(ad_dt_), true, &t);
                }
            });
            capture_segment_graph(adj_reverse_[b], [&] {
                for (u32 k = cnt; k-- > 0;) backward_step(tape_at(k, b));
            });
        }
        adj_len_ = cnt;
        adj_n_ = n_;
        adj_dt_ = ad_dt_;
        adj_eps_ = ad_eps_;
        adj_cx_ = cx_; adj_cv_ = cv_; adj_ci_ = ci_;
    }

    void drop_adjoint_graph() {
        for (SegmentGraph* sg : {&adj_replay_[0], &adj_replay_[1], &adj_reverse_[0], &adj_reverse_[1]}) {
            if (sg->e) cudaGraphExecDestroy(sg->e);
            if (sg->g) cudaGraphDestroy(sg->g);
            sg->e = nullptr;
            sg->g = nullptr;
        }
    }
    // Records of step k of a segment in record buffer buf (buffers of
    // ad_every_ steps each).
    StepTape<R> tape_at(u32 k, u32 buf = 0) {
        const size_t np = tape_stride();
        const size_t kd = cfg_.max_divergence_iters, kr = cfg_.max_density_iters;
        unsigned char* q = tape_.p + tape_step_bytes() * (size_t(buf) * ad_every_ + k);
        auto take = [&](size_t bytes) {
            unsigned char* r = q;
            q += align256(bytes);
            return r;
        };
        StepTape<R> t;
        t.stride = np;
        t.x = reinterpret_cast<V4*>(take(np * sizeof(V4)));
        t.g = reinterpret_cast<V4*>(take(np * sizeof(V4)));
        t.vx = reinterpret_cast<V4*>(take(np * sizeof(V4)));
        t.va = reinterpret_cast<V4*>(take(np * sizeof(V4)));
        const size_t its[2] = {kd, kr};
        for (int w = 0; w < 2; ++w) {
            t.xkf[w] = reinterpret_cast<V4*>(q); for (size_t i = 0; i < its[w]; ++i) take(np * sizeof(V4));
            t.v[w] = reinterpret_cast<V4*>(q); for (size_t i = 0; i < its[w]; ++i) take(np * sizeof(V4));
            t.kap[w] = reinterpret_cast<R*>(q); for (size_t i = 0; i < its[w]; ++i) take(np * sizeof(R));
            t.adv[w] = reinterpret_cast<R*>(q); for (size_t i = 0; i < its[w]; ++i) take(np * sizeof(R));
        }
        t.id = reinterpret_cast<u32*>(take(np * sizeof(u32)));
        t.amask = take(np);
        t.cs = reinterpret_cast<u32*>(take((keys_ + 1) * sizeof(u32)));
        return t;
    }

    // Reverse of step_once for one recorded step: the adjoint of the step's
    // output state (xg_, vg_ in original order) becomes that of its input.
    void backward_step(const StepTape<R>& t) {
        const int n = int(n_);
        const int b128 = blocks_for(n, 128), b256 = blocks_for(n, 256);
        const R dt = R(ad_dt_);
        const BoundaryDev bd = bdev();
        const size_t st = t.stride;
        int cur = 0;
        launch(DFSPH_KERNEL_ADJOINT, adjoint_advect_kernel<R>, b256, 256, n, (const u32*)t.id, (const V4*)t.va,
               (const unsigned char*)t.amask, dt, (const V4*)xg_.p, (const V4*)vg_.p, xbar_.p, vbar_[cur].p,
               rhobar_.p, alphabar_.p);
        // two lanes per particle when one lane would give at most four
        // 128-thread blocks per SM: those launches are latency-bound, larger
        // ones lose more to the lanes' shuffles than they gain
        const bool wide = n <= 4 * 128 * sm_count();
        const int b2 = blocks_for(2 * n, 128);
        auto apply_rate = [&](int w, u32 it, auto divergence) {
            constexpr bool D = decltype(divergence)::value;
            const V4* xkf = (const V4*)(t.xkf[w] + it * st);
            const R* kap = (const R*)(t.kap[w] + it * st);
            const R* adv = (const R*)(t.adv[w] + it * st);
            const V4* vel = (const V4*)(t.v[w] + it * st);
            if (wide) {
                launch(DFSPH_KERNEL_ADJOINT, adjoint_apply_kernel<R, D, 2>, b2, 128, n, xkf, (const V4*)t.x,
                       (const V4*)t.g, kap, adv, (const V4*)vbar_[cur].p, (const u32*)t.cs, g_, phys_, bd, dt,
                       xbar_.p, rhobar_.p, alphabar_.p, xr_.p);
                launch(DFSPH_KERNEL_ADJOINT, adjoint_rate_kernel<R, 2>, b2, 128, n, (const V4*)xr_.p, vel,
                       (const u32*)t.cs, g_, phys_, bd, vbar_[cur].p, xbar_.p);
            } else {
                launch(DFSPH_KERNEL_ADJOINT, adjoint_apply_kernel<R, D, 1>, b128, 128, n, xkf, (const V4*)t.x,
                       (const V4*)t.g, kap, adv, (const V4*)vbar_[cur].p, (const u32*)t.cs, g_, phys_, bd, dt,
                       xbar_.p, rhobar_.p, alphabar_.p, xr_.p);
                launch(DFSPH_KERNEL_ADJOINT, adjoint_rate_kernel<R, 1>, b128, 128, n, (const V4*)xr_.p, vel,
                       (const u32*)t.cs, g_, phys_, bd, vbar_[cur].p, xbar_.p);
            }
        };
        for (u32 it = cfg_.max_density_iters; it-- > 0;) apply_rate(1, it, std::false_type{});
        launch(DFSPH_KERNEL_ADJOINT, adjoint_xsph_kernel<R>, b128, 128, n, (const V4*)t.x, (const V4*)t.vx,
               (const V4*)vbar_[cur].p, vbar_[cur ^ 1].p, (const u32*)t.cs, g_, phys_, R(cfg_.damping), dt,
               R(ad_eps_), xbar_.p,
               rhobar_.p, eps_part_.p, eps_ctr_.p, eps_acc_.p);
        cur ^= 1;
        for (u32 it = cfg_.max_divergence_iters; it-- > 0;) apply_rate(0, it, std::true_type{});
        launch(DFSPH_KERNEL_ADJOINT, adjoint_density_prep_kernel<R>, b256, 256, n, (const V4*)t.x, (const V4*)t.g,
               (const R*)rhobar_.p, (const R*)alphabar_.p, xq_.p, gq_.p);
        launch(DFSPH_KERNEL_ADJOINT, adjoint_density_kernel<R>, b128, 128, n, (const V4*)xq_.p, (const V4*)gq_.p,
               (const V4*)vbar_[cur].p, (const V4*)xbar_.p, (const u32*)t.id, (const u32*)t.cs, g_, phys_, bd, xg_.p,
               vg_.p);
    }

    static constexpr u32 kSentinelCap = 4096;

    template <class K, class... A> void launch(int kclass, K kernel, int grid, int block, A... args) {
        if (grid <= 0) return;
        const bool prof = !capturing_ && ((profile_mask_ >> kclass) & 1u);
        cudaEvent_t a = nullptr, b = nullptr;
        if (prof) {
            a = take_event();
            b = take_event();
            DFSPH_CUDA(cudaEventRecord(a, stream_));
        }
        if (!prof && (kclass <= DFSPH_KERNEL_ADVECT || kclass == DFSPH_KERNEL_ADJOINT)) {
            // the step's and the adjoint's kernels (they all begin with pdl_wait): launched with
            // programmatic stream serialization, so a kernel's launch and
            // block scheduling overlap the drain of the one before it
            cudaLaunchConfig_t lc = {};
            lc.gridDim = dim3(unsigned(grid));
            lc.blockDim = dim3(unsigned(block));
            lc.stream = stream_;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            at[0].val.programmaticStreamSerializationAllowed = 1;
            lc.attrs = at;
            lc.numAttrs = 1;
            DFSPH_CUDA(cudaLaunchKernelEx(&lc, kernel, args...));
        } else {
            kernel<<<grid, block, 0, stream_>>>(args...);
            DFSPH_LAUNCHED();
        }
        if (capturing_) ++graph_kernels_;
        else ++launches_;
        if (prof) {
            DFSPH_CUDA(cudaEventRecord(b, stream_));
            records_.push_back({kclass, a, b});
        }
    }

    // The integrator's arguments, for a solve that may carry it in its last
    // iteration (done is set when it did).
    struct FusedAdvect {
        Domain<R> d;
        u32* mvs;
        int cx0;
        bool count;
        bool done;
    };
    // the integrator's compensation carries when this step uses them
    const u32* comp_id() const { return comp_ ? id_[ci_].p : nullptr; }
    V4* comp_xc() const { return comp_ ? xc_.p : nullptr; }
    void reset_key_range() {
        DFSPH_CUDA(cudaMemsetAsync(krange_.p, 0xFF, KRANGE_SLOTS * sizeof(u32), stream_));
        DFSPH_CUDA(cudaMemsetAsync(krange_.p + KRANGE_SLOTS, 0, KRANGE_SLOTS * sizeof(u32), stream_));
    }
    // ranged fluid scans only in the x-major order (Morton ranks of
    // neighbouring cells are not near each other)
    u32* fluid_krange() const { return g_.rank ? nullptr : krange_.p; }
    // cell_start in full, for readers beyond the particles' stencils. The
    // flag stays set: every later ranged scan (graph replays included, which
    // run no host code) leaves stale entries again.
    void complete_cell_start() {
        if (!cs_ranged_) return;
        const size_t m = keys_;
        launch(DFSPH_KERNEL_IO, complete_cell_start_kernel, blocks_for(m, 256), 256, cell_start_.p, u32(m),
               (const u32*)cs_range_.p);
    }
    void reset_compensation() {
        if (comp_ && cap_) DFSPH_CUDA(cudaMemsetAsync(xc_.p, 0, size_t(cap_) * sizeof(V4), stream_));
    }

    // A neighbour pass at the tuned block size: the instantiation bounded by
    // 256 threads for 256-thread blocks, the one bounded by 128 otherwise
    // (a tighter bound leaves the compiler more registers per thread).
    template <class K1, class K2, class... A> void launch_pass(int kclass, K1 k128, K2 k256, A... args) {
        const int b = bs_[kclass];
        if (b > 128) launch(kclass, k256, blocks_for(n_, b), b, args...);
        else launch(kclass, k128, blocks_for(n_, b), b, args...);
    }

    struct Record { int kclass; cudaEvent_t a, b; };
    cudaEvent_t take_event() {
        if (free_events_.empty()) {
            cudaEvent_t e;
            DFSPH_CUDA(cudaEventCreate(&e));
            return e;
        }
        cudaEvent_t e = free_events_.back();
        free_events_.pop_back();
        return e;
    }

    // ---- CUDA graphs: every step returns the ping-pong buffers to where it
    // found them (step_once), so a captured pair of steps replays with the
    // same pointers.
    bool adaptive() const {
        return (cfg_.max_density_iters > 0 && cfg_.eta_density > 0.0f) ||
               (cfg_.max_divergence_iters > 0 && cfg_.eta_divergence > 0.0f);
    }
    bool graph_ok() const {
        // adaptive solves run as device-resident loops inside the graph
        return cfg_.use_cuda_graph && profile_mask_ == 0 && have_state_ && n_ > 0;
    }
    void drop_graph() {
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        if (graph_) cudaGraphDestroy(graph_);
        graph_exec_ = nullptr;
        graph_ = nullptr;
        if (frame_exec_) cudaGraphExecDestroy(frame_exec_);
        if (frame_graph_) cudaGraphDestroy(frame_graph_);
        frame_exec_ = nullptr;
        frame_graph_ = nullptr;
    }

    // TimeStepper::next_dt (core/include/water/core/timestep.h:23-28) on the host.
    float host_next_dt(const dfsph_frame_config& fc, float max_velocity, float remaining) const {
        const float v = std::max(max_velocity, 1e-6f);
        const float dt_cfl = fc.cfl_lambda * cfg_.particle_radius / v;
        const float dt_min = fc.stepper_frame_dt / static_cast<float>(fc.max_substeps);
        return std::min({fc.dt_max, dt_cfl, remaining, std::max(dt_cfl, dt_min)});
    }

    // Graph of one frame: frame_begin -> WHILE(cond) { one substep with the
    // device dt; frame_control } -> frame_end. The substep is captured once;
    // steps leave the buffer parity unchanged, so every iteration replays the
    // same pointers. Rebuilt when the stream, the state or the parity changes.
    // Before a capture: every cooperative solve that the captured steps would
    // launch is launched once eagerly, with no iterations (it reads the state
    // and writes only a scratch control block), so that the capture records
    // only cooperative launches this device has accepted; a refused one makes
    // the capture use the per-pass solve.
    void verify_cooperative() {
        if (!have_state_ || n_ == 0) return;
        if (!probe_ctl_.p) {
            probe_ctl_.alloc(1);
            DFSPH_CUDA(cudaMemsetAsync(probe_ctl_.p, 0, sizeof(IterCtl), stream_));
        }
        StepDt<R> sd{};
        sd.dt = R(1);
        sd.dev = nullptr;
        const StopTest none{double(n_), 0.0, 0};
        if (cfg_.max_divergence_iters > 0 && coop_ok_[1] == 0)
            solve_cooperative<true>(sd, 0, none, 0, probe_ctl_.p, kap_v_.p, rho_dot_.p, cell_start_.p, true);
        if (cfg_.max_density_iters > 0 && coop_ok_[0] == 0)
            solve_cooperative<false>(sd, 0, none, 1, probe_ctl_.p, kap_.p, rho_adv_.p, cell_start_.p, true);
    }

    void ensure_frame_graph() {
        if (frame_exec_ && cx_ == fg_cx_ && cv_ == fg_cv_ && ci_ == fg_ci_) return;
        verify_cooperative();
        if (frame_exec_) cudaGraphExecDestroy(frame_exec_);
        if (frame_graph_) cudaGraphDestroy(frame_graph_);
        frame_exec_ = nullptr;
        frame_graph_ = nullptr;
        if (!capture_stream_) DFSPH_CUDA(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
        const int cx = cx_, cv = cv_, ci = ci_;
        const cudaStream_t caller = stream_;
        const unsigned long long k0 = graph_kernels_;
        cudaGraph_t g = nullptr;
        DFSPH_CUDA(cudaGraphCreate(&g, 0));
        bool in_capture = false;
        try {
            FrameCtl* f = fctl_.p;
            const IterCtl* c = ctl_.p;
            void* begin_args[] = {&f, &c};
            cudaKernelNodeParams kp = {};
            kp.func = reinterpret_cast<void*>(frame_begin_kernel);
            kp.gridDim = dim3(1);
            kp.blockDim = dim3(32);
            kp.kernelParams = begin_args;
            cudaGraphNode_t nb = nullptr;
            DFSPH_CUDA(cudaGraphAddKernelNode(&nb, g, nullptr, 0, &kp));
            cudaGraphConditionalHandle h = 0;
            DFSPH_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault));
            cudaGraphNodeParams cp = {};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t nc = nullptr;
            DFSPH_CUDA(cudaGraphAddNode(&nc, g, &nb, nullptr, 1, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            DFSPH_CUDA(cudaStreamBeginCaptureToGraph(capture_stream_, body, nullptr, nullptr, 0,
                                                     cudaStreamCaptureModeThreadLocal));
            in_capture = true;
            stream_ = capture_stream_;
            capturing_ = true;
            step_once(R(0), true, nullptr, f);
            launch(DFSPH_KERNEL_OTHER, frame_control_kernel, 1, 32, f, c, h, 1);
            capturing_ = false;
            stream_ = caller;
            in_capture = false;
            cudaGraph_t captured = nullptr;
            DFSPH_CUDA(cudaStreamEndCapture(capture_stream_, &captured));
            void* end_args[] = {&f};
            kp.func = reinterpret_cast<void*>(frame_end_kernel);
            kp.kernelParams = end_args;
            cudaGraphNode_t ne = nullptr;
            DFSPH_CUDA(cudaGraphAddKernelNode(&ne, g, &nc, 1, &kp));
            if (cx_ != cx || cv_ != cv || ci_ != ci) throw Error(DFSPH_ERR_STATE, "a step changed buffer parity");
            DFSPH_CUDA(cudaGraphInstantiate(&frame_exec_, g, 0));
        } catch (...) {
            if (in_capture) {
                cudaGraph_t x = nullptr;
                cudaStreamEndCapture(capture_stream_, &x);
            }
            cudaGraphDestroy(g);
            cudaGetLastError();
            capturing_ = false;
            stream_ = caller;
            cx_ = cx; cv_ = cv; ci_ = ci;
            graph_kernels_ = k0;
            frame_exec_ = nullptr;
            throw;
        }
        frame_graph_ = g;
        frame_body_kernels_ = graph_kernels_ - k0;
        graph_kernels_ = k0;
        fg_cx_ = cx_; fg_cv_ = cv_; fg_ci_ = ci_;
    }
    void ensure_graph(float dt) {
        // a replayed adjoint segment leaves the ping-pong parity where a plain
        // step would not, so the graph is only reused at its capture parity
        if (graph_exec_ && graph_dt_ == dt && cx_ == graph_cx_ && cv_ == graph_cv_ && ci_ == graph_ci_) return;
        drop_graph();
        verify_cooperative();
        const int cx = cx_, cv = cv_, ci = ci_;
        const bool counted = counts_valid_, stepped = stepped_;
        // Capture on a private stream (the caller's may be the legacy default
        // stream, which cannot be captured); replays go to the caller's stream.
        if (!capture_stream_) DFSPH_CUDA(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
        const cudaStream_t caller = stream_;
        graph_kernels_ = 0;
        DFSPH_CUDA(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal));
        stream_ = capture_stream_;
        capturing_ = true;
        try {
            step_once(R(dt), true);
            step_once(R(dt), true);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(capture_stream_, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            capturing_ = false;
            stream_ = caller;
            cx_ = cx; cv_ = cv; ci_ = ci;
            counts_valid_ = counted;
            stepped_ = stepped;
            throw;
        }
        capturing_ = false;
        stream_ = caller;
        DFSPH_CUDA(cudaStreamEndCapture(capture_stream_, &graph_));
        if (cx_ != cx || cv_ != cv || ci_ != ci) throw Error(DFSPH_ERR_STATE, "graph capture changed buffer parity");
        DFSPH_CUDA(cudaGraphInstantiate(&graph_exec_, graph_, 0));
        graph_dt_ = dt;
        graph_cx_ = cx_; graph_cv_ = cv_; graph_ci_ = ci_;
    }

    // The integrator leaves the next step's per-cell counts in count_; any new
    // input invalidates them and count_ must be zero before the next count.
    void drop_pending_counts() {
        if (!counts_valid_) return;
        DFSPH_CUDA(cudaMemsetAsync(count_.p, 0, keys_ * sizeof(u32), stream_));
        reset_key_range();
        counts_valid_ = false;
    }

    // Host data goes through a device staging buffer; device data is used in place.
    const float* upload(const float* xyz, const float* vel, u32 n, int mem) {
        if (mem == DFSPH_MEM_DEVICE || n == 0) return xyz;
        if (mem != DFSPH_MEM_HOST) throw Error(DFSPH_ERR_INVALID_ARGUMENT, "mem must be host or device");
        DFSPH_CUDA(cudaMemcpyAsync(staging_.p, xyz, size_t(n) * 3 * sizeof(float), cudaMemcpyHostToDevice, stream_));
        if (vel)
            DFSPH_CUDA(cudaMemcpyAsync(staging_.p + 3 * size_t(n), vel, size_t(n) * 3 * sizeof(float),
                                       cudaMemcpyHostToDevice, stream_));
        // the caller may free its host buffer after return
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        return staging_.p;
    }

    void launch_import(u32 n, const float* pos, const float* vel, V4* xk, V4* vr, u32* id) {
        launch(DFSPH_KERNEL_IO, import_kernel<R>, blocks_for(n, 256), 256, int(n), pos, vel, xk, vr, id);
    }

    // Scratch 4-vectors for the wall sort's unused velocity lane.
    V4* vr_scratch() { ensure_bscratch(); return bscratch_[0].p; }
    V4* vr_scratch2() { ensure_bscratch(); return bscratch_[1].p; }
    void ensure_bscratch() {
        if (bscratch_[0].n < bcap_) { bscratch_[0].alloc(bcap_); bscratch_[1].alloc(bcap_); }
    }

    // Wall particles with at least one fluid particle within the kernel
    // support, against the fluid grid of the last step (a diagnostic for the
    // algorithmic byte count of the wall terms).
    u32 active_boundary() {
        if (nb_ == 0 || n_ == 0 || !stepped_) return 0;
        complete_cell_start();  // it walks the stencils of all wall particles
        u32* d = static_cast<u32*>(scratch_bytes(sizeof(u32)));
        DFSPH_CUDA(cudaMemsetAsync(d, 0, sizeof(u32), stream_));
        with_slot_order([&](auto order) {
            launch(DFSPH_KERNEL_OTHER, active_boundary_kernel<R, decltype(order)::value>, blocks_for(nb_, 128), 128,
                   int(nb_), xb_[0].p, xk_[cx_].p, cell_start_.p, g_, phys_, int(scenes_), d);
        });
        u32 h = 0;
        DFSPH_CUDA(cudaMemcpyAsync(&h, d, sizeof(u32), cudaMemcpyDeviceToHost, stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
        return h;
    }

    void* scratch_bytes(size_t bytes) {
        if (readback_.n < bytes) readback_.alloc(bytes);
        return readback_.p;
    }

    // Exclusive scan of the counts of m keys into cell_start[0..m] (closing
    // entry included). At a step start it also resets the iteration controls.
    // ranged: only the tiles within the counted key range (plus the stencil
    // margin) are scanned; the other entries of cell_start keep stale values
    // that no stencil reads (complete_cell_start fills them for export)
    void scan(u32* cell_start, size_t m, bool step_start, u32* krange = nullptr) {
        // only the context's own cell_start is scanned by range: cs_range_
        // describes it (an adjoint replay's per-step copies are scanned whole,
        // and the key range they leave behind only widens the next one)
        if (cell_start != cell_start_.p) krange = nullptr;
        const u32 tiles = static_cast<u32>((m + SCAN_TILE - 1) / SCAN_TILE);
        launch(DFSPH_KERNEL_GRID_SCAN, scan_tile_sums, int(tiles), SCAN_BLOCK, count_.p, u32(m), tile_sums_.p,
               (const u32*)krange, margin_);
        launch(DFSPH_KERNEL_GRID_SCAN, scan_tile_offsets, 1, 1024, tile_sums_.p, tiles, cell_start + m,
               step_start ? ctl_.p : nullptr, step_start ? 3 : 0,
               step_start && scenes_ > 1 ? maxv_scene_.p : nullptr, step_start && scenes_ > 1 ? int(scenes_) : 0,
               krange, u32(m), margin_, krange ? cs_range_.p : nullptr);
        launch(DFSPH_KERNEL_GRID_SCAN, scan_tiles, int(tiles), SCAN_BLOCK, count_.p, u32(m), tile_sums_.p, cell_start,
               krange ? (const u32*)cs_range_.p : nullptr);
        if (cell_start == cell_start_.p) cs_ranged_ = krange != nullptr;
    }

    BoundaryDev bdev() const {
        BoundaryDev b;
        b.xb = xb_[0].p;
        b.bcs = bcs_.p;
        b.mask = bmask_.p;
        b.has = nb_ > 0 ? 1 : 0;
        return b;
    }

    void read_ctl() {
        DFSPH_CUDA(cudaMemcpyAsync(host_ctl_, ctl_.p, 3 * sizeof(IterCtl), cudaMemcpyDeviceToHost, stream_));
        DFSPH_CUDA(cudaStreamSynchronize(stream_));
    }

    static u32 iters_done(const IterCtl& c, u32 launched) {
        return c.stop_iter == ~0u ? launched : std::min(launched, c.stop_iter + 1);
    }

    // One Jacobi solve: `max_iters` iterations of (rate, apply). With eta > 0
    // the kernels stop themselves once the mean error is below eta rho0; the
    // host additionally stops launching after the device reports convergence.
    template <bool DIV>
    u32 solve(const StepDt<R>& sd, u32 max_iters, float eta, IterCtl* ctl, R* kap_out, R* adv_out, const u32* cs,
              const StepTape<R>* tp, FusedAdvect* fa = nullptr) {
        const int n = int(n_);
        const bool adaptive = eta > 0.0f;
        // eta rho0 in the working type (dfsph.cu:255: cfg_.eta_density * cfg_.rest_density in f32)
        const bool f32 = sizeof(R) == sizeof(float);
        const StopTest thr{double(n), f32 ? double(eta * cfg_.rest_density)
                                          : double(eta) * double(cfg_.rest_density), f32 ? 1 : 0};
        const u32 first_check = DIV ? 0u : 1u;  // density: from the 2nd iteration (dfsph.cu:255)
        if (!tp) {
            // small scenes: the whole solve in one cooperative launch (with
            // eta = 0 its stop decision never fires: max_iters iterations)
            if (solve_cooperative<DIV>(sd, max_iters, thr, first_check, ctl, kap_out, adv_out, cs)) return max_iters;
            if (adaptive && capturing_)
                return solve_on_device<DIV>(sd, max_iters, thr, first_check, ctl, kap_out, adv_out, cs);
        }
        const int w = DIV ? 0 : 1;
        u32 launched = 0;
        for (u32 it = 0; it < max_iters; ++it) {
            // a replayed segment keeps every iteration's (x, kf), kappa and
            // rate in its tape; positions do not change within the step
            V4* xin = xk_[cx_].p;
            V4* xout = tp ? tp->xkf[w] + it * tp->stride : xk_[cx_ ^ 1].p;
            R* kap_it = tp ? tp->kap[w] + it * tp->stride : kap_out;
            R* adv_it = tp ? tp->adv[w] + it * tp->stride : adv_out;
            V4* tv = tp ? tp->v[w] + it * tp->stride : nullptr;
            with_slot_order([&](auto order) {
                constexpr bool M = decltype(order)::value;
                if (adaptive)
                    launch_pass(DFSPH_KERNEL_PRESSURE_RATE, pressure_rate_kernel<R, DIV, true, false, 128, M>,
                                pressure_rate_kernel<R, DIV, true, false, 256, M>, n, xin, xout, vr_[cv_].p, alpha_.p,
                                adv_it, kap_it, cs, g_, phys_, bdev(), sd, red_partials(), ctl, it, first_check, thr, tv,
                                (const u32*)nullptr);
                else
                    launch_pass(DFSPH_KERNEL_PRESSURE_RATE, pressure_rate_kernel<R, DIV, false, false, 128, M>,
                                pressure_rate_kernel<R, DIV, false, false, 256, M>, n, xin, xout, vr_[cv_].p, alpha_.p,
                                adv_it, kap_it, cs, g_, phys_, bdev(), sd, red_partials(), ctl, it, first_check, thr, tv,
                                (const u32*)nullptr);
            });
            if (!tp) cx_ ^= 1;
            // the last iteration of a fixed-count solve may carry the
            // integrator, when the other position buffer is the one the step
            // must end in
            if (fa && !adaptive && it + 1 == max_iters && cx_ != fa->cx0) {
                with_slot_order([&](auto order) {
                    constexpr bool M = decltype(order)::value;
                    with_compensation(comp_, [&](auto comp) {
                        constexpr bool C = decltype(comp)::value;
                        if (fa->count)
                            launch_pass(DFSPH_KERNEL_PRESSURE_APPLY, apply_advect_kernel<R, true, 128, M, C>,
                                        apply_advect_kernel<R, true, 256, M, C>, n, (const V4*)xout, xk_[cx_ ^ 1].p,
                                        vr_[cv_].p, (const R*)kap_it, cs, g_, phys_, bdev(), sd, fa->d, key_.p,
                                        rank_.p, count_.p, ctl_.p, fa->mvs, comp_id(), comp_xc(), fluid_krange());
                        else
                            launch_pass(DFSPH_KERNEL_PRESSURE_APPLY, apply_advect_kernel<R, false, 128, M, C>,
                                        apply_advect_kernel<R, false, 256, M, C>, n, (const V4*)xout,
                                        xk_[cx_ ^ 1].p, vr_[cv_].p, (const R*)kap_it, cs, g_, phys_, bdev(), sd, fa->d,
                                        key_.p, rank_.p, count_.p, ctl_.p, fa->mvs, comp_id(), comp_xc(),
                                        fluid_krange());
                    });
                });
                cx_ ^= 1;
                fa->done = true;
                launched = it + 1;
                break;
            }
            with_slot_order([&](auto order) {
                constexpr bool M = decltype(order)::value;
                launch_pass(DFSPH_KERNEL_PRESSURE_APPLY, pressure_apply_kernel<R, false, 128, M>,
                            pressure_apply_kernel<R, false, 256, M>, n, xout, vr_[cv_].p, kap_it, cs, g_, phys_, bdev(),
                            sd, ctl, it, (const V4*)nullptr, (const u32*)nullptr);
            });
            launched = it + 1;
            if (adaptive && it + 1 > first_check) {  // it >= first_check
                // The reference reads the error back every iteration
                // (dfsph.cu:296-299); the device already decided, the host
                // only stops launching.
                DFSPH_CUDA(cudaMemcpyAsync(&host_ctl_[DIV ? 1 : 2], ctl, sizeof(IterCtl), cudaMemcpyDeviceToHost,
                                           stream_));
                DFSPH_CUDA(cudaStreamSynchronize(stream_));
                if (host_ctl_[DIV ? 1 : 2].stop_iter != ~0u) break;
            }
        }
        return launched;
    }

    // One step. Every step leaves the ping-pong buffers where it found them
    // (the sorted index is rebuilt in place, and the integrator writes the
    // other position buffer when the step flipped it an odd number of times),
    // so any captured sequence of steps replays with the same pointers.
    // With fdev the kernels read dt from the device frame control.
    // An adaptive solve inside a graph capture: a WHILE node whose body is one
    // iteration (rate, apply, iteration_control_kernel); the kernels take the
    // iteration number from the device and alternate the two position buffers
    // by its parity, so the body replays with fixed pointers. Both buffers hold
    // the step's positions afterwards (every rate pass copies them), so the
    // host-side parity does not depend on the iteration count.
    // An adaptive solve as one cooperative launch of jacobi_solve_kernel when
    // its blocks (at the rate pass's block size) fit one per SM; false when
    // they do not or when the passes are being timed one by one.
    // Like the graph-resident loop it leaves the step's positions in both
    // buffers and the iteration count in IterCtl::iters.
    // With probe = true the launch runs no iteration (it only builds its run
    // tables): verify_cooperative uses it to learn, outside any capture,
    // whether the device accepts the launch.
    template <bool DIV>
    bool solve_cooperative(const StepDt<R>& sd, u32 max_iters, const StopTest& thr, u32 first_check, IterCtl* ctl,
                           R* kap_out, R* adv_out, const u32* cs, bool probe = false) {
        if ((max_iters == 0 && !probe) || profile_mask_ != 0) return false;
        if (g_.rank) return false;  // its run tables hold the 9 column runs of the x-major order
        int& accepted = coop_ok_[DIV ? 1 : 0];
        // a capture records only launches that this device has accepted
        // eagerly: a refusal inside a capture would fail the capture or, on a
        // partitioned GPU, the graph's replays
        if (capturing_ && accepted != 1) return false;
        if (accepted < 0) return false;
        const int lb = bs_[DFSPH_KERNEL_PRESSURE_RATE];  // the per-pass reduction's block size
        if (lb != 128 && lb != 256) return false;
        const int n = int(n_);
        if (blocks_for(n, lb) > JACOBI_SOLVE_MAX_BLOCKS) return false;
        // neighbour records staged per block: 2 x stage_cap fluid records
        // (96 KB) and wall_cap wall records (32 KB)
        constexpr size_t kStageBytes = 128 * 1024;
        const u32 stage_cap = static_cast<u32>(96 * 1024 / (2 * sizeof(V4)));
        const u32 wall_cap = static_cast<u32>(32 * 1024 / sizeof(V4));
        // the smallest block (32, 64, 128 or 224 particles, four lanes each)
        // that needs at most one block per SM: the passes are latency-bound
        // at this size, so spreading the particles over more SMs shortens them
        static constexpr int kBlocks[4] = {32, 64, 128, 224};
        int pick = -1;
        for (int k = 0; k < 4 && pick < 0; ++k) {
            int& cap = coop_blocks_[DIV ? 1 : 0][k];
            if (cap < 0) {
                int per_sm = 0, sms = 0;
                auto probe = [&](auto kernel, int threads) {
                    DFSPH_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    int(kStageBytes)));
                    DFSPH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, kStageBytes));
                };
                // four lanes per particle and one more warp: the stop decision
                if (k == 0) probe(jacobi_solve_kernel<R, DIV, 32>, 4 * 32 + 32);
                else if (k == 1) probe(jacobi_solve_kernel<R, DIV, 64>, 4 * 64 + 32);
                else if (k == 2) probe(jacobi_solve_kernel<R, DIV, 128>, 4 * 128 + 32);
                else probe(jacobi_solve_kernel<R, DIV, 224>, 4 * 224 + 32);
                DFSPH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
                // at most one block per SM: beyond that the passes are long
                // enough to hide their launches, and the per-pass kernels
                // keep their neighbour gathers in L1
                cap = std::min(per_sm, 1) * sms;
            }
            if (blocks_for(n, kBlocks[k]) <= cap) pick = k;
        }
        if (pick < 0) return false;
        const int cb = kBlocks[pick];
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(unsigned(blocks_for(n, cb)));
        lc.blockDim = dim3(unsigned(4 * cb + 32));
        lc.dynamicSmemBytes = kStageBytes;
        lc.stream = stream_;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        V4* xa = xk_[cx_].p;
        V4* xb = xk_[cx_ ^ 1].p;
        auto go = [&](auto kernel) {
            return cudaLaunchKernelEx(&lc, kernel, n, xa, xb, vr_[cv_].p, (const R*)alpha_.p, adv_out, kap_out, cs,
                                      g_, phys_, bdev(), sd, red_partials(), ctl, max_iters, first_check, thr,
                                      stage_cap, wall_cap, u32(lb), WaitCfg{wait_limit_ns_, wait_missing_, dev_err_.p});
        };
        cudaError_t e;
        if (cb == 32) e = go(jacobi_solve_kernel<R, DIV, 32>);
        else if (cb == 64) e = go(jacobi_solve_kernel<R, DIV, 64>);
        else if (cb == 128) e = go(jacobi_solve_kernel<R, DIV, 128>);
        else e = go(jacobi_solve_kernel<R, DIV, 224>);
        if (e == cudaErrorCooperativeLaunchTooLarge && !capturing_) {
            // fewer SMs than the device reports (a partitioned GPU): the
            // per-pass solve from now on
            cudaGetLastError();
            for (int k = 0; k < 4; ++k) coop_blocks_[DIV ? 1 : 0][k] = 0;
            accepted = -1;
            return false;
        }
        DFSPH_CUDA(e);
        if (!capturing_) accepted = 1;
        coop_used_ = true;
        if (!probe) ++coop_launches_;
        if (capturing_) ++graph_kernels_;
        else ++launches_;
        return true;
    }

    template <bool DIV>
    u32 solve_on_device(const StepDt<R>& sd, u32 max_iters, const StopTest& thr, u32 first_check, IterCtl* ctl, R* kap_out,
                        R* adv_out, const u32* cs) {
        if (max_iters == 0) return 0;
        if (g_.rank)
            throw Error(DFSPH_ERR_STATE, "adaptive solves inside CUDA graphs (device-resident loops) need the x-major "
                                         "slot order");
        const int n = int(n_);
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        DFSPH_CUDA(cudaStreamGetCaptureInfo(stream_, &st, nullptr, &g, &deps, nullptr, &nd));
        if (st != cudaStreamCaptureStatusActive) throw Error(DFSPH_ERR_STATE, "device-resident solve outside a capture");
        cudaGraphConditionalHandle h = 0;
        DFSPH_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault));
        launch(DFSPH_KERNEL_OTHER, loop_arm_kernel, 1, 32, h);
        DFSPH_CUDA(cudaStreamGetCaptureInfo(stream_, &st, nullptr, &g, &deps, nullptr, &nd));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        DFSPH_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp));
        DFSPH_CUDA(cudaStreamUpdateCaptureDependencies(stream_, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        if (!loop_stream_) DFSPH_CUDA(cudaStreamCreateWithFlags(&loop_stream_, cudaStreamNonBlocking));
        const cudaStream_t outer = stream_;
        DFSPH_CUDA(cudaStreamBeginCaptureToGraph(loop_stream_, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal));
        stream_ = loop_stream_;
        try {
            V4* xa = xk_[cx_].p;
            V4* xb = xk_[cx_ ^ 1].p;
            const u32* dit = &ctl->iters;
            launch_pass(DFSPH_KERNEL_PRESSURE_RATE, pressure_rate_kernel<R, DIV, true, true, 128>, pressure_rate_kernel<R, DIV, true, true, 256>, n,
                   (const V4*)xa, xb, vr_[cv_].p, alpha_.p, adv_out, kap_out, cs, g_, phys_, bdev(), sd, red_partials(),
                   ctl, 0u, first_check, thr, (V4*)nullptr, dit);
            launch_pass(DFSPH_KERNEL_PRESSURE_APPLY, pressure_apply_kernel<R, true, 128>, pressure_apply_kernel<R, true, 256>, n, (const V4*)xb,
                   vr_[cv_].p, kap_out, cs, g_, phys_, bdev(), sd, (const IterCtl*)ctl, 0u, (const V4*)xa, dit);
            launch(DFSPH_KERNEL_OTHER, iteration_control_kernel, 1, 32, ctl, max_iters, h);
        } catch (...) {
            stream_ = outer;
            cudaGraph_t x = nullptr;
            cudaStreamEndCapture(loop_stream_, &x);
            throw;
        }
        stream_ = outer;
        cudaGraph_t body = nullptr;
        DFSPH_CUDA(cudaStreamEndCapture(loop_stream_, &body));
        return max_iters;  // at most; the device counts the iterations run
    }

    void step_once(R dt, bool count_next, const StepTape<R>* tp = nullptr, const FrameCtl* fdev = nullptr) {
        if (!have_state_) throw Error(DFSPH_ERR_STATE, "no fluid state: call dfsph_set_fluid first");
        const int n = int(n_);
        if (n == 0) return;  // dfsph.cu:121-122
        stepped_ = true;
        if (!capturing_) iters_on_device_ = false;
        u32* cs = tp ? tp->cs : cell_start_.p;
        const int cx0 = cx_;
        StepDt<R> sd;
        sd.dt = dt;
        sd.damping = R(cfg_.damping);  // the kernels derive e^{-damping dt} (damping_decay)
        sd.gx = R(cfg_.gravity[0]);
        sd.gy = R(cfg_.gravity[1]);
        sd.gz = R(cfg_.gravity[2]);
        sd.dev = fdev;
        const Tape1<R> t1{tp ? tp->x : nullptr, tp ? tp->g : nullptr, tp ? tp->id : nullptr};
        const NvtxRange step_range("dfsph step");
        // 1. grid build (CellGrid::build, core/src/cell_grid.cu:73-138)
        if (!counts_valid_)
            launch(DFSPH_KERNEL_GRID_COUNT, count_kernel<R>, blocks_for(n, 256), 256, n, xk_[cx_].p, g_, key_.p,
                   rank_.p, count_.p, fluid_krange());
        scan(cs, keys_, /*step start*/ true, fluid_krange());
        launch(DFSPH_KERNEL_GRID_SCATTER, scatter_kernel, blocks_for(n, 256), 256, n, key_.p, rank_.p, cs,
               id_[ci_].p, tmp_src_.p, tmp_id_.p);
        launch(DFSPH_KERNEL_GRID_REORDER, reorder_kernel<R>, blocks_for(n, 256), 256, n, tmp_src_.p, tmp_id_.p,
               key_.p, cs, cells1_, kSentinelCap, xk_[cx_].p, vr_[cv_].p, xk_[cx_ ^ 1].p, vr_[cv_ ^ 1].p,
               id_[ci_].p, key_sorted_.p, ctl_.p);
        cx_ ^= 1; cv_ ^= 1;
        counts_valid_ = false;
        // 2. density + alpha (dfsph.cu:137-186)
        const BoundaryDev bd = bdev();
        const bool kahan = cfg_.precision == DFSPH_PRECISION_FP32_KAHAN || comp_;
        const u32* idn = id_[ci_].p;
        with_slot_order([&](auto order) {
            constexpr bool M = decltype(order)::value;
            if (cfg_.record_diagnostics) {
                if (kahan)
                    launch_pass(DFSPH_KERNEL_DENSITY_ALPHA, density_alpha_kernel<R, true, true, 128, M>,
                                density_alpha_kernel<R, true, true, 256, M>, n, xk_[cx_].p, vr_[cv_].p, alpha_.p, cs,
                                g_, phys_, bd, nbr_f_.p, nbr_b_.p, nbr_sig_.p, idn, t1);
                else
                    launch_pass(DFSPH_KERNEL_DENSITY_ALPHA, density_alpha_kernel<R, false, true, 128, M>,
                                density_alpha_kernel<R, false, true, 256, M>, n, xk_[cx_].p, vr_[cv_].p, alpha_.p, cs,
                                g_, phys_, bd, nbr_f_.p, nbr_b_.p, nbr_sig_.p, idn, t1);
            } else {
                if (kahan)
                    launch_pass(DFSPH_KERNEL_DENSITY_ALPHA, density_alpha_kernel<R, true, false, 128, M>,
                                density_alpha_kernel<R, true, false, 256, M>, n, xk_[cx_].p, vr_[cv_].p, alpha_.p, cs,
                                g_, phys_, bd, (u32*)nullptr, (u32*)nullptr, (u32*)nullptr, idn, t1);
                else
                    launch_pass(DFSPH_KERNEL_DENSITY_ALPHA, density_alpha_kernel<R, false, false, 128, M>,
                                density_alpha_kernel<R, false, false, 256, M>, n, xk_[cx_].p, vr_[cv_].p, alpha_.p, cs,
                                g_, phys_, bd, (u32*)nullptr, (u32*)nullptr, (u32*)nullptr, idn, t1);
            }
        });
        // 3. divergence solve (the reference's plan; 0 iterations = the reference)
        last_divergence_launched_ = 0;
        if (cfg_.max_divergence_iters > 0)
            last_divergence_launched_ = solve<true>(sd, cfg_.max_divergence_iters, cfg_.eta_divergence, ctl_.p + 1,
                                                    kap_v_.p, rho_dot_.p, cs, tp);
        // 4. gravity + damping + XSPH (dfsph.cu:188-213)
        const bool xsph = explicit_eps_ ? any_xsph_ : cfg_.viscosity > 0.0f;
        with_slot_order([&](auto order) {
            constexpr bool M = decltype(order)::value;
            launch_pass(DFSPH_KERNEL_FORCES_XSPH, forces_xsph_kernel<R, 128, M>, forces_xsph_kernel<R, 256, M>, n,
                        xk_[cx_].p, vr_[cv_].p, vr_[cv_ ^ 1].p, cs, g_, phys_, sd, R(cfg_.viscosity),
                        scenes_ > 1 ? (const R*)eps_scene_.p : (const R*)nullptr, xsph ? 1 : 0,
                        tp ? tp->vx : nullptr);
        });
        cv_ ^= 1;
        // 5. density solve (dfsph.cu:215-260), its last iteration fused with
        // the integrator where possible
        const Domain<R> dom{R(cfg_.domain_min[0]), R(cfg_.domain_min[1]), R(cfg_.domain_min[2]),
                            R(cfg_.domain_max[0]), R(cfg_.domain_max[1]), R(cfg_.domain_max[2])};
        u32* mvs = scenes_ > 1 ? maxv_scene_.p : nullptr;
        FusedAdvect fa{dom, mvs, cx0, count_next, false};
        last_density_launched_ = solve<false>(sd, cfg_.max_density_iters, cfg_.eta_density, ctl_.p + 2, kap_.p,
                                              rho_adv_.p, cs, tp, (tp || !fuse_advect_) ? nullptr : &fa);
        if (fa.done) {
            counts_valid_ = count_next;
            return;
        }
        // 6. advect + max |v| (+ next step's cell counts)
        const V4* xin = xk_[cx_].p;
        V4* xout = cx_ != cx0 ? xk_[cx_ ^ 1].p : xk_[cx_].p;
        cx_ = cx0;
        // taped steps (the adjoint's replays) never compensate: the adjoint
        // refuses DFSPH_PRECISION_FP32_COMPENSATED contexts
        const bool comp = comp_ && !tp;
        with_slot_order([&](auto order) {
            constexpr bool M = decltype(order)::value;
            with_compensation(comp, [&](auto cflag) {
                constexpr bool C = decltype(cflag)::value;
                if (count_next)
                    launch(DFSPH_KERNEL_ADVECT, advect_kernel<R, true, M, C>, blocks_for(n, 256), 256, n, xin, xout,
                           vr_[cv_].p, sd, dom, g_, key_.p, rank_.p, count_.p, ctl_.p, mvs, tp ? tp->va : nullptr,
                           tp ? tp->amask : nullptr, comp ? comp_id() : nullptr, comp ? comp_xc() : nullptr,
                           fluid_krange());
                else
                    launch(DFSPH_KERNEL_ADVECT, advect_kernel<R, false, M, C>, blocks_for(n, 256), 256, n, xin, xout,
                           vr_[cv_].p, sd, dom, g_, key_.p, rank_.p, count_.p, ctl_.p, mvs, tp ? tp->va : nullptr,
                           tp ? tp->amask : nullptr, comp ? comp_id() : nullptr, comp ? comp_xc() : nullptr,
                           fluid_krange());
            });
        });
        if (count_next) counts_valid_ = true;
    }

    dfsph_config cfg_;
    int device_;
    int sm_count_ = 0;  // queried on first use
    bool store_run_ = false;  // the last state change was a dfsph_step_store call
    cudaStream_t stream_;
    GridGeom geom_;
    GridDev<R> g_;   // fluid grid (scene-aware)
    GridDev<R> gb_;  // wall grid
    Phys<R> phys_;
    float mass_f_ = 0;
    u32 cap_ = 0, bcap_ = 0, n_ = 0, nb_ = 0, n_tiles_ = 0;
    u32 scenes_ = 1, cells1_ = 0;
    size_t keys_ = 0;
    std::vector<u32> scene_counts_;
    bool explicit_eps_ = false, any_xsph_ = false;
    int cx_ = 0, cv_ = 0, ci_ = 0;
    bool counts_valid_ = false, have_state_ = false, stepped_ = false;
    u32 last_density_launched_ = 0, last_divergence_launched_ = 0;
    unsigned long long launches_ = 0;
    u32 profile_mask_ = 0;
    std::vector<Record> records_;
    std::vector<cudaEvent_t> free_events_;
    // CUDA graph of two steps
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    float graph_dt_ = 0.0f;
    unsigned long long graph_kernels_ = 0;
    bool capturing_ = false;
    cudaStream_t capture_stream_ = nullptr;

    DevBuf<V4> xk_[2], vr_[2], xb_[2], bscratch_[2];
    DevBuf<u32> id_[2], bid_[2];
    DevBuf<R> alpha_, rho_adv_, kap_, kap_v_, rho_dot_, eps_scene_;
    DevBuf<u32> key_, rank_, tmp_src_, tmp_id_, key_sorted_, nbr_f_, nbr_b_, nbr_sig_, maxv_scene_;
    DevBuf<unsigned short> slot_scene_;
    DevBuf<u32> bkey_, brank_, bkey_sorted_, btmp_src_, btmp_id_;
    DevBuf<u32> count_, cell_start_, tile_sums_, bcs_;
    DevBuf<unsigned char> bmask_;
    DevBuf<u32> morton_rank_;  // Morton slot order: sort key of every x-major cell
    DevBuf<double> partials_;
    DevBuf<IterCtl> ctl_;
    DevBuf<u32> dev_err_;  // device error word (DEV_ERR_*), sticky until check_device_status
    unsigned long long wait_limit_ns_ = 1000000000ull;  // bounded device waits: 1 s
    u32 wait_missing_ = 0;  // test hook: blocks the grid barrier waits for in vain
    bool coop_used_ = false;
    unsigned long long coop_launches_ = 0;  // cooperative solves launched or captured
    DevBuf<float> staging_;
    DevBuf<unsigned char> readback_;
    IterCtl* host_ctl_ = nullptr;
    // differentiable rollout: checkpoints (x, v per slot, original order),
    // per-step records of one segment, adjoint accumulators
    bool ad_valid_ = false;
    u32 ad_n_ = 0, ad_steps_ = 0, ad_every_ = 1;
    float ad_dt_ = 0.0f, ad_eps_ = 0.0f;
    DevBuf<V4> ck_;
    DevBuf<unsigned char> tape_, ad_staging_;
    SegmentGraph adj_replay_[2], adj_reverse_[2];
    u32 adj_len_ = 0, adj_n_ = 0;
    float adj_dt_ = 0.0f, adj_eps_ = 0.0f;
    int adj_cx_ = 0, adj_cv_ = 0, adj_ci_ = 0;
    cudaStream_t replay_stream_ = nullptr;  // replays overlap the reverse of the segment after them
    cudaEvent_t ev_start_ = nullptr, ev_replayed_[2] = {nullptr, nullptr}, ev_reversed_[2] = {nullptr, nullptr};
    DevBuf<V4> xg_, vg_, xbar_, vbar_[2], xr_, xq_, gq_;
    DevBuf<R> rhobar_, alphabar_;
    DevBuf<double> eps_part_, eps_acc_;
    DevBuf<u32> eps_ctr_;
    double* eps_host_ = nullptr;
    int graph_cx_ = 0, graph_cv_ = 0, graph_ci_ = 0;
    // device-stepped frames
    DevBuf<FrameCtl> fctl_;
    DevBuf<u32> frame_sub_;
    FrameCtl* host_fctl_ = nullptr;
    cudaGraph_t frame_graph_ = nullptr;
    cudaGraphExec_t frame_exec_ = nullptr;
    int fg_cx_ = 0, fg_cv_ = 0, fg_ci_ = 0;
    unsigned long long frame_body_kernels_ = 0;
    int last_frame_graph_ = 0;
    cudaStream_t loop_stream_ = nullptr;
    bool iters_on_device_ = false;
    // blocks of jacobi_solve_kernel one launch may hold, [DIV][32, 64, 128,
    // 224 particles] (-1: not probed yet)
    int coop_blocks_[2][4] = {{-1, -1, -1, -1}, {-1, -1, -1, -1}};
    // [DIV]: 1 once a cooperative solve launched outside a capture, -1 once
    // one was refused, 0 before either (captures need 1)
    int coop_ok_[2] = {0, 0};
    DevBuf<IterCtl> probe_ctl_;  // written by the no-iteration launches of verify_cooperative
    bool fuse_advect_ = true;  // last density iteration carries the integrator when it can
    // DFSPH_PRECISION_FP32_COMPENSATED: the integrator's per-particle carries
    // (original particle order), zero on every new fluid state
    const bool comp_ = cfg_.precision == DFSPH_PRECISION_FP32_COMPENSATED;
    // the key range of the particles counted for the next fluid grid build
    // (KRANGE_SLOTS lows, then highs), the cells its scan covered, and
    // whether cell_start holds stale entries outside them
    DevBuf<u32> krange_;
    DevBuf<u32> cs_range_;
    u32 margin_ = 0;
    bool cs_ranged_ = false;
    DevBuf<V4> xc_;
    DevBuf<V4> tune_xc_;
    DevBuf<V4> tune_ck_;
    DevBuf<IterCtl> tune_ctl_;
    // threads per block of each kernel class (the neighbour passes are tuned;
    // the defaults are the choice measured on the 1M-particle dam break)
    int bs_[DFSPH_KERNEL_CLASSES] = {256, 256, 256, 256, 256, 256, 128, 128, 256, 256, 256, 128};
};

}  // namespace dfsph
