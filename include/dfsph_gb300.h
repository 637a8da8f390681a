/*
 * dfsph_gb300.h — C ABI of the GB300-native DFSPH step.
 *
 * Plain C: pointers, sizes and status codes; no C++ or torch types cross this
 * boundary, nothing throws across it and nothing traps on the device. Every
 * entry point returns DFSPH_OK (0) or a DFSPH_ERR_* code; the message of the
 * last failure on a context is available from dfsph_last_error().
 *
 * Each declaration names the reference interface of Qervas/water_simulation
 * that it replaces (file:line within that project). The C++ façade in
 * include/water/ (ParticleStore, DFSPHSolver, CellGrid, load_scene,
 * sample_aabb_boundary) is written on top of these calls.
 *
 * Memory arguments carry a `mem` flag: DFSPH_MEM_HOST for host pointers
 * (pageable or pinned), DFSPH_MEM_DEVICE for device pointers of the context's
 * device. All device work runs on the context's stream.
 */
#ifndef DFSPH_GB300_H
#define DFSPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DFSPH_OK                    0
#define DFSPH_ERR_INVALID_ARGUMENT  1  /* bad pointer / size / enum          */
#define DFSPH_ERR_CUDA              2  /* a CUDA runtime call failed          */
#define DFSPH_ERR_OUT_OF_RANGE      3  /* count beyond capacity (std::out_of_range in the reference) */
#define DFSPH_ERR_STATE             4  /* call not valid in the current state */
#define DFSPH_ERR_DEVICE_TIMEOUT    5  /* a bounded device wait gave up       */
#define DFSPH_ERR_NONFINITE         6  /* NaN/Inf detected in the state       */
#define DFSPH_ERR_NO_DEVICE         7  /* no CUDA device / driver             */
#define DFSPH_ERR_IO                8  /* a state file could not be read or written */

#define DFSPH_MEM_HOST   0
#define DFSPH_MEM_DEVICE 1

/* arithmetic of the step */
#define DFSPH_PRECISION_FP32        0  /* plain FP32                                        */
#define DFSPH_PRECISION_FP32_KAHAN  1  /* FP32 state, compensated density sums               */
#define DFSPH_PRECISION_FP64        2  /* the same kernels instantiated in FP64 (GPU oracle) */
/* FP32 state with compensated density sums and compensated position updates
 * (no counterpart in the reference): the integrator keeps, per particle, what
 * rounding x + v dt to float dropped and adds it back at the next step
 * (Kahan summation over the steps), so position rounding no longer
 * accumulates. The carries restart at zero on every new fluid state
 * (dfsph_set_fluid*, dfsph_step_store, dfsph_load_state) and are not part of
 * the state file. The adjoint refuses such a context (DFSPH_ERR_STATE). */
#define DFSPH_PRECISION_FP32_COMPENSATED 3

/* ---- configuration ----------------------------------------------------- */
/* Mirrors water::solvers::DFSPHSolver::Config
 * (solvers/dfsph/include/water/solvers/dfsph.h:19-33) field for field, then
 * the GB300 extensions. dfsph_config_init() fills the reference defaults. */
typedef struct dfsph_config {
    float    rest_density;          /* 1000                                   */
    float    particle_radius;       /* 0.0015                                 */
    float    smoothing_length;      /* 0.003 (cell length = this)             */
    float    viscosity;             /* XSPH epsilon, 1e-3; <= 0 disables XSPH  */
    float    damping;               /* 0.5 1/s                                */
    float    surface_tension;       /* accepted, unused (as in the reference) */
    float    gravity[3];            /* (0, -9.81, 0)                          */
    uint32_t max_density_iters;     /* 100                                    */
    uint32_t max_divergence_iters;  /* 100 in the reference Config, where it is
                                       unused; set 0 for the reference's step */
    float    eta_density;           /* 1e-3; 0 => exactly max_density_iters    */
    float    eta_divergence;        /* 1e-3                                   */
    float    domain_min[3];         /* (0,0,0)                                */
    float    domain_max[3];         /* (1,1,1)                                */
    /* GB300 extensions */
    uint32_t precision;             /* DFSPH_PRECISION_*                      */
    uint32_t capacity;              /* max fluid particles (ParticleStore capacity) */
    uint32_t boundary_capacity;     /* max boundary particles                 */
    uint32_t record_diagnostics;    /* 1 => keep per-step neighbour counts     */
    uint32_t n_scenes;              /* independent scenes stepped together (0 or 1: one);
                                       they share geometry, wall particles and dt */
    uint32_t use_cuda_graph;        /* 1 => dfsph_step replays a captured CUDA graph of
                                       two steps (only with eta = 0, no profiling) */
    uint32_t slot_order;            /* DFSPH_ORDER_*: the order of the sorted particle slots */
} dfsph_config;

/* Slot orders (dfsph_config.slot_order). The reference sorts by the x-major cell
 * key (core/src/cell_grid.cu:10-30); SpatialAccel's Morton order
 * (core/src/spatial_accel.cu:11-40) is kept as a variant for comparison: cells
 * ranked by the Morton code of their (x, y, z) cell coordinates. Both orders
 * give every particle the same candidates in the same sequence (the stencil is
 * walked cell by cell in x-major order either way), so with fixed iteration
 * counts the two steps give the same fields bit for bit; only the memory
 * layout, and with it the cache behaviour, differs. In Morton order the grid
 * fields (cell keys, cell_start, sorted indices) are indexed by Morton rank
 * and small scenes keep the per-pass Jacobi solve. */
#define DFSPH_ORDER_CELL_KEY 0
#define DFSPH_ORDER_MORTON   1

typedef struct dfsph_ctx dfsph_ctx;

/* Fields readable with dfsph_get_field(), always in the caller's ORIGINAL
 * particle order (the order of dfsph_set_fluid), except the grid arrays. */
#define DFSPH_FIELD_POSITION          0  /* float[3*n]  ParticleStore::positions()              */
#define DFSPH_FIELD_VELOCITY          1  /* float[3*n]  ParticleStore::velocities()             */
#define DFSPH_FIELD_DENSITY           2  /* float[n]    "dfsph_density"     (dfsph.cu:80)         */
#define DFSPH_FIELD_ALPHA             3  /* float[n]    "dfsph_alpha"       (dfsph.cu:81)         */
#define DFSPH_FIELD_KAPPA             4  /* float[n]    "dfsph_kappa"       (dfsph.cu:82)         */
#define DFSPH_FIELD_DENSITY_ADV       5  /* float[n]    "dfsph_density_adv" (dfsph.cu:83)         */
#define DFSPH_FIELD_CELL_KEY          6  /* uint32[n]   cell key of each particle at the last grid build */
#define DFSPH_FIELD_SORTED_INDEX      7  /* uint32[n]   CellGrid::sorted_indices()                */
#define DFSPH_FIELD_CELL_START        8  /* uint32[C+1] CellGrid::cell_start()                    */
#define DFSPH_FIELD_NBR_FLUID         9  /* uint32[n]   fluid candidates visited by the 27-cell stencil (needs record_diagnostics) */
#define DFSPH_FIELD_NBR_BOUNDARY     10  /* uint32[n]   boundary candidates visited                */
#define DFSPH_FIELD_BOUNDARY_MASS    11  /* float[nb]   "dfsph_boundary_mass" (dfsph.cu:91-92), boundary input order */
#define DFSPH_FIELD_KAPPA_V          12  /* float[n]    divergence-solver kappa                    */
#define DFSPH_FIELD_BOUNDARY_CELL_START   13  /* uint32[C+1] boundary CellGrid::cell_start()      */
#define DFSPH_FIELD_BOUNDARY_SORTED_INDEX 14  /* uint32[nb] boundary CellGrid::sorted_indices()   */
#define DFSPH_FIELD_NBR_SIGNATURE    15  /* uint32[n]   signature of the candidate set visited at the last
                                            density pass: sum of mixed ids (needs record_diagnostics);
                                            equal sets give equal signatures, so comparing two runs
                                            finds the particles whose stencil membership differs */

/* Scalars readable with dfsph_get_scalar(). */
#define DFSPH_SCALAR_MAX_VELOCITY          0  /* DFSPHSolver::max_velocity() (dfsph.h:40) */
#define DFSPH_SCALAR_PARTICLE_MASS         1  /* DFSPHSolver::particle_mass() (dfsph.h:44) */
#define DFSPH_SCALAR_LAST_DENSITY_ITERS    2  /* DFSPHSolver::last_density_iters() (dfsph.h:50) */
#define DFSPH_SCALAR_LAST_DIVERGENCE_ITERS 3
#define DFSPH_SCALAR_DENSITY_ERROR         4  /* last mean max(0, rho*-rho0), FP64 sum */
#define DFSPH_SCALAR_DIVERGENCE_ERROR      5  /* last mean max(0, rho_dot),  FP64 sum */
#define DFSPH_SCALAR_TOTAL_CELLS           6  /* CellGrid::total_cells() (cell_grid.h:28-33) */
#define DFSPH_SCALAR_STENCIL_INV_CELL      7  /* device reciprocal that centres the stencil */
#define DFSPH_SCALAR_FLUID_COUNT           8
#define DFSPH_SCALAR_BOUNDARY_COUNT        9
#define DFSPH_SCALAR_KERNEL_LAUNCHES      10  /* kernels launched by this context so far */
#define DFSPH_SCALAR_FLAGS                11  /* bit0: a convergence sum was NaN; bit1: more than
                                                 4096 out-of-grid particles, kept in arrival order */

#define DFSPH_SCALAR_ACTIVE_BOUNDARY      12  /* boundary particles with a fluid particle within
                                                 2h of them (counted on demand, last grid) */
#define DFSPH_SCALAR_FRAME_GRAPH          13  /* 1: the last dfsph_step_frames ran as device-stepped
                                                 graphs; 0: as the host loop */
#define DFSPH_SCALAR_COOP_SOLVES          15  /* Jacobi solves this context ran as one cooperative launch
                                                 (a small scene's solve; counted at launch, or once at
                                                 capture for a graph) */
#define DFSPH_SCALAR_BOUNDS_VIOLATIONS    14  /* neighbour runs outside their cell_start range seen
                                                 by the bounds-checked build (-DDFSPH_BOUNDS_CHECK),
                                                 all contexts of the library; -1 in the normal build */

/* Kernel classes for dfsph_profile_* (bit k of the mask selects class k). */
#define DFSPH_KERNEL_GRID_COUNT       0   /* cell keys + per-cell counts          */
#define DFSPH_KERNEL_GRID_SCAN        1   /* cell_start scan (3 launches)          */
#define DFSPH_KERNEL_GRID_SCATTER     2   /* provisional slots                    */
#define DFSPH_KERNEL_GRID_REORDER     3   /* canonical order + state gather       */
#define DFSPH_KERNEL_DENSITY_ALPHA    4   /* density + alpha                      */
#define DFSPH_KERNEL_PRESSURE_RATE    5   /* Jacobi first half (rho*, kappa)       */
#define DFSPH_KERNEL_PRESSURE_APPLY   6   /* Jacobi second half (dv)               */
#define DFSPH_KERNEL_FORCES_XSPH      7   /* gravity + damping + XSPH              */
#define DFSPH_KERNEL_ADVECT           8   /* integrator + max |v| (+ next counts)  */
#define DFSPH_KERNEL_IO               9   /* import / export / readback           */
#define DFSPH_KERNEL_OTHER           10
#define DFSPH_KERNEL_ADJOINT         11   /* reverse-mode kernels of dfsph_adjoint_backward */
#define DFSPH_KERNEL_CLASSES         12

/* Reference defaults of DFSPHSolver::Config (dfsph.h:19-33). */
int dfsph_config_init(dfsph_config* cfg);

/* Replaces the DFSPHSolver constructor (solvers/dfsph/src/dfsph.cu:71-100)
 * minus the caller-owned stores: grid geometry of make_grid (dfsph.cu:55-65),
 * particle mass rho0*(2r)^3 (dfsph.cu:76-78) and every device buffer, sized for
 * cfg->capacity fluid and cfg->boundary_capacity boundary particles.
 * `stream` is a cudaStream_t (NULL = the legacy default stream). */
int dfsph_create(const dfsph_config* cfg, int device, void* stream, dfsph_ctx** out);
void dfsph_destroy(dfsph_ctx* ctx);
int dfsph_set_stream(dfsph_ctx* ctx, void* stream);

/* Boundary particles: the boundary ParticleStore's positions, the boundary grid
 * built once and the Akinci mass m_b = rho0 / max(sum W, 1e-9)
 * (dfsph.cu:90-99,102-116; dfsph_kernels.cu:40-65). n = 0 removes the boundary. */
int dfsph_set_boundary(dfsph_ctx* ctx, const float* xyz, uint32_t n, int mem);

/* Fluid state: ParticleStore::resize + the position/velocity uploads of
 * sim_cli (apps/sim_cli/main.cpp:180-184). `vel` may be NULL (zero velocity,
 * as a freshly registered attribute). n > capacity => DFSPH_ERR_OUT_OF_RANGE
 * (ParticleStore::resize, core/src/particle_store.cu:11-17). With mem =
 * DFSPH_MEM_HOST, page-locked 16-byte-aligned arrays are read in place by a
 * kernel, other host memory through a staging copy; either way the arrays may
 * be freed when the call returns. */
int dfsph_set_fluid(dfsph_ctx* ctx, const float* xyz, const float* vel, uint32_t n, int mem);

/* Scene batching (no counterpart in the reference: it steps one scene per
 * solver). For a context created with n_scenes = S > 1: counts[S] particles per
 * scene, xyz/vel concatenated scene after scene (sum(counts) <= capacity).
 * Every scene keeps its own cell keys (scene s owns keys [s(C+1), (s+1)(C+1))),
 * so scenes never interact; one launch per kernel steps all of them.
 * Fields read with dfsph_get_field come back concatenated the same way. */
int dfsph_set_fluid_batch(dfsph_ctx* ctx, uint32_t n_scenes, const uint32_t* counts, const float* xyz,
                          const float* vel, int mem);
/* Per-scene XSPH coefficient (host array of n_scenes). */
int dfsph_set_scene_viscosity(dfsph_ctx* ctx, const float* viscosity, uint32_t n_scenes);
/* Per-scene max |v| after the last step (host array of n_scenes). */
int dfsph_get_scene_max_velocity(dfsph_ctx* ctx, float* out, uint32_t n_scenes);

/* DFSPHSolver::step(dt) (dfsph.cu:120-133), n_steps times, on the state held
 * by the context. Asynchronous unless a convergence check needs the host
 * (eta > 0); results stay on the device. */
int dfsph_step(dfsph_ctx* ctx, float dt, uint32_t n_steps);

/* One DFSPHSolver::step(dt) on caller-owned ParticleStore buffers: AoS float3
 * device arrays in the caller's order, read at entry and written back at exit
 * together with the four solver attributes (any attribute pointer may be NULL).
 * This is the entry the C++ façade's DFSPHSolver::step uses. */
int dfsph_step_store(dfsph_ctx* ctx, float* pos, float* vel, uint32_t n, float dt,
                     float* density, float* alpha, float* kappa, float* density_adv);

/* ---- CFL frames (no counterpart in the reference's library: sim_cli's loop,
 * apps/sim_cli/main.cpp:171-181, with TimeStepper::next_dt,
 * core/include/water/core/timestep.h:23-28) ------------------------------- */
typedef struct dfsph_frame_config {
    float    frame_dt;                /* length of one frame: sim_cli's 1 / scene fps      */
    float    stepper_frame_dt;        /* TimeStepper::Config::frame_dt (1/24 s); the dt
                                         floor is stepper_frame_dt / max_substeps        */
    float    dt_max;                  /* TimeStepper::Config::dt_max (1/24 s)              */
    float    cfl_lambda;              /* TimeStepper::Config::cfl_lambda (0.4)             */
    uint32_t max_substeps;            /* TimeStepper::Config::max_substeps (16)            */
    float    min_velocity;            /* sim_cli's floor on max |v| before next_dt (0.5)   */
    uint32_t max_substeps_per_frame;  /* sim_cli's substep cap per frame (64)              */
} dfsph_frame_config;

/* sim_cli's values (above; frame_dt = 1/24 s). */
int dfsph_frame_config_init(dfsph_frame_config* fc);

/* n_frames frames: per frame, substeps of dt = next_dt(max(max|v|, min_velocity),
 * particle_radius, remaining) until remaining <= 1e-6 or the cap, exactly
 * sim_cli's loop. With use_cuda_graph = 1 and fixed iteration counts each frame
 * is one graph launch whose substep size is chosen on the device after every
 * substep (no host synchronisation inside a frame); otherwise the host runs
 * the loop. substeps (host, n_frames entries, may be NULL) receives the
 * substep count of each frame. Returns after the last frame. */
int dfsph_step_frames(dfsph_ctx* ctx, const dfsph_frame_config* fc, uint32_t n_frames, uint32_t* substeps);

/* Field readback (density_at/alpha_at/boundary_mass_at, dfsph.cu:330-353, as
 * whole arrays). dst_bytes is checked against the field's size. Float particle
 * fields bound for page-locked 16-byte-aligned host memory are written there
 * in place by a kernel; other host memory receives a copy. Returns when the
 * data is in dst. */
int dfsph_get_field(dfsph_ctx* ctx, int field, void* dst, size_t dst_bytes, int mem);
/* Positions and velocities (float[3n] each, original order; either pointer may
 * be NULL) in one call: the host copies of the ParticleStore arrays that the
 * reference's sim_cli makes after a frame (apps/sim_cli/main.cpp:186-189,
 * positions there). No counterpart in the reference's API. Bound for
 * page-locked 16-byte-aligned host memory, both are written in place by one
 * kernel with one synchronisation; otherwise as two dfsph_get_field calls.
 * Returns when the data is in pos and vel. */
int dfsph_get_state(dfsph_ctx* ctx, float* pos, float* vel, int mem);
int dfsph_get_scalar(dfsph_ctx* ctx, int which, double* out);

/* Per-kernel device timing with CUDA events on the context's stream (no
 * counterpart in the reference, which has no instrumentation). Launches of the
 * classes in `mask` are bracketed by events until the mask is cleared;
 * dfsph_profile_read() synchronises, sums the recorded durations of one class
 * and forgets them. */
int dfsph_profile_enable(dfsph_ctx* ctx, uint32_t mask);
int dfsph_profile_read(dfsph_ctx* ctx, int kernel_class, double* total_ms, uint64_t* launches);

/* ---- differentiable rollout (no counterpart in the reference) -------------
 * Reverse-mode derivative of dfsph_step through every stage: density + alpha,
 * both Jacobi solvers with their fixed iteration counts, wall terms, XSPH and
 * the integrator (max(.,0) and clamps use the forward pass's active sets).
 * Needs one scene and fixed iteration counts (eta_density = 0, and
 * eta_divergence = 0 when max_divergence_iters > 0), else DFSPH_ERR_STATE.
 * Arrays hold the working type T: float for DFSPH_PRECISION_FP32 and
 * FP32_KAHAN, double for DFSPH_PRECISION_FP64; positions and velocities are
 * T[3n] in the caller's original particle order. */
/* Fluid state in the working type (dfsph_set_fluid without the float rounding
 * of an FP64 context). vel may be NULL (zero). */
int dfsph_adjoint_set_state(dfsph_ctx* ctx, const void* pos, const void* vel, uint32_t n, int mem);
/* Current state in the working type. Either pointer may be NULL. */
int dfsph_adjoint_get_state(dfsph_ctx* ctx, void* pos, void* vel, int mem);
/* n_steps steps of dfsph_step from the current state, keeping a checkpoint of
 * (x, v) in device memory every checkpoint_every steps (and the final state).
 * The context then holds x_T, v_T. The XSPH coefficient in use is recorded. */
int dfsph_adjoint_forward(dfsph_ctx* ctx, float dt, uint32_t n_steps, uint32_t checkpoint_every);
/* Given dL/dx_T and dL/dv_T (vel_bar may be NULL = 0), writes dL/dx_0,
 * dL/dv_0 (either output may be NULL) and *xsph_bar = dL/d(XSPH coefficient)
 * accumulated in FP64 (may be NULL). Each segment between checkpoints is
 * replayed once with its per-step records (neighbour structure included),
 * then differentiated step by step in reverse; the replay of the next segment
 * runs beside the reverse of the current one, so the records of two segments
 * are held at once (about 2 x checkpoint_every x 300 bytes per particle in
 * FP32). Stream-ordered on the context's stream (plus a side stream of its
 * own). The context is left at the rollout's final state. */
int dfsph_adjoint_backward(dfsph_ctx* ctx, const void* pos_bar, const void* vel_bar, void* pos0_bar,
                           void* vel0_bar, double* xsph_bar, int mem);

/* State file (no counterpart in the reference, whose frame files hold positions
 * only and cannot be resumed from): a header ("DFSPHST1", version, bytes per
 * real, scene count, fluid and wall counts, the last max |v|), the per-scene fluid counts,
 * positions and velocities in the working type (original particle order) and
 * the wall positions as float (input order), then, from a
 * DFSPH_PRECISION_FP32_COMPENSATED context, its per-particle position carries
 * (3 floats each, original order; header flag bit 0). dfsph_load_state
 * replaces the walls and the fluid of a context with the same scene count
 * (reals of the other width are converted; a context of another precision
 * skips the carries); the next step continues the saved run exactly. */
int dfsph_save_state(dfsph_ctx* ctx, const char* path);
int dfsph_load_state(dfsph_ctx* ctx, const char* path);

/* Launch-shape tuning (no counterpart in the reference). Times the four
 * neighbour passes (density + alpha, both Jacobi halves, XSPH) at 64, 128 and
 * 256 threads per block on `steps` steps of the context's own state, each
 * candidate from the same snapshot, keeps the fastest per pass and restores
 * the state. block_sizes (may be NULL) receives the threads per block of every
 * kernel class (DFSPH_KERNEL_CLASSES entries). */
int dfsph_autotune(dfsph_ctx* ctx, float dt, uint32_t steps, int32_t* block_sizes);
int dfsph_get_block_sizes(dfsph_ctx* ctx, int32_t* block_sizes);

/* Wait for the context's stream; returns a pending device error if any,
 * DFSPH_ERR_DEVICE_TIMEOUT when a bounded device wait gave up (below). */
int dfsph_synchronize(dfsph_ctx* ctx);

/* Bounded device waits. Replaces the host synchronisation of the reference's
 * density solve, which reads the error back after every iteration
 * (solvers/dfsph/src/dfsph.cu:296-299): a small scene's Jacobi solve runs as
 * one cooperative launch whose blocks meet at a grid barrier twice per
 * iteration. Every such wait gives up after limit_ns nanoseconds (default
 * 1e9), sets the context's device error word and returns; the next
 * dfsph_synchronize, dfsph_get_field or dfsph_step_frames returns
 * DFSPH_ERR_DEVICE_TIMEOUT and clears the word. The state of the step that
 * timed out is not valid; set it again (dfsph_set_fluid, dfsph_load_state) to
 * continue. No trap, fault or endless wait is left on the device. */
int dfsph_set_wait_limit(dfsph_ctx* ctx, uint64_t limit_ns);
/* Test hook (no use outside tests): the grid barrier also waits for
 * missing_blocks blocks that do not exist, so every wait runs out after the
 * limit and the timeout path runs without a GPU fault. 0 restores the normal
 * barrier. */
int dfsph_test_stall_waits(dfsph_ctx* ctx, uint32_t missing_blocks);

const char* dfsph_last_error(const dfsph_ctx* ctx);
const char* dfsph_status_string(int status);

/* ---- stand-alone pieces -------------------------------------------------- */

/* water::solvers::sample_aabb_boundary (solvers/dfsph/src/boundary_sampler.cpp:6-32;
 * declaration solvers/dfsph/include/water/solvers/boundary_sampler.h:24-25).
 * Writes min(count, cap) points to out (xyz, host) and returns count (>= 0). */
int64_t dfsph_sample_aabb_boundary(const float lo[3], const float hi[3], float spacing,
                                   int n_layers, float* out, int64_t cap);

/* make_grid geometry (dfsph.cu:55-65). */
int dfsph_grid_geometry(const dfsph_config* cfg, float origin[3], int dims[3]);

/* CellGrid::build (core/src/cell_grid.cu:73-138) on device arrays: keys
 * (sorted, as CellGrid leaves cell_ids_), sorted_indices[n] and
 * cell_start[dims.x*dims.y*dims.z + 1]; sorted_keys_dev and sorted_indices_dev
 * may be NULL. Temporaries are stream-ordered allocations on `stream`; the call
 * returns after the work is enqueued there. n = 0 leaves cell_start untouched,
 * as CellGrid::build does for count == 0 (cell_grid.cu:74-77). */
int dfsph_build_cell_grid(const float* xyz_dev, uint32_t n, const float origin[3],
                          const int dims[3], float cell_length, uint32_t* sorted_keys_dev,
                          uint32_t* sorted_indices_dev, uint32_t* cell_start_dev,
                          void* stream);


/* SpatialAccel's Morton order (core/src/spatial_accel.cu:11-40,110-179): 30-bit
 * Morton codes of positions normalised to [scene_min, scene_max] (10 bits per
 * axis, x highest), stably sorted; writes the sorted codes and the permutation
 * (device arrays, either may be NULL). The sort key variant kept for comparison
 * with the cell-key order. Temporaries are stream-ordered on `stream`. */
int dfsph_morton_sort(const float* xyz_dev, uint32_t n, const float scene_min[3],
                      const float scene_max[3], uint32_t* sorted_codes_dev,
                      uint32_t* sorted_indices_dev, void* stream);

/* SpatialAccel::build (core/src/spatial_accel.cu:110-179; the class in
 * core/include/water/core/spatial_accel.h:19-54): Morton order as
 * dfsph_morton_sort, internal nodes by Karras' construction with equal codes
 * ordered by sorted slot, leaf boxes position +- leaf_radius, plus the
 * bottom-up internal-box pass the reference leaves for later. Node ids as in
 * the reference: internal 0..n-2 (root 0), leaf of sorted slot k = n-1+k.
 * Device arrays: codes[n], sorted_indices[n], left[n-1], right[n-1],
 * parent[2n-1] (root: 0xFFFFFFFF), boxes[6(2n-1)] (min xyz, max xyz per node),
 * scratch[n-1]. n < 2^30. Stream-ordered on `stream`. */
int dfsph_lbvh_build(const float* xyz_dev, uint32_t n, const float scene_min[3], const float scene_max[3],
                     float leaf_radius, uint32_t* codes_dev, uint32_t* sorted_indices_dev, uint32_t* left_dev,
                     uint32_t* right_dev, uint32_t* parent_dev, float* boxes_dev, uint32_t* scratch_dev,
                     void* stream);
/* Refit after the particles moved: leaf boxes from xyz_dev (original order),
 * internal boxes bottom-up on the topology of the last build. */
int dfsph_lbvh_refit(const float* xyz_dev, uint32_t n, float leaf_radius, const uint32_t* sorted_indices_dev,
                     const uint32_t* left_dev, const uint32_t* right_dev, const uint32_t* parent_dev,
                     float* boxes_dev, uint32_t* scratch_dev, void* stream);

/* The Akinci 2013 cohesion kernel C(r, l) of core/include/water/core/sph_kernels.cuh
 * :43-51 (declared there, called by nothing), evaluated for n distances
 * (device arrays). */
int dfsph_cohesion_kernel(const float* r_dev, uint32_t n, float support, float* out_dev, void* stream);

/* No counterpart in the reference. The same cell-grid build as
 * dfsph_build_cell_grid for callers that cannot allocate device memory (a
 * host callback or graph node that must not enter the allocator, a plugin
 * whose host owns every allocation, a fixed memory budget): it uses a scratch
 * area compiled into the library (DFSPH_STATIC_GRID_SCRATCH_BYTES of device
 * memory that every GPU loading the library keeps until exit) and calls no
 * allocator. Limits: n <= DFSPH_STATIC_GRID_MAX_PARTICLES and
 * dims.x*dims.y*dims.z <= DFSPH_STATIC_GRID_MAX_CELLS, else
 * DFSPH_ERR_OUT_OF_RANGE. All calls share the scratch: calls that overlap on
 * the GPU race. The first call on a device looks the scratch address up (a
 * runtime query); make it before any stream capture. The address is kept for
 * the life of the process: after cudaDeviceReset on that device (which
 * unloads the library's device memory) this entry point must not be called
 * again. As in dfsph_build_cell_grid, ordering the particles of one cell takes
 * time proportional to the square of that cell's occupancy (out-of-grid
 * particles all share one key), so inputs that pile many particles into one
 * cell make a slow call. */
#define DFSPH_STATIC_GRID_MAX_PARTICLES 131072u
#define DFSPH_STATIC_GRID_MAX_CELLS     1048576u
#define DFSPH_STATIC_GRID_SCRATCH_BYTES (7u * 1024u * 1024u)
int dfsph_build_cell_grid_static(const float* xyz_dev, uint32_t n, const float origin[3],
                                 const int dims[3], float cell_length, uint32_t* sorted_keys_dev,
                                 uint32_t* sorted_indices_dev, uint32_t* cell_start_dev,
                                 void* stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* DFSPH_GB300_H */
