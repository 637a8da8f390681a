// Device kernels of the GB300 DFSPH step.
//
// Layout in HBM (all arrays in cell-sorted order, rebuilt every step):
//   xk[s] = (x, y, z, kfac)   kfac = kappa / max(rho^2, 1e-9) of the running
//                             Jacobi iteration (ping-pong between two buffers)
//   vr[s] = (vx, vy, vz, rho)
//   alpha[s], rho_adv[s], kap[s], kap_v[s], id[s] (original particle index)
//   cell_start[C+1] exactly as the reference's CellGrid::cell_start()
//   boundary: xb[s] = (x, y, z, m_b), bcs[C+1], bmask[C]
// One thread owns one particle; every neighbour pass visits the reference's
// 27-cell stencil as 9 contiguous runs of sorted slots, so neighbour loads walk
// consecutive 16-byte records that the warp's other particles share in L1.
#pragma once

#include "common.cuh"

namespace dfsph {

template <class R> struct Phys {
    R l;          // smoothing length (= cell length)
    R inv_l;
    R support2;   // (2l)^2: the spline is zero beyond it
    R sigma;      // 1 / (pi l^3)
    R grad_c;     // sigma / l
    R mass;       // fluid particle mass rho0 (2r)^3
    R rho0;
    R two_l;      // 2l
    R wA2, wA3;   // W = sigma + r^2 (wA2 + wA3 r) for r < l
    R wB;         // W = wB (2l - r)^3 for l <= r < 2l
    R gA, gB;     // F = gA r + gB for r < l
    R gC;         // F = gC (2l - r)^2 / r for l <= r < 2l
};

// The approximate reciprocal square root instruction with subnormal inputs
// and outputs flushed to zero (PTX rsqrt.approx.ftz.f32). Every caller clamps
// its argument at 1e-24, and for any float from 1e-24 up neither the argument
// nor its reciprocal square root (1e12 down to 5e-20) is subnormal, so the
// flush never applies. The results are those of rsqrtf (positions and
// velocities bit-identical after 40 steps of the 1M-particle dam break),
// without rsqrtf's handling of subnormal arguments: 3 instructions fewer per
// pair term, 2.6 M fewer warp instructions per neighbour pass at 1M particles.
__device__ __forceinline__ float rsqrt_r(float v) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ double rsqrt_r(double v) { return rsqrt(v); }

template <class R> __device__ __forceinline__ R4<R> ld(const R4<R>* p) { return *p; }
template <> __device__ __forceinline__ R4<float> ld(const R4<float>* p) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    return {v.x, v.y, v.z, v.w};
}
// A record that other threads of the same launch write between grid barriers
// (a persistent solve): a coherent cached load (ld.global.ca), never the
// read-only path, which the compiler may pick for a plain load through a
// const __restrict__ pointer. The barrier's device-scope release/acquire
// pair (then __syncthreads) orders it after the writes of the previous phase.
template <class R> __device__ __forceinline__ R4<R> ld_coh(const R4<R>* p);
template <> __device__ __forceinline__ R4<float> ld_coh(const R4<float>* p) {
    const float4 v = __ldca(reinterpret_cast<const float4*>(p));
    return {v.x, v.y, v.z, v.w};
}
template <> __device__ __forceinline__ R4<double> ld_coh(const R4<double>* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldca(q), b = __ldca(q + 1);
    return {a.x, a.y, b.x, b.y};
}

// Where a persistent solve (jacobi_solve_kernel) finds a particle's
// neighbours: copies of its block's neighbour records in shared memory (slots
// lo ..; x null means the records are read from global memory), and the
// particle's stencil runs, computed once per launch.
template <class R> struct NbrSrc {
    const R4<R>* x = nullptr;
    const R4<R>* v = nullptr;
    u32 lo = 0;
    // run k of the particle is [rb[k * stride], re[k * stride]); runs past
    // its last one are empty
    const u32* rb = nullptr;
    const u32* re = nullptr;
    int stride = 0;
    // the same for the wall runs (wrb/wre) and, when staged, the wall records
    // of slots wlo .. (wx)
    const u32* wrb = nullptr;
    const u32* wre = nullptr;
    const R4<R>* wx = nullptr;
    u32 wlo = 0;
};

// ---------------------------------------------------------------------------
// Pair terms. With r = |x_i - x_j| the cubic spline and its gradient factor
// F(r) = (sigma/l) w'(r/l) / r (so that gradW = F(r) r_ij) are, per branch,
//   r <  l :  W = sigma + r^2 (wA2 + wA3 r)      F = gA r + gB
//   r >= l :  W = wB (2l - r)^3                  F = gC (2l - r)^2 / r
// with (2l - r) clamped at 0, so both vanish beyond the support without a
// branch. r comes from rsqrt(max(r2, 1e-24)): a particle paired with itself
// (or a coincident one) has r_ij = 0, so every gradient term it adds is exactly
// zero, which is how the reference's explicit self-skips and its r < 1e-12
// guard (sph_kernels.cuh:29) come out here.
// ---------------------------------------------------------------------------
// Minimum resident blocks for __launch_bounds__ of the FP32 density + alpha
// pass and the fused last apply + integrator: six 256-thread (twelve
// 128-thread) blocks per SM, which holds them at 40 registers (48 otherwise;
// measured on the 1M dam break: density + alpha -1.3 us, the fused pass
// -3 us, step -0.5 %). The XSPH pass spills at 40 registers and runs slower
// there; the FP64 build and the diagnostic density pass (neighbour counts and
// candidate-set signatures) are left unbounded.
template <class R> constexpr int fp32_min_blocks(int lb) { return sizeof(R) == sizeof(float) ? 1536 / lb : 1; }

template <class R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }

// a / b for b in [1e-9, 1e30]: a fast approximate quotient where the working
// type is float, the IEEE divide where it is double.
// In FP32: a times the approximate reciprocal of b (PTX rcp.approx.ftz.f32).
// The one caller passes b >= 1e-9, so the reciprocal is never taken of a
// subnormal; the product is an ordinary multiply, exact for subnormal a.
// Same results as __fdividef on the 1M-particle dam break (positions and
// velocities hashed after 55 steps), 2.6 M fewer warp instructions in the
// XSPH pass.
__device__ __forceinline__ float fast_div(float a, float b) {
    float rb;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(b));
    return a * rb;
}
__device__ __forceinline__ double fast_div(double a, double b) { return a / b; }

template <class R> __device__ __forceinline__ R pair_r(R r2, R& rinv) {
    rinv = rsqrt_r(rmax(r2, R(1e-24)));
    return r2 * rinv;
}
template <class R> __device__ __forceinline__ R grad_factor(R r, R rinv, const Phys<R>& p) {
    const R t = rmax(p.two_l - r, R(0));
    const R outer = p.gC * t * t * rinv;
    const R inner = p.gA * r + p.gB;
    return r < p.l ? inner : outer;
}
template <class R> __device__ __forceinline__ R kernel_w(R r, const Phys<R>& p) {
    const R t = rmax(p.two_l - r, R(0));
    const R outer = p.wB * t * t * t;
    const R inner = p.sigma + r * r * (p.wA3 * r + p.wA2);
    return r < p.l ? inner : outer;
}


// The pair terms of the Jacobi passes. Their dot products are written out as
// explicit roundings (no contraction left to the compiler, whose choice of
// which product to fuse can depend on the code around an inlined call), and
// each term is added to its sum with an explicit fused multiply-add, so that
// a pass that evaluates a particle's candidates on several lanes and adds them
// on one (jacobi_solve_kernel) gets the same bits as the one-lane passes.
__device__ __forceinline__ float fma_r(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_r(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_r(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_r(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_r(double a, double b) { return __dsub_rn(a, b); }
// a.x b.x + a.y b.y + a.z b.z as fma(az, bz, fma(ay, by, ax bx))
template <class R> __device__ __forceinline__ R dot3(R ax, R ay, R az, R bx, R by, R bz) {
    return fma_r(az, bz, fma_r(ay, by, mul_r(ax, bx)));
}
// pair_r and grad_factor with every rounding explicit
template <class R> __device__ __forceinline__ R pair_r_x(R r2, R& rinv) {
    rinv = rsqrt_r(rmax(r2, R(1e-24)));
    return mul_r(r2, rinv);
}
template <class R> __device__ __forceinline__ R grad_factor_x(R r, R rinv, const Phys<R>& p) {
    const R t = rmax(sub_r(p.two_l, r), R(0));
    const R outer = mul_r(mul_r(mul_r(p.gC, t), t), rinv);
    const R inner = fma_r(p.gA, r, p.gB);
    return r < p.l ? inner : outer;
}

// a.x - b.x and a.y - b.y. In FP32 both differences are one f32x2
// instruction (sm_100 and later pair FP32 operations; each lane is the IEEE
// round-to-nearest operation, so the lanes are the scalar differences bit
// for bit): the x and y of a record arrive in a register pair from its
// 16-byte load, so no register moves are needed. a - b is computed as
// fma(b, -1, a), whose product is exact and whose one rounding is the
// subtraction's.
template <class R> struct XY { R x, y; };
template <class R> __device__ __forceinline__ XY<R> diff_xy(const R4<R>& a, const R4<R>& b) {
    if constexpr (sizeof(R) == sizeof(float)) {
        const float2 d = __ffma2_rn(make_float2(b.x, b.y), make_float2(-1.0f, -1.0f), make_float2(a.x, a.y));
        return {d.x, d.y};
    } else {
        return {a.x - b.x, a.y - b.y};
    }
}

// (acc.x, acc.y) = (fma(f, x, acc.x), fma(f, y, acc.y)): one f32x2 instruction
// in FP32, each lane the IEEE fused multiply-add, so the sums are the scalar
// ones bit for bit. Used where the x and y terms come from diff_xy (already a
// register pair): density + alpha and the pressure apply pass, 1.7 M and 0.9 M
// fewer warp instructions per launch at 1M particles. In the XSPH pass, whose
// weight is a quotient, the same packing cost instructions and was left out.
template <class R> __device__ __forceinline__ void fma_xy(R f, R x, R y, XY<R>& acc) {
    if constexpr (sizeof(R) == sizeof(float)) {
        const float2 a = __ffma2_rn(make_float2(f, f), make_float2(x, y), make_float2(acc.x, acc.y));
        acc = {a.x, a.y};
    } else {
        acc = {fma_r(f, x, acc.x), fma_r(f, y, acc.y)};
    }
}

// rate pass, fluid candidate j: rd = fma(f, d, rd)
template <class R>
__device__ __forceinline__ void rate_fluid_terms(const R4<R>& pi, const R4<R>& vi, const R4<R>& pj,
                                                 const R4<R>& vj, const Phys<R>& p, R& f, R& d) {
    const XY<R> rxy = diff_xy(pi, pj);
    const R rx = rxy.x, ry = rxy.y, rz = pi.z - pj.z;
    R rinv;
    const R r = pair_r_x(dot3(rx, ry, rz, rx, ry, rz), rinv);
    f = grad_factor_x(r, rinv, p);
    const XY<R> dv = diff_xy(vi, vj);
    d = dot3(dv.x, dv.y, vi.z - vj.z, rx, ry, rz);
}
// rate pass, wall candidate j (wall velocity 0): rb = fma(f, d, rb)
template <class R>
__device__ __forceinline__ void rate_wall_terms(const R4<R>& pi, const R4<R>& vi, const R4<R>& pj,
                                                const Phys<R>& p, R& f, R& d) {
    const XY<R> rxy = diff_xy(pi, pj);
    const R rx = rxy.x, ry = rxy.y, rz = pi.z - pj.z;
    R rinv;
    const R r = pair_r_x(dot3(rx, ry, rz, rx, ry, rz), rinv);
    f = mul_r(pj.w, grad_factor_x(r, rinv, p));
    d = dot3(vi.x, vi.y, vi.z, rx, ry, rz);
}
// apply pass, candidate j with the pair weight w = kfac_i + kfac_j (fluid)
// or m_b (wall): a = fma(f, r_ij, a) per component
template <class R>
__device__ __forceinline__ void apply_terms(const R4<R>& pi, const R4<R>& pj, R w, const Phys<R>& p, R& f, R& rx,
                                            R& ry, R& rz) {
    const XY<R> rxy = diff_xy(pi, pj);
    rx = rxy.x; ry = rxy.y; rz = pi.z - pj.z;
    R rinv;
    const R r = pair_r_x(dot3(rx, ry, rz, rx, ry, rz), rinv);
    f = mul_r(w, grad_factor_x(r, rinv, p));
}

// ---------------------------------------------------------------------------
// Reductions: FP64 block partial sums with a deterministic last-block finish.
// ---------------------------------------------------------------------------
constexpr int MAXV_SLOTS = 32;

struct IterCtl {
    double err_sum;       // sum of the last finished reduction
    u32 stop_iter;        // iteration after which the solver stopped (~0u: running)
    u32 blocks_done;      // last-block counter
    u32 iters;            // iterations run by a device-resident solve loop
    u32 maxv_slot[32];    // max |v| as float bits (non-negative floats order as
                          // ints), spread over MAXV_SLOTS words; the max of the
                          // words is the step's max |v|
    u32 flags;            // bit0: non-finite seen; bit1: sentinel order not canonical
    u32 bar_arrive;       // arrivals at the cooperative solve's grid barrier (cleared every step)
};

// ---------------------------------------------------------------------------
// Bounded device waits. The only kernel that waits on other blocks is the
// cooperative Jacobi solve (jacobi_solve_kernel), whose blocks are all
// resident (cooperative launch). Its grid barrier gives up after a time limit
// instead of spinning forever: the block that gives up sets the context's
// device error word, every other waiting block sees the word and returns too,
// and the host reports DFSPH_ERR_DEVICE_TIMEOUT at its next synchronising
// call. No wait, fault or trap is left behind, so the context stays usable.
// ---------------------------------------------------------------------------
constexpr u32 DEV_ERR_BARRIER_TIMEOUT = 1u;

struct WaitCfg {
    unsigned long long limit_ns;  // give up a wait after this many nanoseconds
    u32 missing;                  // blocks the barrier also waits for (0; tests set more to make every wait run out)
    u32* err;                     // the context's device error word (sticky until the host clears it)
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier number k (0, 1, 2, ...) of a cooperative launch, called by every
// thread of every block. Thread 0 of a block counts its arrival with a
// release add (the block's writes, ordered before it by __syncthreads, are
// published with it) on a counter that only grows (barrier k is complete at
// (k + 1) x (blocks + missing) arrivals) and polls it with acquire loads until
// then, the time limit, or another block's give-up; the block's threads read
// after the closing __syncthreads. Returns false, the same in every thread of
// the block, when the wait gave up; the caller returns then. (Release/acquire
// in place of two full fences around a relaxed add: 1.13 against 1.27 us per
// barrier over 77 blocks, measured with no work between barriers.)
__device__ __forceinline__ bool grid_barrier(u32* arrive, u32 k, const WaitCfg& w, int* sh_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(arrive) : "memory");
        const u32 target = (k + 1u) * (gridDim.x + w.missing);
        const unsigned long long t0 = global_ns();
        for (;;) {
            u32 seen;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(seen) : "l"(arrive) : "memory");
            if (seen >= target) break;
            if (*((volatile const u32*)w.err) & DEV_ERR_BARRIER_TIMEOUT) { ok = 0; break; }
            if (global_ns() - t0 > w.limit_ns) {
                atomicOr(w.err, DEV_ERR_BARRIER_TIMEOUT);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        *sh_ok = ok;
    }
    __syncthreads();
    return *sh_ok != 0;
}

template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < BLOCK / 32; ++w) t += sh[w];
    }
    return t;  // valid in thread 0
}

// Neighbour passes are instantiated for at most 128 and at most 256 threads
// per block (LB) and launch with 64, 128 or 256 threads, whichever the
// autotuner measured fastest for the workload.
constexpr int MAX_PASS_BLOCK = 256;

// block_sum for any block of whole warps up to MAX_PASS_BLOCK threads.
__device__ __forceinline__ double block_sum_dyn(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < int(blockDim.x >> 5); ++w) t += sh[w];
    return t;  // valid in thread 0
}

// The stop test of the reference's solvers (dfsph.cu:254-258,296-299): the
// mean error below eta rho0. The reference sums in FP32 (CUB) and compares
// in float; here the sum is FP64 and, in the FP32 builds, the mean is rounded
// to float and compared with eta rho0 evaluated in float, as the reference
// compares. The FP64 build compares in double.
struct StopTest {
    double n;    // particles in the mean
    double thr;  // eta rho0 in the working type
    int f32;     // 1: round the mean to float before the comparison
};
__device__ __forceinline__ bool below_threshold(double s, const StopTest& t) {
    const double m = s / t.n;
    return (t.f32 ? double(float(m)) : m) < t.thr;
}

// The order in which the block partials of an error reduction are added, the
// same in the per-pass last block (finish_reduction) and in the cooperative
// solve's decision warp. Up to REDUCE_SERIAL_MAX partials one lane adds them
// in block order (a few FP64 additions: quicker than a warp-wide tree on
// this GPU's few FP64 units); beyond, lane l of one warp adds partials l,
// l + 32, l + 64, ... in turn (from 0), then this shuffle tree adds the 32
// lane sums. Valid in lane 0; every lane of the warp calls it.
constexpr u32 REDUCE_SERIAL_MAX = 64;
__device__ __forceinline__ double lane_sums_total(double s) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    return s;
}

// The 32 arrival counters of finish_reduction, each on its own 128-byte line,
// sit in the REDUCE_GROUP_WORDS words in front of the partials (zero between
// reductions: the block that completes a group clears its counter).
constexpr u32 REDUCE_GROUP_WORDS = 32 * 32;

// Every thread of every block calls this (the block's partial valid in thread
// 0); the last block to arrive adds all partials in lane_sums_total's order
// with its first warp, so the result does not depend on block scheduling and
// the tail is gridDim.x / 32 loads per lane, not gridDim.x in sequence.
// Arrivals are counted in two levels (block b on counter b % 32, then the
// block completing a group on ctl->blocks_done), so no single address takes
// one atomic per block. Decides convergence: stop when (iter >= first_check)
// and the mean passes the stop test.
static __device__ __forceinline__ void finish_reduction(double partial, double* partials, IterCtl* ctl,
                                                 u32 iter, u32 first_check, StopTest rule) {
    __shared__ int last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = partial;
        __threadfence();
        u32* group = reinterpret_cast<u32*>(partials) - REDUCE_GROUP_WORDS + 32u * (blockIdx.x & 31u);
        const u32 members = (gridDim.x - (blockIdx.x & 31u) + 31u) / 32u;
        int l = 0;
        if (atomicAdd(group, 1u) == members - 1u) {
            *group = 0u;  // every member has arrived: ready for the next reduction
            __threadfence();
            l = atomicAdd(&ctl->blocks_done, 1u) == min(gridDim.x, 32u) - 1u;
        }
        last = l;
    }
    __syncthreads();
    if (!last || threadIdx.x >= 32) return;
    __threadfence();
    double s = 0;
    if (gridDim.x <= REDUCE_SERIAL_MAX) {
        if (threadIdx.x == 0)
            for (u32 b = 0; b < gridDim.x; ++b) s += *((volatile const double*)&partials[b]);
    } else {
        for (u32 b = threadIdx.x; b < gridDim.x; b += 32) s += *((volatile const double*)&partials[b]);
        s = lane_sums_total(s);
    }
    if (threadIdx.x == 0) {
        ctl->err_sum = s;
        ctl->blocks_done = 0;
        if (iter >= first_check && below_threshold(s, rule)) ctl->stop_iter = iter;
        if (!(s == s)) ctl->flags |= 1u;
    }
}

// A CFL frame stepped on the device: the substep size is chosen after every
// substep from the in-kernel max |v| (the reference's TimeStepper::next_dt,
// core/include/water/core/timestep.h:23-28, with sim_cli's 0.5 m/s floor and
// 64-substep cap, apps/sim_cli/main.cpp:171-181), so no host round trip is
// needed between substeps.
struct FrameCtl {
    float dt;            // substep size in use
    float remaining;     // time left in the frame
    u32 substeps;        // substeps taken in this frame
    u32 frames_done;
    u32 fresh;           // 1: no step taken yet (max |v| reads as 0)
    u32 max_frames;      // length of substeps_out
    float decay_f;       // e^{-damping dt} of the substep
    double decay_d;
    float frame_dt, dt_max, cfl_lambda, radius, dt_min, v_floor, damping;
    u32 max_per_frame;
    u32 more;            // 1: the frame continues (read by the host-driven loop)
    u32* substeps_out;   // substeps per frame (device), or null
};

// Step size and the quantities derived from it, either fixed by the host
// (dev == null) or read from the device frame control at kernel start.
template <class R> struct StepDt {
    R dt, damping, gx, gy, gz;   // gravity
    const FrameCtl* dev;
};

// e^{-damping dt} as the reference evaluates it: apply_gravity_kernel
// (solvers/dfsph/src/dfsph_kernels.cu:347-355) computes expf(-damping * dt)
// on the device, built with -use_fast_math, which makes expf the fast
// exponential __expf. Host-stepped and device-stepped substeps both take it
// from here, so they agree to the bit. The FP64 build uses exp.
__device__ __forceinline__ float damping_decay(float damping, float dt) { return __expf(__fmul_rn(-damping, dt)); }
__device__ __forceinline__ double damping_decay(double damping, double dt) { return exp(-damping * dt); }

template <class R> __device__ __forceinline__ R mul_rn(R a, R b);
template <> __device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

template <class R> __device__ __forceinline__ R step_dt(const StepDt<R>& s) {
    return s.dev ? R(*((volatile const float*)&s.dev->dt)) : s.dt;
}
template <class R> __device__ __forceinline__ R step_decay(const StepDt<R>& s) {
    if (!s.dev) return damping_decay(s.damping, s.dt);
    return sizeof(R) == sizeof(float) ? R(*((volatile const float*)&s.dev->decay_f))
                                      : R(*((volatile const double*)&s.dev->decay_d));
}

__device__ __forceinline__ bool stopped_before(const IterCtl* ctl, u32 iter) {
    // Iteration `iter` runs only while no earlier iteration decided to stop.
    return *((volatile const u32*)&ctl->stop_iter) < iter;
}

// ---------------------------------------------------------------------------
// Grid build: counting sort by cell key, deterministic within a cell.
// ---------------------------------------------------------------------------

// Keys of the state in slot order, with the rank of each particle among the
// particles of its cell (atomic, order fixed later) and the per-cell counts.
// Key range of the particles counted for the next grid build: per block the
// lowest and highest key go to one of KRANGE_SLOTS word pairs (krange[s] the
// lows, krange[KRANGE_SLOTS + s] the highs), so that the atomics of all
// blocks do not meet on one word. An out-of-grid particle (key = the scene's
// last cell) makes the range the whole array: its stencil is clamped to the
// grid's faces, anywhere along them.
constexpr int KRANGE_SLOTS = 32;
__device__ __forceinline__ void key_bounds(u32 k, u32 cells1, u32& lo, u32& hi) {
    if (k % cells1 == cells1 - 1) {
        lo = 0u;
        hi = ~0u;
    } else {
        lo = k;
        hi = k;
    }
}
template <int BLOCK>
__device__ __forceinline__ void key_range_block(u32 lo, u32 hi, u32* __restrict__ krange) {
    __shared__ u32 wlo[BLOCK / 32], whi[BLOCK / 32];
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if ((threadIdx.x & 31) == 0) {
        wlo[threadIdx.x >> 5] = lo;
        whi[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        u32 l = ~0u, h = 0u;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) {
            l = min(l, wlo[w]);
            h = max(h, whi[w]);
        }
        if (l <= h) {
            atomicMin(krange + blockIdx.x % KRANGE_SLOTS, l);
            atomicMax(krange + KRANGE_SLOTS + blockIdx.x % KRANGE_SLOTS, h);
        }
    }
}
// The cells a grid build must scan: the counted keys widened by the stencil
// margin (every cell a stencil centred up to one cell off a particle's key
// cell can read, cell_start[c + 1] included); [a, b) = [0, 0) when nothing
// was counted. Called by the 32 lanes of one warp (one slot pair each).
__device__ __forceinline__ void scan_range(const u32* __restrict__ krange, u32 m, u32 margin, u32& a, u32& b) {
    const u32 lane = threadIdx.x & 31u;
    const u32 lo = __reduce_min_sync(0xffffffffu, krange[lane]);
    const u32 hi = __reduce_max_sync(0xffffffffu, krange[KRANGE_SLOTS + lane]);
    if (lo > hi) {
        a = b = 0u;
        return;
    }
    a = lo > margin ? lo - margin : 0u;
    const unsigned long long e = (unsigned long long)hi + margin + 2u;
    b = e < m ? u32(e) : m;
}

template <class R>
__global__ void __launch_bounds__(256) count_kernel(int n, const R4<R>* __restrict__ xk,
                                                    GridDev<R> g, u32* __restrict__ key,
                                                    u32* __restrict__ rank, u32* __restrict__ count,
                                                    u32* __restrict__ krange) {
    pdl_wait();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    u32 lo = ~0u, hi = 0u;
    if (s < n) {
        const R4<R> p = ld(xk + s);
        const u32 c = cell_key(p.x, p.y, p.z, g);
        const u32 k = (g.rank ? __ldg(g.rank + c) : c) + scene_of(g, s) * g.cells1;
        key[s] = k;
        rank[s] = atomicAdd(count + k, 1u);
        key_bounds(k, g.cells1, lo, hi);
    }
    if (krange) key_range_block<256>(lo, hi, krange);
}

// Exclusive scan of count[0..m) into cell_start[0..m] in three launches without
// inter-block waits: per-tile sums, a one-block scan of the tile sums, then the
// per-tile scans. count is cleared on the way for the next build.
constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

static __global__ void __launch_bounds__(SCAN_BLOCK) scan_tile_sums(const u32* __restrict__ count, u32 m,
                                                             u32* __restrict__ tile_sums,
                                                             const u32* __restrict__ krange, u32 margin) {
    pdl_wait();
    __shared__ u32 sh[SCAN_BLOCK / 32];
    __shared__ u32 range[2];
    const u32 base = blockIdx.x * SCAN_TILE;
    if (krange) {
        // tiles outside the counted key range hold only zero counts
        if (threadIdx.x < 32) {
            u32 a, b;
            scan_range(krange, m, margin, a, b);
            if (threadIdx.x == 0) {
                range[0] = a;
                range[1] = b;
            }
        }
        __syncthreads();
        if (base >= range[1] || base + SCAN_TILE <= range[0]) {
            if (threadIdx.x == 0) tile_sums[blockIdx.x] = 0u;
            return;
        }
    }
    u32 t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const u32 c = base + k * SCAN_BLOCK + threadIdx.x;
        if (c < m) t += count[c];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        u32 s = 0;
        for (int w = 0; w < SCAN_BLOCK / 32; ++w) s += sh[w];
        tile_sums[blockIdx.x] = s;
    }
}

// One block: exclusive scan of n_tiles values in place; writes the total to
// tile_sums[n_tiles] and, when given, to *total_out (the closing entry of
// cell_start). It also resets the solver's iteration controls and per-scene
// maxima for the step when given (every step's grid build runs it exactly
// once, before any solver kernel).
static __global__ void __launch_bounds__(1024) scan_tile_offsets(u32* __restrict__ tile_sums, u32 n_tiles,
                                                          u32* __restrict__ total_out, IterCtl* ctl, int n_ctl,
                                                          u32* __restrict__ maxv_scene, int n_scenes,
                                                          u32* __restrict__ krange, u32 m, u32 margin,
                                                          u32* __restrict__ cs_range) {
    pdl_wait();
    __shared__ u32 warp_tot[32];
    __shared__ u32 carry;
    if (threadIdx.x == 0) carry = 0;
    // the scanned cells, for scan_tiles and for completing cell_start on export
    if (cs_range && threadIdx.x < 32) {
        u32 a = 0u, b = m;
        if (krange) scan_range(krange, m, margin, a, b);
        if (threadIdx.x == 0) {
            cs_range[0] = a;
            cs_range[1] = b;
        }
    }
    __syncthreads();
    for (u32 base = 0; base < n_tiles; base += blockDim.x) {
        const u32 i = base + threadIdx.x;
        const u32 v = (i < n_tiles) ? tile_sums[i] : 0u;
        u32 x = v;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            u32 w = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const u32 y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_tot[lane] = w;  // inclusive prefix of warp totals
        }
        __syncthreads();
        const u32 before = (warp > 0 ? warp_tot[warp - 1] : 0u) + carry;
        if (i < n_tiles) tile_sums[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
    for (int s = threadIdx.x; s < n_scenes; s += blockDim.x) maxv_scene[s] = 0u;
    // the range is consumed: start the next build's from empty
    if (krange && threadIdx.x < 2 * KRANGE_SLOTS) krange[threadIdx.x] = threadIdx.x < KRANGE_SLOTS ? ~0u : 0u;
    if (threadIdx.x == 0) {
        tile_sums[n_tiles] = carry;
        if (total_out) *total_out = carry;
        for (int k = 0; k < n_ctl; ++k) {
            ctl[k].err_sum = 0.0;
            ctl[k].stop_iter = ~0u;
            ctl[k].blocks_done = 0u;
            ctl[k].iters = 0u;
            for (int w = 0; w < MAXV_SLOTS; ++w) ctl[k].maxv_slot[w] = 0u;
            ctl[k].flags = 0u;
            ctl[k].bar_arrive = 0u;
        }
    }
}

// Padded shared-memory index: one spare word per 32 keeps both the coalesced
// (stride-1 across threads) and the per-thread (stride-16) accesses free of
// bank conflicts.
__device__ __forceinline__ u32 scan_pad(u32 i) { return i + (i >> 5); }

static __global__ void __launch_bounds__(SCAN_BLOCK) scan_tiles(u32* __restrict__ count, u32 m,
                                                         const u32* __restrict__ tile_offsets,
                                                         u32* __restrict__ cell_start,
                                                         const u32* __restrict__ cs_range) {
    pdl_wait();
    __shared__ u32 warp_tot[SCAN_BLOCK / 32];
    __shared__ u32 tile[SCAN_TILE + SCAN_TILE / 32];
    const u32 base = blockIdx.x * SCAN_TILE;
    // tiles outside the scanned range keep their (never read) entries; their
    // counts are zero already
    if (cs_range && (base >= cs_range[1] || base + SCAN_TILE <= cs_range[0])) return;
    // coalesced load of the tile (and clear the counts for the next build)
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const u32 li = k * SCAN_BLOCK + threadIdx.x;
        const u32 c = base + li;
        u32 x = 0;
        if (c < m) {
            x = count[c];
            count[c] = 0u;
        }
        tile[scan_pad(li)] = x;
    }
    __syncthreads();
    // each thread owns SCAN_ITEMS consecutive cells of the tile
    const u32 l0 = threadIdx.x * SCAN_ITEMS;
    u32 v[SCAN_ITEMS];
    u32 t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = tile[scan_pad(l0 + k)];
        t += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32 x = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    u32 wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += warp_tot[w];
    u32 run = tile_offsets[blockIdx.x] + wpre + x - t;
    // exclusive prefixes back into the tile (each thread its own words), then
    // a coalesced store
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        tile[scan_pad(l0 + k)] = run;
        run += v[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const u32 li = k * SCAN_BLOCK + threadIdx.x;
        const u32 c = base + li;
        if (c < m) cell_start[c] = tile[scan_pad(li)];
    }
}

// cell_start outside the last ranged scan: 0 before it, the total after it
// (an empty cell starts where the next particle's cell starts).
static __global__ void __launch_bounds__(256) complete_cell_start_kernel(u32* __restrict__ cell_start, u32 m,
                                                                         const u32* __restrict__ cs_range) {
    const u32 c = blockIdx.x * 256u + threadIdx.x;
    if (c >= m) return;
    if (c < cs_range[0]) cell_start[c] = 0u;
    else if (c >= cs_range[1]) cell_start[c] = cell_start[m];
}

// Provisional slot of every particle: cell start + atomic rank.
static __global__ void __launch_bounds__(256) scatter_kernel(int n, const u32* __restrict__ key,
                                                      const u32* __restrict__ rank,
                                                      const u32* __restrict__ cell_start,
                                                      const u32* __restrict__ id_old,
                                                      u32* __restrict__ tmp_src, u32* __restrict__ tmp_id) {
    pdl_wait();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const u32 d = cell_start[key[s]] + rank[s];
    tmp_src[d] = static_cast<u32>(s);
    tmp_id[d] = id_old[s];
}

// Final slot = cell start + number of cell mates with a smaller original index,
// which reproduces the reference's stable (key, index) order
// (core/src/cell_grid.cu:98-110 sorts iota values stably). The state is
// gathered into the new order on the way. cell_start has one closing entry
// (= n) after the last key. Out-of-grid particles of a scene (its last key,
// cells1 - 1 modulo cells1) beyond `sentinel_cap` keep the provisional order
// and raise flag bit 1.
template <class R>
__global__ void __launch_bounds__(256) reorder_kernel(
    int n, const u32* __restrict__ tmp_src, const u32* __restrict__ tmp_id,
    const u32* __restrict__ key_old, const u32* __restrict__ cell_start, u32 cells1,
    u32 sentinel_cap, const R4<R>* __restrict__ xk_old, const R4<R>* __restrict__ vr_old,
    R4<R>* __restrict__ xk_new, R4<R>* __restrict__ vr_new, u32* __restrict__ id_new,
    u32* __restrict__ key_sorted, IterCtl* ctl) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const u32 src = tmp_src[t];
    const u32 my = tmp_id[t];
    const u32 c = key_old[src];
    const u32 b = cell_start[c];
    const u32 e = cell_start[c + 1];
    u32 dst = static_cast<u32>(t);
    if (e - b > 1) {
        if ((c % cells1) == cells1 - 1 && e - b > sentinel_cap) {
            if (t == static_cast<int>(b)) atomicOr(&ctl->flags, 2u);
        } else {
            u32 r = 0;
            for (u32 u = b; u < e; ++u) r += (tmp_id[u] < my) ? 1u : 0u;
            dst = b + r;
        }
    }
    xk_new[dst] = ld(xk_old + src);
    vr_new[dst] = ld(vr_old + src);
    id_new[dst] = my;
    key_sorted[dst] = c;
}

// ---------------------------------------------------------------------------
// Import / export between the caller's original-order AoS arrays and the
// sorted SoA state.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(256) import_kernel(int n, const float* __restrict__ pos,
                                                     const float* __restrict__ vel,
                                                     R4<R>* __restrict__ xk, R4<R>* __restrict__ vr,
                                                     u32* __restrict__ id) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    xk[i] = {R(pos[3 * i]), R(pos[3 * i + 1]), R(pos[3 * i + 2]), R(0)};
    if (vel)
        vr[i] = {R(vel[3 * i]), R(vel[3 * i + 1]), R(vel[3 * i + 2]), R(0)};
    else
        vr[i] = {R(0), R(0), R(0), R(0)};
    id[i] = static_cast<u32>(i);
}

template <class R>
__global__ void __launch_bounds__(256) export_kernel(int n, const u32* __restrict__ id,
                                                     const R4<R>* __restrict__ xk,
                                                     const R4<R>* __restrict__ vr,
                                                     const R* __restrict__ alpha,
                                                     const R* __restrict__ kap,
                                                     const R* __restrict__ rho_adv,
                                                     float* pos, float* vel, float* density,
                                                     float* alpha_out, float* kappa_out,
                                                     float* rho_adv_out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const u32 i = id[s];
    const R4<R> p = xk[s];
    const R4<R> v = vr[s];
    if (pos) { pos[3 * i] = float(p.x); pos[3 * i + 1] = float(p.y); pos[3 * i + 2] = float(p.z); }
    if (vel) { vel[3 * i] = float(v.x); vel[3 * i + 1] = float(v.y); vel[3 * i + 2] = float(v.z); }
    if (density) density[i] = float(v.w);
    if (alpha_out) alpha_out[i] = float(alpha[s]);
    if (kappa_out) kappa_out[i] = float(kap[s]);
    if (rho_adv_out) rho_adv_out[i] = float(rho_adv[s]);
}

// Import from, and export to, caller memory that the GPU reads and writes in
// place (page-locked host memory): the xyz triples of a block's 256
// particles move as 16-byte accesses through shared memory, the few floats
// past the block's last whole 16 bytes (the tail of the last block) as single
// words. Base pointers are 16-byte aligned (checked by the host).
__device__ __forceinline__ void load_triples(const float* __restrict__ src, int base, int cnt, float* tile) {
    const int nf = 3 * cnt, n4 = nf / 4, t = threadIdx.x;
    const float4* s4 = reinterpret_cast<const float4*>(src + 3 * size_t(base));
    if (t < n4) reinterpret_cast<float4*>(tile)[t] = s4[t];
    if (t < nf - 4 * n4) tile[4 * n4 + t] = src[3 * size_t(base) + 4 * n4 + t];
}
__device__ __forceinline__ void store_triples(float* __restrict__ dst, int base, int cnt, const float* tile) {
    const int nf = 3 * cnt, n4 = nf / 4, t = threadIdx.x;
    float4* d4 = reinterpret_cast<float4*>(dst + 3 * size_t(base));
    if (t < n4) d4[t] = reinterpret_cast<const float4*>(tile)[t];
    if (t < nf - 4 * n4) dst[3 * size_t(base) + 4 * n4 + t] = tile[4 * n4 + t];
}

// Positions and velocities in one pass to page-locked host memory (original
// order; either output may be null): export_mapped_kernel for both fields
// from one inverse permutation.
template <class R>
__global__ void __launch_bounds__(256) export_state_mapped_kernel(int n, const u32* __restrict__ inv,
                                                                  const R4<R>* __restrict__ xk,
                                                                  const R4<R>* __restrict__ vr,
                                                                  float* __restrict__ pos, float* __restrict__ vel) {
    __shared__ __align__(16) float tp[3 * 256];
    __shared__ __align__(16) float tv[3 * 256];
    const int base = blockIdx.x * 256;
    const int cnt = min(256, n - base);
    const int t = threadIdx.x;
    if (t < cnt) {
        const u32 s = inv[base + t];
        if (pos) {
            const R4<R> x = xk[s];
            tp[3 * t] = float(x.x);
            tp[3 * t + 1] = float(x.y);
            tp[3 * t + 2] = float(x.z);
        }
        if (vel) {
            const R4<R> v = vr[s];
            tv[3 * t] = float(v.x);
            tv[3 * t + 1] = float(v.y);
            tv[3 * t + 2] = float(v.z);
        }
    }
    __syncthreads();
    if (pos) store_triples(pos, base, cnt, tp);
    if (vel) store_triples(vel, base, cnt, tv);
}

// import_kernel on caller memory read in place (vel null: zero velocities)
template <class R>
__global__ void __launch_bounds__(256) import_mapped_kernel(int n, const float* __restrict__ pos,
                                                            const float* __restrict__ vel,
                                                            R4<R>* __restrict__ xk, R4<R>* __restrict__ vr,
                                                            u32* __restrict__ id) {
    __shared__ __align__(16) float tp[3 * 256];
    __shared__ __align__(16) float tv[3 * 256];
    const int base = blockIdx.x * 256;
    const int cnt = min(256, n - base);
    load_triples(pos, base, cnt, tp);
    if (vel) load_triples(vel, base, cnt, tv);
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= cnt) return;
    const int i = base + t;
    xk[i] = {R(tp[3 * t]), R(tp[3 * t + 1]), R(tp[3 * t + 2]), R(0)};
    if (vel)
        vr[i] = {R(tv[3 * t]), R(tv[3 * t + 1]), R(tv[3 * t + 2]), R(0)};
    else
        vr[i] = {R(0), R(0), R(0), R(0)};
    id[i] = static_cast<u32>(i);
}

// slot of every original index: inv[id[s]] = s
static __global__ void __launch_bounds__(256) invert_kernel(int n, const u32* __restrict__ id,
                                                            u32* __restrict__ inv) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) inv[id[s]] = static_cast<u32>(s);
}

// A per-slot field in original order, written in place to caller memory:
// lane < 0 the xyz triple of in, lane 0..3 one lane of in, or (in null) the
// scalar array sc. Thread t of the block takes original index base + t.
template <class R>
__global__ void __launch_bounds__(256) export_mapped_kernel(int n, const u32* __restrict__ inv,
                                                            const R4<R>* __restrict__ in, int lane,
                                                            const R* __restrict__ sc, float* __restrict__ out) {
    __shared__ __align__(16) float tile[3 * 256];
    const int base = blockIdx.x * 256;
    const int cnt = min(256, n - base);
    const int t = threadIdx.x;
    if (!in) {
        if (t < cnt) out[base + t] = float(sc[inv[base + t]]);
        return;
    }
    if (lane >= 0) {
        if (t < cnt) {
            const R4<R> v = in[inv[base + t]];
            out[base + t] = float(lane == 0 ? v.x : lane == 1 ? v.y : lane == 2 ? v.z : v.w);
        }
        return;
    }
    if (t < cnt) {
        const R4<R> v = in[inv[base + t]];
        tile[3 * t] = float(v.x);
        tile[3 * t + 1] = float(v.y);
        tile[3 * t + 2] = float(v.z);
    }
    __syncthreads();
    store_triples(out, base, cnt, tile);
}

// Scatter a per-slot array to original order (double output for FP64 reads).
template <class T, class O>
__global__ void __launch_bounds__(256) unsort_kernel(int n, const u32* __restrict__ id,
                                                     const T* __restrict__ in, O* __restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    out[id[s]] = O(in[s]);
}

template <class R, class O>
__global__ void __launch_bounds__(256) unsort_vec_kernel(int n, const u32* __restrict__ id,
                                                         const R4<R>* __restrict__ in, int lane,
                                                         O* __restrict__ out) {
    // lane < 0: xyz triple; lane in 0..3: one component
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const R4<R> v = in[s];
    const u32 i = id[s];
    if (lane < 0) {
        out[3 * i] = O(v.x); out[3 * i + 1] = O(v.y); out[3 * i + 2] = O(v.z);
    } else {
        out[i] = O(lane == 0 ? v.x : lane == 1 ? v.y : lane == 2 ? v.z : v.w);
    }
}

// ---------------------------------------------------------------------------
// Boundary: Akinci mass (dfsph_kernels.cu:40-65) and the per-cell flag telling
// whether any boundary particle lies in the 27-cell stencil of a cell.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(128) boundary_mass_kernel(int nb, const R4<R>* __restrict__ xb_in,
                                                            R4<R>* __restrict__ xb_out,
                                                            const u32* __restrict__ bcs, GridDev<R> g,
                                                            Phys<R> p) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nb) return;
    const R4<R> pi = ld(xb_in + s);
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    R sum_w = 0;
    for_each_run(c, g, bcs, [&](u32 b, u32 e) {
        for (u32 j = b; j < e; ++j) {
            const R4<R> pj = ld(xb_in + j);
            const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            R rinv;
            sum_w += kernel_w(pair_r(rx * rx + ry * ry + rz * rz, rinv), p);
        }
    });
    xb_out[s] = {pi.x, pi.y, pi.z, p.rho0 / (sum_w > R(1e-9) ? sum_w : R(1e-9))};
}

template <class R>
__global__ void __launch_bounds__(256) boundary_mask_kernel(u32 total, const u32* __restrict__ bcs,
                                                            GridDev<R> g, unsigned char* __restrict__ mask) {
    const u32 c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= total) return;
    const int cz = static_cast<int>(c % static_cast<u32>(g.nz));
    const u32 rest = c / static_cast<u32>(g.nz);
    const int cy = static_cast<int>(rest % static_cast<u32>(g.ny));
    const int cx = static_cast<int>(rest / static_cast<u32>(g.ny));
    u32 any = 0;
    for_each_run(Centre{cx, cy, cz}, g, bcs, [&](u32 b, u32 e) { any |= (e > b) ? 1u : 0u; });
    mask[c] = static_cast<unsigned char>(any);
}

// 1 per boundary particle that has a fluid particle within the support.
template <class R, bool MORTON = false>
__global__ void __launch_bounds__(128) active_boundary_kernel(int nb, const R4<R>* __restrict__ xb,
                                                              const R4<R>* __restrict__ xk,
                                                              const u32* __restrict__ cs, GridDev<R> g,
                                                              Phys<R> p, int n_scenes, u32* __restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nb) return;
    const R4<R> pi = ld(xb + s);
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    u32 any = 0;
    for (int sc = 0; sc < n_scenes && !any; ++sc)
        for_each_fluid_run<MORTON>(c, g, cs + size_t(sc) * g.cells1, [&](u32 b, u32 e) {
            for (u32 j = b; j < e && !any; ++j) {
                const R4<R> pj = ld(xk + j);
                const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
                if (rx * rx + ry * ry + rz * rz < p.support2) any = 1;
            }
        });
    if (any) atomicAdd(out, 1u);
}

// Boundary runs of a fluid particle are visited unless its stencil centre is an
// in-grid cell whose mask says the stencil holds no boundary particle.
template <class R>
__device__ __forceinline__ bool boundary_near(const Centre& c, const GridDev<R>& g,
                                              const unsigned char* __restrict__ mask) {
    if (c.x < 0 || c.x >= g.nx || c.y < 0 || c.y >= g.ny || c.z < 0 || c.z >= g.nz) return true;
    const u32 cell = (static_cast<u32>(c.x) * static_cast<u32>(g.ny) + static_cast<u32>(c.y)) *
                         static_cast<u32>(g.nz) + static_cast<u32>(c.z);
    return __ldg(mask + cell) != 0;
}

// Per-step records written by the forward kernels when the adjoint replays a
// segment (null pointers otherwise): positions with rho, (G, den) of alpha and
// the slot -> original index map of the step's sorted order.
template <class R> struct Tape1 {
    R4<R>* x;
    R4<R>* g;
    u32* id;
};

struct BoundaryDev {
    const void* xb;             // R4<R>*, (x, y, z, m_b), sorted
    const u32* bcs;             // boundary cell_start
    const unsigned char* mask;  // per cell
    int has;
};

// ---------------------------------------------------------------------------
// Density + alpha (density_kernel dfsph_kernels.cu:68-112 fused with
// alpha_kernel :117-169): rho = sum m W (self included) + sum m_b W;
// alpha = rho / (|sum m gradW|^2 + sum |m gradW|^2). KAHAN compensates the
// density sums.
// ---------------------------------------------------------------------------
// A 32-bit integer mix (the "lowbias32" finaliser of C. Wellons' hash
// prospector): the candidate-set signature adds the mixed ids of a
// particle's candidates, so two builds that visit the same set agree.
__device__ __forceinline__ u32 mix32(u32 x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

template <class R, bool KAHAN, bool DIAG, int LB, bool MORTON = false>
__global__ void __launch_bounds__(LB, DIAG ? 1 : fp32_min_blocks<R>(LB)) density_alpha_kernel(
    int n, const R4<R>* __restrict__ xk, R4<R>* __restrict__ vr, R* __restrict__ alpha,
    const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, BoundaryDev bd, u32* __restrict__ nbr_f,
    u32* __restrict__ nbr_b, u32* __restrict__ nbr_sig, const u32* __restrict__ id, Tape1<R> tp) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const R4<R> pi = ld(xk + i);
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    R ws = 0, wc = 0;
    R gx = 0, gy = 0, gz = 0, gq = 0;
    XY<R> gxy = {0, 0};
    u32 cf = 0, cb = 0, sig = 0;
    for_each_fluid_run<MORTON>(c, g, cs + scene_of(g, i) * g.cells1, [&](u32 b, u32 e) {
        if (DIAG) {
            cf += e - b;
            for (u32 j = b; j < e; ++j) sig += mix32(__ldg(id + j));
        }
#pragma unroll 2
        for (u32 j = b; j < e; ++j) {
            const R4<R> pj = ld(xk + j);
            const XY<R> rxy = diff_xy(pi, pj);
            const R rx = rxy.x, ry = rxy.y, rz = pi.z - pj.z;
            R rinv;
            const R r = pair_r(rx * rx + ry * ry + rz * rz, rinv);
            const R w = kernel_w(r, p);
            if (KAHAN) {
                const R y = w - wc;
                const R t = ws + y;
                wc = (t - ws) - y;
                ws = t;
            } else {
                ws += w;
            }
            const R f = grad_factor(r, rinv, p);
            fma_xy(f, rx, ry, gxy);
            gz = fma_r(f, rz, gz);
            gq += f * f * (rx * rx + ry * ry + rz * rz);
        }
    });
    gx = gxy.x;
    gy = gxy.y;
    R rho = p.mass * ws;
    gx *= p.mass; gy *= p.mass; gz *= p.mass;
    gq *= p.mass * p.mass;
    if (bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        R bs = 0, bsc = 0;
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
            if (DIAG) cb += e - b;
            for (u32 j = b; j < e; ++j) {
                const R4<R> pj = ld(xb + j);
                const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
                const R r2 = rx * rx + ry * ry + rz * rz;
                R rinv;
                const R r = pair_r(r2, rinv);
                const R mw = pj.w * kernel_w(r, p);
                if (KAHAN) {
                    const R y = mw - bsc;
                    const R t = bs + y;
                    bsc = (t - bs) - y;
                    bs = t;
                } else {
                    bs += mw;
                }
                const R f = pj.w * grad_factor(r, rinv, p);
                gx += f * rx; gy += f * ry; gz += f * rz;
                gq += f * f * r2;
            }
        });
        rho += bs;
    } else if (DIAG && bd.has) {
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) { cb += e - b; });
    }
    if (DIAG && bd.has) {
        // wall candidates by their sorted slot (the wall order is fixed)
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
            for (u32 j = b; j < e; ++j) sig += mix32(j ^ 0x80000000u);
        });
    }
    const R denom = gx * gx + gy * gy + gz * gz + gq;
    R4<R> v = vr[i];
    v.w = rho;
    vr[i] = v;
    alpha[i] = denom > R(1e-9) ? rho / denom : R(0);
    if (DIAG) { nbr_f[i] = cf; nbr_b[i] = cb; nbr_sig[i] = sig; }
    if (tp.x) {
        tp.x[i] = {pi.x, pi.y, pi.z, rho};
        tp.g[i] = {gx, gy, gz, denom};
        tp.id[i] = id[i];
    }
}

// ---------------------------------------------------------------------------
// External forces + XSPH (apply_gravity_kernel dfsph_kernels.cu:347-355, then
// xsph_viscosity_kernel :305-341) in one Jacobi pass: v' = v e^{-d dt} + g dt
// and, because g dt cancels in v'_j - v'_i, the XSPH term of v' equals
// e^{-d dt} times the XSPH term of v. Reads vr_in, writes vr_out.
// ---------------------------------------------------------------------------
template <class R, int LB, bool MORTON = false>
__global__ void __launch_bounds__(LB) forces_xsph_kernel(
    int n, const R4<R>* __restrict__ xk, const R4<R>* __restrict__ vr_in, R4<R>* __restrict__ vr_out,
    const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, StepDt<R> sd, R eps,
    const R* __restrict__ eps_scene, int do_xsph, R4<R>* __restrict__ tape_v) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const R dt = step_dt(sd);
    const R decay = step_decay(sd);
    // g dt rounded on its own, as the host computes it
    const R gdx = mul_rn(sd.gx, dt), gdy = mul_rn(sd.gy, dt), gdz = mul_rn(sd.gz, dt);
    const R4<R> vi = ld(vr_in + i);
    if (tape_v) tape_v[i] = vi;
    R dx = 0, dy = 0, dz = 0;
    if (do_xsph) {
        const R4<R> pi = ld(xk + i);
        const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
        for_each_fluid_run<MORTON>(c, g, cs + scene_of(g, i) * g.cells1, [&](u32 b, u32 e) {
            for (u32 j = b; j < e; ++j) {
                const R4<R> pj = ld(xk + j);
                const R4<R> vj = ld(vr_in + j);
                const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
                R rinv;
                const R w = kernel_w(pair_r(rx * rx + ry * ry + rz * rz, rinv), p);
                const R ravg = R(0.5) * (vi.w + vj.w);
                const R cc = fast_div(w, rmax(ravg, R(1e-9)));
                dx += cc * (vj.x - vi.x);
                dy += cc * (vj.y - vi.y);
                dz += cc * (vj.z - vi.z);
            }
        });
        const R e = eps_scene ? eps_scene[scene_of(g, i)] : eps;
        const R s = e * p.mass * decay;
        dx *= s; dy *= s; dz *= s;
    }
    vr_out[i] = {vi.x * decay + gdx + dx, vi.y * decay + gdy + dy, vi.z * decay + gdz + dz, vi.w};
}

// One particle of the rate pass: rho_adv, kappa and (x, kappa / rho^2) of
// particle i; returns its error term (the reduction's input).
template <class R, bool DIVERGENCE, bool MORTON = false>
__device__ __forceinline__ double rate_particle(int i, const R4<R>* __restrict__ xk_in, R4<R>* __restrict__ xk_out,
                                                const R4<R>* __restrict__ vr, const R* __restrict__ alpha,
                                                R* __restrict__ rho_adv, R* __restrict__ kap,
                                                const u32* __restrict__ cs, const GridDev<R>& g, const Phys<R>& p,
                                                const BoundaryDev& bd, R dt, R4<R>* __restrict__ tape_v) {
    double err = 0;
    const R4<R> pi = ld(xk_in + i);
    const R4<R> vi = ld(vr + i);
    if (tape_v) tape_v[i] = vi;
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    R rd = 0;
    auto pair = [&](const R4<R>& pj, const R4<R>& vj) {
        R f, d;
        rate_fluid_terms(pi, vi, pj, vj, p, f, d);
        rd = fma_r(f, d, rd);
    };
    for_each_fluid_run<MORTON>(c, g, cs + scene_of(g, i) * g.cells1, [&](u32 b, u32 e) {
#pragma unroll 2
        for (u32 j = b; j < e; ++j) pair(ld(xk_in + j), ld(vr + j));
    });
    rd *= p.mass;
    if (bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        R rb = 0;
        auto wall = [&](const R4<R>& pj) {
            R f, d;
            rate_wall_terms(pi, vi, pj, p, f, d);
            rb = fma_r(f, d, rb);
        };
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
            for (u32 j = b; j < e; ++j) wall(ld(xb + j));
        });
        rd += rb;
    }
    const R rho = vi.w;
    R k;
    if (!DIVERGENCE) {
        const R rp = fma_r(dt, rd, rho);
        rho_adv[i] = rp;
        const R over = rmax(rp - p.rho0, R(0));
        k = over * alpha[i] / (dt * dt);
        err = double(over);
    } else {
        const R s = rmax(rd, R(0));
        rho_adv[i] = rd;  // the divergence solver's rho_dot scratch
        k = s * alpha[i] / dt;
        err = double(s);
    }
    kap[i] = k;
    xk_out[i] = {pi.x, pi.y, pi.z, k / rmax(rho * rho, R(1e-9))};
    return err;
}

// ---------------------------------------------------------------------------
// Jacobi pressure iteration, first half: rho_dot = sum_j m (v_i - v_j).gradW
// (fluid) + sum_b m_b v_i.gradW (density_change_kernel dfsph_kernels.cu:176-232).
// DIVERGENCE = false: rho* = rho + dt rho_dot, kappa = max(0, rho* - rho0)
// alpha / dt^2, error term max(0, rho* - rho0). DIVERGENCE = true (solver of
// the reference's plan): kappa_v = max(0, rho_dot) alpha / dt, error term
// max(0, rho_dot). Writes xk_out = (x, kappa / max(rho^2, 1e-9)); xk_in is
// not written.
// ---------------------------------------------------------------------------
template <class R, bool DIVERGENCE, bool REDUCE, bool DEVLOOP, int LB, bool MORTON = false>
__global__ void __launch_bounds__(LB) pressure_rate_kernel(
    int n, const R4<R>* __restrict__ xk_in, R4<R>* __restrict__ xk_out,
    const R4<R>* __restrict__ vr, const R* __restrict__ alpha, R* __restrict__ rho_adv,
    R* __restrict__ kap, const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, BoundaryDev bd,
    StepDt<R> sd, double* __restrict__ partials, IterCtl* ctl, u32 iter, u32 first_check, StopTest rule,
    R4<R>* __restrict__ tape_v, const u32* dev_iter) {
    pdl_wait();
    __shared__ double sh[LB / 32];
    // Inside a device-resident loop (DEVLOOP) the iteration comes from the
    // device and even iterations read xk_in / write xk_out, odd ones the other
    // way round.
    if (DEVLOOP) {
        iter = *((volatile const u32*)dev_iter);
        if (iter & 1u) {
            R4<R>* t = xk_out;
            xk_out = const_cast<R4<R>*>(xk_in);
            xk_in = t;
        }
    }
    if (stopped_before(ctl, iter)) return;
    const R dt = step_dt(sd);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double err = 0;
    if (i < n)
        err = rate_particle<R, DIVERGENCE, MORTON>(i, xk_in, xk_out, vr, alpha, rho_adv, kap, cs, g, p, bd, dt,
                                                   tape_v);
    if (REDUCE) {
        const double t = block_sum_dyn(err, sh);
        finish_reduction(t, partials, ctl, iter, first_check, rule);
    }
}

// Second half (apply_kappa_kernel dfsph_kernels.cu:237-301):
// v_i -= dt sum_j m (kfac_i + kfac_j) gradW over fluid and
// dt sum_b m_b (kfac_i + kappa_i / max(rho0^2, 1e-9)) gradW over the boundary.
// One particle of the apply pass: its velocity after the pressure update.
template <class R, bool MORTON = false>
__device__ __forceinline__ R4<R> apply_velocity(int i, const R4<R>* __restrict__ xk, const R4<R>* __restrict__ vr,
                                                const R* __restrict__ kap, const u32* __restrict__ cs,
                                                const GridDev<R>& g, const Phys<R>& p, const BoundaryDev& bd, R dt) {
    const R4<R> pi = ld(xk + i);
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    XY<R> axy = {0, 0};
    R az = 0;
    auto pair = [&](const R4<R>& pj) {
        R f, rx, ry, rz;
        apply_terms(pi, pj, pi.w + pj.w, p, f, rx, ry, rz);
        fma_xy(f, rx, ry, axy);
        az = fma_r(f, rz, az);
    };
    for_each_fluid_run<MORTON>(c, g, cs + scene_of(g, i) * g.cells1, [&](u32 b, u32 e) {
        for (u32 j = b; j < e; ++j) pair(ld(xk + j));
    });
    const R sf = -dt * p.mass;
    R ax = axy.x * sf, ay = axy.y * sf;
    az *= sf;
    if (bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        const R kb = pi.w + kap[i] / rmax(p.rho0 * p.rho0, R(1e-9));
        R bx = 0, by = 0, bz = 0;
        auto wall = [&](const R4<R>& pj) {
            R f, rx, ry, rz;
            apply_terms(pi, pj, pj.w, p, f, rx, ry, rz);
            bx = fma_r(f, rx, bx); by = fma_r(f, ry, by); bz = fma_r(f, rz, bz);
        };
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
            for (u32 j = b; j < e; ++j) wall(ld(xb + j));
        });
        const R sb = -dt * kb;
        ax = fma_r(sb, bx, ax); ay = fma_r(sb, by, ay); az = fma_r(sb, bz, az);
    }
    R4<R> v = vr[i];
    v.x += ax; v.y += ay; v.z += az;
    return v;
}

template <class R, bool DEVLOOP, int LB, bool MORTON = false>
__global__ void __launch_bounds__(LB) pressure_apply_kernel(
    int n, const R4<R>* __restrict__ xk, R4<R>* __restrict__ vr, const R* __restrict__ kap,
    const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, BoundaryDev bd, StepDt<R> sd, const IterCtl* ctl,
    u32 iter, const R4<R>* xk_odd, const u32* dev_iter) {
    pdl_wait();
    if (DEVLOOP) {
        iter = *((volatile const u32*)dev_iter);
        if (iter & 1u) xk = xk_odd;
    }
    if (stopped_before(ctl, iter)) return;
    const R dt = step_dt(sd);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vr[i] = apply_velocity<R, MORTON>(i, xk, vr, kap, cs, g, p, bd, dt);
}

// The rate and apply passes of jacobi_solve_kernel with one particle per quad
// of lanes (lanes 4k .. 4k + 3 of a warp, q = lane % 4). The candidates come
// from the launch's run tables (src), in the one-lane order: for every run,
// groups of four consecutive slots, lane q evaluating slot j0 + q. The group's
// terms are exchanged within the quad and every lane adds them, in slot order,
// with the one-lane pass's fused multiply-adds, so each lane ends with the
// one-lane sum bit for bit while it evaluates only a quarter of the
// particle's pair terms. Records come from shared memory when staged, else
// through ld_coh.
template <class R>
__device__ __forceinline__ R quad_get(unsigned qmask, R v, int src_lane) {
    return __shfl_sync(qmask, v, src_lane);
}

template <class R, bool DIVERGENCE>
__device__ __forceinline__ double rate_particle_quad(int i, int q, unsigned qmask, const R4<R>* xk_in,
                                                     R4<R>* xk_out, const R4<R>* vr, const R* __restrict__ alpha,
                                                     R* rho_adv, R* kap, const GridDev<R>& g, const Phys<R>& p,
                                                     const BoundaryDev& bd, R dt, const NbrSrc<R>& src) {
    const R4<R> pi = ld_coh(xk_in + i);
    const R4<R> vi = ld_coh(vr + i);
    const int base = int(threadIdx.x & 31u) & ~3;
    R rd = 0;
#pragma unroll 1
    for (int k = 0; k < 9; ++k) {
        const u32 b = src.rb[k * src.stride], e = src.re[k * src.stride];
        for (u32 j0 = b; j0 < e; j0 += 4) {
            const u32 j = j0 + u32(q);
            R f = 0, d = 0;
            if (j < e) {
                const R4<R> pj = src.x ? src.x[j - src.lo] : ld_coh(xk_in + j);
                const R4<R> vj = src.x ? src.v[j - src.lo] : ld_coh(vr + j);
                rate_fluid_terms(pi, vi, pj, vj, p, f, d);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const R fu = quad_get(qmask, f, base + u), du = quad_get(qmask, d, base + u);
                if (j0 + u < e) rd = fma_r(fu, du, rd);
            }
        }
    }
    rd *= p.mass;
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    if (bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        R rb = 0;
#pragma unroll 1
        for (int k = 0; k < 9; ++k) {
            const u32 b = src.wrb[k * src.stride], e = src.wre[k * src.stride];
            for (u32 j0 = b; j0 < e; j0 += 4) {
                const u32 j = j0 + u32(q);
                R f = 0, d = 0;
                if (j < e) rate_wall_terms(pi, vi, src.wx ? src.wx[j - src.wlo] : ld(xb + j), p, f, d);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const R fu = quad_get(qmask, f, base + u), du = quad_get(qmask, d, base + u);
                    if (j0 + u < e) rb = fma_r(fu, du, rb);
                }
            }
        }
        rd += rb;
    }
    if (q != 0) return 0.0;
    const R rho = vi.w;
    R kk;
    double err;
    if (!DIVERGENCE) {
        const R rp = fma_r(dt, rd, rho);
        rho_adv[i] = rp;
        const R over = rmax(rp - p.rho0, R(0));
        kk = over * alpha[i] / (dt * dt);
        err = double(over);
    } else {
        const R sv = rmax(rd, R(0));
        rho_adv[i] = rd;
        kk = sv * alpha[i] / dt;
        err = double(sv);
    }
    kap[i] = kk;
    xk_out[i] = {pi.x, pi.y, pi.z, kk / rmax(rho * rho, R(1e-9))};
    return err;
}

template <class R>
__device__ __forceinline__ R4<R> apply_velocity_quad(int i, int q, unsigned qmask, const R4<R>* xk,
                                                     const R4<R>* vr, const R* kap, const GridDev<R>& g,
                                                     const Phys<R>& p, const BoundaryDev& bd, R dt,
                                                     const NbrSrc<R>& src) {
    const R4<R> pi = ld_coh(xk + i);
    const int base = int(threadIdx.x & 31u) & ~3;
    R ax = 0, ay = 0, az = 0;
#pragma unroll 1
    for (int k = 0; k < 9; ++k) {
        const u32 b = src.rb[k * src.stride], e = src.re[k * src.stride];
        for (u32 j0 = b; j0 < e; j0 += 4) {
            const u32 j = j0 + u32(q);
            R f = 0, rx = 0, ry = 0, rz = 0;
            if (j < e) {
                const R4<R> pj = src.x ? src.x[j - src.lo] : ld_coh(xk + j);
                apply_terms(pi, pj, pi.w + pj.w, p, f, rx, ry, rz);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int l = base + u;
                const R fu = quad_get(qmask, f, l), xu = quad_get(qmask, rx, l), yu = quad_get(qmask, ry, l),
                        zu = quad_get(qmask, rz, l);
                if (j0 + u < e) { ax = fma_r(fu, xu, ax); ay = fma_r(fu, yu, ay); az = fma_r(fu, zu, az); }
            }
        }
    }
    const R sf = -dt * p.mass;
    ax *= sf; ay *= sf; az *= sf;
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    if (bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        const R kb = pi.w + kap[i] / rmax(p.rho0 * p.rho0, R(1e-9));
        R bx = 0, by = 0, bz = 0;
#pragma unroll 1
        for (int k = 0; k < 9; ++k) {
            const u32 b = src.wrb[k * src.stride], e = src.wre[k * src.stride];
            for (u32 j0 = b; j0 < e; j0 += 4) {
                const u32 j = j0 + u32(q);
                R f = 0, rx = 0, ry = 0, rz = 0;
                if (j < e) {
                    const R4<R> pj = src.wx ? src.wx[j - src.wlo] : ld(xb + j);
                    apply_terms(pi, pj, pj.w, p, f, rx, ry, rz);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int l = base + u;
                    const R fu = quad_get(qmask, f, l), xu = quad_get(qmask, rx, l), yu = quad_get(qmask, ry, l),
                            zu = quad_get(qmask, rz, l);
                    if (j0 + u < e) { bx = fma_r(fu, xu, bx); by = fma_r(fu, yu, by); bz = fma_r(fu, zu, bz); }
                }
            }
        }
        const R sb = -dt * kb;
        ax = fma_r(sb, bx, ax); ay = fma_r(sb, by, ay); az = fma_r(sb, bz, az);
    }
    R4<R> v = vr[i];
    v.x += ax; v.y += ay; v.z += az;
    return v;
}

// A whole adaptive Jacobi solve in one cooperative launch, every block
// resident (small scenes, where a solve of many short passes is bound by
// launches): per iteration the rate pass, a grid barrier, the stop decision
// and the apply pass, and a second barrier. Even iterations read positions
// from xa and write (x, kappa / rho^2) to xb, odd ones the other way round, as
// the graph-resident loop does. A block holds P particles, one per quad of
// lanes (rate_particle_quad, apply_velocity_quad), P as small as keeps one
// block per SM so that a small scene spreads over many SMs, plus one warp
// that takes the stop decision while the particle lanes run the apply pass,
// which every iteration runs whatever the decision. The per-pass kernels'
// block size pass_block fixes how the error terms are summed, and the
// decision rebuilds that sum exactly: the error terms of every 32 consecutive
// particles are summed with block_sum_dyn's warp shuffle tree into wsums;
// after the barrier the decision warp rebuilds the per-pass partials from them
// (each the sum of its pass_block / 32 warp sums in warp order) and adds those
// in finish_reduction's order (lane_sums_total). The error sum, and with it the iteration
// count, is therefore the per-pass solve's bit for bit, and all blocks take the
// same decision. Records written inside the launch are read with ld_coh; a
// block whose stencils read at most stage_cap consecutive slots copies them
// into shared memory once per pass (dynamic shared memory: 2 x stage_cap
// records).
constexpr int JACOBI_SOLVE_MAX_BLOCKS = 256;
template <class R, bool DIV, int P>
__global__ void __launch_bounds__(4 * P + 32) jacobi_solve_kernel(
    int n, R4<R>* xa, R4<R>* xb, R4<R>* vr, const R* __restrict__ alpha, R* rho_adv, R* kap,
    const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, BoundaryDev bd, StepDt<R> sd, double* wsums,
    IterCtl* ctl, u32 max_iters, u32 first_check, StopTest rule, u32 stage_cap,
    u32 wall_cap, u32 pass_block, WaitCfg wait) {
    static_assert(P % 32 == 0, "whole warps of particles");
    constexpr int W = 4 * P;  // particle lanes
    extern __shared__ __align__(16) unsigned char jacobi_stage[];
    R4<R>* sx = reinterpret_cast<R4<R>*>(jacobi_stage);
    R4<R>* sv = sx + stage_cap;
    R4<R>* swx = sv + stage_cap;  // wall records, staged once per launch
    __shared__ double part[REDUCE_SERIAL_MAX];  // the decision's partials, when added by one lane
    __shared__ double errs[P];
    __shared__ int stop;
    __shared__ u32 span_lo, span_hi;
    __shared__ u32 run_b[9 * P], run_e[9 * P];
    __shared__ u32 wrun_b[9 * P], wrun_e[9 * P];
    __shared__ u32 wspan_lo, wspan_hi;
    __shared__ int bar_ok;
    u32 bar_k = 0;  // grid barriers passed
    // threads W .. W + 31: the decision warp
    const bool worker = threadIdx.x < W;
    // a barrier of the particle lanes alone (named barrier 1)
    auto workers_sync = [] { asm volatile("bar.sync 1, %0;" ::"r"(W) : "memory"); };
    const R dt = step_dt(sd);
    const int pl = int(threadIdx.x >> 2);  // particle of the block (workers)
    const int q = int(threadIdx.x & 3u);
    const unsigned qmask = 0xFu << (threadIdx.x & 28u);
    const int i = worker ? int(blockIdx.x) * P + pl : n;
    const u32 n_warps = (static_cast<u32>(n) + 31u) / 32u;
    const u32 wpb = pass_block / 32u;                     // warps per per-pass block
    const u32 n_pass = (n_warps + wpb - 1u) / wpb;        // per-pass blocks
    // the slot range [lo, hi) that this block's stencils read (the grid does
    // not change during the solve); staged in shared memory when it fits
    if (threadIdx.x == 0) {
        span_lo = 0xFFFFFFFFu;
        span_hi = 0u;
        wspan_lo = 0xFFFFFFFFu;
        wspan_hi = 0u;
        stop = 0;
    }
    __syncthreads();
    if (worker && q == 0) {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            run_b[k * P + pl] = 0u;
            run_e[k * P + pl] = 0u;
            wrun_b[k * P + pl] = 0u;
            wrun_e[k * P + pl] = 0u;
        }
    }
    if (q == 0 && i < n) {
        const R4<R> pi = ld_coh(xa + i);
        u32 lo = 0xFFFFFFFFu, hi = 0u;
        int k = 0;  // runs come in column order; empty and off-grid ones are skipped
        for_each_run(stencil_centre(pi.x, pi.y, pi.z, g), g, cs + scene_of(g, i) * g.cells1, [&](u32 b, u32 e) {
            if (b < e) {
                run_b[k * P + pl] = b;
                run_e[k * P + pl] = e;
                ++k;
                lo = min(lo, b);
                hi = max(hi, e);
            }
        });
        if (hi > lo) {
            atomicMin(&span_lo, lo);
            atomicMax(&span_hi, hi);
        }
        // the wall runs of a particle near the walls (they never change)
        const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
        if (bd.has && boundary_near(c, g, bd.mask)) {
            u32 wl = 0xFFFFFFFFu, wh = 0u;
            int kw = 0;
            for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
                if (b < e) {
                    wrun_b[kw * P + pl] = b;
                    wrun_e[kw * P + pl] = e;
                    ++kw;
                    wl = min(wl, b);
                    wh = max(wh, e);
                }
            });
            if (wh > wl) {
                atomicMin(&wspan_lo, wl);
                atomicMax(&wspan_hi, wh);
            }
        }
    }
    __syncthreads();
    const u32 wlo = wspan_lo, whi = wspan_hi;
    const bool wstaged = whi > wlo && whi - wlo <= wall_cap;
    if (wstaged && worker) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        for (u32 k = threadIdx.x; k < whi - wlo; k += W) swx[k] = ld(xb + wlo + k);
    }
    __syncthreads();
    const u32 lo = span_lo, hi = span_hi;
    const bool staged = hi > lo && hi - lo <= stage_cap;
    const u32 count = staged ? hi - lo : 0u;
    NbrSrc<R> src;
    if (worker) {
        src.rb = run_b + pl;
        src.re = run_e + pl;
        src.stride = P;
        src.wrb = wrun_b + pl;
        src.wre = wrun_e + pl;
        src.wx = wstaged ? swx : nullptr;
        src.wlo = wlo;
        if (staged) {
            src.x = sx;
            src.v = sv;
            src.lo = lo;
        }
    }
    u32 it = 0;
    while (it < max_iters) {
        const R4<R>* xin = (it & 1u) ? xb : xa;
        R4<R>* xout = (it & 1u) ? xa : xb;
        if (worker) {
            if (staged) {
                for (u32 k = threadIdx.x; k < count; k += W) {
                    sx[k] = ld_coh(xin + lo + k);
                    sv[k] = ld_coh(vr + lo + k);
                }
                workers_sync();
            }
            double err = 0;
            if (i < n)
                err = rate_particle_quad<R, DIV>(i, q, qmask, xin, xout, vr, alpha, rho_adv, kap, g, p, bd, dt,
                                                 src);
            if (q == 0) errs[pl] = err;
            workers_sync();
            if (threadIdx.x < P) {
                // the warp's share of block_sum_dyn over 32 consecutive
                // particles: the same shuffle tree
                double e = errs[threadIdx.x];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
                const u32 warp = (blockIdx.x * P + threadIdx.x) >> 5;
                if ((threadIdx.x & 31) == 0 && warp < n_warps) wsums[warp] = e;
            }
        }
        if (!grid_barrier(&ctl->bar_arrive, bar_k++, wait, &bar_ok)) return;
        if (!worker) {
            // the decision: the per-pass partials, each from its warps' sums
            // in warp order (warps past the last particle add +0 there),
            // added in finish_reduction's order (lane_sums_total)
            const u32 lane = threadIdx.x - W;
            double s = 0;
            if (n_pass <= REDUCE_SERIAL_MAX) {
                for (u32 b = lane; b < n_pass; b += 32) {
                    const u32 w0 = b * wpb, w1 = min(w0 + wpb, n_warps);
                    double t = 0;
                    for (u32 w = w0; w < w1; ++w) t += __ldcg(wsums + w);
                    part[b] = t;
                }
                __syncwarp();
                if (lane == 0)
                    for (u32 b = 0; b < n_pass; ++b) s += part[b];
            } else {
                for (u32 b = lane; b < n_pass; b += 32) {
                    const u32 w0 = b * wpb, w1 = min(w0 + wpb, n_warps);
                    double t = 0;
                    for (u32 w = w0; w < w1; ++w) t += __ldcg(wsums + w);
                    s += t;
                }
                s = lane_sums_total(s);
            }
            if (lane == 0) {
                const bool done = it >= first_check && below_threshold(s, rule);
                stop = done ? 1 : 0;
                if (blockIdx.x == 0) {
                    ctl->err_sum = s;
                    if (done) ctl->stop_iter = it;
                    if (!(s == s)) ctl->flags |= 1u;
                }
            }
        } else {
            if (staged) {
                // the block's rate pass finished reading sx, sv before the barrier
                for (u32 k = threadIdx.x; k < count; k += W) sx[k] = ld_coh(xout + lo + k);
                workers_sync();
            }
            if (i < n) {
                const R4<R> v = apply_velocity_quad(i, q, qmask, xout, vr, kap, g, p, bd, dt, src);
                if (q == 0) vr[i] = v;
            }
        }
        ++it;
        // velocities complete before the next rate pass; stop visible
        if (!grid_barrier(&ctl->bar_arrive, bar_k++, wait, &bar_ok)) return;
        if (stop != 0) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->iters = it;
}

// ---------------------------------------------------------------------------
// Integrator (advect_kernel dfsph_kernels.cu:363-386, MAX_VELOCITY_CLAMP = 5,
// dfsph.cu:268) fused with the max-|v| reduction (dfsph.cu:303-326) and, when
// COUNT, the next step's cell keys and per-cell counts. Positions are read
// from xk and written to xk_out (the same buffer, or the other one when that
// returns the position buffers to where the step found them).
// ---------------------------------------------------------------------------
template <class R> struct Domain {
    R lox, loy, loz, hix, hiy, hiz;
};

__device__ __forceinline__ float add_r(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_r(double a, double b) { return __dadd_rn(a, b); }

// x + dx with the rounding error of earlier updates carried in c (Kahan
// summation over the steps): the position in the working type stays the
// rounded sum, c holds what that rounding dropped, and the next update adds
// it back. Every operation is written as an explicit rounding.
template <class R> __device__ __forceinline__ R compensated_add(R x, R dx, R& c) {
    const R y = sub_r(dx, c);
    const R t = add_r(x, y);
    c = sub_r(sub_r(t, x), y);
    return t;
}

// One particle of the integrator: writes v and x (to xk_out), the next
// step's cell key and rank when COUNT, the clamp mask when recording; returns
// the bits of |v| (non-negative floats order as integers). COMP: the position
// update is compensated (DFSPH_PRECISION_FP32_COMPENSATED), its carries kept
// per particle in xc in the original particle order (id = original index of
// slot i); a clamped component restarts its carry at zero.
template <class R, bool COUNT, bool MORTON = false, bool COMP = false>
__device__ __forceinline__ u32 integrate_particle(int i, R4<R> v, const R4<R>& x, R dt, const Domain<R>& d,
                                                  const GridDev<R>& g, R4<R>* __restrict__ vr, R4<R>* xk_out,
                                                  u32* __restrict__ key, u32* __restrict__ rank,
                                                  u32* __restrict__ count, unsigned char* __restrict__ tape_mask,
                                                  const u32* __restrict__ id, R4<R>* __restrict__ xc, u32& klo,
                                                  u32& khi) {
    // mask bits (recorded for the adjoint): 0-2 position clamped on x/y/z,
    // 3-5 velocity component zeroed, 6 speed clamped
    u32 mk = 0;
    const R maxv = R(5);
    const R sp = sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    if (sp > maxv) {
        const R s = maxv / sp;
        v.x *= s; v.y *= s; v.z *= s;
        mk |= 64u;
    }
    R px, py, pz;
    R4<R> c{};
    u32 oid = 0;
    if constexpr (COMP) {
        oid = id[i];
        c = xc[oid];
        px = compensated_add(x.x, mul_r(v.x, dt), c.x);
        py = compensated_add(x.y, mul_r(v.y, dt), c.y);
        pz = compensated_add(x.z, mul_r(v.z, dt), c.z);
    } else {
        px = x.x + v.x * dt;
        py = x.y + v.y * dt;
        pz = x.z + v.z * dt;
    }
    const R eps = R(1e-3);
    if (px < d.lox + eps) { px = d.lox + eps; mk |= 1u; if (v.x < R(0)) { v.x = R(0); mk |= 8u; } }
    if (py < d.loy + eps) { py = d.loy + eps; mk |= 2u; if (v.y < R(0)) { v.y = R(0); mk |= 16u; } }
    if (pz < d.loz + eps) { pz = d.loz + eps; mk |= 4u; if (v.z < R(0)) { v.z = R(0); mk |= 32u; } }
    if (px > d.hix - eps) { px = d.hix - eps; mk |= 1u; if (v.x > R(0)) { v.x = R(0); mk |= 8u; } }
    if (py > d.hiy - eps) { py = d.hiy - eps; mk |= 2u; if (v.y > R(0)) { v.y = R(0); mk |= 16u; } }
    if (pz > d.hiz - eps) { pz = d.hiz - eps; mk |= 4u; if (v.z > R(0)) { v.z = R(0); mk |= 32u; } }
    if constexpr (COMP) {
        if (mk & 1u) c.x = R(0);
        if (mk & 2u) c.y = R(0);
        if (mk & 4u) c.z = R(0);
        xc[oid] = c;
    }
    if (tape_mask) tape_mask[i] = static_cast<unsigned char>(mk);
    vr[i] = {v.x, v.y, v.z, v.w};
    xk_out[i] = {px, py, pz, R(0)};
    if (COUNT) {
        const u32 k = sort_key<MORTON>(g, cell_key(px, py, pz, g)) + scene_of(g, i) * g.cells1;
        key[i] = k;
        rank[i] = atomicAdd(count + k, 1u);
        key_bounds(k, g.cells1, klo, khi);
    }
    return __float_as_uint(float(sqrt(v.x * v.x + v.y * v.y + v.z * v.z)));
}

// Max |v| of the block's particles: per scene (lanes of one scene are
// contiguous slots; their lowest lane does the one atomic) and overall (one
// atomic per block into one of MAXV_SLOTS words, since one word for every
// block serialises the atomics in L2). NaN bits dominate every finite
// magnitude. Every thread of the block calls it.
template <int BLOCK>
__device__ __forceinline__ void max_velocity_epilogue(bool valid, u32 vbits, u32 scene, IterCtl* ctl,
                                                      u32* __restrict__ maxv_scene) {
    __shared__ u32 wmax[BLOCK / 32];
    if (maxv_scene) {
        const u32 peers = __match_any_sync(0xffffffffu, scene);
        const u32 m = __reduce_max_sync(peers, vbits);
        if (valid && (threadIdx.x & 31) == __ffs(peers) - 1 && m) atomicMax(maxv_scene + scene, m);
    }
    const u32 m = __reduce_max_sync(0xffffffffu, vbits);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        u32 b = 0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) b = max(b, wmax[w]);
        if (b) atomicMax(&ctl->maxv_slot[blockIdx.x % MAXV_SLOTS], b);
    }
}

template <class R, bool COUNT, bool MORTON = false, bool COMP = false>
__global__ void __launch_bounds__(256) advect_kernel(
    int n, const R4<R>* xk, R4<R>* xk_out, R4<R>* __restrict__ vr, StepDt<R> sd, Domain<R> d, GridDev<R> g,
    u32* __restrict__ key, u32* __restrict__ rank, u32* __restrict__ count, IterCtl* ctl,
    u32* __restrict__ maxv_scene, R4<R>* __restrict__ tape_v, unsigned char* __restrict__ tape_mask,
    const u32* __restrict__ id, R4<R>* __restrict__ xc, u32* __restrict__ krange) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const R dt = step_dt(sd);
    u32 vbits = 0;
    u32 scene = 0xffffffffu;  // lanes past the end form their own group
    u32 klo = ~0u, khi = 0u;
    if (i < n) {
        const R4<R> v = vr[i];
        if (tape_v) tape_v[i] = v;
        vbits = integrate_particle<R, COUNT, MORTON, COMP>(i, v, xk[i], dt, d, g, vr, xk_out, key, rank, count,
                                                           tape_mask, id, xc, klo, khi);
        scene = scene_of(g, i);
    }
    max_velocity_epilogue<256>(i < n, vbits, scene, ctl, maxv_scene);
    if (COUNT && krange) key_range_block<256>(klo, khi, krange);
}

// The last apply pass of a fixed-iteration density solve fused with the
// integrator: the particle's new velocity goes straight into the integrator
// (same values as the two passes: the apply pass's velocity, positions from
// the same buffer). xk_out is the other position buffer, which nothing in
// this pass reads.
template <class R, bool COUNT, int LB, bool MORTON = false, bool COMP = false>
__global__ void __launch_bounds__(LB, fp32_min_blocks<R>(LB)) apply_advect_kernel(
    int n, const R4<R>* __restrict__ xk, R4<R>* xk_out, R4<R>* __restrict__ vr, const R* __restrict__ kap,
    const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, BoundaryDev bd, StepDt<R> sd, Domain<R> d,
    u32* __restrict__ key, u32* __restrict__ rank, u32* __restrict__ count, IterCtl* ctl,
    u32* __restrict__ maxv_scene, const u32* __restrict__ id, R4<R>* __restrict__ xc,
    u32* __restrict__ krange) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const R dt = step_dt(sd);
    u32 vbits = 0;
    u32 scene = 0xffffffffu;
    u32 klo = ~0u, khi = 0u;
    if (i < n) {
        const R4<R> v = apply_velocity<R, MORTON>(i, xk, vr, kap, cs, g, p, bd, dt);
        vbits = integrate_particle<R, COUNT, MORTON, COMP>(i, v, ld(xk + i), dt, d, g, vr, xk_out, key, rank,
                                                           count, nullptr, id, xc, klo, khi);
        scene = scene_of(g, i);
    }
    max_velocity_epilogue<LB>(i < n, vbits, scene, ctl, maxv_scene);
    if (COUNT && krange) key_range_block<LB>(klo, khi, krange);
}

}  // namespace dfsph
