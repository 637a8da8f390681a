// Device-resident loops: CFL frames and adaptive Jacobi solves stepped on the
// device. The reference's sim_cli picks every
// substep on the host after reading max |v| back (apps/sim_cli/main.cpp
// :171-181, TimeStepper::next_dt in core/include/water/core/timestep.h:23-28);
// here the same float arithmetic runs in a one-thread kernel after each
// substep, against the max |v| the integrator left in IterCtl, and a CUDA
// graph WHILE node repeats the substep until the frame is done. The
// reference's solvers read the mean error back after every iteration
// (dfsph.cu:296-299); inside a graph a WHILE node repeats rate + apply until
// the device-side convergence test stops it.
#pragma once

#include "kernels.cuh"

namespace dfsph {

// std::max / std::min as the reference evaluates them (a NaN operand
// propagates the way the comparisons do).
__device__ __forceinline__ float std_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float std_min(float a, float b) { return (b < a) ? b : a; }

// min(dt_max, lambda r / v, remaining, max(lambda r / v, frame_dt / max_substeps)),
// v = max(max |v|, 1e-6), in that order (std::min over an initializer list).
__device__ __forceinline__ float cfl_next_dt(const FrameCtl& f, float max_velocity, float remaining) {
    const float v = std_max(max_velocity, 1e-6f);
    const float dt_cfl = __fdiv_rn(__fmul_rn(f.cfl_lambda, f.radius), v);
    float m = f.dt_max;
    m = std_min(m, dt_cfl);
    m = std_min(m, remaining);
    m = std_min(m, std_max(dt_cfl, f.dt_min));
    return m;
}

__device__ __forceinline__ float read_max_velocity(const IterCtl* ctl) {
    u32 b = 0;
    for (int w = 0; w < MAXV_SLOTS; ++w) b = max(b, ((volatile const u32*)ctl->maxv_slot)[w]);
    return __uint_as_float(b);
}

// Next substep from max |v| (floored at v_floor as sim_cli does).
__device__ __forceinline__ void choose_substep(FrameCtl* f, float max_velocity) {
    const float dt = cfl_next_dt(*f, std_max(max_velocity, f->v_floor), f->remaining);
    f->dt = dt;
    f->decay_f = damping_decay(f->damping, dt);
    f->decay_d = damping_decay(double(f->damping), double(dt));
}

static __global__ void frame_begin_kernel(FrameCtl* f, const IterCtl* ctl) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    f->remaining = f->frame_dt;
    f->substeps = 0;
    choose_substep(f, f->fresh ? 0.0f : read_max_velocity(ctl));
}

// After a substep: t_remaining -= dt, ++sub, and either the next dt or the
// end of the frame. Inside the frame graph the decision goes to the WHILE
// node's condition; on the host path to f->more.
static __global__ void frame_control_kernel(FrameCtl* f, const IterCtl* ctl, cudaGraphConditionalHandle h,
                                            int use_handle) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    f->fresh = 0;
    f->remaining = f->remaining - f->dt;
    f->substeps += 1;
    const bool more = f->remaining > 1e-6f && f->substeps < f->max_per_frame;
    if (more) choose_substep(f, read_max_velocity(ctl));
    if (use_handle) cudaGraphSetConditional(h, more ? 1u : 0u);
    f->more = more ? 1u : 0u;
}

// End of one iteration of a device-resident Jacobi loop (a WHILE node around
// rate + apply): counts it and keeps the loop going while fewer than
// max_iters ran and no iteration decided to stop (finish_reduction's
// convergence test, dfsph.cu:254-258).
static __global__ void iteration_control_kernel(IterCtl* ctl, u32 max_iters, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const u32 it = ctl->iters + 1u;
    ctl->iters = it;
    const bool more = it < max_iters && *((volatile const u32*)&ctl->stop_iter) == ~0u;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

// Sets a WHILE node's condition before the node runs. A condition's default
// value is applied once per launch of the whole graph, so a loop nested in
// another loop's body (a solve inside a frame's substep) must be re-armed
// every time its parent body runs.
static __global__ void loop_arm_kernel(cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, 1u);
}

static __global__ void frame_end_kernel(FrameCtl* f) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (f->substeps_out && f->frames_done < f->max_frames) f->substeps_out[f->frames_done] = f->substeps;
    f->frames_done += 1;
}

}  // namespace dfsph
