// Reverse-mode derivative (adjoint) of one DFSPH step. The reference has no
// differentiable path; this is the hand-written adjoint of the step that
// kernels.cuh computes, with the iteration counts of both Jacobi solvers fixed.
//
// Forward step, per particle i in the step's sorted order (j over the 27-cell
// stencil, self included; b over wall particles; gradW_ij = F(r) r_ij):
//   rho_i  = m sum_j W_ij + sum_b m_b W_ib
//   G_i    = m sum_j gradW_ij + sum_b m_b gradW_ib      Bg_i = the wall part of G_i
//   den_i  = |G_i|^2 + m^2 sum_j |gradW_ij|^2 + sum_b m_b^2 |gradW_ib|^2
//   alpha_i = rho_i / den_i                              (0 when den_i <= 1e-9)
//   per solver iteration (divergence: K_d, density: K_rho):
//     rd_i  = m sum_j (v_i - v_j).gradW_ij + v_i.Bg_i
//     kappa_i = max(rd_i, 0) alpha_i / dt                      (divergence)
//             = max(rho_i + dt rd_i - rho0, 0) alpha_i / dt^2  (density)
//     kf_i  = kappa_i / max(rho_i^2, 1e-9)
//     v_i  -= dt m sum_j (kf_i + kf_j) gradW_ij + dt (kf_i + kappa_i / rho0^2) Bg_i
//   XSPH between the solvers:
//     v_i' = d v_i + g dt + eps m d sum_j W_ij / max((rho_i + rho_j) / 2, 1e-9) (v_j - v_i)
//   integrator: speed clamp at 5 m/s, x += v dt, per-axis domain clamps.
//
// The pair sets are symmetric (j in the stencil of i exactly when i is in the
// stencil of j, the stencil being the cells around each particle's own cell),
// so every transposed scatter of the forward pass is evaluated here as a gather
// over the same stencil and no atomics are needed. With
// J(r) = dgradW/dr = F I + D r r^T, D = F'(r)/r, the adjoints are:
//   apply:   kf_bar_i  = -dt (m sum_j F (vb_i - vb_j).r + vb_i.Bg_i)
//            x_bar_i  += -dt m sum_j (kf_i + kf_j) J (vb_i - vb_j) - dt (kf_i + kappa_i/rho0^2) sum_b m_b J vb_i
//            kappa_bar = kf_bar / max(rho^2, 1e-9) - dt/rho0^2 vb_i.Bg_i, rho_bar_i += -2 kf_bar_i kf_i / rho_i
//            then through max(.,0) with the active set of the forward pass
//   rate:    v_bar_i  += m sum_j (rdb_i + rdb_j) gradW_ij + rdb_i Bg_i
//            x_bar_i  += m sum_j (rdb_i + rdb_j) J (v_i - v_j) + rdb_i sum_b m_b J v_i
//   XSPH:    v_bar_i   = d vb_i + eps m d sum_j c_ij (vb_j - vb_i),  c_ij = W_ij / rho_ij
//            x_bar_i  += eps m d sum_j F r (vb_i - vb_j).(v_j - v_i) / rho_ij
//            rho_bar_i += -eps m d / 2 sum_j W (vb_i - vb_j).(v_j - v_i) / rho_ij^2
//            eps_bar  += m d sum_i vb_i . sum_j c_ij (v_j - v_i)          (FP64)
//   density: x_bar_i  += m sum_j (rb_i + rb_j) gradW + rb_i Bg_i
//                      + m sum_j J (Gb_i - Gb_j) + sum_b m_b J Gb_i
//                      + 2 m^2 sum_j (Qb_i + Qb_j) F (F + D r^2) r + 2 Qb_i sum_b m_b^2 F (F + D r^2) r
//            with Gb = 2 den_bar G, Qb = den_bar, den_bar = -alpha_bar alpha / den.
// Self pairs have r = 0 and every term above vanishes for them.
#pragma once

#include "kernels.cuh"

namespace dfsph {

// F(r) and D(r) = F'(r) / r per branch of the cubic spline (see "Pair terms"):
//   r <  l :  F = gA r + gB               F' = gA
//   r >= l :  F = gC (2l - r)^2 / r       F' = -gC (2l - r)(2l + r) / r^2
template <class R> __device__ __forceinline__ void grad_factor_jac(R r, R rinv, const Phys<R>& p, R& F, R& D) {
    const R t = rmax(p.two_l - r, R(0));
    const R fo = p.gC * t * t * rinv;
    const R dov = -p.gC * t * (p.two_l + r) * rinv * rinv * rinv;
    const bool in = r < p.l;
    F = in ? p.gA * r + p.gB : fo;
    D = in ? p.gA * rinv : dov;
}

// Per-step records of a replayed segment (sorted order of the step).
template <class R> struct StepTape {
    R4<R>* x;               // (x, y, z, rho)
    R4<R>* g;               // (G, den)
    u32* id;                // slot -> original index
    u32* cs;                // cell_start of the step
    R4<R>* vx;              // velocity entering XSPH (w = rho)
    R4<R>* va;              // velocity entering the integrator
    unsigned char* amask;   // integrator clamp bits
    R4<R>* xkf[2];          // per solver (0 divergence, 1 density): (x, kf) of iteration k at + k * stride
    R4<R>* v[2];            // velocity entering iteration k (w = rho)
    R* kap[2];              // kappa of iteration k
    R* adv[2];              // rd (divergence) or rho* (density) of iteration k
    size_t stride;
};

// Integrator: gathers the adjoint of the step's output state (original order)
// into the step's sorted order and takes it through the clamps.
template <class R>
__global__ void __launch_bounds__(256) adjoint_advect_kernel(
    int n, const u32* __restrict__ id, const R4<R>* __restrict__ va, const unsigned char* __restrict__ amask, R dt,
    const R4<R>* __restrict__ xg, const R4<R>* __restrict__ vg, R4<R>* __restrict__ xbar, R4<R>* __restrict__ vbar,
    R* __restrict__ rhobar, R* __restrict__ alphabar) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const u32 o = id[i];
    const R4<R> xo = xg[o];
    const R4<R> vo = vg[o];
    const u32 m = amask[i];
    R ux = (m & 8u) ? R(0) : vo.x;
    R uy = (m & 16u) ? R(0) : vo.y;
    R uz = (m & 32u) ? R(0) : vo.z;
    if (!(m & 1u)) ux += dt * xo.x;
    if (!(m & 2u)) uy += dt * xo.y;
    if (!(m & 4u)) uz += dt * xo.z;
    xbar[i] = {(m & 1u) ? R(0) : xo.x, (m & 2u) ? R(0) : xo.y, (m & 4u) ? R(0) : xo.z, R(0)};
    if (m & 64u) {
        // u = 5 v / |v|:  du/dv = (5 / |v|) (I - vh vh^T)
        const R4<R> v = va[i];
        const R sp = sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        const R hx = v.x / sp, hy = v.y / sp, hz = v.z / sp;
        const R d = hx * ux + hy * uy + hz * uz;
        const R s = R(5) / sp;
        ux = s * (ux - hx * d);
        uy = s * (uy - hy * d);
        uz = s * (uz - hz * d);
    }
    vbar[i] = {ux, uy, uz, R(0)};
    rhobar[i] = R(0);
    alphabar[i] = R(0);
}

// Sum of a value over the L lanes (consecutive, L a power of two) that share a
// particle, by a fixed butterfly: every lane ends with the same bits.
template <int L, class T> __device__ __forceinline__ T lane_sum(T v) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Adjoint of the apply half of one Jacobi iteration plus the pointwise part of
// its rate half. Reads vbar (adjoint of the iteration's output velocity, which
// is also the adjoint of its input through the identity), writes the rate
// adjoint rdb into xr = (x, rdb) and accumulates x_bar, rho_bar, alpha_bar.
// L lanes per particle (1, or 2 for scenes small enough that one lane per
// particle leaves most SMs idle): lane q takes candidates b + q, b + q + L, ...
// of every run, and the lanes' partial sums are added by lane_sum.
template <class R, bool DIVERGENCE, int L>
__global__ void __launch_bounds__(128) adjoint_apply_kernel(
    int n, const R4<R>* __restrict__ xkf, const R4<R>* __restrict__ tx, const R4<R>* __restrict__ tg,
    const R* __restrict__ kap, const R* __restrict__ adv, const R4<R>* __restrict__ vbar,
    const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, BoundaryDev bd, R dt, R4<R>* __restrict__ xbar,
    R* __restrict__ rhobar, R* __restrict__ alphabar, R4<R>* __restrict__ xr) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / L;
    const u32 q = u32(t % L);
    if (L == 1 && i >= n) return;
    const bool valid = i < n;
    const int ii = valid ? i : 0;
    const R4<R> pi = ld(xkf + ii);
    const R4<R> vb = ld(vbar + ii);
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    R s1 = 0, X = 0, Y = 0, Z = 0;
    if (valid) for_each_run(c, g, cs + scene_of(g, ii) * g.cells1, [&](u32 b, u32 e) {
        for (u32 j = b + q; j < e; j += L) {
            const R4<R> pj = ld(xkf + j);
            const R4<R> wj = ld(vbar + j);
            const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            R rinv;
            const R r = pair_r(rx * rx + ry * ry + rz * rz, rinv);
            R F, D;
            grad_factor_jac(r, rinv, p, F, D);
            const R dx = vb.x - wj.x, dy = vb.y - wj.y, dz = vb.z - wj.z;
            const R rdv = rx * dx + ry * dy + rz * dz;
            s1 += F * rdv;
            const R cf = pi.w + pj.w;
            const R t = D * rdv;
            X += cf * (F * dx + t * rx);
            Y += cf * (F * dy + t * ry);
            Z += cf * (F * dz + t * rz);
        }
    });
    R bgv = 0, JX = 0, JY = 0, JZ = 0;
    if (valid && bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
            for (u32 j = b + q; j < e; j += L) {
                const R4<R> pj = ld(xb + j);
                const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
                R rinv;
                const R r = pair_r(rx * rx + ry * ry + rz * rz, rinv);
                R F, D;
                grad_factor_jac(r, rinv, p, F, D);
                const R rv = rx * vb.x + ry * vb.y + rz * vb.z;
                bgv += pj.w * F * rv;
                const R t = D * rv;
                JX += pj.w * (F * vb.x + t * rx);
                JY += pj.w * (F * vb.y + t * ry);
                JZ += pj.w * (F * vb.z + t * rz);
            }
        });
    }
    if (L > 1) {
        s1 = lane_sum<L>(s1); X = lane_sum<L>(X); Y = lane_sum<L>(Y); Z = lane_sum<L>(Z);
        bgv = lane_sum<L>(bgv); JX = lane_sum<L>(JX); JY = lane_sum<L>(JY); JZ = lane_sum<L>(JZ);
        if (!valid || q != 0) return;
    }
    const R kfb = -dt * (p.mass * s1 + bgv);
    const R kap_i = kap[i];
    const R rho0sq = rmax(p.rho0 * p.rho0, R(1e-9));
    const R sa = -dt * p.mass;
    const R sb = -dt * (pi.w + kap_i / rho0sq);
    R4<R> xo = xbar[i];
    xo.x += sa * X + sb * JX;
    xo.y += sa * Y + sb * JY;
    xo.z += sa * Z + sb * JZ;
    xbar[i] = xo;
    const R4<R> ti = tx[i];
    const R rho = ti.w;
    const R rho2 = rho * rho;
    const R kb = kfb / rmax(rho2, R(1e-9)) - dt / rho0sq * bgv;
    R rb = rho2 > R(1e-9) ? R(-2) * kfb * pi.w / rho : R(0);
    const R den = tg[i].w;
    const R alpha = den > R(1e-9) ? rho / den : R(0);
    R ab, rdb;
    if (!DIVERGENCE) {
        const R rs = adv[i];
        const R over = rmax(rs - p.rho0, R(0));
        const R idt2 = R(1) / (dt * dt);
        ab = kb * over * idt2;
        const R rsb = rs > p.rho0 ? kb * alpha * idt2 : R(0);
        rb += rsb;
        rdb = dt * rsb;
    } else {
        const R rd = adv[i];
        const R s = rmax(rd, R(0));
        ab = kb * s / dt;
        rdb = rd > R(0) ? kb * alpha / dt : R(0);
    }
    rhobar[i] += rb;
    alphabar[i] += ab;
    xr[i] = {pi.x, pi.y, pi.z, rdb};
}

// Adjoint of the rate half's neighbour sum: adds to v_bar and x_bar. L lanes
// per particle as in adjoint_apply_kernel.
template <class R, int L>
__global__ void __launch_bounds__(128) adjoint_rate_kernel(
    int n, const R4<R>* __restrict__ xr, const R4<R>* __restrict__ vel, const u32* __restrict__ cs, GridDev<R> g,
    Phys<R> p, BoundaryDev bd, R4<R>* __restrict__ vbar, R4<R>* __restrict__ xbar) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / L;
    const u32 q = u32(t % L);
    if (L == 1 && i >= n) return;
    const bool valid = i < n;
    const int ii = valid ? i : 0;
    const R4<R> pi = ld(xr + ii);
    const R4<R> vi = ld(vel + ii);
    const Centre c = stencil_centre(pi.x, pi.y, pi.z, g);
    R VX = 0, VY = 0, VZ = 0, X = 0, Y = 0, Z = 0;
    if (valid) for_each_run(c, g, cs + scene_of(g, ii) * g.cells1, [&](u32 b, u32 e) {
        for (u32 j = b + q; j < e; j += L) {
            const R4<R> pj = ld(xr + j);
            const R4<R> vj = ld(vel + j);
            const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            R rinv;
            const R r = pair_r(rx * rx + ry * ry + rz * rz, rinv);
            R F, D;
            grad_factor_jac(r, rinv, p, F, D);
            const R cf = pi.w + pj.w;
            const R cF = cf * F;
            VX += cF * rx; VY += cF * ry; VZ += cF * rz;
            const R dx = vi.x - vj.x, dy = vi.y - vj.y, dz = vi.z - vj.z;
            const R t = cf * D * (rx * dx + ry * dy + rz * dz);
            X += cF * dx + t * rx;
            Y += cF * dy + t * ry;
            Z += cF * dz + t * rz;
        }
    });
    R BX = 0, BY = 0, BZ = 0, JX = 0, JY = 0, JZ = 0;
    if (valid && bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
            for (u32 j = b + q; j < e; j += L) {
                const R4<R> pj = ld(xb + j);
                const R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
                R rinv;
                const R r = pair_r(rx * rx + ry * ry + rz * rz, rinv);
                R F, D;
                grad_factor_jac(r, rinv, p, F, D);
                const R mF = pj.w * F;
                BX += mF * rx; BY += mF * ry; BZ += mF * rz;
                const R t = pj.w * D * (rx * vi.x + ry * vi.y + rz * vi.z);
                JX += mF * vi.x + t * rx;
                JY += mF * vi.y + t * ry;
                JZ += mF * vi.z + t * rz;
            }
        });
    }
    if (L > 1) {
        VX = lane_sum<L>(VX); VY = lane_sum<L>(VY); VZ = lane_sum<L>(VZ);
        X = lane_sum<L>(X); Y = lane_sum<L>(Y); Z = lane_sum<L>(Z);
        BX = lane_sum<L>(BX); BY = lane_sum<L>(BY); BZ = lane_sum<L>(BZ);
        JX = lane_sum<L>(JX); JY = lane_sum<L>(JY); JZ = lane_sum<L>(JZ);
        if (!valid || q != 0) return;
    }
    const R rdb = pi.w;
    R4<R> vo = vbar[i];
    vo.x += p.mass * VX + rdb * BX;
    vo.y += p.mass * VY + rdb * BY;
    vo.z += p.mass * VZ + rdb * BZ;
    vbar[i] = vo;
    R4<R> xo = xbar[i];
    xo.x += p.mass * X + rdb * JX;
    xo.y += p.mass * Y + rdb * JY;
    xo.z += p.mass * Z + rdb * JZ;
    xbar[i] = xo;
}

// Adds a block's FP64 partial (valid in thread 0) into *acc; called by every
// thread of a 128-thread block. The last block to finish adds the partials
// with all its threads, each a fixed stride of blocks, then a block sum: a
// fixed order, so the result does not depend on scheduling (and the last
// block's tail is a few strided loads, not one load per block in sequence).
static __device__ __forceinline__ void accumulate_partial(double partial, double* partials, u32* counter,
                                                          double* acc, double* sh) {
    __shared__ int last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = partial;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0;
    for (u32 b = threadIdx.x; b < gridDim.x; b += 128) s += *((volatile const double*)&partials[b]);
    s = block_sum<128>(s, sh);
    if (threadIdx.x == 0) {
        *acc += s;
        *counter = 0;
    }
}

// 1 / b as the forward XSPH pass forms its quotient w / b (fast_div): the
// approximate reciprocal in FP32, so that w * rcp_as_forward(b) is the
// forward's bits, and a division in FP64.
__device__ __forceinline__ float rcp_as_forward(float b) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
    return r;
}
__device__ __forceinline__ double rcp_as_forward(double b) { return 1.0 / b; }

// Adjoint of gravity + damping + XSPH (forces_xsph_kernel).
template <class R>
__global__ void __launch_bounds__(128) adjoint_xsph_kernel(
    int n, const R4<R>* __restrict__ tx, const R4<R>* __restrict__ vx, const R4<R>* __restrict__ vbar_in,
    R4<R>* __restrict__ vbar_out, const u32* __restrict__ cs, GridDev<R> g, Phys<R> p, R damping, R dt, R eps,
    R4<R>* __restrict__ xbar, R* __restrict__ rhobar, double* __restrict__ partials, u32* counter,
    double* eps_acc) {
    pdl_wait();
    const R decay = damping_decay(damping, dt);  // the forward pass's factor
    __shared__ double sh[4];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double part = 0;
    if (i < n) {
        const R4<R> xi = ld(tx + i);
        const R4<R> vi = ld(vx + i);
        const R4<R> wi = ld(vbar_in + i);
        const Centre c = stencil_centre(xi.x, xi.y, xi.z, g);
        R AX = 0, AY = 0, AZ = 0, EX = 0, EY = 0, EZ = 0, X = 0, Y = 0, Z = 0, P = 0;
        for_each_run(c, g, cs + scene_of(g, i) * g.cells1, [&](u32 b, u32 e) {
            for (u32 j = b; j < e; ++j) {
                const R4<R> xj = ld(tx + j);
                const R4<R> vj = ld(vx + j);
                const R4<R> wj = ld(vbar_in + j);
                const R rx = xi.x - xj.x, ry = xi.y - xj.y, rz = xi.z - xj.z;
                R rinv;
                const R r = pair_r(rx * rx + ry * ry + rz * rz, rinv);
                const R w = kernel_w(r, p);
                const R f = grad_factor(r, rinv, p);
                const R ra = R(0.5) * (vi.w + vj.w);
                const R inv = rcp_as_forward(rmax(ra, R(1e-9)));
                const R cc = w * inv;
                AX += cc * (wj.x - wi.x); AY += cc * (wj.y - wi.y); AZ += cc * (wj.z - wi.z);
                const R ux = vj.x - vi.x, uy = vj.y - vi.y, uz = vj.z - vi.z;
                EX += cc * ux; EY += cc * uy; EZ += cc * uz;
                const R q = (wi.x - wj.x) * ux + (wi.y - wj.y) * uy + (wi.z - wj.z) * uz;
                const R fq = f * inv * q;
                X += fq * rx; Y += fq * ry; Z += fq * rz;
                if (ra > R(1e-9)) P += cc * inv * q;
            }
        });
        const R s = eps * p.mass * decay;
        vbar_out[i] = {decay * wi.x + s * AX, decay * wi.y + s * AY, decay * wi.z + s * AZ, R(0)};
        R4<R> xo = xbar[i];
        xo.x += s * X; xo.y += s * Y; xo.z += s * Z;
        xbar[i] = xo;
        rhobar[i] += R(-0.5) * s * P;
        part = double(p.mass) * double(decay) *
               (double(wi.x) * double(EX) + double(wi.y) * double(EY) + double(wi.z) * double(EZ));
    }
    const double t = block_sum<128>(part, sh);
    accumulate_partial(t, partials, counter, eps_acc, sh);
}

// alpha = rho / den: folds alpha_bar into rho_bar and the adjoints of G and of
// the squared-gradient sum, packed for the density gather.
template <class R>
__global__ void __launch_bounds__(256) adjoint_density_prep_kernel(
    int n, const R4<R>* __restrict__ tx, const R4<R>* __restrict__ tg, const R* __restrict__ rhobar,
    const R* __restrict__ alphabar, R4<R>* __restrict__ xq, R4<R>* __restrict__ gq) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const R4<R> ti = tx[i];
    const R4<R> gi = tg[i];
    R rb = rhobar[i];
    R db = 0;
    if (gi.w > R(1e-9)) {
        const R ab = alphabar[i];
        const R alpha = ti.w / gi.w;
        rb += ab / gi.w;
        db = -ab * alpha / gi.w;
    }
    xq[i] = {ti.x, ti.y, ti.z, rb};
    gq[i] = {R(2) * db * gi.x, R(2) * db * gi.y, R(2) * db * gi.z, db};
}

// Adjoint of density + alpha with respect to the positions; finishes the step
// by scattering the adjoint of its input state to original order.
template <class R>
__global__ void __launch_bounds__(128) adjoint_density_kernel(
    int n, const R4<R>* __restrict__ xq, const R4<R>* __restrict__ gq, const R4<R>* __restrict__ vbar,
    const R4<R>* __restrict__ xbar, const u32* __restrict__ id, const u32* __restrict__ cs, GridDev<R> g, Phys<R> p,
    BoundaryDev bd, R4<R>* __restrict__ xg, R4<R>* __restrict__ vg) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const R4<R> xi = ld(xq + i);
    const R4<R> gi = ld(gq + i);
    const Centre c = stencil_centre(xi.x, xi.y, xi.z, g);
    R AX = 0, AY = 0, AZ = 0, BX = 0, BY = 0, BZ = 0, CX = 0, CY = 0, CZ = 0;
    for_each_run(c, g, cs + scene_of(g, i) * g.cells1, [&](u32 b, u32 e) {
        for (u32 j = b; j < e; ++j) {
            const R4<R> xj = ld(xq + j);
            const R4<R> gj = ld(gq + j);
            const R rx = xi.x - xj.x, ry = xi.y - xj.y, rz = xi.z - xj.z;
            const R r2 = rx * rx + ry * ry + rz * rz;
            R rinv;
            const R r = pair_r(r2, rinv);
            R F, D;
            grad_factor_jac(r, rinv, p, F, D);
            const R a = (xi.w + xj.w) * F;
            AX += a * rx; AY += a * ry; AZ += a * rz;
            const R dx = gi.x - gj.x, dy = gi.y - gj.y, dz = gi.z - gj.z;
            const R t = D * (rx * dx + ry * dy + rz * dz);
            BX += F * dx + t * rx; BY += F * dy + t * ry; BZ += F * dz + t * rz;
            const R q = (gi.w + gj.w) * F * (F + D * r2);
            CX += q * rx; CY += q * ry; CZ += q * rz;
        }
    });
    const R m = p.mass;
    R ox = m * (AX + BX) + R(2) * m * m * CX;
    R oy = m * (AY + BY) + R(2) * m * m * CY;
    R oz = m * (AZ + BZ) + R(2) * m * m * CZ;
    if (bd.has && boundary_near(c, g, bd.mask)) {
        const R4<R>* xb = static_cast<const R4<R>*>(bd.xb);
        R bx = 0, by = 0, bz = 0;
        for_each_run(c, wall_grid(g), bd.bcs, [&](u32 b, u32 e) {
            for (u32 j = b; j < e; ++j) {
                const R4<R> pj = ld(xb + j);
                const R rx = xi.x - pj.x, ry = xi.y - pj.y, rz = xi.z - pj.z;
                const R r2 = rx * rx + ry * ry + rz * rz;
                R rinv;
                const R r = pair_r(r2, rinv);
                R F, D;
                grad_factor_jac(r, rinv, p, F, D);
                const R mF = pj.w * F;
                // rho: rb_i m_b F r; G: m_b J Gb_i; squared gradients: 2 Qb_i m_b^2 F (F + D r^2) r
                const R t = pj.w * D * (rx * gi.x + ry * gi.y + rz * gi.z);
                const R q = R(2) * gi.w * pj.w * mF * (F + D * r2);
                const R s = xi.w * mF + t + q;
                bx += s * rx + mF * gi.x;
                by += s * ry + mF * gi.y;
                bz += s * rz + mF * gi.z;
            }
        });
        ox += bx; oy += by; oz += bz;
    }
    const R4<R> xa = xbar[i];
    const u32 o = id[i];
    xg[o] = {xa.x + ox, xa.y + oy, xa.z + oz, R(0)};
    vg[o] = vbar[i];
}

// Original-order state <-> packed 4-vectors of the working type.
template <class R>
__global__ void __launch_bounds__(256) pack3_kernel(int n, const R* __restrict__ a, R4<R>* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = a ? R4<R>{a[3 * i], a[3 * i + 1], a[3 * i + 2], R(0)} : R4<R>{R(0), R(0), R(0), R(0)};
}

template <class R>
__global__ void __launch_bounds__(256) unpack3_kernel(int n, const R4<R>* __restrict__ in, R* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const R4<R> v = in[i];
    out[3 * i] = v.x; out[3 * i + 1] = v.y; out[3 * i + 2] = v.z;
}

// Checkpoint of the sorted state in original order, and its restore.
template <class R>
__global__ void __launch_bounds__(256) save_state_kernel(int n, const u32* __restrict__ id,
                                                         const R4<R>* __restrict__ xk, const R4<R>* __restrict__ vr,
                                                         R4<R>* __restrict__ ox, R4<R>* __restrict__ ov) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const u32 i = id[s];
    const R4<R> x = xk[s];
    const R4<R> v = vr[s];
    ox[i] = {x.x, x.y, x.z, R(0)};
    ov[i] = {v.x, v.y, v.z, R(0)};
}

template <class R>
__global__ void __launch_bounds__(256) load_state_kernel(int n, const R4<R>* __restrict__ x,
                                                         const R4<R>* __restrict__ v, R4<R>* __restrict__ xk,
                                                         R4<R>* __restrict__ vr, u32* __restrict__ id) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    xk[i] = x[i];
    vr[i] = v[i];
    id[i] = static_cast<u32>(i);
}

}  // namespace dfsph
