// Adjoint (reverse-mode) RK4 over a regular-grid time-series field.
//
// Gradients of a loss of the final positions with respect to the initial
// positions and to the snapshot values.  The forward pass stores positions
// every K steps (the tracking kernel's recording); this kernel walks one
// segment backwards: it recomputes the segment's states from its checkpoint
// with the forward arithmetic into a per-thread array, then for every step
// recomputes the four stage positions and runs the RK4 reverse sweep
//     x' = B(x + h/6 (k1 + 2k2 + 2k3 + k4)),   k_i = v(x_i, t_i)
// with vector-Jacobian products of the trilinear, time-blended field
//     v(x) = sum_c w_c(x) (wa A_c + wb B_c).
// J^T g uses dw_c/dx; dL/dA_c += wa w_c g and dL/dB_c += wb w_c g go to a
// gradient buffer with the snapshot-pair record layout through vector atomics.
#include <stdint.h>

#include "jt_grid.cuh"
#include "jt_internal.h"
#include "jt_kernels.cuh"

namespace jt {

// Effective weights (ca, cb) of A and B in the blend entry: v = ca*A + cb*B.
__device__ __forceinline__ void blend_coefs(const jt_blend& e, float& ca, float& cb) {
    switch (e.form) {
        case JT_BLEND_LERP_FWD: ca = 1.0f - e.wb; cb = e.wb; break;          // A + w(B - A)
        case JT_BLEND_LERP_BWD: ca = -e.wb; cb = 1.0f + e.wb; break;         // B + w(B - A)
        case JT_BLEND_SAME_A: ca = e.wa + e.wb; cb = 0.0f; break;
        case JT_BLEND_SAME_B: ca = 0.0f; cb = e.wa + e.wb; break;
        default: ca = e.wa; cb = e.wb; break;
    }
}

__device__ __forceinline__ void red_v4(float* p, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}
__device__ __forceinline__ void red_v2(float* p, float a, float b) {
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(a), "f"(b) : "memory");
}

// Axis data of the adjoint: cell, weight, and d(weight)/dx (0 where the
// clamp mode clipped the coordinate).
struct AxisD {
    int i0, i1;
    float w, dfdx;
};

__device__ __forceinline__ AxisD axis_d(float x, float org, float d, float inv_d, int n, int mode) {
    AxisD r;
    bool valid;
    int flags = 0;
    grid_axis<true>(x, org, d, inv_d, n, mode, 0.0f, r.i0, r.i1, r.w, valid, flags);
    if (mode == JT_GRID_PERIODIC) {
        r.dfdx = inv_d;
    } else {
        const float f = (x - org) * inv_d;
        r.dfdx = (f > 0.0f && f < (float)(n > 1 ? n - 1 : 0)) ? inv_d : 0.0f;
    }
    return r;
}

// J^T g at p for entry e, scattering the snapshot gradient.
__device__ __forceinline__ V3 grid_vjp(const jt_grid_field& F, const V3& p, const jt_blend& e, const V3& g,
                                       float* __restrict__ grad) {
    const AxisD ax = axis_d(p.x, F.origin[0], F.spacing[0], F.inv_spacing[0], F.nx, F.bounds_mode);
    const AxisD ay = axis_d(p.y, F.origin[1], F.spacing[1], F.inv_spacing[1], F.ny, F.bounds_mode);
    const AxisD az = axis_d(p.z, F.origin[2], F.spacing[2], F.inv_spacing[2], F.nz, F.bounds_mode);
    float ca, cb;
    blend_coefs(e, ca, cb);
    const int pr = min(max(e.pair, 0), F.n_pairs - 1);
    const int64_t base = (int64_t)pr * F.pair_stride;
    V3 jtg{0.f, 0.f, 0.f};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
        const int i = bx ? ax.i1 : ax.i0, j = by ? ay.i1 : ay.i0, k = bz ? az.i1 : az.i0;
        const float wx = bx ? ax.w : 1.0f - ax.w, wy = by ? ay.w : 1.0f - ay.w, wz = bz ? az.w : 1.0f - az.w;
        const int64_t rec = base + ((int64_t)(i * F.ny + j) * F.nz + k);
        const PairVal pv = load_pair<JT_STORE_F32>(F.pairs, rec);
        // blended corner value dotted with g
        const float vx = ca * pv.axy.x + cb * pv.bxy.x, vy = ca * pv.axy.y + cb * pv.bxy.y;
        const float vz = ca * pv.az + cb * pv.bz;
        const float vg = vx * g.x + vy * g.y + vz * g.z;
        const float sx = bx ? 1.0f : -1.0f, sy = by ? 1.0f : -1.0f, sz = bz ? 1.0f : -1.0f;
        jtg.x += sx * ax.dfdx * wy * wz * vg;
        jtg.y += sy * ay.dfdx * wx * wz * vg;
        jtg.z += sz * az.dfdx * wx * wy * vg;
        const float w = wx * wy * wz;
        const float wa = w * ca, wb = w * cb;
        float* r = grad + 8 * rec;  // {Ax, Ay, Bx, By, Az, Bz, -, -}
        red_v4(r, wa * g.x, wa * g.y, wb * g.x, wb * g.y);
        red_v2(r + 4, wa * g.z, wb * g.z);
    }
    return jtg;
}

// d(boundary)/dx per axis for the box kinds: periodic and none pass the
// cotangent through, clamp zeroes it where the coordinate was clipped,
// reflective flips its sign on an odd number of folds.
__device__ __forceinline__ float bc_deriv(int kind, float x, float lo, float hi) {
    switch (kind) {
        case JT_BC_CLAMP: return (x < lo || x > hi) ? 0.0f : 1.0f;
        case JT_BC_ABSORBING: return (x < lo || x > hi) ? 0.0f : 1.0f;
        case JT_BC_REFLECTIVE: {
            const float width = fmaxf(hi - lo, 0.0f);
            const float ws = width > 0.0f ? width : 1.0f;
            const float y = np_mod(x - lo, 2.0f * ws);
            return y <= width ? 1.0f : -1.0f;
        }
        default: return 1.0f;
    }
}

// One backward segment [s0, s1): lambda holds dL/dx_{s1} on entry, dL/dx_{s0} on exit.
__global__ void __launch_bounds__(kBlock) k_adjoint_rk4(jt_grid_field F, jt_boundary B, jt_adjoint_params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n_particles) return;
    typedef GridField<true, JT_STORE_F32> Fw;
    const Fw f{F};
    typedef Ar<true> A;
    const int nseg = P.step_end - P.step_begin;
    float xs[JT_ADJOINT_MAX_SEGMENT][3];
    V3 x{P.ckpt[3 * (int64_t)i], P.ckpt[3 * (int64_t)i + 1], P.ckpt[3 * (int64_t)i + 2]};
    const StepConst k{P.dt, P.dt_half, P.dt_sixth};
    int flags = 0;
    V3 cz{0.f, 0.f, 0.f};
    for (int s = 0; s < nseg; ++s) {  // recompute the segment's states
        xs[s][0] = x.x; xs[s][1] = x.y; xs[s][2] = x.z;
        integrate<true, JT_RK4, false>(f, P.schedule + 4 * (int64_t)(P.step_begin + s), k, x, cz, flags);
        apply_boundary<true>(B, x.x, x.y, x.z);
    }
    V3 lam{P.lambda[3 * (int64_t)i], P.lambda[3 * (int64_t)i + 1], P.lambda[3 * (int64_t)i + 2]};
    for (int s = nseg - 1; s >= 0; --s) {
        const jt_blend* e = P.schedule + 4 * (int64_t)(P.step_begin + s);
        const jt_blend e0 = e[0], e1 = e[1], e2 = e[2];
        const V3 x0{xs[s][0], xs[s][1], xs[s][2]};
        // forward stages (same arithmetic as the forward pass)
        const V3 k1 = f(x0, e0, flags);
        const V3 x2{A::axpy(x0.x, k.dth, k1.x), A::axpy(x0.y, k.dth, k1.y), A::axpy(x0.z, k.dth, k1.z)};
        const V3 k2 = f(x2, e1, flags);
        const V3 x3{A::axpy(x0.x, k.dth, k2.x), A::axpy(x0.y, k.dth, k2.y), A::axpy(x0.z, k.dth, k2.z)};
        const V3 k3 = f(x3, e1, flags);
        const V3 x4{A::axpy(x0.x, k.dt, k3.x), A::axpy(x0.y, k.dt, k3.y), A::axpy(x0.z, k.dt, k3.z)};
        // through the boundary: pre-boundary position of this step
        if (B.inlet_mode == JT_INLET_OFF && !B.absorbing_joint) {
            const V3 k4 = f(x4, e2, flags);
            const float pre[3] = {x0.x + k.dt6 * (k1.x + 2.0f * k2.x + 2.0f * k3.x + k4.x),
                                  x0.y + k.dt6 * (k1.y + 2.0f * k2.y + 2.0f * k3.y + k4.y),
                                  x0.z + k.dt6 * (k1.z + 2.0f * k2.z + 2.0f * k3.z + k4.z)};
            lam.x *= bc_deriv(B.axis_kind[0], pre[0], B.lo[0], B.hi[0]);
            lam.y *= bc_deriv(B.axis_kind[1], pre[1], B.lo[1], B.hi[1]);
            lam.z *= bc_deriv(B.axis_kind[2], pre[2], B.lo[2], B.hi[2]);
        }
        // reverse sweep
        const float c6 = k.dt6, c3 = 2.0f * k.dt6;
        V3 g4{c6 * lam.x, c6 * lam.y, c6 * lam.z};
        V3 g3{c3 * lam.x, c3 * lam.y, c3 * lam.z};
        V3 g2{c3 * lam.x, c3 * lam.y, c3 * lam.z};
        V3 g1{c6 * lam.x, c6 * lam.y, c6 * lam.z};
        V3 lx = lam;
        const V3 d4 = grid_vjp(F, x4, e2, g4, P.grad);          // k4 = v(x4)
        lx = V3{lx.x + d4.x, lx.y + d4.y, lx.z + d4.z};
        g3 = V3{g3.x + k.dt * d4.x, g3.y + k.dt * d4.y, g3.z + k.dt * d4.z};
        const V3 d3 = grid_vjp(F, x3, e1, g3, P.grad);          // k3 = v(x3)
        lx = V3{lx.x + d3.x, lx.y + d3.y, lx.z + d3.z};
        g2 = V3{g2.x + k.dth * d3.x, g2.y + k.dth * d3.y, g2.z + k.dth * d3.z};
        const V3 d2 = grid_vjp(F, x2, e1, g2, P.grad);          // k2 = v(x2)
        lx = V3{lx.x + d2.x, lx.y + d2.y, lx.z + d2.z};
        g1 = V3{g1.x + k.dth * d2.x, g1.y + k.dth * d2.y, g1.z + k.dth * d2.z};
        const V3 d1 = grid_vjp(F, x0, e0, g1, P.grad);          // k1 = v(x0)
        lam = V3{lx.x + d1.x, lx.y + d1.y, lx.z + d1.z};
    }
    P.lambda[3 * (int64_t)i] = lam.x;
    P.lambda[3 * (int64_t)i + 1] = lam.y;
    P.lambda[3 * (int64_t)i + 2] = lam.z;
}

}  // namespace jt

using namespace jt;

extern "C" int jt_adjoint_rk4(const jt_field* field, const jt_boundary* bc, const jt_adjoint_params* p, void* stream) {
    if (field == nullptr || field->kind != JT_FIELD_GRID || field->grid == nullptr)
        return set_error(JT_ERR_UNSUPPORTED, "the adjoint runs on regular-grid fields");
    const jt_grid_field& F = *field->grid;
    if (F.storage != JT_STORE_F32) return set_error(JT_ERR_UNSUPPORTED, "the adjoint needs float32 snapshot storage");
    if (F.pairs == nullptr || F.n_pairs < 1) return set_error(JT_ERR_INVALID, "field has no snapshot pairs");
    if (bc == nullptr || p == nullptr) return set_error(JT_ERR_INVALID, "boundary and params are required");
    if (bc->inlet_mode != JT_INLET_OFF || bc->absorbing_joint)
        return set_error(JT_ERR_UNSUPPORTED, "the adjoint supports the per-axis box boundaries");
    if (p->n_particles < 0) return set_error(JT_ERR_INVALID, "n_particles must be >= 0");
    const int nseg = p->step_end - p->step_begin;
    if (p->step_begin < 0 || nseg < 0 || nseg > JT_ADJOINT_MAX_SEGMENT)
        return set_error(JT_ERR_INVALID, "segment [%d,%d) must hold 0..%d steps", p->step_begin, p->step_end,
                         JT_ADJOINT_MAX_SEGMENT);
    if (p->n_particles == 0 || nseg == 0) return JT_OK;
    if (p->schedule == nullptr || p->ckpt == nullptr || p->lambda == nullptr || p->grad == nullptr)
        return set_error(JT_ERR_INVALID, "schedule, ckpt, lambda and grad are required");
    k_adjoint_rk4<<<grid_blocks(p->n_particles), kBlock, 0, (cudaStream_t)stream>>>(F, *bc, *p);
    return cuda_status(cudaGetLastError(), "adjoint kernel launch");
}
