// Adjoint (reverse-mode) RK4 over a regular-grid time-series field.
//
// Gradients of a loss of the final positions with respect to the initial
// positions and to the snapshot values.  The forward pass stores positions
// every K steps (the tracking kernel's recording); this kernel walks one
// segment backwards: it recomputes the segment from its checkpoint with the
// forward arithmetic, keeping every step's stage positions in a per-thread
// array, then runs the RK4 reverse sweep
//     x' = B(x + h/6 (k1 + 2k2 + 2k3 + k4)),   k_i = v(x_i, t_i)
// with vector-Jacobian products of the trilinear, time-blended field
//     v(x) = sum_c w_c(x) (ca A_c + cb B_c).
// J^T g uses dw_c/dx.  The snapshot gradient dL/dA_c += ca w_c g,
// dL/dB_c += cb w_c g is gathered as w_c g per stage time and node (one
// vector atomic per corner) and folded with (ca, cb) afterwards.
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

// The three axes of a point: cells, weights and weight derivatives.
struct Ax3 {
    AxisD x, y, z;
};

__device__ __forceinline__ Ax3 axes_of(const jt_grid_field& F, const V3& p) {
    return Ax3{axis_d(p.x, F.origin[0], F.spacing[0], F.inv_spacing[0], F.nx, F.bounds_mode),
               axis_d(p.y, F.origin[1], F.spacing[1], F.inv_spacing[1], F.ny, F.bounds_mode),
               axis_d(p.z, F.origin[2], F.spacing[2], F.inv_spacing[2], F.nz, F.bounds_mode)};
}

__device__ __forceinline__ bool same_cell(const Ax3& a, const Ax3& b) {
    return a.x.i0 == b.x.i0 && a.y.i0 == b.y.i0 && a.z.i0 == b.z.i0;
}

// Two schedule entries blend the same pair with the same coefficients.
__device__ __forceinline__ bool same_entry(const jt_blend& a, const jt_blend& b) {
    return a.pair == b.pair && a.form == b.form && __float_as_int(a.wa) == __float_as_int(b.wa) &&
           __float_as_int(a.wb) == __float_as_int(b.wb);
}

// w_c * g into the accumulator records of the eight corners (no loads).
__device__ __forceinline__ void scatter(const jt_grid_field& F, const Ax3& a, const V3& g, float4* __restrict__ acc) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
        const int i = bx ? a.x.i1 : a.x.i0, j = by ? a.y.i1 : a.y.i0, k = bz ? a.z.i1 : a.z.i0;
        const float w = (bx ? a.x.w : 1.0f - a.x.w) * (by ? a.y.w : 1.0f - a.y.w) * (bz ? a.z.w : 1.0f - a.z.w);
        const int64_t node = (int64_t)(i * F.ny + j) * F.nz + k;
        red_v4(reinterpret_cast<float*>(acc + node), w * g.x, w * g.y, w * g.z, 0.0f);
    }
}

// J^T g at the point with axes a for entry e.  With acc set, the snapshot
// gradient of this stage, w_c * g per corner node c, is added to acc (one
// float4 record per node: x, y, z, unused); with `other` set (a second point
// of the same stage time in the same cell), w'_c * g' is added in the same
// atomic.  The blend coefficients of A and B are applied when the
// accumulators are folded into the pair-record gradient.
//
// STAGE: the blended corner values come from a pre-blended float32 stage
// field (stage + slot * nodes, one float4 per node) instead of the pair
// records: half the bytes, no blend arithmetic.
template <bool STAGE>
__device__ __forceinline__ V3 grid_vjp(const jt_grid_field& F, const Ax3& a, const jt_blend& e, const V3& g,
                                       float4* __restrict__ acc, const Ax3* other, const V3& g_other,
                                       const float4* __restrict__ stage) {
    float ca = 0.f, cb = 0.f;
    if (!STAGE) blend_coefs(e, ca, cb);
    const int pr = min(max(e.pair, 0), F.n_pairs - 1);
    const int64_t base = (int64_t)pr * F.pair_stride;
    V3 jtg{0.f, 0.f, 0.f};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
        const int i = bx ? a.x.i1 : a.x.i0, j = by ? a.y.i1 : a.y.i0, k = bz ? a.z.i1 : a.z.i0;
        const float wx = bx ? a.x.w : 1.0f - a.x.w, wy = by ? a.y.w : 1.0f - a.y.w;
        const float wz = bz ? a.z.w : 1.0f - a.z.w;
        const int64_t node = (int64_t)(i * F.ny + j) * F.nz + k;
        // blended corner value dotted with g
        float vx, vy, vz;
        if (STAGE) {
            const float4 v = __ldg(stage + node);
            vx = v.x; vy = v.y; vz = v.z;
        } else {
            const PairVal pv = load_pair<JT_STORE_F32>(F.pairs, base + node);
            vx = ca * pv.axy.x + cb * pv.bxy.x;
            vy = ca * pv.axy.y + cb * pv.bxy.y;
            vz = ca * pv.az + cb * pv.bz;
        }
        const float vg = vx * g.x + vy * g.y + vz * g.z;
        const float sx = bx ? 1.0f : -1.0f, sy = by ? 1.0f : -1.0f, sz = bz ? 1.0f : -1.0f;
        jtg.x += sx * a.x.dfdx * wy * wz * vg;
        jtg.y += sy * a.y.dfdx * wx * wz * vg;
        jtg.z += sz * a.z.dfdx * wx * wy * vg;
        if (acc != nullptr) {
            const float w = wx * wy * wz;
            float gx = w * g.x, gy = w * g.y, gz = w * g.z;
            if (other != nullptr) {
                const float ow = (bx ? other->x.w : 1.0f - other->x.w) * (by ? other->y.w : 1.0f - other->y.w) *
                                 (bz ? other->z.w : 1.0f - other->z.w);
                gx += ow * g_other.x;
                gy += ow * g_other.y;
                gz += ow * g_other.z;
            }
            red_v4(reinterpret_cast<float*>(acc + node), gx, gy, gz, 0.0f);
        }
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

// Per recomputed step: the RK4 stage positions x0, x2 = x0 + h/2 k1,
// x3 = x0 + h/2 k2, x4 = x0 + h k3 and (PRE) the pre-boundary end point,
// with the forward pass's exact arithmetic (integrate<true, JT_RK4>).
template <bool PRE>
struct StepRec {
    float v[PRE ? 15 : 12];
};

#ifndef JT_ADJOINT_MIN_BLOCKS
#define JT_ADJOINT_MIN_BLOCKS 3
#endif

// One backward segment [s0, s1): lambda holds dL/dx_{s1} on entry, dL/dx_{s0}
// on exit; acc (or NULL) receives the per-stage snapshot gradients, three
// records per step (stage times t, t + h/2, t + h), (3*nseg, nodes) float4.
// PRE: some axis has a boundary whose derivative is not 1 (clamp,
// absorbing, reflective), so the pre-boundary end point is kept.
// STAGE: P.stage holds the segment's float32 stage fields (3 per step, slot
// 3*s + k for stage k of local step s), used for the recompute (bit-identical
// to blending the pair records) and the vector-Jacobian products.
template <bool PRE, bool STAGE>
__global__ void __launch_bounds__(kBlock, JT_ADJOINT_MIN_BLOCKS)
    k_adjoint_rk4(jt_grid_field F, jt_boundary B, jt_adjoint_params P, float4* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n_particles) return;
    typedef GridField<true, JT_STORE_F32> Fw;
    const Fw f{F};
    jt_grid_field FS = F;  // the stage fields as a grid descriptor
    FS.storage = JT_STORE_STAGE_F32;
    FS.pairs = P.stage;
    FS.n_pairs = 3 * (P.step_end - P.step_begin);
    const StageGridField<true, JT_STORE_STAGE_F32> fs = StageGridField<true, JT_STORE_STAGE_F32>::create(FS, 0);
    const float4* stage4 = reinterpret_cast<const float4*>(P.stage);
    typedef Ar<true> A;
    const int nseg = P.step_end - P.step_begin;
    const int64_t nodes = F.pair_stride;
    StepRec<PRE> rec[JT_ADJOINT_MAX_SEGMENT];
    V3 x{P.ckpt[3 * (int64_t)i], P.ckpt[3 * (int64_t)i + 1], P.ckpt[3 * (int64_t)i + 2]};
    const StepConst k{P.dt, P.dt_half, P.dt_sixth};
    int flags = 0;
    for (int s = 0; s < nseg; ++s) {  // recompute the segment, keeping the stage positions
        const jt_blend* e = P.schedule + 4 * (int64_t)(P.step_begin + s);
        float* r = rec[s].v;
        V3 sm{0.f, 0.f, 0.f}, xs = x;
#pragma unroll 1
        for (int st = 0; st < 4; ++st) {
            r[3 * st] = xs.x; r[3 * st + 1] = xs.y; r[3 * st + 2] = xs.z;
            const int sk = st == 0 ? 0 : (st == 3 ? 2 : 1);
            V3 kk;
            if (STAGE) {
                jt_blend es{};
                es.pair = 3 * s + sk;
                kk = fs(xs, es, flags);
            } else {
                kk = f(xs, e[sk], flags);
            }
            if (st == 0) {
                sm = kk;
            } else if (st == 3) {
                sm = V3{A::add(sm.x, kk.x), A::add(sm.y, kk.y), A::add(sm.z, kk.z)};
            } else {
                sm = V3{A::add(sm.x, A::mul(2.0f, kk.x)), A::add(sm.y, A::mul(2.0f, kk.y)),
                        A::add(sm.z, A::mul(2.0f, kk.z))};
            }
            const float h = st < 2 ? k.dth : k.dt;
            xs = V3{A::axpy(x.x, h, kk.x), A::axpy(x.y, h, kk.y), A::axpy(x.z, h, kk.z)};
        }
        x = V3{A::add(x.x, A::mul(k.dt6, sm.x)), A::add(x.y, A::mul(k.dt6, sm.y)),
               A::add(x.z, A::mul(k.dt6, sm.z))};
        if (PRE) { r[12] = x.x; r[13] = x.y; r[14] = x.z; }
        apply_boundary<true>(B, x.x, x.y, x.z);
    }
    V3 lam{P.lambda[3 * (int64_t)i], P.lambda[3 * (int64_t)i + 1], P.lambda[3 * (int64_t)i + 2]};
    // The scatter of k1 = v(x0) at step s waits for step s-1: its stage time
    // t_s usually carries the same blend entry as t_{s-1} + h (k4 of step
    // s-1) and x0 lies next to x4 of step s-1, so one atomic per corner
    // often carries both.  pend_* hold the waiting scatter.
    bool pend = false;
    Ax3 pend_ax;
    V3 pend_g{0.f, 0.f, 0.f};
    float4* pend_acc = nullptr;
    const jt_blend* pend_e = nullptr;
    const V3 none{0.f, 0.f, 0.f};
    for (int s = nseg - 1; s >= 0; --s) {
        const jt_blend* e = P.schedule + 4 * (int64_t)(P.step_begin + s);
        const jt_blend e0 = e[0], e1 = e[1], e2 = e[2];
        const float* r = rec[s].v;
        const V3 x0{r[0], r[1], r[2]}, x2{r[3], r[4], r[5]}, x3{r[6], r[7], r[8]}, x4{r[9], r[10], r[11]};
        // through the boundary at the pre-boundary end point
        if (PRE) {
            lam.x *= bc_deriv(B.axis_kind[0], r[PRE ? 12 : 0], B.lo[0], B.hi[0]);
            lam.y *= bc_deriv(B.axis_kind[1], r[PRE ? 13 : 1], B.lo[1], B.hi[1]);
            lam.z *= bc_deriv(B.axis_kind[2], r[PRE ? 14 : 2], B.lo[2], B.hi[2]);
        }
        float4* a0 = acc != nullptr ? acc + (int64_t)(3 * s) * nodes : nullptr;
        float4* a1 = acc != nullptr ? a0 + nodes : nullptr;
        float4* a2 = acc != nullptr ? a1 + nodes : nullptr;
        // reverse sweep
        const float c6 = k.dt6, c3 = 2.0f * k.dt6;
        V3 lx = lam;
        const Ax3 ax4 = axes_of(F, x4);
        const bool join = pend && same_entry(*pend_e, e2) && same_cell(pend_ax, ax4);
        if (pend && !join) scatter(F, pend_ax, pend_g, pend_acc);
        const float4* s0 = STAGE ? stage4 + (int64_t)(3 * s) * nodes : nullptr;
        const float4* s1 = STAGE ? s0 + nodes : nullptr;
        const float4* s2 = STAGE ? s1 + nodes : nullptr;
        const V3 d4 = grid_vjp<STAGE>(F, ax4, e2, V3{c6 * lam.x, c6 * lam.y, c6 * lam.z}, join ? pend_acc : a2,
                                      join ? &pend_ax : nullptr, pend_g, s2);                         // k4 = v(x4)
        lx = V3{lx.x + d4.x, lx.y + d4.y, lx.z + d4.z};
        const V3 g3{c3 * lam.x + k.dt * d4.x, c3 * lam.y + k.dt * d4.y, c3 * lam.z + k.dt * d4.z};
        // k3 = v(x3) and k2 = v(x2) share the stage time t + h/2 and almost
        // always the cell: one atomic per corner carries both contributions
        const Ax3 ax3 = axes_of(F, x3), ax2 = axes_of(F, x2);
        const bool merge = same_cell(ax3, ax2);
        const V3 d3 = grid_vjp<STAGE>(F, ax3, e1, g3, merge ? nullptr : a1, nullptr, none, s1);
        lx = V3{lx.x + d3.x, lx.y + d3.y, lx.z + d3.z};
        const V3 g2{c3 * lam.x + k.dth * d3.x, c3 * lam.y + k.dth * d3.y, c3 * lam.z + k.dth * d3.z};
        const V3 d2 = grid_vjp<STAGE>(F, ax2, e1, g2, a1, merge ? &ax3 : nullptr, g3, s1);
        lx = V3{lx.x + d2.x, lx.y + d2.y, lx.z + d2.z};
        const V3 g1{c6 * lam.x + k.dth * d2.x, c6 * lam.y + k.dth * d2.y, c6 * lam.z + k.dth * d2.z};
        const Ax3 ax0 = axes_of(F, x0);
        const V3 d1 = grid_vjp<STAGE>(F, ax0, e0, g1, nullptr, nullptr, none, s0);          // k1 = v(x0)
        lam = V3{lx.x + d1.x, lx.y + d1.y, lx.z + d1.z};
        pend = acc != nullptr;
        pend_ax = ax0;
        pend_g = g1;
        pend_acc = a0;
        pend_e = e;
    }
    if (pend) scatter(F, pend_ax, pend_g, pend_acc);
    P.lambda[3 * (int64_t)i] = lam.x;
    P.lambda[3 * (int64_t)i + 1] = lam.y;
    P.lambda[3 * (int64_t)i + 2] = lam.z;
}

// Fold the per-stage accumulators of a segment into the pair-record gradient:
// dL/dA += ca * G, dL/dB += cb * G with (ca, cb) the stage's blend
// coefficients.  One thread per node walks the stages in order, so no two
// threads touch one record.
__global__ void __launch_bounds__(kBlock) k_adjoint_fold(jt_grid_field F, const jt_blend* __restrict__ sched,
                                                          int nseg, const float4* __restrict__ acc,
                                                          float* __restrict__ grad) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nodes = F.pair_stride;
    if (node >= nodes) return;
    int cur = -1;
    float sa[3] = {0.f, 0.f, 0.f}, sb[3] = {0.f, 0.f, 0.f};
    for (int j = 0; j < 3 * nseg; ++j) {
        const jt_blend e = sched[4 * (j / 3) + (j % 3)];
        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        if (pr != cur) {
            if (cur >= 0) {
                float* r = grad + 8 * ((int64_t)cur * F.pair_stride + node);
                r[0] += sa[0]; r[1] += sa[1]; r[2] += sb[0]; r[3] += sb[1]; r[4] += sa[2]; r[5] += sb[2];
            }
            cur = pr;
            sa[0] = sa[1] = sa[2] = sb[0] = sb[1] = sb[2] = 0.f;
        }
        float ca, cb;
        blend_coefs(e, ca, cb);
        const float4 g = acc[(int64_t)j * nodes + node];
        sa[0] += ca * g.x; sa[1] += ca * g.y; sa[2] += ca * g.z;
        sb[0] += cb * g.x; sb[1] += cb * g.y; sb[2] += cb * g.z;
    }
    if (cur >= 0) {
        float* r = grad + 8 * ((int64_t)cur * F.pair_stride + node);
        r[0] += sa[0]; r[1] += sa[1]; r[2] += sb[0]; r[3] += sb[1]; r[4] += sa[2]; r[5] += sb[2];
    }
}

}  // namespace jt

using namespace jt;

extern "C" size_t jt_adjoint_workspace_bytes(int64_t n_nodes, int32_t n_steps) {
    if (n_nodes < 0 || n_steps < 0 || n_steps > JT_ADJOINT_MAX_SEGMENT) return 0;
    return (size_t)3 * (size_t)n_steps * (size_t)n_nodes * sizeof(float4);
}

extern "C" int jt_adjoint_rk4(const jt_field* field, const jt_boundary* bc, const jt_adjoint_params* p, void* stream) {
    if (field == nullptr || field->kind != JT_FIELD_GRID || field->grid == nullptr)
        return set_error(JT_ERR_UNSUPPORTED, "the adjoint runs on regular-grid fields");
    const jt_grid_field& F = *field->grid;
    if (int rc = check_grid_shape(F)) return rc;
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
    if (p->schedule == nullptr || p->ckpt == nullptr || p->lambda == nullptr)
        return set_error(JT_ERR_INVALID, "schedule, ckpt and lambda are required");
    const size_t need = jt_adjoint_workspace_bytes(F.pair_stride, nseg);
    if (p->grad != nullptr && (p->work == nullptr || p->work_bytes < (int64_t)need))
        return set_error(JT_ERR_INVALID, "the snapshot gradient needs a workspace of %zu bytes", need);
    if (p->grad != nullptr && ((uintptr_t)p->work & 15u) != 0)
        return set_error(JT_ERR_INVALID, "the adjoint workspace must be 16-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    float4* acc = p->grad != nullptr ? reinterpret_cast<float4*>(p->work) : nullptr;
    if (acc != nullptr) {
        const cudaError_t e = cudaMemsetAsync(acc, 0, need, s);
        if (e != cudaSuccess) return cuda_status(e, "adjoint workspace memset");
    }
    bool pre = false;
    for (int a = 0; a < 3; ++a) pre |= bc->axis_kind[a] != JT_BC_PERIODIC && bc->axis_kind[a] != JT_BC_NONE;
    const unsigned gb = grid_blocks(p->n_particles);
    if (p->stage != nullptr) {
        if (pre) k_adjoint_rk4<true, true><<<gb, kBlock, 0, s>>>(F, *bc, *p, acc);
        else k_adjoint_rk4<false, true><<<gb, kBlock, 0, s>>>(F, *bc, *p, acc);
    } else {
        if (pre) k_adjoint_rk4<true, false><<<gb, kBlock, 0, s>>>(F, *bc, *p, acc);
        else k_adjoint_rk4<false, false><<<gb, kBlock, 0, s>>>(F, *bc, *p, acc);
    }
    int rc = cuda_status(cudaGetLastError(), "adjoint kernel launch");
    if (rc != JT_OK || acc == nullptr) return rc;
    k_adjoint_fold<<<grid_blocks(F.pair_stride), kBlock, 0, s>>>(F, p->schedule + 4 * (int64_t)p->step_begin, nseg,
                                                                  acc, p->grad);
    return cuda_status(cudaGetLastError(), "adjoint fold launch");
}
