// Shared device code of the tracking kernels: float32 arithmetic policies,
// NumPy-compatible remainder, time-blend decoding, boundary conditions and
// the fused integrator step.  Every formula names the reference expression
// (path:line inside the JAXTrace project) whose float32 rounding it follows.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/jaxtrace_gb300.h"

namespace jt {

// Tuning switches.  JT_LERP_NOINLINE=1 moves the rarely taken extrapolation
// blend out of line (measured 2x slower: the call forces a stack frame on the
// hot path); JT_STAGE_UNROLL unrolls the RK stage loop of every field (measured
// slower for the pair-gather, mesh and FEM bodies: more registers, more
// instruction-cache misses); a field type opts in with kUnrollStages.
#ifndef JT_LERP_NOINLINE
#define JT_LERP_NOINLINE 0
#endif
#if JT_LERP_NOINLINE
#define JT_LERP_INLINE __device__ __noinline__
#else
#define JT_LERP_INLINE __device__ __forceinline__
#endif
#ifndef JT_STAGE_UNROLL
#define JT_STAGE_UNROLL 1
#endif
#define JT_PRAGMA(x) _Pragma(#x)
#define JT_UNROLL(n) JT_PRAGMA(unroll n)

// ---------------------------------------------------------------------------
// Arithmetic policies.  Exact: every operation rounded to nearest on its own,
// never contracted into an FMA -- the order and rounding of NumPy float32
// array expressions.  Fast: the compiler may contract, and lerps use FMA.
// ---------------------------------------------------------------------------
template <bool EXACT>
struct Ar;

template <>
struct Ar<true> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    // a*wa + b*wb, both products rounded before the sum
    static __device__ __forceinline__ float dot2(float a, float wa, float b, float wb) {
        return __fadd_rn(__fmul_rn(a, wa), __fmul_rn(b, wb));
    }
    // a + w*b with the product rounded
    static __device__ __forceinline__ float axpy(float a, float w, float b) {
        return __fadd_rn(a, __fmul_rn(w, b));
    }
};

template <>
struct Ar<false> {
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float dot2(float a, float wa, float b, float wb) {
        return fmaf(a, wa, b * wb);
    }
    static __device__ __forceinline__ float axpy(float a, float w, float b) { return fmaf(w, b, a); }
};

// NumPy float32 remainder (np.mod / jnp.mod): fmod, then move the result to
// the sign of the divisor (Python convention).  fmodf is exact; the one add
// is rounded, so the result may equal b itself (e.g. a = -1e-9, b = 32).
__device__ __forceinline__ float np_mod(float a, float b) {
    if (a >= 0.0f && a < b) return a;  // fmod(a,b) == a exactly on this range
    float m = fmodf(a, b);
    if (m != 0.0f) {
        if ((b < 0.0f) != (m < 0.0f)) m = __fadd_rn(m, b);
    } else {
        m = copysignf(0.0f, b);
    }
    return m;
}

// np.clip(x, lo, hi) for float32: NaN propagates.
__device__ __forceinline__ float np_clip(float x, float lo, float hi) {
    x = (x < lo) ? lo : x;
    x = (x > hi) ? hi : x;
    return x;
}

struct V3 {
    float x, y, z;
};

// Morton (Z-order) key of a cell: bit b of axis a goes to bit 3b+a.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000ff;
    v = (v | (v << 8)) & 0x0300f00f;
    v = (v | (v << 4)) & 0x030c30c3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}
__device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

// ---------------------------------------------------------------------------
// Snapshot-pair records.
// ---------------------------------------------------------------------------
// Record layout (8 slots, float32 or 16-bit): {Ax, Ay, Bx, By, Az, Bz, 0, 0}
// so that (Ax,Ay) and (Bx,By) arrive in aligned register pairs for the
// packed float32x2 instructions.
struct PairVal {
    float2 axy, bxy;
    float az, bz;
};

template <int STORE>
__device__ __forceinline__ PairVal load_pair(const void* base, int64_t rec);

// One 256-bit read-only load (a whole 32-byte record in one request).
__device__ __forceinline__ void ldg256(const void* p, uint32_t (&w)[8]) {
    asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
        : "l"(p));
}

template <>
__device__ __forceinline__ PairVal load_pair<JT_STORE_F32>(const void* base, int64_t rec) {
    uint32_t w[8];
    ldg256(reinterpret_cast<const float4*>(base) + 2 * rec, w);
    return PairVal{make_float2(__uint_as_float(w[0]), __uint_as_float(w[1])),
                   make_float2(__uint_as_float(w[2]), __uint_as_float(w[3])), __uint_as_float(w[4]),
                   __uint_as_float(w[5])};
}

// bfloat16 -> float32 is exact: the 16 bits become the high half of the word.
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

template <int STORE>
__device__ __forceinline__ PairVal decode3(uint32_t w0, uint32_t w1, uint32_t w2) {
    if (STORE == JT_STORE_BF16) {
        return PairVal{make_float2(bf16_lo(w0), bf16_hi(w0)), make_float2(bf16_lo(w1), bf16_hi(w1)), bf16_lo(w2),
                       bf16_hi(w2)};
    }
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&w0));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&w1));
    const float2 z = __half22float2(*reinterpret_cast<const __half2*>(&w2));
    return PairVal{a, b, z.x, z.y};
}

// 16-bit yz-quad record of the grid field (48 B): nodes (i,j,k), (i,j,k1),
// (i,j1,k), (i,j1,k1), j1 and k1 as the sampler computes them, three words
// each in that order.  Words 0-7 are part A (32 B, records [0, part_b)) and
// words 8-11 part B (16 B, after every part-A record), so one 256-bit and
// one 128-bit load fetch the quad; 48 B for four corners instead of 64 B.
template <int STORE>
__device__ __forceinline__ void load_quad(const void* base, int64_t part_b, int64_t rec, PairVal& p00,
                                          PairVal& p01, PairVal& p10, PairVal& p11) {
    uint32_t w[8];
    ldg256(reinterpret_cast<const uint4*>(base) + 2 * rec, w);
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(base) + 2 * part_b + rec);
    p00 = decode3<STORE>(w[0], w[1], w[2]);
    p01 = decode3<STORE>(w[3], w[4], w[5]);
    p10 = decode3<STORE>(w[6], w[7], v.x);
    p11 = decode3<STORE>(v.y, v.z, v.w);
}

// 16-bit single-node record (16 B), used by the mesh and nearest fields.
template <>
__device__ __forceinline__ PairVal load_pair<JT_STORE_BF16>(const void* base, int64_t rec) {
    const uint4 r = __ldg(reinterpret_cast<const uint4*>(base) + rec);
    return decode3<JT_STORE_BF16>(r.x, r.y, r.z);
}

template <>
__device__ __forceinline__ PairVal load_pair<JT_STORE_F16>(const void* base, int64_t rec) {
    const uint4 r = __ldg(reinterpret_cast<const uint4*>(base) + rec);
    return decode3<JT_STORE_F16>(r.x, r.y, r.z);
}

// a*wa + b*wb on (x,y) pairs.  The exact mode rounds every product and sum on
// its own with scalar instructions (a packed multiply followed by a packed
// add was measured to differ from separately rounded scalar operations in a
// quarter of the results, so it cannot stand in for NumPy's arithmetic); the
// fast modes use the packed FFMA2/FMUL2 instructions.
template <bool EXACT>
__device__ __forceinline__ float2 dot2p(float2 a, float2 wa, float2 b, float2 wb) {
    if (EXACT) {
        return make_float2(__fadd_rn(__fmul_rn(a.x, wa.x), __fmul_rn(b.x, wb.x)),
                           __fadd_rn(__fmul_rn(a.y, wa.y), __fmul_rn(b.y, wb.y)));
    }
    return __ffma2_rn(a, wa, __fmul2_rn(b, wb));
}

__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }

// Linear extrapolation outside the snapshot times (rarely taken).
template <bool EXACT, int STORE>
JT_LERP_INLINE V3 blend_lerp(const PairVal& p, const jt_blend& e) {
    typedef Ar<EXACT> A;
    float ax = p.axy.x, ay = p.axy.y, az = p.az, bx = p.bxy.x, by = p.bxy.y, bz = p.bz;
    if (STORE != JT_STORE_F32) {
        ax = A::mul(ax, e.sa); ay = A::mul(ay, e.sa); az = A::mul(az, e.sa);
        bx = A::mul(bx, e.sb); by = A::mul(by, e.sb); bz = A::mul(bz, e.sb);
    }
    if (e.form == JT_BLEND_LERP_FWD) {
        return V3{A::axpy(ax, e.wb, A::sub(bx, ax)), A::axpy(ay, e.wb, A::sub(by, ay)),
                  A::axpy(az, e.wb, A::sub(bz, az))};
    }
    return V3{A::axpy(bx, e.wb, A::sub(bx, ax)), A::axpy(by, e.wb, A::sub(by, ay)),
              A::axpy(bz, e.wb, A::sub(bz, az))};
}

// Blend of one snapshot pair at the time the schedule entry describes:
// time_series.py:367  ((1-alpha)*V[il] + alpha*V[ir]).astype(float32)
// time_series.py:336  V0 + alpha*(V1-V0)        (linear extrapolation, left)
// time_series.py:352  V1 + alpha*(V1-V0)        (linear extrapolation, right)
template <bool EXACT, int STORE>
__device__ __forceinline__ V3 blend(const PairVal& p, const jt_blend& e) {
    typedef Ar<EXACT> A;
    if (e.form == JT_BLEND_WEIGHTED) {
        const float2 xy = dot2p<EXACT>(p.axy, splat(e.wa), p.bxy, splat(e.wb));
        return V3{xy.x, xy.y, A::dot2(p.az, e.wa, p.bz, e.wb)};
    }
    const float ax = p.axy.x, ay = p.axy.y, bx0 = p.bxy.x, by0 = p.bxy.y;
    if (e.form == JT_BLEND_SAME_A) {
        return V3{A::dot2(ax, e.wa, ax, e.wb), A::dot2(ay, e.wa, ay, e.wb), A::dot2(p.az, e.wa, p.az, e.wb)};
    }
    if (e.form == JT_BLEND_SAME_B) {
        return V3{A::dot2(bx0, e.wa, bx0, e.wb), A::dot2(by0, e.wa, by0, e.wb), A::dot2(p.bz, e.wa, p.bz, e.wb)};
    }
    return blend_lerp<EXACT, STORE>(p, e);
}

// ---------------------------------------------------------------------------
// Boundary conditions (tracking/boundary.py), float32 as the NumPy path.
// ---------------------------------------------------------------------------
template <bool EXACT>
__device__ __forceinline__ float bc_axis(int kind, float x, float lo, float hi, float outside) {
    typedef Ar<EXACT> A;
    switch (kind) {
        case JT_BC_PERIODIC: {
            // boundary.py:118-123  lo + mod(x - lo, where(width>0, width, 1))
            float width = A::sub(hi, lo);
            width = width > 0.0f ? width : 0.0f;
            float ws = width > 0.0f ? width : 1.0f;
            return A::add(lo, np_mod(A::sub(x, lo), ws));
        }
        case JT_BC_REFLECTIVE: {
            // boundary.py:165-172  sawtooth fold with period 2*width
            float width = A::sub(hi, lo);
            width = width > 0.0f ? width : 0.0f;
            float ws = width > 0.0f ? width : 1.0f;
            float y = np_mod(A::sub(x, lo), A::mul(2.0f, ws));
            float yr = (y <= width) ? y : A::sub(A::mul(2.0f, width), y);
            return A::add(lo, yr);
        }
        case JT_BC_CLAMP:
            // boundary.py:143  clip(x, lo, hi)
            return np_clip(x, lo, hi);
        case JT_BC_ABSORBING:
            // boundary.py:198-208 on one axis (mixed_boundary, :415)
            return (x < lo || x > hi) ? outside : x;
        default:
            return x;
    }
}

// Nearest lattice coordinate: argmin(|coords - c|) with ties to the lower
// index (boundary.py:1309).  The lattice is ascending, so |fl(g[j]-c)| falls
// then rises; start from the bracketing pair and walk left over ties.
__device__ __forceinline__ float nearest_lattice(const float* g, int n, float c) {
    if (n <= 1) return __ldg(g);
    if (c != c) return __ldg(g);  // all distances NaN: argmin returns 0
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(g + mid) < c) lo = mid + 1; else hi = mid;
    }
    int best;
    if (lo == 0) {
        best = 0;
    } else if (lo == n) {
        best = n - 1;
    } else {
        float dl = fabsf(__fsub_rn(__ldg(g + lo - 1), c));
        float dr = fabsf(__fsub_rn(__ldg(g + lo), c));
        best = (dr < dl) ? lo : lo - 1;
    }
    float db = fabsf(__fsub_rn(__ldg(g + best), c));
    while (best > 0) {
        float d = fabsf(__fsub_rn(__ldg(g + best - 1), c));
        if (!(d <= db)) break;
        db = d;
        --best;
    }
    return __ldg(g + best);
}

// The continuous inlet's bounds in its own frame: the flow axis a and the two
// others o0 < o1 (o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2), with the mirror
// offsets 2*lo and 2*hi (exact in float32).  Built once per launch on the host
// so that the kernel reads them as launch constants instead of selecting them
// by a run-time axis at every step.
struct InletFrame {
    float amin, amax, lo0, hi0, lo1, hi1, lo0x2, hi0x2, lo1x2, hi1x2;
};

__host__ __device__ inline InletFrame inlet_frame(const jt_boundary& B) {
    const int a = B.inlet_axis;
    const int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
    const int aa = a == 0 ? 0 : (a == 1 ? 1 : 2);
    InletFrame I;
    I.amin = B.lo[aa];
    I.amax = B.hi[aa];
    I.lo0 = B.lo[o0];
    I.hi0 = B.hi[o0];
    I.lo1 = B.lo[o1];
    I.hi1 = B.hi[o1];
    I.lo0x2 = 2.0f * I.lo0;
    I.hi0x2 = 2.0f * I.hi0;
    I.lo1x2 = 2.0f * I.lo1;
    I.hi1x2 = 2.0f * I.hi1;
    return I;
}

// Continuous inlet with grid-preserving replacement (boundary.py:1517-1599).
template <bool EXACT>
__device__ __forceinline__ void bc_inlet(const jt_boundary& B, const InletFrame& I, float& x, float& y, float& z) {
    typedef Ar<EXACT> A;
    // the particle's coordinates in the inlet frame, picked with selects so
    // that nothing is indexed by a run-time axis (no local-memory copy of B)
    const int a = B.inlet_axis;
    float fa = a == 0 ? x : (a == 1 ? y : z);
    float u0 = a == 0 ? y : x;
    float u1 = a == 2 ? y : z;
    const float amin = I.amin, amax = I.amax, lo0 = I.lo0, hi0 = I.hi0, lo1 = I.lo1, hi1 = I.hi1;
    const bool exited = B.inlet_positive ? (fa > amax) : (fa < amin);
    if (exited && B.inlet_mode == JT_INLET_GRID) {
        const float g0 = nearest_lattice(B.inlet_coords[0], B.inlet_res[0], u0);
        const float g1 = nearest_lattice(B.inlet_coords[1], B.inlet_res[1], u1);
        fa = B.inlet_positive ? amin : amax;
        u0 = g0;
        u1 = g1;
    }
    // boundary.py:1580-1587  backward crossings are nudged inside
    if (B.inlet_positive) {
        if (fa < amin) fa = B.inlet_nudge;
    } else {
        if (fa > amax) fa = B.inlet_nudge;
    }
    // boundary.py:1590-1597  one mirror on the other axes (2*lo - u, 2*hi - u)
    if (u0 < lo0) u0 = A::sub(I.lo0x2, u0);
    else if (u0 > hi0) u0 = A::sub(I.hi0x2, u0);
    if (u1 < lo1) u1 = A::sub(I.lo1x2, u1);
    else if (u1 > hi1) u1 = A::sub(I.hi1x2, u1);
    if (a == 0) {
        x = fa; y = u0; z = u1;
    } else if (a == 1) {
        x = u0; y = fa; z = u1;
    } else {
        x = u0; y = u1; z = fa;
    }
}

// bc_inlet for its most common form, fixed at compile time: grid
// replacement, flow along +x.  The same operations as bc_inlet with a = 0,
// without the run-time selects by axis, direction and mode.
template <bool EXACT>
__device__ __forceinline__ void bc_inlet_xpos(const jt_boundary& B, const InletFrame& I, float& x, float& y,
                                              float& z) {
    typedef Ar<EXACT> A;
    if (x > I.amax) {
        y = nearest_lattice(B.inlet_coords[0], B.inlet_res[0], y);
        z = nearest_lattice(B.inlet_coords[1], B.inlet_res[1], z);
        x = I.amin;
    }
    if (x < I.amin) x = B.inlet_nudge;
    if (y < I.lo0) y = A::sub(I.lo0x2, y);
    else if (y > I.hi0) y = A::sub(I.hi0x2, y);
    if (z < I.lo1) z = A::sub(I.lo1x2, z);
    else if (z > I.hi1) z = A::sub(I.hi1x2, z);
}

// Boundary forms a kernel can be specialised for (BK): any (read from the
// descriptor at run time) or the +x grid inlet.
enum { JT_BK_ANY = 0, JT_BK_INLET_XPOS = 1 };

template <bool EXACT>
__device__ __forceinline__ void apply_boundary(const jt_boundary& B, const InletFrame& I, float& x, float& y,
                                               float& z) {
    if (B.inlet_mode != JT_INLET_OFF) {
        bc_inlet<EXACT>(B, I, x, y, z);
        return;
    }
    if (B.absorbing_joint) {
        // boundary.py:198-208: any coordinate outside marks the whole particle
        bool out = x < B.lo[0] || y < B.lo[1] || z < B.lo[2] || x > B.hi[0] || y > B.hi[1] ||
                   z > B.hi[2];
        if (out) { x = B.outside_value; y = B.outside_value; z = B.outside_value; }
        return;
    }
    x = bc_axis<EXACT>(B.axis_kind[0], x, B.lo[0], B.hi[0], B.outside_value);
    y = bc_axis<EXACT>(B.axis_kind[1], y, B.lo[1], B.hi[1], B.outside_value);
    z = bc_axis<EXACT>(B.axis_kind[2], z, B.lo[2], B.hi[2], B.outside_value);
}

template <bool EXACT>
__device__ __forceinline__ void apply_boundary(const jt_boundary& B, float& x, float& y, float& z) {
    apply_boundary<EXACT>(B, inlet_frame(B), x, y, z);
}

// ---------------------------------------------------------------------------
// One integrator step, generic over the field evaluator.
//   RK4  rk4.py:82-106   k1..k4, x + (dt/6)*(((k1 + 2k2) + 2k3) + k4)
//   RK2  rk2.py:283-309  x + dt * v(x + dt/2 * v(x, t), t_mid)
//   Euler euler.py:146-157  x + dt * v(x, t)
// `s` points at the step's schedule entries (stage 0, mid, full).
// Compensated mode keeps a Kahan term c per coordinate for the final update.
// ---------------------------------------------------------------------------
struct StepConst {
    float dt, dth, dt6;
};

// Whether a field's evaluations are unrolled over the integrator stages: a
// field type may set kUnrollStages (a short evaluation body, where the loop's
// own instructions cost more than the larger code), otherwise the stage loop
// follows JT_STAGE_UNROLL.
template <class F, class = void>
struct UnrollStagesOf {
    static constexpr bool value = false;
};
template <class F>
struct UnrollStagesOf<F, decltype(void(F::kUnrollStages))> {
    static constexpr bool value = F::kUnrollStages;
};

// RK4 stage st: evaluate at xs, fold k into the weighted sum sm and move xs to
// the next stage position (rk4.py:82-106).
template <bool EXACT, class Field>
__device__ __forceinline__ void rk4_stage(const Field& f, const jt_blend* s, const StepConst& k, int st,
                                          const V3& x, V3& xs, V3& sm, int& flags) {
    typedef Ar<EXACT> A;
    const jt_blend e = s[st == 0 ? 0 : (st == 3 ? 2 : 1)];
    const V3 kk = f(xs, e, flags);
    if (st == 0) {
        sm = kk;
    } else if (st == 3) {
        sm = V3{A::add(sm.x, kk.x), A::add(sm.y, kk.y), A::add(sm.z, kk.z)};
    } else {
        sm = V3{A::axpy(sm.x, 2.0f, kk.x), A::axpy(sm.y, 2.0f, kk.y), A::axpy(sm.z, 2.0f, kk.z)};
    }
    const float h = st < 2 ? k.dth : k.dt;
    xs = V3{A::axpy(x.x, h, kk.x), A::axpy(x.y, h, kk.y), A::axpy(x.z, h, kk.z)};
}

// RK2 stage st: evaluate at xs and move xs to the midpoint (rk2.py:283-309).
template <bool EXACT, class Field>
__device__ __forceinline__ void rk2_stage(const Field& f, const jt_blend* s, const StepConst& k, int st,
                                          const V3& x, V3& xs, V3& v, int& flags) {
    typedef Ar<EXACT> A;
    const jt_blend e = s[st];
    v = f(xs, e, flags);
    xs = V3{A::axpy(x.x, k.dth, v.x), A::axpy(x.y, k.dth, v.y), A::axpy(x.z, k.dth, v.z)};
}

template <bool EXACT, int INTEG, bool COMP, class Field>
__device__ __forceinline__ void integrate(const Field& f, const jt_blend* s, const StepConst& k,
                                          V3& x, V3& c, int& flags) {
    typedef Ar<EXACT> A;
    V3 inc;  // the increment added to x
    if (INTEG == JT_RK4) {
        // One field-evaluation body, four trips: stage positions x + dth*k1,
        // x + dth*k2, x + dt*k3 and the sum ((k1 + 2k2) + 2k3) + k4 in the
        // reference's left-to-right order.
        V3 sm{0.f, 0.f, 0.f}, xs = x;
        if (UnrollStagesOf<Field>::value) {
#pragma unroll
            for (int st = 0; st < 4; ++st) rk4_stage<EXACT>(f, s, k, st, x, xs, sm, flags);
        } else {
JT_UNROLL(JT_STAGE_UNROLL)
            for (int st = 0; st < 4; ++st) rk4_stage<EXACT>(f, s, k, st, x, xs, sm, flags);
        }
        inc = V3{A::mul(k.dt6, sm.x), A::mul(k.dt6, sm.y), A::mul(k.dt6, sm.z)};
    } else if (INTEG == JT_RK2) {
        V3 xs = x, v{0.f, 0.f, 0.f};
        if (UnrollStagesOf<Field>::value) {
#pragma unroll
            for (int st = 0; st < 2; ++st) rk2_stage<EXACT>(f, s, k, st, x, xs, v, flags);
        } else {
JT_UNROLL(JT_STAGE_UNROLL)
            for (int st = 0; st < 2; ++st) rk2_stage<EXACT>(f, s, k, st, x, xs, v, flags);
        }
        inc = V3{A::mul(k.dt, v.x), A::mul(k.dt, v.y), A::mul(k.dt, v.z)};
    } else {
        const jt_blend e0 = s[0];
        V3 v = f(x, e0, flags);
        inc = V3{A::mul(k.dt, v.x), A::mul(k.dt, v.y), A::mul(k.dt, v.z)};
    }
    if (COMP) {
        // Kahan (1965) compensated summation of the position increments.
        float yx = inc.x - c.x, yy = inc.y - c.y, yz = inc.z - c.z;
        float tx = x.x + yx, ty = x.y + yy, tz = x.z + yz;
        c.x = __fsub_rn(__fsub_rn(tx, x.x), yx);
        c.y = __fsub_rn(__fsub_rn(ty, x.y), yy);
        c.z = __fsub_rn(__fsub_rn(tz, x.z), yz);
        x = V3{tx, ty, tz};
    } else {
        x = V3{A::add(x.x, inc.x), A::add(x.y, inc.y), A::add(x.z, inc.z)};
    }
}

// Whether a field's tracking kernels record velocities (a field type may
// set kRecordsVelocity false when its host never asks: the unused fifth
// evaluation then leaves the kernel).
template <class F, class = void>
struct RecordsVelocityOf {
    static constexpr bool value = true;
};
template <class F>
struct RecordsVelocityOf<F, decltype(void(F::kRecordsVelocity))> {
    static constexpr bool value = F::kRecordsVelocity;
};

// OR the per-thread status flags into the device status word, one atomic
// per warp.
__device__ __forceinline__ void report_flags(int32_t* status, int flags) {
    if (status == nullptr) return;
    const unsigned m = __activemask();
    const int f = __reduce_or_sync(m, flags);
    if (f != 0 && (threadIdx.x & 31) == (__ffs(m) - 1)) atomicOr(status, f);
}

// Ensemble of particle i: largest e with offsets[e] <= i.
__device__ __forceinline__ int find_ensemble(const int32_t* off, int n_ens, int i) {
    int lo = 0, hi = n_ens - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Persistent tracking kernel body: one particle per thread, the time loop in
// registers, boundary fused after every step, optional strided recording.
// PATH: P.path is set (the per-particle path length is accumulated); a
// template argument so that runs without it keep the register budget.
template <bool EXACT, int INTEG, bool PATH, int BK, class Field>
__device__ __forceinline__ void track_body(const Field& f, const jt_boundary& B, const InletFrame& I,
                                           const jt_track_params& P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n_particles) return;
    const bool comp = (P.arith == JT_ARITH_COMPENSATED) && P.comp != nullptr;
    const jt_blend* sched = P.schedule;
    if (P.ens_offsets != nullptr && P.n_ens > 0) {
        const int pid = P.ids != nullptr ? __ldg(P.ids + i) : i;
        sched += (int64_t)find_ensemble(P.ens_offsets, P.n_ens, pid) * P.schedule_stride;
    }
    float* pp = P.pos + 3 * (int64_t)i;
    V3 x{pp[0], pp[1], pp[2]};
    V3 c{0.f, 0.f, 0.f};
    if (comp) {
        const float* cp = P.comp + 3 * (int64_t)i;
        c = V3{cp[0], cp[1], cp[2]};
    }
    const StepConst k{P.dt, P.dt_half, P.dt_sixth};
    int flags = 0;
    const int64_t n = P.n_particles;
    // per-particle path length (Trajectory.compute_path_length over rows
    // recorded every step): float32 |x_after - x_before| summed in step order
    float plen = 0.0f;
    int64_t pid = 0;
    if (PATH) {
        pid = P.ids != nullptr ? (int64_t)P.ids[i] : (int64_t)i;
        plen = P.path[pid];
    }
    for (int s = P.step_begin; s < P.step_end; ++s) {
        const jt_blend* e = sched + 4 * (int64_t)s;
        const V3 xo = x;
        if (comp) integrate<EXACT, INTEG, true>(f, e, k, x, c, flags);
        else integrate<EXACT, INTEG, false>(f, e, k, x, c, flags);
        if constexpr (BK == JT_BK_INLET_XPOS) bc_inlet_xpos<EXACT>(B, I, x.x, x.y, x.z);
        else apply_boundary<EXACT>(B, I, x.x, x.y, x.z);
        if (PATH) {
            const float dx = __fsub_rn(x.x, xo.x), dy = __fsub_rn(x.y, xo.y), dz = __fsub_rn(x.z, xo.z);
            plen = __fadd_rn(plen, __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                        __fmul_rn(dz, dz))));
        }
        if (P.traj != nullptr) {
            const int cnt = s + 1;
            if (cnt % P.record_every == 0) {
                const int row = (P.record_compact ? cnt / P.record_every : cnt) - P.row_base;
                if (row >= 0 && row < P.n_rows) {
                    const int64_t id = P.ids != nullptr ? (int64_t)P.ids[i] : (int64_t)i;
                    float* o = P.traj + ((int64_t)row * n + id) * 3;
                    o[0] = x.x; o[1] = x.y; o[2] = x.z;
                    if (RecordsVelocityOf<Field>::value && P.vel != nullptr) {
                        const jt_blend er = e[3];
                        V3 v = f(x, er, flags);
                        float* ov = P.vel + ((int64_t)row * n + id) * 3;
                        ov[0] = v.x; ov[1] = v.y; ov[2] = v.z;
                    }
                }
            }
        }
    }
    pp[0] = x.x; pp[1] = x.y; pp[2] = x.z;
    if (PATH) P.path[pid] = plen;
    if (comp) {
        float* cp = P.comp + 3 * (int64_t)i;
        cp[0] = c.x; cp[1] = c.y; cp[2] = c.z;
    }
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) flags |= JT_STATUS_NONFINITE;
    report_flags(P.status, flags);
}

}  // namespace jt
