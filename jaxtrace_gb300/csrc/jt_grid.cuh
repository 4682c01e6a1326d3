// Regular-grid field: trilinear interpolation of time-blended snapshots.
// Follows StructuredGridSampler.sample (fields/structured.py:284-349) applied
// to TimeSeriesField.sample_at_time (fields/time_series.py:326-367): the
// reference blends every node in time and then interpolates; here only the
// eight gathered corners are blended, with identical float32 rounding.
//
// Throughput: x and y components travel as float32x2 pairs through packed
// FMUL2/FADD2/FFMA2 instructions (each lane rounded like the scalar op, so
// the exact mode stays bit-identical), z components pair up across corners.
#pragma once

#include "jt_common.cuh"

namespace jt {

// Continuous index, cell and weight of one axis (structured.py:289-322).
// FMA_IDX (fast arithmetic only): the index as one FMA, x * inv_d + nofs with
// nofs = -x_min * inv_d.
template <bool EXACT, bool FMA_IDX = false>
__device__ __forceinline__ void grid_axis(float x, float org, float d, float inv_d, int n, int mode, float vhi,
                                          int& i0, int& i1, float& w, bool& valid, int& flags, float nofs = 0.0f) {
    typedef Ar<EXACT> A;
    // (x - x_min) / dx; the fast modes multiply by the reciprocal
    float f = EXACT ? __fdiv_rn(__fsub_rn(x, org), d) : (FMA_IDX ? fmaf(x, inv_d, nofs) : (x - org) * inv_d);
    if (mode == JT_GRID_PERIODIC) {
        const int nn = n > 1 ? n : 1;
        f = np_mod(f, (float)nn);          // np.mod(fx, max(Nx,1))
        const float fl = floorf(f);
        int i = (int)fl;                   // NaN converts to 0
        w = A::sub(f, fl);                 // fx - i0.astype(float32)
        if (i >= nn) {                     // mod rounded up to N: the reference
            i -= nn;                       // indexes out of bounds here; wrap
            flags |= JT_STATUS_INDEX_WRAPPED;
        }
        if (i < 0) i = 0;
        i0 = i;
        i1 = (i + 1 == nn) ? 0 : i + 1;    // (i0 + 1) % max(Nx,1)
        valid = true;
    } else {
        valid = (x >= org) && (x <= vhi);  // structured.py:299-302
        const float hi = (float)(n > 1 ? n - 1 : 0);
        // np.clip(fx, 0, max(Nx-1,0)); the fast modes clip with min/max, which
        // send NaN to cell 0 instead of carrying it in the weight (the
        // particle's position stays NaN either way)
        f = EXACT ? np_clip(f, 0.0f, hi) : fminf(fmaxf(f, 0.0f), hi);
        const float fl = floorf(f);
        // fl is an integer in [0, n-1] (n <= 2^24, so n-1 is exact), or NaN,
        // which converts to 0: the cell is always in range
        const int i = __float2int_rz(fl);
        w = A::sub(f, fl);
        i0 = i;
        i1 = (i + 1 > n - 1) ? (n - 1) : i + 1;  // np.clip(i0+1, 0, max(Nx-1,0))
    }
}

// A corner value after the time blend: (x,y) packed, z apart.
struct CV {
    float2 xy;
    float z;
};

template <bool EXACT, int STORE>
__device__ __forceinline__ CV blend_cv(const PairVal& p, const jt_blend& e, float2 WA, float2 WB, bool weighted) {
    if (weighted) {
        // wa*A + wb*B per component
        const float2 xy = dot2p<EXACT>(p.axy, WA, p.bxy, WB);
        return CV{xy, Ar<EXACT>::dot2(p.az, WA.x, p.bz, WB.x)};
    }
    const V3 v = blend<EXACT, STORE>(p, e);
    return CV{make_float2(v.x, v.y), v.z};
}

// structured.py:334-342: lerp in x, then y, then z; every product rounded
// before its sum in the exact mode.  x,y travel as packed pairs; z pairs up
// across corners: (c00z, c01z) and (c10z, c11z), then (c0z, c1z).
template <bool EXACT>
__device__ __forceinline__ V3 trilinear(const CV& v000, const CV& v100, const CV& v010, const CV& v110,
                                        const CV& v001, const CV& v101, const CV& v011, const CV& v111, float wx,
                                        float wy, float wz) {
    typedef Ar<EXACT> A;
    const float ox = A::sub(1.0f, wx), oy = A::sub(1.0f, wy), oz = A::sub(1.0f, wz);
    const float2 OX = splat(ox), WX = splat(wx), OY = splat(oy), WY = splat(wy), OZ = splat(oz), WZ = splat(wz);
    const float2 c00 = dot2p<EXACT>(v000.xy, OX, v100.xy, WX);
    const float2 c10 = dot2p<EXACT>(v010.xy, OX, v110.xy, WX);
    const float2 c01 = dot2p<EXACT>(v001.xy, OX, v101.xy, WX);
    const float2 c11 = dot2p<EXACT>(v011.xy, OX, v111.xy, WX);
    const float2 c0 = dot2p<EXACT>(c00, OY, c10, WY);
    const float2 c1 = dot2p<EXACT>(c01, OY, c11, WY);
    const float2 rxy = dot2p<EXACT>(c0, OZ, c1, WZ);
    const float2 cz0 = dot2p<EXACT>(make_float2(v000.z, v001.z), OX, make_float2(v100.z, v101.z), WX);
    const float2 cz1 = dot2p<EXACT>(make_float2(v010.z, v011.z), OX, make_float2(v110.z, v111.z), WX);
    const float2 cz = dot2p<EXACT>(cz0, OY, cz1, WY);
    return V3{rxy.x, rxy.y, A::dot2(cz.x, oz, cz.y, wz)};
}

// b - a on a pair, as one packed FMA with -1 (exact: a single rounding).
__device__ __forceinline__ float2 sub2(float2 b, float2 a) { return __ffma2_rn(a, make_float2(-1.0f, -1.0f), b); }

// Fast-arithmetic trilinear in lerp form, a + w (b - a) per level: the same
// x, then y, then z order without the (1 - w) weights.
__device__ __forceinline__ V3 trilinear_lerp(const CV& v000, const CV& v100, const CV& v010, const CV& v110,
                                             const CV& v001, const CV& v101, const CV& v011, const CV& v111, float wx,
                                             float wy, float wz) {
    const float2 WX = splat(wx), WY = splat(wy), WZ = splat(wz);
    const float2 c00 = __ffma2_rn(WX, sub2(v100.xy, v000.xy), v000.xy);
    const float2 c10 = __ffma2_rn(WX, sub2(v110.xy, v010.xy), v010.xy);
    const float2 c01 = __ffma2_rn(WX, sub2(v101.xy, v001.xy), v001.xy);
    const float2 c11 = __ffma2_rn(WX, sub2(v111.xy, v011.xy), v011.xy);
    const float2 c0 = __ffma2_rn(WY, sub2(c10, c00), c00);
    const float2 c1 = __ffma2_rn(WY, sub2(c11, c01), c01);
    const float2 rxy = __ffma2_rn(WZ, sub2(c1, c0), c0);
    const float2 z0 = make_float2(v000.z, v001.z), z1 = make_float2(v010.z, v011.z);
    const float2 cz0 = __ffma2_rn(WX, sub2(make_float2(v100.z, v101.z), z0), z0);
    const float2 cz1 = __ffma2_rn(WX, sub2(make_float2(v110.z, v111.z), z1), z1);
    const float2 cz = __ffma2_rn(WY, sub2(cz1, cz0), cz0);
    return V3{rxy.x, rxy.y, fmaf(wz, cz.y - cz.x, cz.x)};
}

// One 32-byte float16 yz-quad record.
struct alignas(32) Quad32 {
    uint4 lo, hi;
};

__device__ __forceinline__ float2 h2f2(uint32_t w) { return __half22float2(*reinterpret_cast<const __half2*>(&w)); }

template <bool EXACT, int STORE>
struct GridField {
    jt_grid_field F;

    static GridField create(const jt_grid_field& d, int) { return GridField{d}; }

    __device__ __forceinline__ V3 operator()(const V3& p, const jt_blend& e, int& flags) const {
        typedef Ar<EXACT> A;
        int i0, i1, j0, j1, k0, k1;
        float wx, wy, wz;
        bool vx, vy, vz;
        grid_axis<EXACT>(p.x, F.origin[0], F.spacing[0], F.inv_spacing[0], F.nx, F.bounds_mode, F.valid_hi[0], i0,
                         i1, wx, vx, flags);
        grid_axis<EXACT>(p.y, F.origin[1], F.spacing[1], F.inv_spacing[1], F.ny, F.bounds_mode, F.valid_hi[1], j0,
                         j1, wy, vy, flags);
        grid_axis<EXACT>(p.z, F.origin[2], F.spacing[2], F.inv_spacing[2], F.nz, F.bounds_mode, F.valid_hi[2], k0,
                         k1, wz, vz, flags);

        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        const int64_t base = (int64_t)pr * F.pair_stride;
        const int ny = F.ny, nz = F.nz;
        const int r00 = (i0 * ny + j0) * nz, r10 = (i1 * ny + j0) * nz;
        const int r01 = (i0 * ny + j1) * nz, r11 = (i1 * ny + j1) * nz;
        // all gathers issued before any use: eight 32-byte float32 node
        // records, or two 48-byte 16-bit yz-quad records (i0 and i1)
        PairVal p000, p100, p010, p110, p001, p101, p011, p111;
        if (STORE == JT_STORE_F32) {
            p000 = load_pair<STORE>(F.pairs, base + (r00 + k0));
            p100 = load_pair<STORE>(F.pairs, base + (r10 + k0));
            p010 = load_pair<STORE>(F.pairs, base + (r01 + k0));
            p110 = load_pair<STORE>(F.pairs, base + (r11 + k0));
            p001 = load_pair<STORE>(F.pairs, base + (r00 + k1));
            p101 = load_pair<STORE>(F.pairs, base + (r10 + k1));
            p011 = load_pair<STORE>(F.pairs, base + (r01 + k1));
            p111 = load_pair<STORE>(F.pairs, base + (r11 + k1));
        } else {
            const int64_t part_b = (int64_t)F.n_pairs * F.pair_stride;
            load_quad<STORE>(F.pairs, part_b, base + (r00 + k0), p000, p001, p010, p011);
            load_quad<STORE>(F.pairs, part_b, base + (r10 + k0), p100, p101, p110, p111);
        }
        const bool wgt = e.form == JT_BLEND_WEIGHTED;
        const float2 WA = splat(e.wa), WB = splat(e.wb);
        const CV v000 = blend_cv<EXACT, STORE>(p000, e, WA, WB, wgt), v100 = blend_cv<EXACT, STORE>(p100, e, WA, WB, wgt);
        const CV v010 = blend_cv<EXACT, STORE>(p010, e, WA, WB, wgt), v110 = blend_cv<EXACT, STORE>(p110, e, WA, WB, wgt);
        const CV v001 = blend_cv<EXACT, STORE>(p001, e, WA, WB, wgt), v101 = blend_cv<EXACT, STORE>(p101, e, WA, WB, wgt);
        const CV v011 = blend_cv<EXACT, STORE>(p011, e, WA, WB, wgt), v111 = blend_cv<EXACT, STORE>(p111, e, WA, WB, wgt);

        V3 r = trilinear<EXACT>(v000, v100, v010, v110, v001, v101, v011, v111, wx, wy, wz);
        if (F.bounds_mode == JT_GRID_ZERO || F.bounds_mode == JT_GRID_NAN) {
            if (!(vx && vy && vz)) {
                const float o = F.bounds_mode == JT_GRID_ZERO ? 0.0f : __int_as_float(0x7fc00000);
                r = V3{o, o, o};
            }
        }
        return r;
    }
};

__device__ __forceinline__ __half2 u2h2(uint32_t w) { return *reinterpret_cast<const __half2*>(&w); }

// a + w (b - a) on half pairs
__device__ __forceinline__ __half2 hlerp2(__half2 w, __half2 a, __half2 b) { return __hfma2(w, __hsub2(b, a), a); }

// Offset yz-quad of a float16 stage field (32 B): the blended values of the
// nodes (j,k), (j,k1), (j1,k), (j1,k1) of one x plane, each stored as
// o + r with a per-quad offset o and float16 residuals r:
//   words 0-3  (rx, ry) of the four nodes      words 4-5  (rz, rz) pairs
//   word 6     ox as float32
//   word 7     a float32 whose value is oy; its low 16 bits are oz as a
//              float16 (the encoder measures oy with them in place)
// The residuals are the spread of four neighbouring values, small beside the
// values, so float16 arithmetic on them rounds far below the values' own
// float16 rounding.  Returns the bilinear (y, then z) value at (wy, wz).
__device__ __forceinline__ V3 quad_yz(const uint32_t (&q)[8], __half2 WY, __half2 WZ) {
    const __half2 ck = hlerp2(WY, u2h2(q[0]), u2h2(q[2]));   // (x, y) at k
    const __half2 ck1 = hlerp2(WY, u2h2(q[1]), u2h2(q[3]));  // (x, y) at k1
    const float2 rxy = __half22float2(hlerp2(WZ, ck, ck1));
    const __half2 zy = hlerp2(WY, u2h2(q[4]), u2h2(q[5]));   // (z at k, z at k1)
    const __half rz = __hfma(__high2half(WZ), __hsub(__high2half(zy), __low2half(zy)), __low2half(zy));
    const float oz = __low2float(u2h2(q[7]));
    const float2 v = __fadd2_rn(make_float2(__uint_as_float(q[6]), __uint_as_float(q[7])), rxy);
    return V3{v.x, v.y, oz + __half2float(rz)};
}

// Pre-blended stage field of a time chunk: one time level per schedule entry
// (slot = e.pair), blended per node ahead of the tracking launch exactly as
// TimeSeriesField.sample_at_time blends every node (time_series.py:326-367)
// before StructuredGridSampler interpolates -- the reference's own order, so
// the exact mode is bit-identical to blending the gathered corners.
//   JT_STORE_STAGE_F32: float4 {x, y, z, 0} per node (16 B);
//   JT_STORE_STAGE_F32Q: float32 yz-quads per node (48 B): a 32 B part with
//     the (x, y) of nodes (j,k), (j,k1), (j1,k), (j1,k1) and, after the part
//     A records of every node of the slot, a 16 B part with their z -- the
//     same float32 values as STAGE_F32 in four loads per evaluation instead
//     of eight;
//   JT_STORE_STAGE_F16: offset yz-quads per node (32 B, quad_yz), values
//     divided by the power-of-two scale carried in e.wa.  Two 256-bit loads
//     per evaluation measured faster than eight 64-bit loads of float16 node
//     records, although those fit L2 and the quads do not.
// Blocks of 256 per SM the stage-field kernels are compiled for, measured on
// the precision configuration: float16 offset quads 6 (42 registers, 12 B
// of spills; 1.6 % faster than 5 without spills), float32 quads 5 in the
// exact arithmetic (2.8 % faster than 4 despite spills) and 4 in the fast
// one (5 was 12 % slower).
#ifndef JT_STAGE16_MIN_BLOCKS
#define JT_STAGE16_MIN_BLOCKS 6
#endif
#ifndef JT_STAGE32_MIN_BLOCKS
#define JT_STAGE32_MIN_BLOCKS 4
#endif
#ifndef JT_STAGE32X_MIN_BLOCKS
#define JT_STAGE32X_MIN_BLOCKS 5
#endif

//
// MODE >= 0 fixes the bounds mode at compile time (clamp and periodic, the
// common ones), which removes the mode tests and the unused validity tests
// from every evaluation; MODE < 0 reads F.bounds_mode at run time.  The fast
// arithmetic maps coordinates to indices with one FMA and interpolates in
// lerp form.
template <bool EXACT, int OUT, int MODE = -1>
struct StageGridField {
    static constexpr int kMinBlocks = OUT == JT_STORE_STAGE_F16
                                          ? JT_STAGE16_MIN_BLOCKS
                                          : (EXACT && OUT == JT_STORE_STAGE_F32Q ? JT_STAGE32X_MIN_BLOCKS
                                                                                 : JT_STAGE32_MIN_BLOCKS);
    // the evaluation is short enough that the kernel is bound by instruction
    // issue: unrolled stages drop the loop's own instructions
    static constexpr bool kUnrollStages = true;
    // the host gathers snapshot pairs when it records velocities
    static constexpr bool kRecordsVelocity = false;
    // the inlet configuration runs on a clamped grid.  Measured on it: float32
    // quads 1.1 % (exact) and 0.7 % (compensated) faster; offset float16
    // quads 2.6 % slower (spills at 6 blocks/SM), so they keep the run-time
    // boundary
    static constexpr bool kInletXpos = MODE == JT_GRID_CLAMP && OUT != JT_STORE_STAGE_F16;
    jt_grid_field F;
    float nofs[3];  // -origin * inv_spacing per axis (fast arithmetic)
    int sx;         // node stride of the x axis, ny * nz

    __host__ __device__ static StageGridField create(const jt_grid_field& d, int) {
        StageGridField s{d, {0.0f, 0.0f, 0.0f}, d.ny * d.nz};
        for (int a = 0; a < 3; ++a) s.nofs[a] = -d.origin[a] * d.inv_spacing[a];
        return s;
    }

    __device__ __forceinline__ V3 operator()(const V3& p, const jt_blend& e, int& flags) const {
        const int mode = MODE >= 0 ? MODE : F.bounds_mode;
        int i0, i1, j0, j1, k0, k1;
        float wx, wy, wz;
        bool vx, vy, vz;
        grid_axis<EXACT, !EXACT>(p.x, F.origin[0], F.spacing[0], F.inv_spacing[0], F.nx, mode, F.valid_hi[0], i0,
                                 i1, wx, vx, flags, nofs[0]);
        grid_axis<EXACT, !EXACT>(p.y, F.origin[1], F.spacing[1], F.inv_spacing[1], F.ny, mode, F.valid_hi[1], j0,
                                 j1, wy, vy, flags, nofs[1]);
        grid_axis<EXACT, !EXACT>(p.z, F.origin[2], F.spacing[2], F.inv_spacing[2], F.nz, mode, F.valid_hi[2], k0,
                                 k1, wz, vz, flags, nofs[2]);
        const int slot = min(max(e.pair, 0), F.n_pairs - 1);
        const int64_t base = (int64_t)slot * F.pair_stride;
        // 32-bit node offsets within the slot (fewer than 2^31 nodes), scaled
        // to bytes by the wide multiply-add of the address
        const int nz = F.nz;
        const int n000 = i0 * sx + (j0 * nz + k0);
        const int n100 = n000 + (i1 - i0) * sx;
        CV v000, v100, v010, v110, v001, v101, v011, v111;
        V3 r;
        if (OUT == JT_STORE_STAGE_F32Q) {
            // slot = pair_stride part-A records (32 B) then pair_stride part-B records (16 B)
            const char* sb = reinterpret_cast<const char*>(F.pairs) + base * 48;
            const char* pb = sb + F.pair_stride * 32;
            uint32_t a0[8], a1[8];
            ldg256(sb + (int64_t)n000 * 32, a0);
            ldg256(sb + (int64_t)n100 * 32, a1);
            const float4 z0 = __ldg(reinterpret_cast<const float4*>(pb) + n000);
            const float4 z1 = __ldg(reinterpret_cast<const float4*>(pb) + n100);
            const auto f2 = [](uint32_t x, uint32_t y) { return make_float2(__uint_as_float(x), __uint_as_float(y)); };
            v000 = CV{f2(a0[0], a0[1]), z0.x}; v001 = CV{f2(a0[2], a0[3]), z0.y};
            v010 = CV{f2(a0[4], a0[5]), z0.z}; v011 = CV{f2(a0[6], a0[7]), z0.w};
            v100 = CV{f2(a1[0], a1[1]), z1.x}; v101 = CV{f2(a1[2], a1[3]), z1.y};
            v110 = CV{f2(a1[4], a1[5]), z1.z}; v111 = CV{f2(a1[6], a1[7]), z1.w};
            r = EXACT ? trilinear<EXACT>(v000, v100, v010, v110, v001, v101, v011, v111, wx, wy, wz)
                      : trilinear_lerp(v000, v100, v010, v110, v001, v101, v011, v111, wx, wy, wz);
        } else if (OUT == JT_STORE_STAGE_F32) {
            const int dy = (j1 - j0) * nz, dz = k1 - k0;
            const float4* b4 = reinterpret_cast<const float4*>(F.pairs) + base;
            const float4 a000 = __ldg(b4 + n000), a100 = __ldg(b4 + n100);
            const float4 a010 = __ldg(b4 + (n000 + dy)), a110 = __ldg(b4 + (n100 + dy));
            const float4 a001 = __ldg(b4 + (n000 + dz)), a101 = __ldg(b4 + (n100 + dz));
            const float4 a011 = __ldg(b4 + (n000 + dy + dz)), a111 = __ldg(b4 + (n100 + dy + dz));
            v000 = CV{make_float2(a000.x, a000.y), a000.z}; v100 = CV{make_float2(a100.x, a100.y), a100.z};
            v010 = CV{make_float2(a010.x, a010.y), a010.z}; v110 = CV{make_float2(a110.x, a110.y), a110.z};
            v001 = CV{make_float2(a001.x, a001.y), a001.z}; v101 = CV{make_float2(a101.x, a101.y), a101.z};
            v011 = CV{make_float2(a011.x, a011.y), a011.z}; v111 = CV{make_float2(a111.x, a111.y), a111.z};
            r = EXACT ? trilinear<EXACT>(v000, v100, v010, v110, v001, v101, v011, v111, wx, wy, wz)
                      : trilinear_lerp(v000, v100, v010, v110, v001, v101, v011, v111, wx, wy, wz);
        } else {
            uint32_t q0[8], q1[8];
            const Quad32* bq = reinterpret_cast<const Quad32*>(F.pairs) + base;
            ldg256(bq + n000, q0);
            ldg256(bq + n100, q1);
            // y and z in float16 pairs on the small residuals of each x plane,
            // x in float32 on the planes' values
            const __half2 WY = __float2half2_rn(wy), WZ = __float2half2_rn(wz);
            const V3 a = quad_yz(q0, WY, WZ);
            const V3 b = quad_yz(q1, WY, WZ);
            const float2 axy = make_float2(a.x, a.y);
            const float2 rxy = __ffma2_rn(splat(wx), sub2(make_float2(b.x, b.y), axy), axy);
            const float rz = fmaf(wx, b.z - a.z, a.z);
            r = V3{rxy.x * e.wa, rxy.y * e.wa, rz * e.wa};
        }
        if (mode == JT_GRID_ZERO || mode == JT_GRID_NAN) {
            if (!(vx && vy && vz)) {
                const float o = mode == JT_GRID_ZERO ? 0.0f : __int_as_float(0x7fc00000);
                r = V3{o, o, o};
            }
        }
        return r;
    }
};

}  // namespace jt
