// Regular-grid field: trilinear interpolation of time-blended snapshots.
// Follows StructuredGridSampler.sample (fields/structured.py:284-349) applied
// to TimeSeriesField.sample_at_time (fields/time_series.py:326-367): the
// reference blends every node in time and then interpolates; here only the
// eight gathered corners are blended, with identical float32 rounding.
#pragma once

#include "jt_common.cuh"

namespace jt {

// Continuous index, cell and weight of one axis (structured.py:289-322).
template <bool EXACT>
__device__ __forceinline__ void grid_axis(float x, float org, float d, int n, int mode, float vhi,
                                          int& i0, int& i1, float& w, bool& valid, int& flags) {
    typedef Ar<EXACT> A;
    float f = A::div(A::sub(x, org), d);  // (x - x_min) / dx
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
        f = np_clip(f, 0.0f, hi);          // np.clip(fx, 0, max(Nx-1,0))
        const float fl = floorf(f);
        int i = (int)fl;
        if (i < 0) i = 0;
        if (i > n - 1) i = n - 1;
        w = A::sub(f, fl);
        i0 = i;
        i1 = (i + 1 > n - 1) ? (n - 1) : i + 1;  // np.clip(i0+1, 0, max(Nx-1,0))
    }
}

template <bool EXACT, int STORE>
struct GridField {
    jt_grid_field F;

    static GridField create(const jt_grid_field& d, int) { return GridField{d}; }

    __device__ __forceinline__ V3 operator()(const V3& p, const jt_blend& e, int& flags) const {
        typedef Ar<EXACT> A;
        int i0, i1, j0, j1, k0, k1;
        float wx, wy, wz;
        bool vx, vy, vz;
        grid_axis<EXACT>(p.x, F.origin[0], F.spacing[0], F.nx, F.bounds_mode, F.valid_hi[0], i0, i1, wx, vx, flags);
        grid_axis<EXACT>(p.y, F.origin[1], F.spacing[1], F.ny, F.bounds_mode, F.valid_hi[1], j0, j1, wy, vy, flags);
        grid_axis<EXACT>(p.z, F.origin[2], F.spacing[2], F.nz, F.bounds_mode, F.valid_hi[2], k0, k1, wz, vz, flags);

        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        const int64_t base = (int64_t)pr * F.pair_stride;
        const int ny = F.ny, nz = F.nz;
        const int64_t r00 = ((int64_t)i0 * ny + j0) * nz, r10 = ((int64_t)i1 * ny + j0) * nz;
        const int64_t r01 = ((int64_t)i0 * ny + j1) * nz, r11 = ((int64_t)i1 * ny + j1) * nz;
        // all eight gathers issued before any use
        const PairVal p000 = load_pair<STORE>(F.pairs, base + r00 + k0);
        const PairVal p100 = load_pair<STORE>(F.pairs, base + r10 + k0);
        const PairVal p010 = load_pair<STORE>(F.pairs, base + r01 + k0);
        const PairVal p110 = load_pair<STORE>(F.pairs, base + r11 + k0);
        const PairVal p001 = load_pair<STORE>(F.pairs, base + r00 + k1);
        const PairVal p101 = load_pair<STORE>(F.pairs, base + r10 + k1);
        const PairVal p011 = load_pair<STORE>(F.pairs, base + r01 + k1);
        const PairVal p111 = load_pair<STORE>(F.pairs, base + r11 + k1);
        const V3 v000 = blend<EXACT, STORE>(p000, e), v100 = blend<EXACT, STORE>(p100, e);
        const V3 v010 = blend<EXACT, STORE>(p010, e), v110 = blend<EXACT, STORE>(p110, e);
        const V3 v001 = blend<EXACT, STORE>(p001, e), v101 = blend<EXACT, STORE>(p101, e);
        const V3 v011 = blend<EXACT, STORE>(p011, e), v111 = blend<EXACT, STORE>(p111, e);

        // structured.py:334-342: lerp in x, then y, then z
        const float ox = A::sub(1.0f, wx), oy = A::sub(1.0f, wy), oz = A::sub(1.0f, wz);
        V3 r;
#define JT_TRI(c)                                                      \
    {                                                                  \
        const float c00 = A::dot2(v000.c, ox, v100.c, wx);             \
        const float c10 = A::dot2(v010.c, ox, v110.c, wx);             \
        const float c01 = A::dot2(v001.c, ox, v101.c, wx);             \
        const float c11 = A::dot2(v011.c, ox, v111.c, wx);             \
        const float c0 = A::dot2(c00, oy, c10, wy);                    \
        const float c1 = A::dot2(c01, oy, c11, wy);                    \
        r.c = A::dot2(c0, oz, c1, wz);                                 \
    }
        JT_TRI(x) JT_TRI(y) JT_TRI(z)
#undef JT_TRI
        if (F.bounds_mode == JT_GRID_ZERO || F.bounds_mode == JT_GRID_NAN) {
            if (!(vx && vy && vz)) {
                const float o = F.bounds_mode == JT_GRID_ZERO ? 0.0f : __int_as_float(0x7fc00000);
                r = V3{o, o, o};
            }
        }
        return r;
    }
};

}  // namespace jt
