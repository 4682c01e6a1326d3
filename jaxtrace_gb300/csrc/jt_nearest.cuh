// Scattered-node field: nearest-node sampling of TimeSeriesField
// (fields/time_series.py:249-259 and :391-412).  The reference takes the
// argmin over all nodes of the float32 squared distance; here a uniform cell
// list limits the search to rings of cells around the query, and the ring
// loop stops once no unvisited cell can hold a point at or below the best
// squared distance.  Ties go to the lowest node index, as argmin does.
#pragma once

#include "jt_common.cuh"

namespace jt {

// Index of the node nearest to q (argmin of the float32 squared distance,
// lowest index on ties; 0 for a NaN query, whose distances are all NaN).
// h_min: the smallest cell edge, scaled down slightly (ring-stop bound).
template <bool EXACT>
__device__ __forceinline__ int nearest_id(const jt_nearest_field& F, float h_min, const V3& q) {
    typedef Ar<EXACT> A;
    if (q.x != q.x || q.y != q.y || q.z != q.z) return 0;
    const float qq[3] = {q.x, q.y, q.z};
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float f = floorf((qq[a] - F.origin[a]) * F.inv_cell[a]);
        int ci = (f != f) ? 0 : (f < 0.0f ? 0 : (f >= (float)F.cells[a] ? F.cells[a] - 1 : (int)f));
        c[a] = ci;
    }
    float best = __int_as_float(0x7f800000);
    int best_id = 0x7fffffff;
    const int rmax = max(F.cells[0], max(F.cells[1], F.cells[2]));
    for (int r = 0; r <= rmax; ++r) {
        if (r >= 2) {
            const float lb = (float)(r - 1) * h_min;
            if (lb * lb > best * 1.00001f) break;
        }
        for (int dz = -r; dz <= r; ++dz) {
            const int cz = c[2] + dz;
            if (cz < 0 || cz >= F.cells[2]) continue;
            for (int dy = -r; dy <= r; ++dy) {
                const int cy = c[1] + dy;
                if (cy < 0 || cy >= F.cells[1]) continue;
                const bool face = (dz == -r || dz == r || dy == -r || dy == r);
                for (int dx = -r; dx <= r; dx += (face ? 1 : 2 * r)) {
                    const int cx = c[0] + dx;
                    if (cx >= 0 && cx < F.cells[0]) {
                        const int cell = (cz * F.cells[1] + cy) * F.cells[0] + cx;
                        const int b = __ldg(F.cell_start + cell), en = __ldg(F.cell_start + cell + 1);
                        for (int s = b; s < en; ++s) {
                            const float4 p = __ldg(reinterpret_cast<const float4*>(F.points) + s);
                            const float ddx = A::sub(q.x, p.x), ddy = A::sub(q.y, p.y), ddz = A::sub(q.z, p.z);
                            const float d = A::add(A::add(A::mul(ddx, ddx), A::mul(ddy, ddy)), A::mul(ddz, ddz));
                            const int id = __ldg(F.point_ids + s);
                            if (d < best || (d == best && id < best_id)) { best = d; best_id = id; }
                        }
                    }
                    if (r == 0) break;
                }
            }
        }
    }
    return best_id == 0x7fffffff ? 0 : best_id;
}

template <bool EXACT, int STORE>
struct NearestField {
    jt_nearest_field F;
    float h_min;  // smallest cell edge

    static NearestField create(const jt_nearest_field& d, float h) { return NearestField{d, h}; }

    __device__ __forceinline__ V3 operator()(const V3& q, const jt_blend& e, int& flags) const {
        const int64_t base = (int64_t)min(max(e.pair, 0), F.n_pairs - 1) * F.pair_stride;
        return blend<EXACT, STORE>(load_pair<STORE>(F.pairs, base + nearest_id<EXACT>(F, h_min, q)), e);
    }
};

}  // namespace jt
