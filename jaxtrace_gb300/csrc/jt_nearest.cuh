// Scattered-node field: nearest-node sampling of TimeSeriesField
// (fields/time_series.py:249-259 and :391-412).  The reference takes the
// argmin over all nodes of the float32 squared distance; here a uniform cell
// list limits the search to rings of cells around the query, and the ring
// loop stops once no unvisited cell can hold a point at or below the best
// squared distance.  Ties go to the lowest node index, as argmin does.
#pragma once

#include "jt_common.cuh"

namespace jt {

// Nodes [b, en) of the sorted node array against the best so far: argmin of
// the float32 squared distance, lowest id on ties.  The id is read only for
// a distance at or below the best (a new best or a tie).
template <bool EXACT>
__device__ __forceinline__ void nearest_scan(const jt_nearest_field& F, const V3& q, int b, int en, float& best,
                                             int& best_id) {
    typedef Ar<EXACT> A;
    for (int s = b; s < en; ++s) {
        const float4 p = __ldg(reinterpret_cast<const float4*>(F.points) + s);
        const float ddx = A::sub(q.x, p.x), ddy = A::sub(q.y, p.y), ddz = A::sub(q.z, p.z);
        const float d = A::add(A::add(A::mul(ddx, ddx), A::mul(ddy, ddy)), A::mul(ddz, ddz));
        if (d <= best) {
            const int id = __ldg(F.point_ids + s);
            if (d < best || id < best_id) { best = d; best_id = id; }
        }
    }
}

// Lower bound of the distance from the query to a neighbouring row of cells
// along one axis, in cell units: 0 for its own row, else the gap from its
// continuous cell coordinate f to the shared cell face, less 1e-3 of a cell
// for the float32 rounding of f and of the nodes' own cell coordinates.
__device__ __forceinline__ float row_gap(int d, float frac) {
    const float g = d < 0 ? frac : (d > 0 ? 1.0f - frac : 0.0f);
    return fmaxf(g - 1e-3f, 0.0f);
}

// Index of the node nearest to q (argmin of the float32 squared distance,
// lowest index on ties; 0 for a NaN query, whose distances are all NaN).
// h_min: the smallest cell edge, scaled down slightly (ring-stop bound).
// Cells are walked in rows along x: a row's cells are consecutive in the
// cell list, so their nodes are one range of the sorted node array.  In the
// first ring a row whose gap from the query already exceeds the best
// distance (with a 1e-4 relative margin) is skipped; no node in it can reach
// the best or tie with it.
template <bool EXACT>
__device__ __forceinline__ int nearest_id(const jt_nearest_field& F, float h_min, const V3& q) {
    if (q.x != q.x || q.y != q.y || q.z != q.z) return 0;
    const float qq[3] = {q.x, q.y, q.z};
    int c[3];
    float frac[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float fc = (qq[a] - F.origin[a]) * F.inv_cell[a];
        const float f = floorf(fc);
        int ci = (f != f) ? 0 : (f < 0.0f ? 0 : (f >= (float)F.cells[a] ? F.cells[a] - 1 : (int)f));
        c[a] = ci;
        // the query's position inside its cell (clamped cells: the nearer face)
        frac[a] = fminf(fmaxf(fc - (float)ci, 0.0f), 1.0f);
    }
    const int nx = F.cells[0], ny = F.cells[1], nz = F.cells[2];
    const float hy = 1.0f / F.inv_cell[1], hz = 1.0f / F.inv_cell[2];
    float best = __int_as_float(0x7f800000);
    int best_id = 0x7fffffff;
    const int rmax = max(nx, max(ny, nz));
    for (int r = 0; r <= rmax; ++r) {
        if (r >= 2) {
            const float lb = (float)(r - 1) * h_min;
            if (lb * lb > best * 1.00001f) break;
        }
        for (int dz = -r; dz <= r; ++dz) {
            const int cz = c[2] + dz;
            if (cz < 0 || cz >= nz) continue;
            for (int dy = -r; dy <= r; ++dy) {
                const int cy = c[1] + dy;
                if (cy < 0 || cy >= ny) continue;
                if (r == 1 && (dy != 0 || dz != 0) && F.inv_cell[1] > 0.0f && F.inv_cell[2] > 0.0f) {
                    const float gy = row_gap(dy, frac[1]) * hy, gz = row_gap(dz, frac[2]) * hz;
                    if ((gy * gy + gz * gz) * 0.9999f > best) continue;
                }
                const int row = (cz * ny + cy) * nx;
                const bool face = (dz == -r || dz == r || dy == -r || dy == r);
                if (face) {  // the whole row [c - r, c + r] as one node range
                    const int x0 = max(c[0] - r, 0), x1 = min(c[0] + r, nx - 1);
                    nearest_scan<EXACT>(F, q, __ldg(F.cell_start + row + x0), __ldg(F.cell_start + row + x1 + 1),
                                        best, best_id);
                } else {     // the two end cells of an inner row
                    if (c[0] - r >= 0) {
                        const int cell = row + c[0] - r;
                        nearest_scan<EXACT>(F, q, __ldg(F.cell_start + cell), __ldg(F.cell_start + cell + 1),
                                            best, best_id);
                    }
                    if (c[0] + r < nx) {
                        const int cell = row + c[0] + r;
                        nearest_scan<EXACT>(F, q, __ldg(F.cell_start + cell), __ldg(F.cell_start + cell + 1),
                                            best, best_id);
                    }
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
