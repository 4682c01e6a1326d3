// Tetrahedral-mesh field with the hash-grid point location of
// FEMTimeSeriesField (fields/fem_time_series.py:16-110) and
// interpolate_in_mesh (fields/fem_interpolator.py:210-328): the query's cell
// of a uniform grid over the node bounding box, that cell's elements in
// ascending order, the first whose box and barycentric test hold the query
// gives P1; with none, the value of the nearest node of the whole mesh.  The
// time blend is the float32 one of TimeSeriesField's JAX path
// (fem_time_series.py:104).
#pragma once

#include "jt_mesh.cuh"
#include "jt_nearest.cuh"

namespace jt {

// NEAR as in MeshFieldT
template <bool EXACT, int STORE, bool NEAR = false>
struct FemFieldT {
    static constexpr int kMinBlocks = JT_MESH_MIN_BLOCKS;
    jt_fem_field F;
    float h_min;  // smallest nearest-node cell edge (ring-stop bound)

    static FemFieldT create(const jt_fem_field& d, float h) { return FemFieldT{d, h}; }

    __device__ __forceinline__ V3 node_value(int node, const jt_blend& e) const {
        const int64_t base = (int64_t)min(max(e.pair, 0), F.nearest.n_pairs - 1) * F.nearest.pair_stride;
        return blend<EXACT, STORE>(load_pair<STORE>(F.nearest.pairs, base + node), e);
    }

    // floor((q - grid_min) / cell_size).astype(int32) clipped to [0, n-1]
    // (fem_interpolator.py:262-263); the float clamp before the conversion
    // is XLA's saturating float->int (NaN lands on 0).
    __device__ __forceinline__ int cell_coord(float q, float lo, float cs, int n) const {
        typedef Ar<EXACT> A;
        const float f = floorf(A::div(A::sub(q, lo), cs));
        return (int)fminf(fmaxf(f, 0.0f), (float)(n - 1));
    }

    // sub-cell of coordinate q inside hash cell c: floor((q - (lo + c*cs)) /
    // (cs/S)) clipped to [0, S-1]; the host lists widen the sub-cells enough
    // to absorb the rounding of this float32 arithmetic
    __device__ __forceinline__ int sub_coord(float q, float lo, float cs, int c, int S) const {
        const float cell_lo = lo + (float)c * cs;
        const float f = floorf((q - cell_lo) * ((float)S / cs));
        return (int)fminf(fmaxf(f, 0.0f), (float)(S - 1));
    }

    __device__ __forceinline__ V3 operator()(const V3& q, const jt_blend& e, int& flags) const {
        const int cx = cell_coord(q.x, F.grid_min[0], F.cell_size[0], F.grid_size[0]);
        const int cy = cell_coord(q.y, F.grid_min[1], F.cell_size[1], F.grid_size[1]);
        const int cz = cell_coord(q.z, F.grid_min[2], F.cell_size[2], F.grid_size[2]);
        const int cell = (cx * F.grid_size[1] + cy) * F.grid_size[2] + cz;
        const int32_t* list = F.cell_elems;
        int b0, b1;
        if (F.sub_div > 0) {
            // the query's sub-cell, clamped into its hash cell
            const int S = F.sub_div;
            const int sx = sub_coord(q.x, F.grid_min[0], F.cell_size[0], cx, S);
            const int sy = sub_coord(q.y, F.grid_min[1], F.cell_size[1], cy, S);
            const int sz = sub_coord(q.z, F.grid_min[2], F.cell_size[2], cz, S);
            const int64_t sc = (int64_t)cell * (S * S * S) + (sx * S + sy) * S + sz;
            b0 = __ldg(F.sub_start + sc);
            b1 = __ldg(F.sub_start + sc + 1);
            list = F.sub_elems;
        } else {
            b0 = __ldg(F.cell_start + cell);
            b1 = __ldg(F.cell_start + cell + 1);
        }
        // lax.scan over the cell's candidates keeps the first hit (:280-305)
        for (int s = b0; s < b1; ++s) {
            float4 b;
            int4 cn;
            bool near;
            const int t = __ldg(list + s);
            if (!tet_bary<EXACT>(q, F.tet_box, F.tet_geom, t, b, cn, near)) continue;
            if (NEAR && !EXACT && near) b = bary_f64(q, F.tet_geom, t);
            return p1_combine<EXACT>(b, node_value(cn.x, e), node_value(cn.y, e), node_value(cn.z, e),
                                     node_value(cn.w, e));
        }
        // global nearest node (:311-316)
        flags |= JT_STATUS_OCTREE_FALLBACK;
        return node_value(nearest_id<EXACT>(F.nearest, h_min, q), e);
    }
};

template <bool EXACT, int STORE>
using FemField = FemFieldT<EXACT, STORE, false>;
template <bool EXACT, int STORE>
using FemFieldNear = FemFieldT<EXACT, STORE, true>;

}  // namespace jt
