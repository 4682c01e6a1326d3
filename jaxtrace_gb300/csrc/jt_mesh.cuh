// Tetrahedral-mesh field: octree point location and P1 interpolation with
// the semantics of fields/octree_fem_interpolator_optimized.py:253-380 and
// the float32 time blend of fields/time_series.py:175-184 (JAX path, which
// that field always uses: octree_fem_time_series_optimized.py:108).
#pragma once

#include "jt_common.cuh"

namespace jt {

// 3x3 determinant of the matrix whose COLUMNS are c0, c1, c2, expanded as
// JAX evaluates jnp.linalg.det for 3x3 inputs (six triple products summed
// left to right).  Used by point_in_tetrahedron_fast (…optimized.py:231-242).
template <bool EXACT>
__device__ __forceinline__ float det3(const V3& c0, const V3& c1, const V3& c2) {
    typedef Ar<EXACT> A;
    const float a00 = c0.x, a01 = c1.x, a02 = c2.x;
    const float a10 = c0.y, a11 = c1.y, a12 = c2.y;
    const float a20 = c0.z, a21 = c1.z, a22 = c2.z;
    const float t1 = A::mul(A::mul(a00, a11), a22);
    const float t2 = A::mul(A::mul(a01, a12), a20);
    const float t3 = A::mul(A::mul(a02, a10), a21);
    const float t4 = A::mul(A::mul(a02, a11), a20);
    const float t5 = A::mul(A::mul(a00, a12), a21);
    const float t6 = A::mul(A::mul(a01, a10), a22);
    return A::sub(A::sub(A::sub(A::add(A::add(t1, t2), t3), t4), t5), t6);
}

// Barycentric test of tetrahedron t (point_in_tetrahedron_fast,
// …optimized.py:218-250, and point_in_tetrahedron, fem_interpolator.py:146-207,
// which compute the same thing): true when the query's box test and the
// tolerance test pass; b receives (b0, b1, b2, b3) as (x, y, z, w) and cn
// the vertex ids.
template <bool EXACT>
__device__ __forceinline__ bool tet_bary(const V3& q, const float* tet_box, const float* tet_geom, int t,
                                         float4& b, int4& cn) {
    typedef Ar<EXACT> A;
    const float4* bx = reinterpret_cast<const float4*>(tet_box) + 2 * (int64_t)t;
    const float4 mn = __ldg(bx), mx = __ldg(bx + 1);
    if (!(q.x >= mn.x && q.y >= mn.y && q.z >= mn.z && q.x <= mx.x && q.y <= mx.y && q.z <= mx.z)) return false;
    const float4* g = reinterpret_cast<const float4*>(tet_geom) + 4 * (int64_t)t;
    const float4 g0 = __ldg(g), g1 = __ldg(g + 1), g2 = __ldg(g + 2);
    const V3 v0{g0.x, g0.y, g0.z};
    const V3 v01{g0.w, g1.x, g1.y}, v02{g1.z, g1.w, g2.x}, v03{g2.y, g2.z, g2.w};
    const V3 v0p{A::sub(q.x, v0.x), A::sub(q.y, v0.y), A::sub(q.z, v0.z)};
    float det = det3<EXACT>(v01, v02, v03);
    if (fabsf(det) < 1e-10f) det = 1.0f;
    b.y = A::div(det3<EXACT>(v0p, v02, v03), det);
    b.z = A::div(det3<EXACT>(v01, v0p, v03), det);
    b.w = A::div(det3<EXACT>(v01, v02, v0p), det);
    b.x = A::sub(A::sub(A::sub(1.0f, b.y), b.z), b.w);
    const float lo = -1e-6f, hi = 0.999999f;  // tol and 1 + tol as float32
    if (!(b.x >= lo && b.y >= lo && b.z >= lo && b.w >= lo && b.x <= hi && b.y <= hi && b.z <= hi && b.w <= hi))
        return false;
    cn = __ldg(reinterpret_cast<const int4*>(g + 3));
    return true;
}

// jnp.dot(bary, node_values): terms accumulated in vertex order.
template <bool EXACT>
__device__ __forceinline__ V3 p1_combine(const float4& b, const V3& n0, const V3& n1, const V3& n2, const V3& n3) {
    typedef Ar<EXACT> A;
    return V3{A::add(A::add(A::add(A::mul(b.x, n0.x), A::mul(b.y, n1.x)), A::mul(b.z, n2.x)), A::mul(b.w, n3.x)),
              A::add(A::add(A::add(A::mul(b.x, n0.y), A::mul(b.y, n1.y)), A::mul(b.z, n2.y)), A::mul(b.w, n3.y)),
              A::add(A::add(A::add(A::mul(b.x, n0.z), A::mul(b.y, n1.z)), A::mul(b.z, n2.z)), A::mul(b.w, n3.z))};
}

#ifndef JT_MESH_MIN_BLOCKS
#define JT_MESH_MIN_BLOCKS 4
#endif

template <bool EXACT, int STORE>
struct MeshField {
    // the dependent gather chain is latency-bound: 4 blocks of 256 (64
    // registers, no spills) keep more warps in flight than the default 3
    static constexpr int kMinBlocks = JT_MESH_MIN_BLOCKS;
    jt_mesh_field F;

    static MeshField create(const jt_mesh_field& d, int) { return MeshField{d}; }

    __device__ __forceinline__ V3 node_value(int node, const jt_blend& e) const {
        const int64_t base = (int64_t)min(max(e.pair, 0), F.n_pairs - 1) * F.pair_stride;
        return blend<EXACT, STORE>(load_pair<STORE>(F.pairs, base + node), e);
    }

    __device__ __forceinline__ V3 operator()(const V3& q, const jt_blend& e, int& flags) const {
        typedef Ar<EXACT> A;
        // fixed-depth descent (…optimized.py:278-302): at most max_depth moves,
        // stopping at a leaf or where the query's octant has no child
        int node = 0;
        for (int d = 0; d < F.max_depth; ++d) {
            const int4 h = __ldg(reinterpret_cast<const int4*>(F.nodes + node));
            if (h.w) break;  // is_leaf
            const int oct = (q.x >= __int_as_float(h.x) ? 1 : 0) + (q.y >= __int_as_float(h.y) ? 2 : 0) +
                            (q.z >= __int_as_float(h.z) ? 4 : 0);
            const int ch = __ldg(&F.nodes[node].children[oct]);
            if (ch < 0) break;
            node = ch;
        }
        const int2 oc = __ldg(reinterpret_cast<const int2*>(&F.nodes[node].elem_offset));
        const int32_t* L = F.elems + oc.x;
        const int cnt = oc.y;
        // candidate scan (…optimized.py:309-360): first candidate whose box
        // holds the query and whose barycentrics pass the tolerance test
        for (int s = 0; s < cnt; ++s) {
            float4 b;
            int4 cn;
            if (!tet_bary<EXACT>(q, F.tet_box, F.tet_geom, __ldg(L + s), b, cn)) continue;
            return p1_combine<EXACT>(b, node_value(cn.x, e), node_value(cn.y, e), node_value(cn.z, e),
                                     node_value(cn.w, e));
        }
        // cheap fallback (…optimized.py:364-376): nearest of the four vertices
        // of the first candidate; an empty list reads slot -1, which indexes
        // the last tetrahedron
        flags |= JT_STATUS_OCTREE_FALLBACK;
        int first = cnt > 0 ? __ldg(L) : -1;
        if (first < 0) first += F.n_tets;
        const int4 cn = __ldg(reinterpret_cast<const int4*>(F.tet_geom) + 4 * (int64_t)first + 3);
        const int ids[4] = {cn.x, cn.y, cn.z, cn.w};
        int best = ids[0];
        float bd = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 pk = __ldg(reinterpret_cast<const float4*>(F.points) + ids[k]);
            const float dx = A::sub(pk.x, q.x), dy = A::sub(pk.y, q.y), dz = A::sub(pk.z, q.z);
            const float d = A::add(A::add(A::mul(dx, dx), A::mul(dy, dy)), A::mul(dz, dz));
            if (k == 0 || d < bd) { bd = d; best = ids[k]; }
        }
        return node_value(best, e);
    }
};

}  // namespace jt
