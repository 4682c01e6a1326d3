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

// float64 determinant of three float32 columns (same expansion as det3)
__device__ __forceinline__ double det3_f64(double a00, double a10, double a20, double a01, double a11, double a21,
                                           double a02, double a12, double a22) {
    return a00 * a11 * a22 + a01 * a12 * a20 + a02 * a10 * a21 - a02 * a11 * a20 - a00 * a12 * a21 -
           a01 * a10 * a22;
}

// Near-degenerate tetrahedra: |det| below this fraction of
// |v1-v0| |v2-v0| |v3-v0| (about 0.7 for a regular tetrahedron) loses float32
// digits in cancellation.  jt_mark_near_degenerate flags them in the pad slot
// after the box minimum (tet_box[8t+3] = 1); in the compensated arithmetic the
// float32 solve still decides which tetrahedron holds the query (the
// reference's decision) and the weights of a flagged one are solved again in
// float64.
constexpr float kNearDegenerate = 1e-2f;

__device__ __forceinline__ bool near_degenerate(const float* g12) {
    const V3 v01{g12[3], g12[4], g12[5]}, v02{g12[6], g12[7], g12[8]}, v03{g12[9], g12[10], g12[11]};
    const float det = det3<true>(v01, v02, v03);
    const float l1 = __fadd_rn(__fadd_rn(__fmul_rn(v01.x, v01.x), __fmul_rn(v01.y, v01.y)), __fmul_rn(v01.z, v01.z));
    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(v02.x, v02.x), __fmul_rn(v02.y, v02.y)), __fmul_rn(v02.z, v02.z));
    const float l3 = __fadd_rn(__fadd_rn(__fmul_rn(v03.x, v03.x), __fmul_rn(v03.y, v03.y)), __fmul_rn(v03.z, v03.z));
    return __fmul_rn(det, det) < __fmul_rn(kNearDegenerate * kNearDegenerate, __fmul_rn(__fmul_rn(l1, l2), l3));
}

// Barycentrics (b1, b2, b3 in y, z, w; b0 in x) of tetrahedron t in float64
// from its stored float32 geometry, rounded once to float32; |det| < 1e-10
// gives det = 1 as in the float32 solve.
static __device__ __noinline__ float4 bary_f64(const V3 q, const float* tet_geom, int t) {
    const float4* g = reinterpret_cast<const float4*>(tet_geom) + 4 * (int64_t)t;
    const float4 g0 = __ldg(g), g1 = __ldg(g + 1), g2 = __ldg(g + 2);
    const V3 v0{g0.x, g0.y, g0.z};
    const V3 a{g0.w, g1.x, g1.y}, b{g1.z, g1.w, g2.x}, c{g2.y, g2.z, g2.w};
    const double px = (double)q.x - (double)v0.x, py = (double)q.y - (double)v0.y, pz = (double)q.z - (double)v0.z;
    double det = det3_f64(a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z);
    if (fabs(det) < 1e-10) det = 1.0;
    const double y = det3_f64(px, py, pz, b.x, b.y, b.z, c.x, c.y, c.z) / det;
    const double z = det3_f64(a.x, a.y, a.z, px, py, pz, c.x, c.y, c.z) / det;
    const double w = det3_f64(a.x, a.y, a.z, b.x, b.y, b.z, px, py, pz) / det;
    return make_float4((float)(1.0 - y - z - w), (float)y, (float)z, (float)w);
}

// Barycentric test of tetrahedron t (point_in_tetrahedron_fast,
// …optimized.py:218-250, and point_in_tetrahedron, fem_interpolator.py:146-207,
// which compute the same thing): true when the query's box test and the
// tolerance test pass; b receives (b0, b1, b2, b3) as (x, y, z, w) and cn
// the vertex ids.
template <bool EXACT>
__device__ __forceinline__ bool tet_bary(const V3& q, const float* tet_box, const float* tet_geom, int t,
                                         float4& b, int4& cn, bool& near) {
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
    near = !EXACT && mn.w != 0.0f;
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

// NEAR: re-solve flagged near-degenerate tetrahedra in float64 (compensated
// arithmetic only); launched only for fields that have flagged ones, so the
// out-of-line call costs nothing elsewhere.
template <bool EXACT, int STORE, bool NEAR = false>
struct MeshFieldT {
    // the dependent gather chain is latency-bound: 4 blocks of 256 (64
    // registers, no spills) keep more warps in flight than the default 3
    static constexpr int kMinBlocks = JT_MESH_MIN_BLOCKS;
    jt_mesh_field F;

    static MeshFieldT create(const jt_mesh_field& d, int) { return MeshFieldT{d}; }

    __device__ __forceinline__ V3 node_value(int node, const jt_blend& e) const {
        const int64_t base = (int64_t)min(max(e.pair, 0), F.n_pairs - 1) * F.pair_stride;
        return blend<EXACT, STORE>(load_pair<STORE>(F.pairs, base + node), e);
    }

    __device__ __forceinline__ V3 operator()(const V3& q, const jt_blend& e, int& flags) const {
        typedef Ar<EXACT> A;
        // fixed-depth descent (…optimized.py:278-302): at most max_depth moves,
        // stopping at a leaf or where the query's octant has no child
        int node = 0;
        int2 oc;
        if (F.desc != nullptr) {
            // the same moves on the breadth-first copy: a child's index is the
            // node's first child plus the present octants below its own
            const int4* D = reinterpret_cast<const int4*>(F.desc);
            for (int d = 0; d < F.max_depth; ++d) {
                const int4 h = __ldg(D + node);
                const unsigned w = (unsigned)h.w, m = w & 0xffu;
                if (m == 0u) break;  // a leaf (or a node without children)
                const int oct = (q.x >= __int_as_float(h.x) ? 1 : 0) + (q.y >= __int_as_float(h.y) ? 2 : 0) +
                                (q.z >= __int_as_float(h.z) ? 4 : 0);
                if (!((m >> oct) & 1u)) break;
                node = (int)(w >> 8) + __popc(m & ((1u << oct) - 1u));
            }
            oc = __ldg(reinterpret_cast<const int2*>(F.dtab) + node);
        } else {
            for (int d = 0; d < F.max_depth; ++d) {
                const int4 h = __ldg(reinterpret_cast<const int4*>(F.nodes + node));
                if (h.w) break;  // is_leaf
                const int oct = (q.x >= __int_as_float(h.x) ? 1 : 0) + (q.y >= __int_as_float(h.y) ? 2 : 0) +
                                (q.z >= __int_as_float(h.z) ? 4 : 0);
                const int ch = __ldg(&F.nodes[node].children[oct]);
                if (ch < 0) break;
                node = ch;
            }
            oc = __ldg(reinterpret_cast<const int2*>(&F.nodes[node].elem_offset));
        }
        const int32_t* L = F.elems + oc.x;
        const int cnt = oc.y;
        // candidate scan (…optimized.py:309-360): first candidate whose box
        // holds the query and whose barycentrics pass the tolerance test
        for (int s = 0; s < cnt; ++s) {
            float4 b;
            int4 cn;
            bool near;
            const int t = __ldg(L + s);
            if (!tet_bary<EXACT>(q, F.tet_box, F.tet_geom, t, b, cn, near)) continue;
            if (NEAR && !EXACT && near) b = bary_f64(q, F.tet_geom, t);
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

template <bool EXACT, int STORE>
using MeshField = MeshFieldT<EXACT, STORE, false>;
template <bool EXACT, int STORE>
using MeshFieldNear = MeshFieldT<EXACT, STORE, true>;

}  // namespace jt
