// Kernel instances for the tetrahedral-mesh field (octree + P1,
// octree_fem_interpolator_optimized.py).
#include "jt_kernels.cuh"
#include "jt_mesh.cuh"

namespace jt {
typedef Launcher<MeshField, jt_mesh_field, int> MeshL;

// fields with flagged near-degenerate tetrahedra run the float64 re-solve
// variants (jt_field_mesh_near.cu) in the compensated arithmetic
int mesh_track(const jt_mesh_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    if (f.near_degenerate && p.arith != JT_ARITH_EXACT) return mesh_track_near(f, b, p, s);
    return MeshL::track(f, 0, f.storage, b, p, s);
}
int mesh_step(const jt_mesh_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
              const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s) {
    if (f.near_degenerate && arith != JT_ARITH_EXACT)
        return mesh_step_near(f, arith, sb, integ, k, dtpp, xin, xout, n, status, s);
    return MeshL::step(f, 0, f.storage, arith, sb, integ, k, dtpp, xin, xout, n, status, s);
}
int mesh_sample(const jt_mesh_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                int m, int32_t* status, cudaStream_t s) {
    if (f.near_degenerate && arith != JT_ARITH_EXACT) return mesh_sample_near(f, arith, e, pos, out, m, status, s);
    return MeshL::sample(f, 0, f.storage, arith, e, pos, out, m, status, s);
}

// Candidate prefilter records (jt_mesh_prefilter), one thread per octree
// node: the node's candidate box (union of its list's tet boxes), then per
// list slot the tet's box relative to it as float16, the lower ends rounded
// down and the upper ends up, each first moved outward by 1e-3 of its
// magnitude (at least 6.2e-8) -- twice the query's float16 rounding error
// (2^-12 relative, or 3e-8 below the normal range) plus its float32 one.
__global__ void __launch_bounds__(kBlock) k_mesh_prefilter(jt_mesh_field F, uint4* __restrict__ eq,
                                                           float4* __restrict__ nq) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= F.n_nodes) return;
    const int2 oc = __ldg(reinterpret_cast<const int2*>(&F.nodes[node].elem_offset));
    float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int s = 0; s < oc.y; ++s) {
        const float4* bx = reinterpret_cast<const float4*>(F.tet_box) + 2 * (int64_t)__ldg(F.elems + oc.x + s);
        const float4 a = __ldg(bx), b = __ldg(bx + 1);
        mn[0] = fminf(mn[0], a.x); mn[1] = fminf(mn[1], a.y); mn[2] = fminf(mn[2], a.z);
        mx[0] = fmaxf(mx[0], b.x); mx[1] = fmaxf(mx[1], b.y); mx[2] = fmaxf(mx[2], b.z);
    }
    float inv[3];
    for (int a = 0; a < 3; ++a) {
        if (oc.y == 0) mn[a] = mx[a] = 0.0f;
        const float ext = mx[a] - mn[a];
        inv[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    nq[2 * node] = make_float4(mn[0], mn[1], mn[2], 0.0f);
    nq[2 * node + 1] = make_float4(inv[0], inv[1], inv[2], 0.0f);
    for (int s = 0; s < oc.y; ++s) {
        const int t = __ldg(F.elems + oc.x + s);
        const float4* bx = reinterpret_cast<const float4*>(F.tet_box) + 2 * (int64_t)t;
        const float4 a = __ldg(bx), b = __ldg(bx + 1);
        const float lo3[3] = {a.x, a.y, a.z}, hi3[3] = {b.x, b.y, b.z};
        __half lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {
            const float l = __fmul_rd(__fsub_rd(lo3[k], mn[k]), inv[k]);
            const float h = __fmul_ru(__fsub_ru(hi3[k], mn[k]), inv[k]);
            lo[k] = __float2half_rd(__fsub_rd(l, fmaxf(fabsf(l), 6.2e-5f) * 1e-3f));
            hi[k] = __float2half_ru(__fadd_ru(h, fmaxf(fabsf(h), 6.2e-5f) * 1e-3f));
        }
        const __half2 w1 = __halves2half2(lo[0], lo[1]), w2 = __halves2half2(hi[0], hi[1]);
        const __half2 w3 = __halves2half2(lo[2], __hneg(hi[2]));
        eq[oc.x + s] = make_uint4((uint32_t)t, *reinterpret_cast<const uint32_t*>(&w1),
                                  *reinterpret_cast<const uint32_t*>(&w2), *reinterpret_cast<const uint32_t*>(&w3));
    }
}

}  // namespace jt

using namespace jt;

extern "C" int jt_mesh_prefilter(const jt_mesh_field* mesh, int32_t n_elem_entries, uint32_t* elem_q, float* node_q,
                                 void* stream) {
    if (mesh == nullptr) return set_error(JT_ERR_INVALID, "mesh field descriptor is NULL");
    if (mesh->n_nodes < 1 || mesh->nodes == nullptr || mesh->elems == nullptr || mesh->tet_box == nullptr)
        return set_error(JT_ERR_INVALID, "mesh field needs octree nodes, element lists and tet boxes");
    if (n_elem_entries < 0) return set_error(JT_ERR_INVALID, "n_elem_entries must be >= 0");
    if (elem_q == nullptr || node_q == nullptr) return set_error(JT_ERR_INVALID, "elem_q and node_q are required");
    k_mesh_prefilter<<<grid_blocks(mesh->n_nodes), kBlock, 0, (cudaStream_t)stream>>>(
        *mesh, reinterpret_cast<uint4*>(elem_q), reinterpret_cast<float4*>(node_q));
    return cuda_status(cudaGetLastError(), "mesh prefilter launch");
}
