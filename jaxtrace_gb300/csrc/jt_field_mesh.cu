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
}  // namespace jt
