// Kernel instances of the tetrahedral-mesh field that re-solve flagged
// near-degenerate tetrahedra in float64 (compensated arithmetic), kept in
// their own translation unit so the build compiles them in parallel.
#include "jt_kernels.cuh"
#include "jt_mesh.cuh"

namespace jt {
typedef Launcher<MeshFieldNear, jt_mesh_field, int> MeshNearL;

int mesh_track_near(const jt_mesh_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    return MeshNearL::track(f, 0, f.storage, b, p, s);
}
int mesh_step_near(const jt_mesh_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
                   const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s) {
    return MeshNearL::step(f, 0, f.storage, arith, sb, integ, k, dtpp, xin, xout, n, status, s);
}
int mesh_sample_near(const jt_mesh_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                     int m, int32_t* status, cudaStream_t s) {
    return MeshNearL::sample(f, 0, f.storage, arith, e, pos, out, m, status, s);
}
}  // namespace jt
