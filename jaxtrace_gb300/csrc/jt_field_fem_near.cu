// Kernel instances of the hash-grid FEM field that re-solve flagged
// near-degenerate tetrahedra in float64 (compensated arithmetic), kept in
// their own translation unit so the build compiles them in parallel.
#include "jt_fem.cuh"
#include "jt_kernels.cuh"

namespace jt {
typedef Launcher<FemFieldNear, jt_fem_field, float> FemNearL;

float nearest_min_cell_edge(const jt_nearest_field& f);

int fem_track_near(const jt_fem_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    return FemNearL::track(f, nearest_min_cell_edge(f.nearest), f.nearest.storage, b, p, s);
}
int fem_step_near(const jt_fem_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
                  const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s) {
    return FemNearL::step(f, nearest_min_cell_edge(f.nearest), f.nearest.storage, arith, sb, integ, k, dtpp, xin,
                          xout, n, status, s);
}
int fem_sample_near(const jt_fem_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                    int m, int32_t* status, cudaStream_t s) {
    return FemNearL::sample(f, nearest_min_cell_edge(f.nearest), f.nearest.storage, arith, e, pos, out, m, status,
                            s);
}
}  // namespace jt
