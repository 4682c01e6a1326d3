// Kernel instances for the hash-grid FEM field (FEMTimeSeriesField,
// fem_time_series.py / fem_interpolator.py).
#include "jt_fem.cuh"
#include "jt_kernels.cuh"

namespace jt {
typedef Launcher<FemField, jt_fem_field, float> FemL;

float nearest_min_cell_edge(const jt_nearest_field& f);

// fields with flagged near-degenerate tetrahedra run the float64 re-solve
// variants (jt_field_fem_near.cu) in the compensated arithmetic
int fem_track(const jt_fem_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    if (f.near_degenerate && p.arith != JT_ARITH_EXACT) return fem_track_near(f, b, p, s);
    return FemL::track(f, nearest_min_cell_edge(f.nearest), f.nearest.storage, b, p, s);
}
int fem_step(const jt_fem_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
             const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s) {
    if (f.near_degenerate && arith != JT_ARITH_EXACT)
        return fem_step_near(f, arith, sb, integ, k, dtpp, xin, xout, n, status, s);
    return FemL::step(f, nearest_min_cell_edge(f.nearest), f.nearest.storage, arith, sb, integ, k, dtpp, xin, xout,
                      n, status, s);
}
int fem_sample(const jt_fem_field& f, int arith, const jt_blend& e, const float* pos, float* out,
               int m, int32_t* status, cudaStream_t s) {
    if (f.near_degenerate && arith != JT_ARITH_EXACT) return fem_sample_near(f, arith, e, pos, out, m, status, s);
    return FemL::sample(f, nearest_min_cell_edge(f.nearest), f.nearest.storage, arith, e, pos, out, m, status, s);
}
}  // namespace jt
