// Kernel instances for the regular-grid field (trilinear, structured.py).
#include "jt_grid.cuh"
#include "jt_kernels.cuh"

namespace jt {
typedef Launcher<GridField, jt_grid_field, int> GridL;

int grid_track(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    if (f.storage == JT_STORE_STAGE_F32 || f.storage == JT_STORE_STAGE_F16 || f.storage == JT_STORE_STAGE_F32Q)
        return stage_track(f, b, p, s);
    return GridL::track(f, 0, f.storage, b, p, s);
}
int grid_step(const jt_grid_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
              const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s) {
    if (f.storage > JT_STORE_F16) return set_error(JT_ERR_UNSUPPORTED, "stage fields are for jt_track only");
    return GridL::step(f, 0, f.storage, arith, sb, integ, k, dtpp, xin, xout, n, status, s);
}
int grid_sample(const jt_grid_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                int m, int32_t* status, cudaStream_t s) {
    if (f.storage > JT_STORE_F16) return set_error(JT_ERR_UNSUPPORTED, "stage fields are for jt_track only");
    return GridL::sample(f, 0, f.storage, arith, e, pos, out, m, status, s);
}
}  // namespace jt
