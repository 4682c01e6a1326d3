// Kernel instances for the nearest-node field (TimeSeriesField spatial
// sampling, time_series.py:391-412).
#include "jt_kernels.cuh"
#include "jt_nearest.cuh"

namespace jt {
typedef Launcher<NearestField, jt_nearest_field, float> NearL;

float nearest_min_cell_edge(const jt_nearest_field& f) {
    float h = 3.4e38f;
    for (int a = 0; a < 3; ++a) {
        if (f.cells[a] > 1 && f.inv_cell[a] > 0.0f) {
            const float e = 1.0f / f.inv_cell[a];
            h = e < h ? e : h;
        }
    }
    // with a single cell on every axis the ring search visits everything at r=0
    return h < 3.4e38f ? h * 0.999f : 0.0f;
}

int nearest_track(const jt_nearest_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    return NearL::track(f, nearest_min_cell_edge(f), f.storage, b, p, s);
}
int nearest_step(const jt_nearest_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
                 const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s) {
    return NearL::step(f, nearest_min_cell_edge(f), f.storage, arith, sb, integ, k, dtpp, xin, xout, n, status, s);
}
int nearest_sample(const jt_nearest_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                   int m, int32_t* status, cudaStream_t s) {
    return NearL::sample(f, nearest_min_cell_edge(f), f.storage, arith, e, pos, out, m, status, s);
}
}  // namespace jt
