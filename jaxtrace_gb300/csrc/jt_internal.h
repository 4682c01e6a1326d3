// Library-internal declarations: error state and the per-field launchers.
#pragma once

#include <cuda_runtime.h>

#include "../../include/jaxtrace_gb300.h"

namespace jt {

// Record `msg` as the calling thread's last error and return `code`.
int set_error(int code, const char* fmt, ...);
// JT_OK for cudaSuccess, else JT_ERR_CUDA with the CUDA error string.
int cuda_status(cudaError_t e, const char* what);
// Grid shape limits the kernels rely on: every axis 1..2^24 nodes (its last
// index is exact in float32, so a clipped coordinate floors to a valid cell)
// and fewer than 2^31 nodes (32-bit node offsets within a snapshot).
int check_grid_shape(const jt_grid_field& g);
// tiles[] of an affine-tile storage against the grid shape, and its base array
int check_tiles(const jt_grid_field& g);

// Device scratch of the library's own (the device builds and their handles,
// the near-degenerate count): through the allocator jt_set_allocator
// installed, else cudaMallocAsync / cudaFreeAsync, ordered on `s`.
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s);
void dev_free(void* p, cudaStream_t s);

// Exclusive scan of n uint32 values in place (n <= scan_capacity()); sums
// holds scan_partials(n) values, sums2 scan_partials2(n) (one up to
// 2^22 items).
int64_t scan_capacity();
int64_t scan_partials(int64_t n);
int64_t scan_partials2(int64_t n);
int exclusive_scan_u32(uint32_t* data, int64_t n, uint32_t* sums, uint32_t* sums2, cudaStream_t st);

struct StageBlends;
struct StepConst;

int grid_track(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s);
int grid_step(const jt_grid_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
              const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s);
int grid_sample(const jt_grid_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                int m, int32_t* status, cudaStream_t s);

int mesh_track(const jt_mesh_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s);
int mesh_step(const jt_mesh_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
              const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s);
int mesh_sample(const jt_mesh_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                int m, int32_t* status, cudaStream_t s);

int mesh_track_near(const jt_mesh_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s);
int mesh_step_near(const jt_mesh_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
                   const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s);
int mesh_sample_near(const jt_mesh_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                     int m, int32_t* status, cudaStream_t s);

int nearest_track(const jt_nearest_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s);
int nearest_step(const jt_nearest_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
                 const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s);
int nearest_sample(const jt_nearest_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                   int m, int32_t* status, cudaStream_t s);

int stage_track(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s);

int fem_track(const jt_fem_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s);
int fem_step(const jt_fem_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
             const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s);
int fem_sample(const jt_fem_field& f, int arith, const jt_blend& e, const float* pos, float* out,
               int m, int32_t* status, cudaStream_t s);
int fem_track_near(const jt_fem_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s);
int fem_step_near(const jt_fem_field& f, int arith, const StageBlends& sb, int integ, StepConst k,
                  const float* dtpp, const float* xin, float* xout, int n, int32_t* status, cudaStream_t s);
int fem_sample_near(const jt_fem_field& f, int arith, const jt_blend& e, const float* pos, float* out,
                    int m, int32_t* status, cudaStream_t s);

}  // namespace jt
