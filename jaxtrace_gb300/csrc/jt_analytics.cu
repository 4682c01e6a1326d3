// Trajectory analytics on the device.
//
// The Lyapunov-like term of compute_mixing_metrics
// (tracking/analysis.py:297-312): over every ordered pair (i, j) of
// particles whose initial distance d0 = |x0_i - x0_j| satisfies
// 0 < d0 < rmax, the mean of log(d1 / d0) with d1 = |x1_i - x1_j|.  The
// reference builds the two N x N distance matrices on the host; here one
// thread owns particle i and walks j in shared-memory tiles, with the
// distances, the ratio and the cutoff test in the reference's float32
// arithmetic (sqrt((dx*dx + dy*dy) + dz*dz), each operation rounded) and
// the log terms summed in float64.
#include <stdint.h>

#include "jt_internal.h"
#include "jt_kernels.cuh"

namespace jt {

constexpr int kPairTile = 256;

__device__ __forceinline__ float dist3(float ax, float ay, float az, float bx, float by, float bz) {
    const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}

__global__ void __launch_bounds__(kPairTile) k_pair_log_ratio(const float* __restrict__ x0, const float* __restrict__ x1,
                                                              int n, float rmax, double* __restrict__ sum,
                                                              unsigned long long* __restrict__ count) {
    __shared__ float s0[kPairTile][3];
    __shared__ float s1[kPairTile][3];
    const int i = blockIdx.x * kPairTile + threadIdx.x;
    const bool live = i < n;
    float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
    if (live) {
        ax = x0[3 * (int64_t)i]; ay = x0[3 * (int64_t)i + 1]; az = x0[3 * (int64_t)i + 2];
        bx = x1[3 * (int64_t)i]; by = x1[3 * (int64_t)i + 1]; bz = x1[3 * (int64_t)i + 2];
    }
    double acc = 0.0;
    unsigned long long cnt = 0;
    for (int base = 0; base < n; base += kPairTile) {
        const int j = base + threadIdx.x;
        if (j < n) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                s0[threadIdx.x][a] = x0[3 * (int64_t)j + a];
                s1[threadIdx.x][a] = x1[3 * (int64_t)j + a];
            }
        }
        __syncthreads();
        const int m = min(kPairTile, n - base);
        if (live) {
            float part = 0.0f;
            int pc = 0;
            for (int k = 0; k < m; ++k) {
                const float d0 = dist3(ax, ay, az, s0[k][0], s0[k][1], s0[k][2]);
                if (d0 > 0.0f && d0 < rmax) {
                    const float d1 = dist3(bx, by, bz, s1[k][0], s1[k][1], s1[k][2]);
                    part += logf(__fdiv_rn(d1, d0));
                    ++pc;
                }
            }
            acc += (double)part;
            cnt += (unsigned long long)pc;
        }
        __syncthreads();
    }
    // warp sums, one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sum, acc);
        atomicAdd(count, cnt);
    }
}

}  // namespace jt

using namespace jt;

extern "C" int jt_pair_log_ratio(const float* x0, const float* x1, int32_t n, float rmax, double* out_sum,
                                 unsigned long long* out_count, void* stream) {
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (out_sum == nullptr || out_count == nullptr) return set_error(JT_ERR_INVALID, "out_sum and out_count are required");
    if (n > 0 && (x0 == nullptr || x1 == nullptr)) return set_error(JT_ERR_INVALID, "x0 and x1 are required");
    if (!(rmax > 0.0f)) return set_error(JT_ERR_INVALID, "rmax must be > 0");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(out_sum, 0, sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(out_count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_status(e, "pair sum reset");
    if (n == 0) return JT_OK;
    const unsigned g = (unsigned)((n + kPairTile - 1) / kPairTile);
    k_pair_log_ratio<<<g, kPairTile, 0, s>>>(x0, x1, n, rmax, out_sum, out_count);
    return cuda_status(cudaGetLastError(), "pair log-ratio kernel launch");
}
