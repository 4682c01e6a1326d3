// Candidate lists of the nearest-node search (jt_nearest_field.cand_*).
//
// For a cell B of the candidate grid (grown by kCandGrow of its edge on
// every side, which covers the float32 rounding of a query's cell
// coordinate), take any node m0 and U^2 = the largest squared distance from
// m0 to B: every query q in B has a node within U.  The float32 argmin w of
// q satisfies |q - w|^2 <= d32(q, w) (1 + e) <= d32(q, m0) (1 + e) <=
// U^2 (1 + e)^2, e < 1e-6 the relative error of a float32 squared distance
// (three subtractions, three products, two sums of non-negative terms), so
// w lies within that distance of B.  The list of B is every node whose
// squared distance to B is at most U^2 (1 + kCandSlack), as {x, y, z, id}
// records in the order of the field's cell list; m0 is the float32 nearest
// node of B's centre, which keeps U small.
#include <math.h>

#include "jt_internal.h"
#include "jt_nearest.cuh"

namespace jt {
namespace {

constexpr int kCandBlock = 128;
constexpr double kCandGrow = 1e-3;   // of a cell edge, on every side
constexpr double kCandSlack = 1e-4;  // relative, on squared distances

struct CandGrid {
    int cells[3];
    double origin[3];
    double edge[3];
};

// cell-list cell of coordinate x on axis a (the list's float32 cell of a
// node may differ by one at a face: callers widen ranges by one cell)
__device__ __forceinline__ int list_cell(const jt_nearest_field& F, int a, double x) {
    const double f = floor((x - (double)F.origin[a]) * (double)F.inv_cell[a]);
    if (!(f > 0.0)) return 0;  // also NaN
    const int last = F.cells[a] - 1;
    return f >= (double)last ? last : (int)f;
}

__device__ __forceinline__ double box_far2(const float4& p, const double* lo, const double* hi) {
    const double dx = fmax(fabs((double)p.x - lo[0]), fabs((double)p.x - hi[0]));
    const double dy = fmax(fabs((double)p.y - lo[1]), fabs((double)p.y - hi[1]));
    const double dz = fmax(fabs((double)p.z - lo[2]), fabs((double)p.z - hi[2]));
    return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ double box_near2(const float4& p, const double* lo, const double* hi) {
    const double px[3] = {(double)p.x, (double)p.y, (double)p.z};
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double g = px[a] < lo[a] ? lo[a] - px[a] : (px[a] > hi[a] ? px[a] - hi[a] : 0.0);
        s += g * g;
    }
    return s;
}

// FILL = false: the list length of each cell into count[c] and its sum
// into *total; FILL = true: the list of cell c into recs[start[c] ..].
// Both passes walk the same nodes in the same order.
template <bool FILL>
__global__ void __launch_bounds__(kCandBlock) k_cand(jt_nearest_field F, CandGrid G, float h_min, int64_t n_cells,
                                                     const int32_t* __restrict__ start, int32_t* __restrict__ count,
                                                     float4* __restrict__ recs, unsigned long long* total) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t n = 0;
    if (c < n_cells) {
        const int64_t cxy = (int64_t)G.cells[0] * G.cells[1];
        const int idx[3] = {(int)(c % G.cells[0]), (int)((c / G.cells[0]) % G.cells[1]), (int)(c / cxy)};
        double lo[3], hi[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = G.origin[a] + ((double)idx[a] - kCandGrow) * G.edge[a];
            hi[a] = G.origin[a] + ((double)idx[a] + 1.0 + kCandGrow) * G.edge[a];
        }
        const V3 mid{(float)(0.5 * (lo[0] + hi[0])), (float)(0.5 * (lo[1] + hi[1])), (float)(0.5 * (lo[2] + hi[2]))};
        int s0;
        nearest_core<true>(F, h_min, mid, false, s0);
        if (s0 >= 0) {
            const double u2 = box_far2(__ldg(reinterpret_cast<const float4*>(F.points) + s0), lo, hi) *
                              (1.0 + kCandSlack);
            const double u = sqrt(u2);
            int clo[3], chi[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                clo[a] = max(list_cell(F, a, lo[a] - u) - 1, 0);
                chi[a] = min(list_cell(F, a, hi[a] + u) + 1, F.cells[a] - 1);
            }
            const int64_t w = FILL ? (int64_t)start[c] : 0;
            for (int z = clo[2]; z <= chi[2]; ++z)
                for (int y = clo[1]; y <= chi[1]; ++y) {
                    const int64_t row = ((int64_t)z * F.cells[1] + y) * F.cells[0];
                    const int b = __ldg(F.cell_start + row + clo[0]), e = __ldg(F.cell_start + row + chi[0] + 1);
                    for (int s = b; s < e; ++s) {
                        const float4 p = __ldg(reinterpret_cast<const float4*>(F.points) + s);
                        if (box_near2(p, lo, hi) <= u2) {
                            if (FILL) recs[w + n] = make_float4(p.x, p.y, p.z, __int_as_float(__ldg(F.point_ids + s)));
                            ++n;
                        }
                    }
                }
        }
        if (!FILL) count[c] = n;
    }
    if (!FILL) {
        // the exact total (the offsets are 32-bit): one atomic per warp
        unsigned long long v = (unsigned long long)n;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(total, v);
    }
}

}  // namespace
}  // namespace jt

using namespace jt;

extern "C" int jt_nearest_candidates(const jt_nearest_field* F, const int32_t* cells, const float* origin,
                                     const float* inv_cell, int32_t* cand_start, float* cand_recs, int64_t* total,
                                     void* stream) {
    if (F == nullptr || cells == nullptr || origin == nullptr || inv_cell == nullptr || cand_start == nullptr ||
        total == nullptr)
        return set_error(JT_ERR_INVALID, "F, cells, origin, inv_cell, cand_start and total are required");
    if (F->n_points < 1 || F->points == nullptr || F->point_ids == nullptr || F->cell_start == nullptr)
        return set_error(JT_ERR_INVALID, "the field's node cell list is required");
    for (int a = 0; a < 3; ++a)
        if (F->cells[a] < 1 || !(F->inv_cell[a] > 0.0f))
            return set_error(JT_ERR_UNSUPPORTED, "candidate lists need nodes spread along every axis");
    CandGrid G{};
    int64_t n_cells = 1;
    for (int a = 0; a < 3; ++a) {
        if (cells[a] < 1 || !(inv_cell[a] > 0.0f) || !isfinite(inv_cell[a]) || !isfinite(origin[a]))
            return set_error(JT_ERR_INVALID, "candidate grid axis %d: cells >= 1, finite origin, inv_cell > 0", a);
        G.cells[a] = cells[a];
        G.origin[a] = (double)origin[a];
        G.edge[a] = 1.0 / (double)inv_cell[a];
        n_cells *= cells[a];
        if (n_cells >= (int64_t)1 << 30) return set_error(JT_ERR_INVALID, "at most 2^30 candidate cells");
    }
    jt_nearest_field f = *F;
    f.cand_start = nullptr;
    f.cand_recs = nullptr;
    const float h = nearest_min_cell_edge(f);
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned blocks = (unsigned)((n_cells + kCandBlock - 1) / kCandBlock);
    if (cand_recs != nullptr) {
        if (((uintptr_t)cand_recs & 15u) != 0) return set_error(JT_ERR_INVALID, "cand_recs must be 16-byte aligned");
        k_cand<true><<<blocks, kCandBlock, 0, s>>>(f, G, h, n_cells, cand_start, nullptr,
                                                   reinterpret_cast<float4*>(cand_recs), nullptr);
        return cuda_status(cudaGetLastError(), "candidate list fill");
    }
    unsigned long long* sum = nullptr;
    uint32_t *sums = nullptr, *sums2 = nullptr;
    cudaError_t e = dev_alloc(reinterpret_cast<void**>(&sum), sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = dev_alloc(reinterpret_cast<void**>(&sums), (size_t)scan_partials(n_cells + 1) * 4 + 16, s);
    if (e == cudaSuccess) e = dev_alloc(reinterpret_cast<void**>(&sums2), (size_t)scan_partials2(n_cells + 1) * 4 + 16, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sum, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(cand_start + n_cells, 0, sizeof(int32_t), s);
    if (e == cudaSuccess) {
        k_cand<false><<<blocks, kCandBlock, 0, s>>>(f, G, h, n_cells, nullptr, cand_start, nullptr, sum);
        e = cudaGetLastError();
    }
    int rc = cuda_status(e, "candidate list count");
    if (rc == JT_OK) rc = exclusive_scan_u32(reinterpret_cast<uint32_t*>(cand_start), n_cells + 1, sums, sums2, s);
    unsigned long long t = 0;
    if (rc == JT_OK) {
        e = cudaMemcpyAsync(&t, sum, sizeof(t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        rc = cuda_status(e, "candidate list total");
    }
    if (sums2 != nullptr) dev_free(sums2, s);
    if (sums != nullptr) dev_free(sums, s);
    if (sum != nullptr) dev_free(sum, s);
    if (rc != JT_OK) return rc;
    if (t >= (1ull << 31)) return set_error(JT_ERR_INVALID, "candidate lists hold %llu entries (at most 2^31 - 1)", t);
    *total = (int64_t)t;
    return JT_OK;
}
