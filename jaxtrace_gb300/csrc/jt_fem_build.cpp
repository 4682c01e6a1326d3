// Host build of the hash grid of FEMTimeSeriesField (build_tetrahedral_mesh,
// fields/fem_interpolator.py:36-143) and of its sub-cell refinement.
//
// Cell lists: an element is listed in every cell its float32 box overlaps,
// with the reference's arithmetic -- the float32 box offset from the float32
// grid minimum, divided by the float64 cell edge, floored, clipped to the
// grid -- in ascending element order per cell (a counting sort over the
// (element, cell) entries taken in element order, which is stable).
//
// Sub-cell lists: each (element, cell) entry is listed in the sub-cells of
// that cell (sub_div^3 per cell) its box, widened by eps (per axis), meets; the
// sub-cell index is floor((box - cell corner) / (edge / sub_div)) in float64,
// clipped.  The element the cell scan would pick holds the query in its box,
// so it is on the query's sub-cell list, and the list keeps ascending order.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "../../include/jaxtrace_gb300.h"
#include "jt_internal.h"

namespace {

struct FemGrid {
    std::vector<int32_t> cell_start, cell_elems, sub_start, sub_elems;
    int32_t max_per_cell = 0;
};

inline int64_t clip64(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

// floor(x) as an int64 clipped to [0, hi]; anything not >= 0 (NaN included)
// gives 0
inline int64_t cell_index(double x, int64_t hi) {
    const double f = floor(x);
    if (!(f >= 0.0)) return 0;
    if (f >= (double)hi) return hi;
    return (int64_t)f;
}

}  // namespace

using jt::set_error;

extern "C" int jt_fem_grid_build(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                                 const int32_t* grid_size, const float* grid_min, const double* cell_edge,
                                 int32_t sub_div, const double* eps, void** handle_out, jt_fem_grid_info* info) {
    if (handle_out == nullptr || info == nullptr) return set_error(JT_ERR_INVALID, "handle_out and info are required");
    *handle_out = nullptr;
    if (n_points < 0 || n_tets < 0) return set_error(JT_ERR_INVALID, "negative sizes");
    if (n_tets > 0 && (points == nullptr || conn == nullptr)) return set_error(JT_ERR_INVALID, "points and conn are required");
    if (grid_size == nullptr || grid_min == nullptr || cell_edge == nullptr)
        return set_error(JT_ERR_INVALID, "grid_size, grid_min and cell_edge are required");
    int64_t gs[3];
    for (int a = 0; a < 3; ++a) {
        if (grid_size[a] < 1) return set_error(JT_ERR_INVALID, "grid_size must be positive");
        gs[a] = grid_size[a];
    }
    const int64_t n_cells = gs[0] * gs[1] * gs[2];
    if (n_cells > (int64_t)1 << 30) return set_error(JT_ERR_INVALID, "too many hash cells");
    if (sub_div < 0 || sub_div > 16) return set_error(JT_ERR_INVALID, "sub_div must be 0..16");
    if (sub_div > 0 && eps == nullptr) return set_error(JT_ERR_INVALID, "eps (3 margins) is required with sub_div");
    for (int64_t t = 0; t < n_tets; ++t)
        for (int k = 0; k < 4; ++k)
            if (conn[4 * t + k] < 0 || conn[4 * t + k] >= n_points)
                return set_error(JT_ERR_INVALID, "connectivity indexes outside the points array");
    FemGrid* G = new (std::nothrow) FemGrid();
    if (G == nullptr) return set_error(JT_ERR_NOMEM, "out of host memory");
    try {
        // element boxes and their cell ranges
        std::vector<float> emin((size_t)n_tets * 3), emax((size_t)n_tets * 3);
        std::vector<int64_t> cmin((size_t)n_tets * 3), cmax((size_t)n_tets * 3);
        for (int64_t t = 0; t < n_tets; ++t) {
            for (int a = 0; a < 3; ++a) {
                float lo = points[3 * (int64_t)conn[4 * t] + a], hi = lo;
                for (int k = 1; k < 4; ++k) {
                    const float v = points[3 * (int64_t)conn[4 * t + k] + a];
                    lo = v < lo ? v : lo;
                    hi = v > hi ? v : hi;
                }
                emin[3 * t + a] = lo;
                emax[3 * t + a] = hi;
                // (float32 offset) / (float64 edge), floored, clipped
                const float dlo = lo - grid_min[a], dhi = hi - grid_min[a];
                cmin[3 * t + a] = cell_index((double)dlo / cell_edge[a], gs[a] - 1);
                cmax[3 * t + a] = cell_index((double)dhi / cell_edge[a], gs[a] - 1);
            }
        }
        // counting sort of the (element, cell) entries by cell, elements ascending
        std::vector<int64_t> count((size_t)n_cells + 1, 0);
        for (int64_t t = 0; t < n_tets; ++t)
            for (int64_t i = cmin[3 * t]; i <= cmax[3 * t]; ++i)
                for (int64_t j = cmin[3 * t + 1]; j <= cmax[3 * t + 1]; ++j)
                    for (int64_t k = cmin[3 * t + 2]; k <= cmax[3 * t + 2]; ++k) ++count[(i * gs[1] + j) * gs[2] + k];
        G->cell_start.assign((size_t)n_cells + 1, 0);
        int64_t total = 0;
        for (int64_t c = 0; c < n_cells; ++c) {
            G->cell_start[c] = (int32_t)total;
            G->max_per_cell = std::max<int32_t>(G->max_per_cell, (int32_t)count[c]);
            total += count[c];
            if (total > INT32_MAX) throw std::bad_alloc();
        }
        G->cell_start[n_cells] = (int32_t)total;
        G->cell_elems.assign((size_t)total, 0);
        std::vector<int32_t> cursor(G->cell_start.begin(), G->cell_start.end() - 1);
        for (int64_t t = 0; t < n_tets; ++t)
            for (int64_t i = cmin[3 * t]; i <= cmax[3 * t]; ++i)
                for (int64_t j = cmin[3 * t + 1]; j <= cmax[3 * t + 1]; ++j)
                    for (int64_t k = cmin[3 * t + 2]; k <= cmax[3 * t + 2]; ++k)
                        G->cell_elems[cursor[(i * gs[1] + j) * gs[2] + k]++] = (int32_t)t;
        // sub-cells
        if (sub_div > 0 && total > 0) {
            const int64_t S = sub_div, S3 = S * S * S;
            const int64_t n_sub = n_cells * S3;
            if (n_sub > (int64_t)1 << 31) throw std::bad_alloc();
            double sub[3];
            for (int a = 0; a < 3; ++a) sub[a] = cell_edge[a] / (double)S;
            auto sub_range = [&](int64_t t, int a, int64_t c, int64_t& lo_i, int64_t& hi_i) {
                if (!(sub[a] > 0.0)) {
                    lo_i = 0;
                    hi_i = S - 1;
                    return;
                }
                const double corner = (double)grid_min[a] + (double)c * cell_edge[a];
                const double e_lo = (double)emin[3 * t + a] - eps[a], e_hi = (double)emax[3 * t + a] + eps[a];
                lo_i = clip64(cell_index((e_lo - corner) / sub[a], S - 1), 0, S - 1);
                hi_i = clip64(cell_index((e_hi - corner) / sub[a], S - 1), 0, S - 1);
            };
            std::vector<int64_t> scount((size_t)n_sub + 1, 0);
            for (int pass = 0; pass < 2; ++pass) {
                std::vector<int64_t> scur;
                if (pass == 1) {
                    G->sub_start.assign((size_t)n_sub + 1, 0);
                    int64_t st = 0;
                    for (int64_t c = 0; c < n_sub; ++c) {
                        G->sub_start[c] = (int32_t)st;
                        st += scount[c];
                        if (st > INT32_MAX) throw std::bad_alloc();
                    }
                    G->sub_start[n_sub] = (int32_t)st;
                    G->sub_elems.assign((size_t)st, 0);
                    scur.assign(G->sub_start.begin(), G->sub_start.end() - 1);
                }
                // entries in element order, as the cell lists were filled
                for (int64_t t = 0; t < n_tets; ++t)
                    for (int64_t i = cmin[3 * t]; i <= cmax[3 * t]; ++i)
                        for (int64_t j = cmin[3 * t + 1]; j <= cmax[3 * t + 1]; ++j)
                            for (int64_t k = cmin[3 * t + 2]; k <= cmax[3 * t + 2]; ++k) {
                                const int64_t cell = (i * gs[1] + j) * gs[2] + k;
                                int64_t x0, x1, y0, y1, z0, z1;
                                sub_range(t, 0, i, x0, x1);
                                sub_range(t, 1, j, y0, y1);
                                sub_range(t, 2, k, z0, z1);
                                for (int64_t sx = x0; sx <= x1; ++sx)
                                    for (int64_t sy = y0; sy <= y1; ++sy)
                                        for (int64_t sz = z0; sz <= z1; ++sz) {
                                            const int64_t sid = cell * S3 + (sx * S + sy) * S + sz;
                                            if (pass == 0) ++scount[sid];
                                            else G->sub_elems[scur[sid]++] = (int32_t)t;
                                        }
                            }
            }
        } else {
            G->sub_start.assign(1, 0);
        }
    } catch (const std::bad_alloc&) {
        delete G;
        return set_error(JT_ERR_NOMEM, "hash grid lists exceed host memory or 2^31 entries");
    }
    info->n_cells = n_cells;
    info->n_entries = (int64_t)G->cell_elems.size();
    info->n_sub_cells = (int64_t)G->sub_start.size() - 1;
    info->n_sub_entries = (int64_t)G->sub_elems.size();
    info->max_per_cell = G->max_per_cell;
    info->pad = 0;
    *handle_out = G;
    return JT_OK;
}

extern "C" int jt_fem_grid_fetch(void* handle, int32_t* cell_start, int32_t* cell_elems, int32_t* sub_start,
                                 int32_t* sub_elems) {
    if (handle == nullptr) return set_error(JT_ERR_INVALID, "handle is NULL");
    const FemGrid* G = static_cast<const FemGrid*>(handle);
    auto copy = [](int32_t* dst, const std::vector<int32_t>& v) {
        if (dst != nullptr && !v.empty()) memcpy(dst, v.data(), v.size() * sizeof(int32_t));
    };
    copy(cell_start, G->cell_start);
    copy(cell_elems, G->cell_elems);
    copy(sub_start, G->sub_start);
    copy(sub_elems, G->sub_elems);
    return JT_OK;
}

extern "C" void jt_fem_grid_free(void* handle) { delete static_cast<FemGrid*>(handle); }
