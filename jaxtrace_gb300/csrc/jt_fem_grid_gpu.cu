// Device build of the FEM hash grid's cell and sub-cell lists, giving the
// same arrays as the host builder (jt_fem_build.cpp), which follows
// build_tetrahedral_mesh (fields/fem_interpolator.py:36-143).
//
// Cell lists: an element is listed in every cell its float32 box overlaps;
// the cell range per axis is floor((float32 box - float32 grid minimum) /
// float64 edge), clipped.  Sub-cell lists: each (element, cell) entry is
// listed in the sub-cells of that cell (sub_div^3 per cell) its box, widened
// by eps per axis, meets; the sub-cell range is floor((box -/+ eps - cell
// corner) / (edge / sub_div)) in float64, clipped.  Every float64 operation
// is a separately rounded intrinsic, as the host code compiled without
// contraction rounds it.
//
// Lists are built by counting (atomics per cell), an exclusive scan of the
// counts, a scatter with atomic cursors, and a rank sort of every list into
// ascending element order -- the order the host's stable counting sort over
// the entries taken in element order gives.  The rank sort costs
// O(list length^2 / 32) per list, so lists longer than kFemMaxList are left
// to the host builder (JT_ERR_UNSUPPORTED).
#include <math.h>
#include <stdint.h>

#include <new>

#include "jt_internal.h"

namespace jt {

constexpr int kFemBlock = 256;
constexpr int kFemMaxList = 4096;

struct FemGridGeom {
    int32_t gs[3];
    float gmin[3];
    double edge[3];
    int32_t S;
    double sub[3];
    double eps[3];
};

__device__ __forceinline__ int cell_index_d(double x, int hi) {
    const double f = floor(x);
    if (!(f >= 0.0)) return 0;
    if (f >= (double)hi) return hi;
    return (int)f;
}

// box (min xyz,0,max xyz,0), geometry (v0, v1-v0, v2-v0, v3-v0, vertex ids)
// and cell range (min ijk, max ijk) of every tetrahedron
__global__ void __launch_bounds__(kFemBlock) k_fem_tets(const float* __restrict__ pts, const int32_t* __restrict__ conn,
                                                        int n_tets, int n_points, FemGridGeom G,
                                                        float* __restrict__ tet_box, float* __restrict__ tet_geom,
                                                        int* __restrict__ crange, int* __restrict__ bad) {
    const int e = blockIdx.x * kFemBlock + threadIdx.x;
    if (e >= n_tets) return;
    int v[4];
    for (int k = 0; k < 4; ++k) {
        v[k] = conn[4 * (int64_t)e + k];
        if (v[k] < 0 || v[k] >= n_points) {
            atomicExch(bad, 1);
            v[k] = 0;
        }
    }
    for (int a = 0; a < 3; ++a) {
        float p[4];
        for (int k = 0; k < 4; ++k) p[k] = pts[3 * (int64_t)v[k] + a];
        float lo = p[0], hi = p[0];
        for (int k = 1; k < 4; ++k) {
            lo = p[k] < lo ? p[k] : lo;
            hi = p[k] > hi ? p[k] : hi;
        }
        tet_box[8 * (int64_t)e + a] = lo;
        tet_box[8 * (int64_t)e + 4 + a] = hi;
        if (tet_geom != nullptr) {
            float* g = tet_geom + 16 * (int64_t)e;
            g[a] = p[0];
            g[3 + a] = __fsub_rn(p[1], p[0]);
            g[6 + a] = __fsub_rn(p[2], p[0]);
            g[9 + a] = __fsub_rn(p[3], p[0]);
        }
        crange[6 * (int64_t)e + a] = cell_index_d(__ddiv_rn((double)__fsub_rn(lo, G.gmin[a]), G.edge[a]), G.gs[a] - 1);
        crange[6 * (int64_t)e + 3 + a] =
            cell_index_d(__ddiv_rn((double)__fsub_rn(hi, G.gmin[a]), G.edge[a]), G.gs[a] - 1);
    }
    tet_box[8 * (int64_t)e + 3] = 0.0f;
    tet_box[8 * (int64_t)e + 7] = 0.0f;
    if (tet_geom != nullptr)
        for (int k = 0; k < 4; ++k) tet_geom[16 * (int64_t)e + 12 + k] = __int_as_float(conn[4 * (int64_t)e + k]);
}

// MODE 0: count per cell; MODE 1: scatter element ids to the cells' ranges
template <int MODE>
__global__ void __launch_bounds__(kFemBlock) k_fem_cells(int n_tets, const int* __restrict__ crange, FemGridGeom G,
                                                         uint32_t* __restrict__ count, const uint32_t* __restrict__ start,
                                                         int* __restrict__ out) {
    const int e = blockIdx.x * kFemBlock + threadIdx.x;
    if (e >= n_tets) return;
    const int* r = crange + 6 * (int64_t)e;
    for (int i = r[0]; i <= r[3]; ++i)
        for (int j = r[1]; j <= r[4]; ++j)
            for (int k = r[2]; k <= r[5]; ++k) {
                const int64_t cell = ((int64_t)i * G.gs[1] + j) * G.gs[2] + k;
                const uint32_t slot = atomicAdd(&count[cell], 1u);
                if (MODE == 1) out[start[cell] + slot] = e;
            }
}

__device__ __forceinline__ void sub_range(const FemGridGeom& G, int a, int c, float emin, float emax, int& lo, int& hi) {
    const int S = G.S;
    if (!(G.sub[a] > 0.0)) {
        lo = 0;
        hi = S - 1;
        return;
    }
    const double corner = __dadd_rn((double)G.gmin[a], __dmul_rn((double)c, G.edge[a]));
    const double e_lo = __dsub_rn((double)emin, G.eps[a]), e_hi = __dadd_rn((double)emax, G.eps[a]);
    lo = cell_index_d(__ddiv_rn(__dsub_rn(e_lo, corner), G.sub[a]), S - 1);
    hi = cell_index_d(__ddiv_rn(__dsub_rn(e_hi, corner), G.sub[a]), S - 1);
}

// MODE 0: count per sub-cell; MODE 1: scatter element ids
template <int MODE>
__global__ void __launch_bounds__(kFemBlock) k_fem_subs(int n_tets, const int* __restrict__ crange,
                                                        const float* __restrict__ tet_box, FemGridGeom G,
                                                        uint32_t* __restrict__ count, const uint32_t* __restrict__ start,
                                                        int* __restrict__ out) {
    const int e = blockIdx.x * kFemBlock + threadIdx.x;
    if (e >= n_tets) return;
    const int* r = crange + 6 * (int64_t)e;
    const float* b = tet_box + 8 * (int64_t)e;
    const int S = G.S;
    const int64_t S3 = (int64_t)S * S * S;
    for (int i = r[0]; i <= r[3]; ++i) {
        int x0, x1;
        sub_range(G, 0, i, b[0], b[4], x0, x1);
        for (int j = r[1]; j <= r[4]; ++j) {
            int y0, y1;
            sub_range(G, 1, j, b[1], b[5], y0, y1);
            for (int k = r[2]; k <= r[5]; ++k) {
                int z0, z1;
                sub_range(G, 2, k, b[2], b[6], z0, z1);
                const int64_t cell = ((int64_t)i * G.gs[1] + j) * G.gs[2] + k;
                for (int sx = x0; sx <= x1; ++sx)
                    for (int sy = y0; sy <= y1; ++sy)
                        for (int sz = z0; sz <= z1; ++sz) {
                            const int64_t sid = cell * S3 + ((int64_t)sx * S + sy) * S + sz;
                            const uint32_t slot = atomicAdd(&count[sid], 1u);
                            if (MODE == 1) out[start[sid] + slot] = e;
                        }
            }
        }
    }
}

// longest list of a CSR start array
__global__ void __launch_bounds__(kFemBlock) k_fem_max_list(int64_t n, const uint32_t* __restrict__ start,
                                                            int* __restrict__ mx) {
    const int64_t i = (int64_t)blockIdx.x * kFemBlock + threadIdx.x;
    int c = i < n ? (int)(start[i + 1] - start[i]) : 0;
    for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
    if ((threadIdx.x & 31) == 0 && c > 0) atomicMax(mx, c);
}

// one warp per list: src[start[w]..start[w+1]) into dst, ascending (distinct ids)
__global__ void __launch_bounds__(kFemBlock) k_fem_rank_sort(int64_t n_lists, const uint32_t* __restrict__ start,
                                                             const int* __restrict__ src, int* __restrict__ dst) {
    const int64_t w = ((int64_t)blockIdx.x * kFemBlock + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_lists) return;
    const uint32_t o = start[w];
    const int c = (int)(start[w + 1] - o);
    for (int i = lane; i < c; i += 32) {
        const int v = src[o + i];
        int rank = 0;
        for (int q = 0; q < c; ++q) rank += src[o + q] < v;
        dst[o + rank] = v;
    }
}

}  // namespace jt

using namespace jt;

namespace {

struct DevFemGrid {
    int32_t* cell_start = nullptr;
    int32_t* cell_elems = nullptr;
    int32_t* sub_start = nullptr;
    int32_t* sub_elems = nullptr;
    int64_t n_cells = 0, n_entries = 0, n_sub = 0, n_sub_entries = 0;
    cudaStream_t s = nullptr;
    ~DevFemGrid() {
        for (void* p : {(void*)cell_start, (void*)cell_elems, (void*)sub_start, (void*)sub_elems})
            if (p != nullptr) dev_free(p, s);
    }
};

// scratch of one build, released on the stream
struct Scratch {
    cudaStream_t s;
    void* ptrs[16] = {};
    int n = 0;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        if (err == cudaSuccess && n >= 16) err = cudaErrorMemoryAllocation;  // more scratch arrays than slots
        if (err == cudaSuccess) err = dev_alloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 16, s);
        if (err != cudaSuccess || p == nullptr) return nullptr;
        ptrs[n++] = p;
        return static_cast<T*>(p);
    }
    ~Scratch() {
        for (int i = 0; i < n; ++i)
            if (ptrs[i] != nullptr) dev_free(ptrs[i], s);
    }
};

template <class T>
T* dev_array(size_t count, cudaStream_t s, cudaError_t& err) {
    void* p = nullptr;
    if (err == cudaSuccess) err = dev_alloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 16, s);
    return static_cast<T*>(p);
}

inline unsigned fem_blocks(int64_t n) { return (unsigned)((n + kFemBlock - 1) / kFemBlock); }

// counts -> CSR start (n_lists + 1 values, the last the total), in place
int csr_start(uint32_t* count, int64_t n_lists, Scratch& sc, uint32_t* total, cudaStream_t s) {
    uint32_t* sums = sc.get<uint32_t>((size_t)scan_partials(n_lists + 1));
    uint32_t* sums2 = sc.get<uint32_t>((size_t)scan_partials2(n_lists + 1));
    if (sc.err != cudaSuccess) return cuda_status(sc.err, "hash grid scan allocation");
    int rc = exclusive_scan_u32(count, n_lists + 1, sums, sums2, s);
    if (rc != JT_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(total, count + n_lists, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_status(e, "hash grid list total");
}

}  // namespace

extern "C" int jt_fem_grid_build_device(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                                        const int32_t* grid_size, const float* grid_min, const double* cell_edge,
                                        int32_t sub_div, const double* eps, float* tet_box, float* tet_geom,
                                        void* stream, void** handle_out, jt_fem_grid_info* info) {
    if (handle_out == nullptr || info == nullptr) return set_error(JT_ERR_INVALID, "handle_out and info are required");
    *handle_out = nullptr;
    if (n_points < 1 || n_tets < 1 || points == nullptr || conn == nullptr || tet_box == nullptr)
        return set_error(JT_ERR_INVALID, "the device build needs points, tetrahedra and a tet_box buffer");
    if (grid_size == nullptr || grid_min == nullptr || cell_edge == nullptr)
        return set_error(JT_ERR_INVALID, "grid_size, grid_min and cell_edge are required");
    if (sub_div < 0 || sub_div > 16) return set_error(JT_ERR_INVALID, "sub_div must be 0..16");
    if (sub_div > 0 && eps == nullptr) return set_error(JT_ERR_INVALID, "eps (3 margins) is required with sub_div");
    FemGridGeom G{};
    int64_t n_cells = 1;
    for (int a = 0; a < 3; ++a) {
        if (grid_size[a] < 1) return set_error(JT_ERR_INVALID, "grid_size must be positive");
        G.gs[a] = grid_size[a];
        G.gmin[a] = grid_min[a];
        G.edge[a] = cell_edge[a];
        G.sub[a] = sub_div > 0 ? cell_edge[a] / (double)sub_div : 0.0;
        G.eps[a] = sub_div > 0 ? eps[a] : 0.0;
        n_cells *= grid_size[a];
    }
    G.S = sub_div;
    const int64_t S3 = (int64_t)sub_div * sub_div * sub_div;
    const int64_t n_sub = sub_div > 0 ? n_cells * S3 : 0;
    if (n_cells + 1 > scan_capacity() || n_sub + 1 > scan_capacity())
        return set_error(JT_ERR_UNSUPPORTED, "hash grid of %lld cells / %lld sub-cells exceeds the device build",
                         (long long)n_cells, (long long)n_sub);
    cudaStream_t s = (cudaStream_t)stream;
    Scratch sc{s};
    int* crange = sc.get<int>(6 * (size_t)n_tets);
    int* bad = sc.get<int>(2);
    uint32_t* ccount = sc.get<uint32_t>((size_t)n_cells + 1);
    if (sc.err != cudaSuccess) return cuda_status(sc.err, "hash grid allocation");
    cudaError_t e = cudaMemsetAsync(bad, 0, 2 * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ccount, 0, sizeof(uint32_t) * ((size_t)n_cells + 1), s);
    if (e != cudaSuccess) return cuda_status(e, "hash grid reset");
    const unsigned gb = fem_blocks(n_tets);
    k_fem_tets<<<gb, kFemBlock, 0, s>>>(points, conn, n_tets, n_points, G, tet_box, tet_geom, crange, bad);
    int host_bad = 0;
    if ((e = cudaMemcpyAsync(&host_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_status(e, "hash grid element pass");
    if (host_bad) return set_error(JT_ERR_INVALID, "connectivity indexes outside the points array");
    k_fem_cells<0><<<gb, kFemBlock, 0, s>>>(n_tets, crange, G, ccount, nullptr, nullptr);
    uint32_t n_entries = 0;
    int rc = csr_start(ccount, n_cells, sc, &n_entries, s);
    if (rc != JT_OK) return rc;
    if ((int64_t)n_entries > INT32_MAX) return set_error(JT_ERR_NOMEM, "hash grid lists exceed 2^31 entries");
    DevFemGrid* H = new (std::nothrow) DevFemGrid();
    if (H == nullptr) return set_error(JT_ERR_NOMEM, "out of host memory");
    H->s = s;
    H->n_cells = n_cells;
    H->n_entries = n_entries;
    // the scanned counts are the cell starts; a second counter array gives the cursors
    H->cell_start = reinterpret_cast<int32_t*>(ccount);
    sc.ptrs[2] = nullptr;  // owned by the handle from here
    H->cell_elems = dev_array<int32_t>(n_entries, s, e);
    int* ctmp = sc.get<int>(n_entries);
    uint32_t* cursor = sc.get<uint32_t>((size_t)n_cells);
    if (e == cudaSuccess) e = sc.err;
    if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * (size_t)n_cells, s);
    if (e != cudaSuccess) {
        delete H;
        return cuda_status(e, "hash grid cell lists");
    }
    k_fem_cells<1><<<gb, kFemBlock, 0, s>>>(n_tets, crange, G, cursor, ccount, ctmp);
    if ((e = cudaMemsetAsync(bad, 0, sizeof(int), s)) != cudaSuccess) {
        delete H;
        return cuda_status(e, "hash grid reset");
    }
    k_fem_max_list<<<fem_blocks(n_cells), kFemBlock, 0, s>>>(n_cells, ccount, bad);
    int max_list = 0;
    if ((e = cudaMemcpyAsync(&max_list, bad, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        delete H;
        return cuda_status(e, "hash grid list lengths");
    }
    if (max_list > kFemMaxList) {
        delete H;
        return set_error(JT_ERR_UNSUPPORTED, "a hash cell lists %d elements (device build handles up to %d)", max_list,
                         kFemMaxList);
    }
    k_fem_rank_sort<<<fem_blocks(n_cells * 32), kFemBlock, 0, s>>>(n_cells, ccount, ctmp, H->cell_elems);
    if (sub_div > 0 && n_entries > 0) {
        uint32_t* scount = dev_array<uint32_t>((size_t)n_sub + 1, s, e);
        H->sub_start = reinterpret_cast<int32_t*>(scount);
        if (e == cudaSuccess) e = cudaMemsetAsync(scount, 0, sizeof(uint32_t) * ((size_t)n_sub + 1), s);
        if (e != cudaSuccess) {
            delete H;
            return cuda_status(e, "hash grid sub-cell counts");
        }
        k_fem_subs<0><<<gb, kFemBlock, 0, s>>>(n_tets, crange, tet_box, G, scount, nullptr, nullptr);
        uint32_t n_sub_entries = 0;
        if ((rc = csr_start(scount, n_sub, sc, &n_sub_entries, s)) != JT_OK) {
            delete H;
            return rc;
        }
        if ((int64_t)n_sub_entries > INT32_MAX) {
            delete H;
            return set_error(JT_ERR_NOMEM, "hash grid sub-cell lists exceed 2^31 entries");
        }
        H->n_sub = n_sub;
        H->n_sub_entries = n_sub_entries;
        H->sub_elems = dev_array<int32_t>(n_sub_entries, s, e);
        int* stmp = sc.get<int>(n_sub_entries);
        uint32_t* scursor = sc.get<uint32_t>((size_t)n_sub);
        if (e == cudaSuccess) e = sc.err;
        if (e == cudaSuccess) e = cudaMemsetAsync(scursor, 0, sizeof(uint32_t) * (size_t)n_sub, s);
        if (e != cudaSuccess) {
            delete H;
            return cuda_status(e, "hash grid sub-cell lists");
        }
        k_fem_subs<1><<<gb, kFemBlock, 0, s>>>(n_tets, crange, tet_box, G, scursor, scount, stmp);
        k_fem_rank_sort<<<fem_blocks(n_sub * 32), kFemBlock, 0, s>>>(n_sub, scount, stmp, H->sub_elems);
    } else {
        H->sub_start = dev_array<int32_t>(1, s, e);
        if (e == cudaSuccess) e = cudaMemsetAsync(H->sub_start, 0, sizeof(int32_t), s);
        if (e != cudaSuccess) {
            delete H;
            return cuda_status(e, "hash grid sub-cell start");
        }
    }
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        delete H;
        return cuda_status(e, "hash grid build kernels");
    }
    info->n_cells = n_cells;
    info->n_entries = n_entries;
    info->n_sub_cells = H->n_sub;
    info->n_sub_entries = H->n_sub_entries;
    info->max_per_cell = max_list;
    info->pad = 0;
    *handle_out = H;
    return JT_OK;
}

extern "C" int jt_fem_grid_fetch_device(void* handle, int32_t* cell_start, int32_t* cell_elems, int32_t* sub_start,
                                        int32_t* sub_elems, void* stream) {
    if (handle == nullptr) return set_error(JT_ERR_INVALID, "handle is NULL");
    const DevFemGrid* H = static_cast<const DevFemGrid*>(handle);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    auto copy = [&](int32_t* dst, const int32_t* src, int64_t n) {
        if (e == cudaSuccess && dst != nullptr && src != nullptr && n > 0)
            e = cudaMemcpyAsync(dst, src, sizeof(int32_t) * (size_t)n, cudaMemcpyDefault, s);
    };
    copy(cell_start, H->cell_start, H->n_cells + 1);
    copy(cell_elems, H->cell_elems, H->n_entries);
    copy(sub_start, H->sub_start, H->n_sub + 1);
    copy(sub_elems, H->sub_elems, H->n_sub_entries);
    return cuda_status(e, "hash grid fetch");
}

extern "C" void jt_fem_grid_free_device(void* handle, void* stream) {
    DevFemGrid* H = static_cast<DevFemGrid*>(handle);
    if (H == nullptr) return;
    H->s = (cudaStream_t)stream;
    delete H;
}
