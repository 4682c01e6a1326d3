// Public C ABI of the tracking path: argument validation, error state and
// dispatch to the per-field kernel launchers.
#include <stdarg.h>
#include <stdio.h>

#include <string>

#include "jt_common.cuh"
#include "jt_internal.h"
#include "jt_kernels.cuh"

namespace jt {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return JT_OK;
    return set_error(JT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Boundary callables applied on their own (boundary.py:215-438, :1517-1599).
__global__ void __launch_bounds__(kBlock) k_boundary(jt_boundary B, float* pos, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* p = pos + 3 * (int64_t)i;
    float x = p[0], y = p[1], z = p[2];
    apply_boundary<true>(B, x, y, z);
    p[0] = x; p[1] = y; p[2] = z;
}

static int check_storage(int s) {
    if (s < JT_STORE_F32 || s > JT_STORE_F16) return set_error(JT_ERR_INVALID, "unknown storage %d", s);
    return JT_OK;
}

static int check_nearest(const jt_nearest_field* q) {
    if (q == nullptr) return set_error(JT_ERR_INVALID, "nearest field descriptor is NULL");
    if (q->n_points < 1 || q->cells[0] < 1 || q->cells[1] < 1 || q->cells[2] < 1)
        return set_error(JT_ERR_INVALID, "nearest field needs points and a positive cell grid");
    if (q->points == nullptr || q->point_ids == nullptr || q->cell_start == nullptr || q->pairs == nullptr ||
        q->n_pairs < 1)
        return set_error(JT_ERR_INVALID, "nearest field has a NULL array");
    if (q->pair_stride < q->n_points) return set_error(JT_ERR_INVALID, "pair_stride smaller than n_points");
    if (((uintptr_t)q->pairs & 31u) != 0)
        return set_error(JT_ERR_INVALID, "pairs must be 32-byte aligned (256-bit records)");
    return check_storage(q->storage);
}

int check_grid_shape(const jt_grid_field& g) {
    if (g.nx < 1 || g.ny < 1 || g.nz < 1)
        return set_error(JT_ERR_INVALID, "grid shape (%d,%d,%d) must be positive", g.nx, g.ny, g.nz);
    const int32_t kAxisMax = 1 << 24;
    if (g.nx > kAxisMax || g.ny > kAxisMax || g.nz > kAxisMax)
        return set_error(JT_ERR_INVALID, "grid axes hold at most 2^24 nodes, got (%d,%d,%d)", g.nx, g.ny, g.nz);
    if ((int64_t)g.nx * g.ny * g.nz > (int64_t)INT32_MAX)
        return set_error(JT_ERR_INVALID, "grid holds %lld nodes, more than 2^31 - 1",
                         (long long)((int64_t)g.nx * g.ny * g.nz));
    return JT_OK;
}

int check_tiles(const jt_grid_field& g) {
    const int32_t n[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; ++a)
        if (g.tiles[a] != (n[a] + JT_TILE - 1) / JT_TILE)
            return set_error(JT_ERR_INVALID, "tiles[%d] = %d, expected (n + %d) / %d = %d", a, g.tiles[a], JT_TILE - 1,
                             JT_TILE, (n[a] + JT_TILE - 1) / JT_TILE);
    if (g.tile_base == nullptr) return set_error(JT_ERR_INVALID, "affine-tile field without tile_base");
    return JT_OK;
}

static int check_field(const jt_field* f) {
    if (f == nullptr) return set_error(JT_ERR_INVALID, "field is NULL");
    switch (f->kind) {
        case JT_FIELD_GRID: {
            const jt_grid_field* g = f->grid;
            if (g == nullptr) return set_error(JT_ERR_INVALID, "grid field descriptor is NULL");
            if (int rc = check_grid_shape(*g)) return rc;
            if (g->bounds_mode < JT_GRID_CLAMP || g->bounds_mode > JT_GRID_PERIODIC)
                return set_error(JT_ERR_INVALID, "unknown bounds_mode %d", g->bounds_mode);
            if (g->n_pairs < 1 || g->pairs == nullptr) return set_error(JT_ERR_INVALID, "grid field has no snapshot pairs");
            if (g->storage == JT_STORE_TILE_BF16 || g->storage == JT_STORE_TILE_F16)
                return set_error(JT_ERR_UNSUPPORTED, "affine-tile snapshots are read by jt_stage_tile_fields only");
            if (g->pair_stride < (int64_t)g->nx * g->ny * g->nz)
                return set_error(JT_ERR_INVALID, "pair_stride smaller than the node count");
            // the gathers read 256-bit records (32-byte aligned); a float32-quad
            // slot of pair_stride records keeps that alignment only for an even stride
            if (((uintptr_t)g->pairs & 31u) != 0)
                return set_error(JT_ERR_INVALID, "pairs must be 32-byte aligned (256-bit records)");
            if (g->storage == JT_STORE_STAGE_F32Q && (g->pair_stride & 1) != 0)
                return set_error(JT_ERR_INVALID, "JT_STORE_STAGE_F32Q needs an even pair_stride (slots of 32-byte records)");
            if (g->storage == JT_STORE_STAGE_F32 || g->storage == JT_STORE_STAGE_F16 ||
                g->storage == JT_STORE_STAGE_F32Q)
                return JT_OK;
            return check_storage(g->storage);
        }
        case JT_FIELD_MESH: {
            const jt_mesh_field* m = f->mesh;
            if (m == nullptr) return set_error(JT_ERR_INVALID, "mesh field descriptor is NULL");
            if (m->n_points < 1 || m->n_tets < 1 || m->n_nodes < 1)
                return set_error(JT_ERR_INVALID, "mesh needs points, tetrahedra and octree nodes");
            if (m->points == nullptr || m->tet_box == nullptr || m->tet_geom == nullptr || m->nodes == nullptr ||
                m->elems == nullptr || m->pairs == nullptr || m->n_pairs < 1)
                return set_error(JT_ERR_INVALID, "mesh field has a NULL array");
            if (m->max_depth < 0) return set_error(JT_ERR_INVALID, "max_depth must be >= 0");
            if (m->pair_stride < m->n_points) return set_error(JT_ERR_INVALID, "pair_stride smaller than n_points");
            if (((uintptr_t)m->pairs & 31u) != 0)
                return set_error(JT_ERR_INVALID, "pairs must be 32-byte aligned (256-bit records)");
            return check_storage(m->storage);
        }
        case JT_FIELD_NEAREST: return check_nearest(f->nearest);
        case JT_FIELD_FEM: {
            const jt_fem_field* h = f->fem;
            if (h == nullptr) return set_error(JT_ERR_INVALID, "FEM field descriptor is NULL");
            if (h->n_tets < 1 || h->grid_size[0] < 1 || h->grid_size[1] < 1 || h->grid_size[2] < 1)
                return set_error(JT_ERR_INVALID, "FEM field needs tetrahedra and a positive hash grid");
            if (h->tet_box == nullptr || h->tet_geom == nullptr || h->cell_start == nullptr ||
                h->cell_elems == nullptr)
                return set_error(JT_ERR_INVALID, "FEM field has a NULL array");
            if (h->sub_div < 0 || h->sub_div > 16 || (h->sub_div > 0 && (h->sub_start == nullptr ||
                                                                         h->sub_elems == nullptr)))
                return set_error(JT_ERR_INVALID, "FEM sub-cell lists: sub_div must be 0..16 with both arrays set");
            return check_nearest(&h->nearest);
        }
        default:
            return set_error(JT_ERR_INVALID, "unknown field kind %d", f->kind);
    }
}

static int check_boundary(const jt_boundary* b) {
    if (b == nullptr) return set_error(JT_ERR_INVALID, "boundary is NULL");
    for (int a = 0; a < 3; ++a)
        if (b->axis_kind[a] < JT_BC_NONE || b->axis_kind[a] > JT_BC_ABSORBING)
            return set_error(JT_ERR_INVALID, "unknown boundary kind %d on axis %d", b->axis_kind[a], a);
    if (b->inlet_mode != JT_INLET_OFF) {
        if (b->inlet_mode != JT_INLET_GRID)
            return set_error(JT_ERR_UNSUPPORTED, "inlet mode %d is not implemented", b->inlet_mode);
        if (b->inlet_axis < 0 || b->inlet_axis > 2) return set_error(JT_ERR_INVALID, "inlet_axis must be 0..2");
        if (b->inlet_res[0] < 1 || b->inlet_res[1] < 1 || b->inlet_coords[0] == nullptr ||
            b->inlet_coords[1] == nullptr)
            return set_error(JT_ERR_INVALID, "grid inlet needs two non-empty lattices");
    }
    return JT_OK;
}

static int check_arith(int a) {
    if (a != JT_ARITH_EXACT && a != JT_ARITH_COMPENSATED) return set_error(JT_ERR_INVALID, "unknown arith %d", a);
    return JT_OK;
}

static int check_integ(int i) {
    if (i < JT_EULER || i > JT_RK4) return set_error(JT_ERR_INVALID, "unknown integrator %d", i);
    return JT_OK;
}

}  // namespace jt

using namespace jt;

namespace jt {

static jt_alloc_fn g_alloc = nullptr;
static jt_free_fn g_free = nullptr;
static void* g_alloc_ctx = nullptr;

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    if (g_alloc == nullptr) return cudaMallocAsync(p, bytes, s);
    *p = g_alloc(bytes, (void*)s, g_alloc_ctx);
    return *p != nullptr ? cudaSuccess : cudaErrorMemoryAllocation;
}

void dev_free(void* p, cudaStream_t s) {
    if (p == nullptr) return;
    if (g_free == nullptr) cudaFreeAsync(p, s);
    else g_free(p, (void*)s, g_alloc_ctx);
}

}  // namespace jt

extern "C" int jt_set_allocator(jt_alloc_fn alloc, jt_free_fn free_fn, void* ctx) {
    if ((alloc == nullptr) != (free_fn == nullptr))
        return set_error(JT_ERR_INVALID, "give both alloc and free, or neither (the default)");
    g_alloc = alloc;
    g_free = free_fn;
    g_alloc_ctx = ctx;
    return JT_OK;
}

extern "C" int jt_abi_version(void) { return JT_ABI_VERSION; }

extern "C" const char* jt_last_error(void) { return g_last_error.c_str(); }

extern "C" int jt_struct_sizes(int64_t* out, int32_t n) {
    const int64_t s[] = {(int64_t)sizeof(jt_blend),         (int64_t)sizeof(jt_grid_field),
                         (int64_t)sizeof(jt_octree_node),   (int64_t)sizeof(jt_mesh_field),
                         (int64_t)sizeof(jt_nearest_field), (int64_t)sizeof(jt_field),
                         (int64_t)sizeof(jt_boundary),      (int64_t)sizeof(jt_track_params),
                         (int64_t)sizeof(jt_sort_grid),     (int64_t)sizeof(jt_sph_params),
                         (int64_t)sizeof(jt_kde_params),    (int64_t)sizeof(jt_adjoint_params),
                         (int64_t)sizeof(jt_octree_info),   (int64_t)sizeof(jt_fem_field)};
    const int k = (int)(sizeof(s) / sizeof(s[0]));
    if (out == nullptr || n < k) return set_error(JT_ERR_INVALID, "jt_struct_sizes needs room for %d values", k);
    for (int i = 0; i < k; ++i) out[i] = s[i];
    return k;
}

extern "C" int jt_track(const jt_field* field, const jt_boundary* bc, const jt_track_params* p, void* stream) {
    int rc;
    if ((rc = check_field(field)) || (rc = check_boundary(bc))) return rc;
    if (p == nullptr) return set_error(JT_ERR_INVALID, "params is NULL");
    if ((rc = check_integ(p->integrator)) || (rc = check_arith(p->arith))) return rc;
    if (p->n_particles < 0) return set_error(JT_ERR_INVALID, "n_particles must be >= 0");
    if (p->step_begin < 0 || p->step_end < p->step_begin)
        return set_error(JT_ERR_INVALID, "bad step range [%d,%d)", p->step_begin, p->step_end);
    if (p->n_particles == 0 || p->step_end == p->step_begin) return JT_OK;
    if (p->schedule == nullptr || p->pos == nullptr) return set_error(JT_ERR_INVALID, "schedule and pos are required");
    if (p->traj != nullptr && (p->record_every < 1 || p->n_rows < 0))
        return set_error(JT_ERR_INVALID, "recording needs record_every >= 1 and n_rows >= 0");
    if (p->vel != nullptr && p->traj == nullptr)
        return set_error(JT_ERR_INVALID, "velocity recording needs a trajectory buffer");
    if (p->vel != nullptr && field->kind == JT_FIELD_GRID &&
        (field->grid->storage == JT_STORE_STAGE_F32 || field->grid->storage == JT_STORE_STAGE_F32Q ||
         field->grid->storage == JT_STORE_STAGE_F16))
        return set_error(JT_ERR_UNSUPPORTED, "stage fields do not record velocities: track on snapshot pairs");
    if (p->block_size != 0 && p->block_size != 64 && p->block_size != 128 && p->block_size != 256)
        return set_error(JT_ERR_INVALID, "block_size must be 0, 64, 128 or 256, got %d", p->block_size);
    if (p->ens_offsets != nullptr && (p->n_ens < 1 || p->schedule_stride < 4LL * p->step_end))
        return set_error(JT_ERR_INVALID, "ensembles need n_ens >= 1 and schedule_stride >= 4*step_end");
    cudaStream_t s = (cudaStream_t)stream;
    switch (field->kind) {
        case JT_FIELD_GRID: return grid_track(*field->grid, *bc, *p, s);
        case JT_FIELD_MESH: return mesh_track(*field->mesh, *bc, *p, s);
        case JT_FIELD_FEM: return fem_track(*field->fem, *bc, *p, s);
        default: return nearest_track(*field->nearest, *bc, *p, s);
    }
}

extern "C" int jt_field_sample(const jt_field* field, const jt_blend* blend, int32_t arith, const float* pos,
                               float* out, int32_t m, int32_t* status, void* stream) {
    int rc;
    if ((rc = check_field(field)) || (rc = check_arith(arith))) return rc;
    if (blend == nullptr) return set_error(JT_ERR_INVALID, "blend is NULL");
    if (m < 0) return set_error(JT_ERR_INVALID, "m must be >= 0");
    if (m == 0) return JT_OK;
    if (pos == nullptr || out == nullptr) return set_error(JT_ERR_INVALID, "pos and out are required");
    cudaStream_t s = (cudaStream_t)stream;
    switch (field->kind) {
        case JT_FIELD_GRID: return grid_sample(*field->grid, arith, *blend, pos, out, m, status, s);
        case JT_FIELD_MESH: return mesh_sample(*field->mesh, arith, *blend, pos, out, m, status, s);
        case JT_FIELD_FEM: return fem_sample(*field->fem, arith, *blend, pos, out, m, status, s);
        default: return nearest_sample(*field->nearest, arith, *blend, pos, out, m, status, s);
    }
}

extern "C" int jt_boundary_apply(const jt_boundary* bc, float* pos, int32_t n, void* stream) {
    int rc;
    if ((rc = check_boundary(bc))) return rc;
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n == 0) return JT_OK;
    if (pos == nullptr) return set_error(JT_ERR_INVALID, "pos is NULL");
    k_boundary<<<grid_blocks(n), kBlock, 0, (cudaStream_t)stream>>>(*bc, pos, n);
    return cuda_status(cudaGetLastError(), "boundary kernel launch");
}

extern "C" int jt_integrator_step(const jt_field* field, const jt_blend* stage_blends, int32_t integrator,
                                  int32_t arith, float dt, const float* dt_per_particle, const float* x_in,
                                  float* x_out, int32_t n, int32_t* status, void* stream) {
    int rc;
    if ((rc = check_field(field)) || (rc = check_integ(integrator)) || (rc = check_arith(arith))) return rc;
    if (stage_blends == nullptr) return set_error(JT_ERR_INVALID, "stage_blends is NULL");
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n == 0) return JT_OK;
    if (x_in == nullptr || x_out == nullptr) return set_error(JT_ERR_INVALID, "x_in and x_out are required");
    StageBlends sb;
    for (int i = 0; i < 3; ++i) sb.e[i] = stage_blends[i];
    // rk4.py:89-92 / rk2.py:292: float32 dt/2 and dt/6
    volatile float dtv = dt;
    StepConst k{dt, 0.5f * dtv, dtv / 6.0f};
    cudaStream_t s = (cudaStream_t)stream;
    switch (field->kind) {
        case JT_FIELD_GRID: return grid_step(*field->grid, arith, sb, integrator, k, dt_per_particle, x_in, x_out, n, status, s);
        case JT_FIELD_MESH: return mesh_step(*field->mesh, arith, sb, integrator, k, dt_per_particle, x_in, x_out, n, status, s);
        case JT_FIELD_FEM: return fem_step(*field->fem, arith, sb, integrator, k, dt_per_particle, x_in, x_out, n, status, s);
        default: return nearest_step(*field->nearest, arith, sb, integrator, k, dt_per_particle, x_in, x_out, n, status, s);
    }
}
