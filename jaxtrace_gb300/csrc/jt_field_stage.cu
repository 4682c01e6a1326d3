// Pre-blended stage fields of a regular grid and the tracking kernel that
// gathers them (StageGridField in jt_grid.cuh).  TimeSeriesField blends
// every node at the query time and StructuredGridSampler then interpolates
// (time_series.py:326-367, structured.py:284-349); k_stage_* do the blend
// once per schedule entry of a time chunk, with the arithmetic the gathered
// corners would get (blend_cv), so the float32 path stays bit-identical.
#include <cuda_fp16.h>

#include "jt_grid.cuh"
#include "jt_internal.h"
#include "jt_kernels.cuh"

namespace jt {

// float32 pairs -> float4 {x, y, z, 0} per node, one thread per node walking
// the chunk's entries (a pair record is reloaded only when the pair changes).
template <bool EXACT>
__global__ void __launch_bounds__(kBlock) k_stage_f32(jt_grid_field F, const jt_blend* __restrict__ ent, int n,
                                                       float4* __restrict__ out) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t N = F.pair_stride;
    if (node >= N) return;
    int cur = -1;
    PairVal pv{};
    for (int j = 0; j < n; ++j) {
        const jt_blend e = ent[j];
        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        if (pr != cur) {
            pv = load_pair<JT_STORE_F32>(F.pairs, (int64_t)pr * N + node);
            cur = pr;
        }
        const CV v = blend_cv<EXACT, JT_STORE_F32>(pv, e, splat(e.wa), splat(e.wb), e.form == JT_BLEND_WEIGHTED);
        out[(int64_t)j * N + node] = make_float4(v.xy.x, v.xy.y, v.z, 0.0f);
    }
}

__device__ __forceinline__ CV scale_cv(CV c, float s) {
    return CV{make_float2(c.xy.x * s, c.xy.y * s), c.z * s};
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// 16-bit yz-quad pairs -> float16 yz-quads of the blended values divided by
// the entry's power-of-two scale.  Blocks of 64 threads at <= 64 registers
// (4,096 per block): one fits beside five blocks of the float16 tracking
// kernel (5 x 256 threads x 48 registers), so the next chunk's fields are
// blended on a side stream while the current chunk is tracked.
constexpr int kStageBlock16 = 64;

template <int STORE>
__global__ void __launch_bounds__(kStageBlock16, 16) k_stage_f16(jt_grid_field F, const jt_blend* __restrict__ ent,
                                                       const float* __restrict__ scales, int n,
                                                       uint4* __restrict__ out) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t N = F.pair_stride;
    if (node >= N) return;
    const int64_t part_b = (int64_t)F.n_pairs * N;
    int cur = -1;
    PairVal p00{}, p01{}, p10{}, p11{};
    for (int j = 0; j < n; ++j) {
        const jt_blend e = ent[j];
        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        if (pr != cur) {
            load_quad<STORE>(F.pairs, part_b, (int64_t)pr * N + node, p00, p01, p10, p11);
            cur = pr;
        }
        // the scale is a power of two, so dividing by it is exact and can be
        // folded into the weights of the common (weighted) form
        const float inv = __frcp_rn(__ldg(scales + j));
        CV c00, c01, c10, c11;
        if (e.form == JT_BLEND_WEIGHTED) {
            const float2 WA = splat(e.wa * inv), WB = splat(e.wb * inv);
            c00 = blend_cv<false, STORE>(p00, e, WA, WB, true);
            c01 = blend_cv<false, STORE>(p01, e, WA, WB, true);
            c10 = blend_cv<false, STORE>(p10, e, WA, WB, true);
            c11 = blend_cv<false, STORE>(p11, e, WA, WB, true);
        } else {
            const float2 WA = splat(e.wa), WB = splat(e.wb);
            c00 = scale_cv(blend_cv<false, STORE>(p00, e, WA, WB, false), inv);
            c01 = scale_cv(blend_cv<false, STORE>(p01, e, WA, WB, false), inv);
            c10 = scale_cv(blend_cv<false, STORE>(p10, e, WA, WB, false), inv);
            c11 = scale_cv(blend_cv<false, STORE>(p11, e, WA, WB, false), inv);
        }
        uint4 a, b;
        a.x = pack_h2(c00.xy.x, c00.xy.y);
        a.y = pack_h2(c01.xy.x, c01.xy.y);
        a.z = pack_h2(c10.xy.x, c10.xy.y);
        a.w = pack_h2(c11.xy.x, c11.xy.y);
        b.x = pack_h2(c00.z, c01.z);
        b.y = pack_h2(c10.z, c11.z);
        b.z = 0u;
        b.w = 0u;
        uint4* o = out + 2 * ((int64_t)j * N + node);
        o[0] = a;
        o[1] = b;
    }
}

// ---------------------------------------------------------------------------
// Affine-tile stage fields.  One thread per residual quad of a tile (80 per
// tile: local x plane 0..4, y and z cell 0..3) walks the chunk's entries; a
// quad's four nodes of snapshots A and B are reloaded only when the pair
// changes.  The blend is linear, so the stage residual is the blend of the
// snapshot residuals and the stage base the blend of the snapshot bases; the
// first thread of each tile blends its base record.  Blocks of 64 threads so
// that the side-stream launch fits beside the tracking blocks.
// ---------------------------------------------------------------------------

// Residual node {x, y, z, 0} of 16-bit storage STORE, decoded to float32.
template <int STORE>
__device__ __forceinline__ void tile_node(const uint2* __restrict__ r, float2& xy, float& z) {
    const uint2 w = __ldg(r);
    if (STORE == JT_STORE_TILE_BF16) {
        xy = make_float2(bf16_lo(w.x), bf16_hi(w.x));
        z = bf16_lo(w.y);
    } else {
        xy = __half22float2(*reinterpret_cast<const __half2*>(&w.x));
        z = __low2float(*reinterpret_cast<const __half2*>(&w.y));
    }
}

template <int STORE>
__global__ void __launch_bounds__(kStageBlock16, 16) k_stage_tile(jt_grid_field F, const jt_blend* __restrict__ ent,
                                                                int n, uint4* __restrict__ out_q,
                                                                float* __restrict__ out_b) {
    const int64_t tiles = (int64_t)F.tiles[0] * F.tiles[1] * F.tiles[2];
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t Q = tiles * JT_TILE_QUADS;
    if (q >= Q) return;
    const int64_t tile = q / JT_TILE_QUADS;
    const int lq = (int)(q - tile * JT_TILE_QUADS);
    const int lx = lq >> 4, ly = (lq >> 2) & 3, lz = lq & 3;
    // local nodes (lx,ly,lz), (lx,ly,lz+1), (lx,ly+1,lz), (lx,ly+1,lz+1)
    const int l0 = (lx * (JT_TILE + 1) + ly) * (JT_TILE + 1) + lz;
    const int lofs[4] = {l0, l0 + 1, l0 + (JT_TILE + 1), l0 + (JT_TILE + 1) + 1};
    const bool head = lq == 0;
    const uint2* res = reinterpret_cast<const uint2*>(F.pairs);
    int cur = -1;
    PairVal pv[4];
    PairVal pb[4];  // the tile base's four triples (o, Gx, Gy, Gz) of A and B
    for (int j = 0; j < n; ++j) {
        const jt_blend e = ent[j];
        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        if (pr != cur) {
            const uint2* ra = res + ((int64_t)pr * tiles + tile) * JT_TILE_NODES;
            const uint2* rb = ra + tiles * JT_TILE_NODES;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                tile_node<STORE>(ra + lofs[c], pv[c].axy, pv[c].az);
                tile_node<STORE>(rb + lofs[c], pv[c].bxy, pv[c].bz);
            }
            if (head) {
                const float* ba = F.tile_base + ((int64_t)pr * tiles + tile) * 16;
                const float* bb = ba + tiles * 16;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    pb[c].axy = make_float2(__ldg(ba + 2 * c), __ldg(ba + 2 * c + 1));
                    pb[c].az = __ldg(ba + 8 + c);
                    pb[c].bxy = make_float2(__ldg(bb + 2 * c), __ldg(bb + 2 * c + 1));
                    pb[c].bz = __ldg(bb + 8 + c);
                }
            }
            cur = pr;
        }
        V3 v[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) v[c] = blend<false, JT_STORE_F32>(pv[c], e);
        uint4 a, b;
        a.x = pack_h2(v[0].x, v[0].y);
        a.y = pack_h2(v[1].x, v[1].y);
        a.z = pack_h2(v[2].x, v[2].y);
        a.w = pack_h2(v[3].x, v[3].y);
        b.x = pack_h2(v[0].z, v[1].z);
        b.y = pack_h2(v[2].z, v[3].z);
        b.z = 0u;
        b.w = 0u;
        uint4* o = out_q + 2 * ((int64_t)j * Q + q);
        o[0] = a;
        o[1] = b;
        if (head) {
            float4* ob = reinterpret_cast<float4*>(out_b + ((int64_t)j * tiles + tile) * 16);
            V3 t[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) t[c] = blend<false, JT_STORE_F32>(pb[c], e);
            ob[0] = make_float4(t[0].x, t[0].y, t[1].x, t[1].y);
            ob[1] = make_float4(t[2].x, t[2].y, t[3].x, t[3].y);
            ob[2] = make_float4(t[0].z, t[1].z, t[2].z, t[3].z);
            ob[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

// The bounds mode as a template argument: clamp and periodic get their own
// kernels, zero and nan share the run-time one.
template <bool E, int O>
using StageClamp = StageGridField<E, O, JT_GRID_CLAMP>;
template <bool E, int O>
using StagePeriodic = StageGridField<E, O, JT_GRID_PERIODIC>;
template <bool E, int O>
using StageAnyMode = StageGridField<E, O, -1>;

template <int MODE>
static cudaError_t tile_launch(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p,
                               cudaStream_t s) {
    const StageTileField<MODE, true> fld = StageTileField<MODE, true>::create(f, 0);
    const int bs = p.block_size > 0 ? p.block_size : kBlock;
    const unsigned g = (unsigned)((p.n_particles + bs - 1) / bs);
    const InletFrame I = inlet_frame(b);
    typedef Launcher<GridField, jt_grid_field, int> L;
    if (p.path != nullptr) return L::template launch_track<false, true>(fld, b, I, p, g, bs, s);
    return L::template launch_track<false, false>(fld, b, I, p, g, bs, s);
}

template <template <bool, int> class FT>
static cudaError_t stage_launch(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p,
                                cudaStream_t s, bool exact) {
    typedef Launcher<FT, jt_grid_field, int> L;
    if (f.storage == JT_STORE_STAGE_F32)
        return exact ? L::template track_s<true, JT_STORE_STAGE_F32>(f, 0, b, p, s)
                     : L::template track_s<false, JT_STORE_STAGE_F32>(f, 0, b, p, s);
    return L::template track_s<false, JT_STORE_STAGE_F16>(f, 0, b, p, s);
}

int stage_track(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    const bool exact = p.arith == JT_ARITH_EXACT;
    if (f.storage == JT_STORE_STAGE_TILE) {
        if (exact) return set_error(JT_ERR_UNSUPPORTED, "exact arithmetic needs float32 stage fields");
        cudaError_t err;
        switch (f.bounds_mode) {
            case JT_GRID_CLAMP: err = tile_launch<JT_GRID_CLAMP>(f, b, p, s); break;
            case JT_GRID_PERIODIC: err = tile_launch<JT_GRID_PERIODIC>(f, b, p, s); break;
            default: err = tile_launch<-1>(f, b, p, s); break;
        }
        return cuda_status(err, "tracking kernel launch");
    }
    if (f.storage != JT_STORE_STAGE_F32 && exact)
        return set_error(JT_ERR_UNSUPPORTED, "exact arithmetic needs float32 stage fields");
    cudaError_t err;
    switch (f.bounds_mode) {
        case JT_GRID_CLAMP: err = stage_launch<StageClamp>(f, b, p, s, exact); break;
        case JT_GRID_PERIODIC: err = stage_launch<StagePeriodic>(f, b, p, s, exact); break;
        default: err = stage_launch<StageAnyMode>(f, b, p, s, exact); break;
    }
    return cuda_status(err, "tracking kernel launch");
}

}  // namespace jt

using namespace jt;

extern "C" int jt_stage_fields(const jt_field* field, const jt_blend* entries, const float* out_scales, int32_t n,
                               int32_t out_storage, void* out, void* stream) {
    if (field == nullptr || field->kind != JT_FIELD_GRID || field->grid == nullptr)
        return set_error(JT_ERR_INVALID, "stage fields need a regular-grid field");
    const jt_grid_field& F = *field->grid;
    if (int rc = check_grid_shape(F)) return rc;
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n == 0) return JT_OK;
    if (entries == nullptr || out == nullptr) return set_error(JT_ERR_INVALID, "entries and out are required");
    if (F.pairs == nullptr || F.n_pairs < 1) return set_error(JT_ERR_INVALID, "field has no snapshot pairs");
    const int64_t N = (int64_t)F.nx * F.ny * F.nz;
    if (F.pair_stride != N) return set_error(JT_ERR_INVALID, "pair_stride must equal the node count");
    const unsigned g = grid_blocks(N);
    const unsigned g16 = (unsigned)((N + kStageBlock16 - 1) / kStageBlock16);
    cudaStream_t s = (cudaStream_t)stream;
    if (out_storage == JT_STORE_STAGE_F32) {
        if (F.storage != JT_STORE_F32)
            return set_error(JT_ERR_UNSUPPORTED, "float32 stage fields come from float32 snapshots");
        k_stage_f32<true><<<g, kBlock, 0, s>>>(F, entries, n, reinterpret_cast<float4*>(out));
    } else if (out_storage == JT_STORE_STAGE_F16) {
        if (out_scales == nullptr) return set_error(JT_ERR_INVALID, "float16 stage fields need out_scales");
        if (F.storage == JT_STORE_BF16)
            k_stage_f16<JT_STORE_BF16><<<g16, kStageBlock16, 0, s>>>(F, entries, out_scales, n,
                                                                     reinterpret_cast<uint4*>(out));
        else if (F.storage == JT_STORE_F16)
            k_stage_f16<JT_STORE_F16><<<g16, kStageBlock16, 0, s>>>(F, entries, out_scales, n,
                                                                    reinterpret_cast<uint4*>(out));
        else
            return set_error(JT_ERR_UNSUPPORTED, "float16 stage fields come from 16-bit snapshots");
    } else {
        return set_error(JT_ERR_INVALID, "out_storage must be JT_STORE_STAGE_F32 or JT_STORE_STAGE_F16");
    }
    return cuda_status(cudaGetLastError(), "stage field launch");
}

extern "C" int jt_stage_tile_fields(const jt_field* field, const jt_blend* entries, int32_t n, void* out_quads,
                                    float* out_base, void* stream) {
    if (field == nullptr || field->kind != JT_FIELD_GRID || field->grid == nullptr)
        return set_error(JT_ERR_INVALID, "stage fields need a regular-grid field");
    const jt_grid_field& F = *field->grid;
    if (int rc = check_grid_shape(F)) return rc;
    if (F.storage != JT_STORE_TILE_BF16 && F.storage != JT_STORE_TILE_F16)
        return set_error(JT_ERR_INVALID, "affine-tile stage fields come from JT_STORE_TILE_* snapshots");
    if (int rc = check_tiles(F)) return rc;
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n == 0) return JT_OK;
    if (entries == nullptr || out_quads == nullptr || out_base == nullptr)
        return set_error(JT_ERR_INVALID, "entries, out_quads and out_base are required");
    if (F.pairs == nullptr || F.n_pairs < 1) return set_error(JT_ERR_INVALID, "field has no snapshots");
    const int64_t tiles = (int64_t)F.tiles[0] * F.tiles[1] * F.tiles[2];
    if (F.pair_stride != tiles * JT_TILE_NODES)
        return set_error(JT_ERR_INVALID, "pair_stride must be tiles * JT_TILE_NODES");
    const int64_t Q = tiles * JT_TILE_QUADS;
    const unsigned g = (unsigned)((Q + kStageBlock16 - 1) / kStageBlock16);
    cudaStream_t s = (cudaStream_t)stream;
    if (F.storage == JT_STORE_TILE_BF16)
        k_stage_tile<JT_STORE_TILE_BF16><<<g, kStageBlock16, 0, s>>>(F, entries, n, reinterpret_cast<uint4*>(out_quads),
                                                                      out_base);
    else
        k_stage_tile<JT_STORE_TILE_F16><<<g, kStageBlock16, 0, s>>>(F, entries, n, reinterpret_cast<uint4*>(out_quads),
                                                                     out_base);
    return cuda_status(cudaGetLastError(), "stage field launch");
}
