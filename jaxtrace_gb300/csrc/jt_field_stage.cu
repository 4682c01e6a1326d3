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

// float32 pairs -> float32 yz-quads (JT_STORE_STAGE_F32Q), one thread per
// node: its quad's four nodes (j,k), (j,k1), (j1,k), (j1,k1) blended with
// the exact arithmetic of k_stage_f32, so the values are the same bits.
template <bool EXACT>
// A float32-quad slot holds S = stage_f32q_stride(N) part-A records (32 B)
// then S part-B records (16 B): S is even, so every slot starts on a 32-byte
// boundary for the tracking kernel's 256-bit loads.
__global__ void __launch_bounds__(kBlock) k_stage_f32q(jt_grid_field F, const jt_blend* __restrict__ ent, int n,
                                                        char* __restrict__ out) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t N = F.pair_stride;
    const int64_t S = N + (N & 1);
    if (node >= N) return;
    const int k = (int)(node % F.nz);
    const int j = (int)((node / F.nz) % F.ny);
    const bool per = F.bounds_mode == JT_GRID_PERIODIC;
    // successors as the sampler computes them (structured.py:311-318)
    const int k1 = per ? (k + 1 == F.nz ? 0 : k + 1) : min(k + 1, F.nz - 1);
    const int j1 = per ? (j + 1 == F.ny ? 0 : j + 1) : min(j + 1, F.ny - 1);
    const int64_t row = node - k - (int64_t)j * F.nz;       // node (i, 0, 0)
    const int64_t ids[4] = {node, row + (int64_t)j * F.nz + k1, row + (int64_t)j1 * F.nz + k,
                            row + (int64_t)j1 * F.nz + k1};
    int cur = -1;
    PairVal pv[4];
    for (int jj = 0; jj < n; ++jj) {
        const jt_blend e = ent[jj];
        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        if (pr != cur) {
#pragma unroll
            for (int c = 0; c < 4; ++c) pv[c] = load_pair<JT_STORE_F32>(F.pairs, (int64_t)pr * N + ids[c]);
            cur = pr;
        }
        CV v[4];
#pragma unroll
        for (int c = 0; c < 4; ++c)
            v[c] = blend_cv<EXACT, JT_STORE_F32>(pv[c], e, splat(e.wa), splat(e.wb), e.form == JT_BLEND_WEIGHTED);
        char* slot = out + (int64_t)jj * S * 48;
        float4* a = reinterpret_cast<float4*>(slot + node * 32);
        a[0] = make_float4(v[0].xy.x, v[0].xy.y, v[1].xy.x, v[1].xy.y);
        a[1] = make_float4(v[2].xy.x, v[2].xy.y, v[3].xy.x, v[3].xy.y);
        reinterpret_cast<float4*>(slot + S * 32)[node] = make_float4(v[0].z, v[1].z, v[2].z, v[3].z);
    }
}

__device__ __forceinline__ CV scale_cv(CV c, float s) {
    return CV{make_float2(c.xy.x * s, c.xy.y * s), c.z * s};
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Offset yz-quad (quad_yz in jt_grid.cuh) of the four nodes' values u,
// already divided by the entry's power-of-two scale: ox the float32 mean of
// the x values; oy the mean of the y values rounded to bfloat16 in the high
// half of word 7, whose low half holds oz, the mean of the z values rounded
// to float16; each residual is the value minus the offset as the tracking
// kernel reads it back (word 7 whole as a float32 for oy), rounded to
// float16.
__device__ __forceinline__ void encode_quad(const V3 (&u)[4], uint4& a, uint4& b) {
    const float ox = 0.25f * ((u[0].x + u[1].x) + (u[2].x + u[3].x));
    const float my = 0.25f * ((u[0].y + u[1].y) + (u[2].y + u[3].y));
    const float mz = 0.25f * ((u[0].z + u[1].z) + (u[2].z + u[3].z));
    const __half hz = __float2half_rn(mz);
    const uint32_t w7 = ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(my)) << 16) | __half_as_ushort(hz);
    const float oy = __uint_as_float(w7), oz = __half2float(hz);
    a.x = pack_h2(u[0].x - ox, u[0].y - oy);
    a.y = pack_h2(u[1].x - ox, u[1].y - oy);
    a.z = pack_h2(u[2].x - ox, u[2].y - oy);
    a.w = pack_h2(u[3].x - ox, u[3].y - oy);
    b.x = pack_h2(u[0].z - oz, u[1].z - oz);
    b.y = pack_h2(u[2].z - oz, u[3].z - oz);
    b.z = __float_as_uint(ox);
    b.w = w7;
}

// 16-bit yz-quad pairs -> offset yz-quads of the blended values divided by
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
        const V3 u[4] = {V3{c00.xy.x, c00.xy.y, c00.z}, V3{c01.xy.x, c01.xy.y, c01.z},
                         V3{c10.xy.x, c10.xy.y, c10.z}, V3{c11.xy.x, c11.xy.y, c11.z}};
        uint4 a, b;
        encode_quad(u, a, b);
        uint4* o = out + 2 * ((int64_t)j * N + node);
        o[0] = a;
        o[1] = b;
    }
}

// ---------------------------------------------------------------------------
// Offset yz-quads from affine-tile snapshots (JT_STORE_TILE_*).  One thread
// per grid node walks the chunk's entries; when the pair changes it rebuilds
// its quad's four node values of snapshots A and B from the tile that holds
// the node's cell (tile base at the nodes' index coordinates plus their
// residuals) and keeps them in registers.  Blocks of 64 threads, as
// k_stage_f16, so the side-stream launch fits beside the tracking blocks.
// ---------------------------------------------------------------------------

// Residual node {x, y, z, 0} of 16-bit storage STORE, decoded to float32.
template <int STORE>
__device__ __forceinline__ V3 tile_residual(const uint2* __restrict__ r) {
    const uint2 w = __ldg(r);
    if (STORE == JT_STORE_TILE_BF16) return V3{bf16_lo(w.x), bf16_hi(w.x), bf16_lo(w.y)};
    const float2 xy = __half22float2(*reinterpret_cast<const __half2*>(&w.x));
    return V3{xy.x, xy.y, __low2float(*reinterpret_cast<const __half2*>(&w.y))};
}

// Index coordinate of a tile's local node l on an axis of n nodes.
__device__ __forceinline__ float tile_coord(int t, int l, int n, bool periodic) {
    const int g = JT_TILE * t + l;
    return (float)(periodic ? g : min(g, n - 1));
}

// The four quad nodes' values of one snapshot: base o + Gx cx + Gy cy + Gz cz
// at their coordinates plus their residuals.
template <int STORE>
__device__ __forceinline__ void tile_values(const uint2* __restrict__ res, const float* __restrict__ rec,
                                            const int (&lofs)[4], float cx, const float (&cy)[2],
                                            const float (&cz)[2], V3 (&v)[4]) {
    const float4 r0 = __ldg(reinterpret_cast<const float4*>(rec));
    const float4 r1 = __ldg(reinterpret_cast<const float4*>(rec) + 1);
    const float4 r2 = __ldg(reinterpret_cast<const float4*>(rec) + 2);
    // {ox, oy, Gx.x, Gx.y}, {Gy.x, Gy.y, Gz.x, Gz.y}, {oz, Gx.z, Gy.z, Gz.z}
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float y = cy[c >> 1], z = cz[c & 1];
        const V3 r = tile_residual<STORE>(res + lofs[c]);
        v[c] = V3{fmaf(r1.z, z, fmaf(r1.x, y, fmaf(r0.z, cx, r0.x))) + r.x,
                  fmaf(r1.w, z, fmaf(r1.y, y, fmaf(r0.w, cx, r0.y))) + r.y,
                  fmaf(r2.w, z, fmaf(r2.z, y, fmaf(r2.y, cx, r2.x))) + r.z};
    }
}

template <int STORE>
__global__ void __launch_bounds__(kStageBlock16, 16) k_stage_tile(jt_grid_field F, const jt_blend* __restrict__ ent,
                                                                const float* __restrict__ scales, int n,
                                                                uint4* __restrict__ out) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t N = (int64_t)F.nx * F.ny * F.nz;
    if (node >= N) return;
    const int k = (int)(node % F.nz);
    const int j = (int)((node / F.nz) % F.ny);
    const int i = (int)(node / ((int64_t)F.nz * F.ny));
    const bool per = F.bounds_mode == JT_GRID_PERIODIC;
    const int tx = i >> 2, ty = j >> 2, tz = k >> 2, li = i & 3, lj = j & 3, lk = k & 3;
    const int64_t tiles = (int64_t)F.tiles[0] * F.tiles[1] * F.tiles[2];
    const int64_t tile = ((int64_t)tx * F.tiles[1] + ty) * F.tiles[2] + tz;
    constexpr int K = JT_TILE + 1;
    // quad nodes (j,k), (j,k1), (j1,k), (j1,k1): local (lj,lk), (lj,lk+1), (lj+1,lk), (lj+1,lk+1)
    const int l0 = (li * K + lj) * K + lk;
    const int lofs[4] = {l0, l0 + 1, l0 + K, l0 + K + 1};
    const float cx = tile_coord(tx, li, F.nx, per);
    const float cy[2] = {tile_coord(ty, lj, F.ny, per), tile_coord(ty, lj + 1, F.ny, per)};
    const float cz[2] = {tile_coord(tz, lk, F.nz, per), tile_coord(tz, lk + 1, F.nz, per)};
    const uint2* res = reinterpret_cast<const uint2*>(F.pairs);
    int cur = -1;
    PairVal pv[4];
    for (int jj = 0; jj < n; ++jj) {
        const jt_blend e = ent[jj];
        const int pr = min(max(e.pair, 0), F.n_pairs - 1);
        if (pr != cur) {
            V3 va[4], vb[4];
            const int64_t sa = (int64_t)pr * tiles + tile, sb = sa + tiles;
            tile_values<STORE>(res + sa * JT_TILE_NODES, F.tile_base + sa * 16, lofs, cx, cy, cz, va);
            tile_values<STORE>(res + sb * JT_TILE_NODES, F.tile_base + sb * 16, lofs, cx, cy, cz, vb);
#pragma unroll
            for (int c = 0; c < 4; ++c)
                pv[c] = PairVal{make_float2(va[c].x, va[c].y), make_float2(vb[c].x, vb[c].y), va[c].z, vb[c].z};
            cur = pr;
        }
        const float inv = __frcp_rn(__ldg(scales + jj));   // a power of two: exact
        V3 u[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const V3 v = blend<false, JT_STORE_F32>(pv[c], e);
            u[c] = V3{v.x * inv, v.y * inv, v.z * inv};
        }
        uint4 a, b;
        encode_quad(u, a, b);
        uint4* o = out + 2 * ((int64_t)jj * N + node);
        o[0] = a;
        o[1] = b;
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

template <template <bool, int> class FT>
static cudaError_t stage_launch(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p,
                                cudaStream_t s, bool exact) {
    typedef Launcher<FT, jt_grid_field, int> L;
    if (f.storage == JT_STORE_STAGE_F32)
        return exact ? L::template track_s<true, JT_STORE_STAGE_F32>(f, 0, b, p, s)
                     : L::template track_s<false, JT_STORE_STAGE_F32>(f, 0, b, p, s);
    if (f.storage == JT_STORE_STAGE_F32Q)
        return exact ? L::template track_s<true, JT_STORE_STAGE_F32Q>(f, 0, b, p, s)
                     : L::template track_s<false, JT_STORE_STAGE_F32Q>(f, 0, b, p, s);
    return L::template track_s<false, JT_STORE_STAGE_F16>(f, 0, b, p, s);
}

int stage_track(const jt_grid_field& f, const jt_boundary& b, const jt_track_params& p, cudaStream_t s) {
    const bool exact = p.arith == JT_ARITH_EXACT;
    if (f.storage == JT_STORE_STAGE_F16 && exact)
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
    if (((uintptr_t)out & 31u) != 0 || ((uintptr_t)F.pairs & 31u) != 0)
        return set_error(JT_ERR_INVALID, "pairs and out must be 32-byte aligned (256-bit records)");
    const int64_t N = (int64_t)F.nx * F.ny * F.nz;
    if (F.pair_stride != N) return set_error(JT_ERR_INVALID, "pair_stride must equal the node count");
    const unsigned g = grid_blocks(N);
    const unsigned g16 = (unsigned)((N + kStageBlock16 - 1) / kStageBlock16);
    cudaStream_t s = (cudaStream_t)stream;
    if (out_storage == JT_STORE_STAGE_F32Q) {
        if (F.storage != JT_STORE_F32)
            return set_error(JT_ERR_UNSUPPORTED, "float32 stage fields come from float32 snapshots");
        k_stage_f32q<true><<<g, kBlock, 0, s>>>(F, entries, n, reinterpret_cast<char*>(out));
    } else if (out_storage == JT_STORE_STAGE_F32) {
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
        return set_error(JT_ERR_INVALID, "out_storage must be JT_STORE_STAGE_F32, _F32Q or _F16");
    }
    return cuda_status(cudaGetLastError(), "stage field launch");
}

extern "C" int jt_stage_tile_fields(const jt_field* field, const jt_blend* entries, const float* out_scales,
                                    int32_t n, void* out, void* stream) {
    if (field == nullptr || field->kind != JT_FIELD_GRID || field->grid == nullptr)
        return set_error(JT_ERR_INVALID, "stage fields need a regular-grid field");
    const jt_grid_field& F = *field->grid;
    if (int rc = check_grid_shape(F)) return rc;
    if (F.storage != JT_STORE_TILE_BF16 && F.storage != JT_STORE_TILE_F16)
        return set_error(JT_ERR_INVALID, "jt_stage_tile_fields reads JT_STORE_TILE_* snapshots");
    if (int rc = check_tiles(F)) return rc;
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n == 0) return JT_OK;
    if (entries == nullptr || out == nullptr || out_scales == nullptr)
        return set_error(JT_ERR_INVALID, "entries, out_scales and out are required");
    if (F.pairs == nullptr || F.n_pairs < 1) return set_error(JT_ERR_INVALID, "field has no snapshots");
    if (((uintptr_t)out & 31u) != 0)
        return set_error(JT_ERR_INVALID, "out must be 32-byte aligned (256-bit records)");
    const int64_t tiles = (int64_t)F.tiles[0] * F.tiles[1] * F.tiles[2];
    if (F.pair_stride != tiles * JT_TILE_NODES)
        return set_error(JT_ERR_INVALID, "pair_stride must be tiles * JT_TILE_NODES");
    const int64_t N = (int64_t)F.nx * F.ny * F.nz;
    const unsigned g = (unsigned)((N + kStageBlock16 - 1) / kStageBlock16);
    cudaStream_t s = (cudaStream_t)stream;
    uint4* o = reinterpret_cast<uint4*>(out);
    if (F.storage == JT_STORE_TILE_BF16)
        k_stage_tile<JT_STORE_TILE_BF16><<<g, kStageBlock16, 0, s>>>(F, entries, out_scales, n, o);
    else
        k_stage_tile<JT_STORE_TILE_F16><<<g, kStageBlock16, 0, s>>>(F, entries, out_scales, n, o);
    return cuda_status(cudaGetLastError(), "stage field launch");
}
