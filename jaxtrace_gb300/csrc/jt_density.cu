// Density passes over a Morton cell list: SPH summation (density/sph.py) and
// Gaussian KDE on a grid or at points (density/kde.py).
//
// SPH: one query per thread; the query's neighbour cells are visited in a
// fixed order, each cell's terms summed in float32 and the cell sums in
// float64.  The sum runs over every particle within the cutoff -- the NumPy
// brute-force semantics (sph.py:282-292), not the JAX hash grid's per-cell
// cap and nearest-512 truncation (neighbors.py:145-159).
//
// KDE grid: exp(-|g-p|^2/2h^2) = ex * ey * ez factorises per axis, so a block
// owning an 8x8x8 tile of grid points computes 24 exponentials per particle
// (8 per axis) instead of 512 and forms the products from shared memory.
// Particles more than `radius` from the tile along an axis lie in cells the
// block never visits; their terms are below exp(-radius^2/2h^2).
#include <stdint.h>

#include "jt_internal.h"
#include "jt_kernels.cuh"

namespace jt {

// Cell coordinate of x on one axis, clamped to [0, 2^bits - 1].
__device__ __forceinline__ int cell_of(float x, float org, float inv, int lim) {
    const float f = floorf((x - org) * inv);
    return (f != f) ? 0 : (f < 0.0f ? 0 : (f > (float)lim ? lim : (int)f));
}

__device__ __forceinline__ uint32_t cell_begin(const uint32_t* __restrict__ end, uint32_t key) {
    return key == 0 ? 0u : __ldg(end + key - 1);
}

// Row-major cell key (x fastest), the JT_ORDER_LINEAR order of the cell list:
// the cells x0..x1 of one (y, z) row hold one contiguous particle range.
__device__ __forceinline__ uint32_t row_key(int x, int y, int z, int bits) {
    return (((uint32_t)z << bits | (uint32_t)y) << bits) | (uint32_t)x;
}

// Particle range [b, e) of the cells x0..x1 in row (y, z).
__device__ __forceinline__ void row_range(const uint32_t* __restrict__ end, int x0, int x1, int y, int z, int bits,
                                          uint32_t& b, uint32_t& e) {
    b = cell_begin(end, row_key(x0, y, z, bits));
    e = __ldg(end + row_key(x1, y, z, bits));
}

// Smoothing kernels of SPHDensityEstimator (sph.py:227-255).
template <int DIM, int KERN>
__device__ __forceinline__ float sph_w(float r, float h) {
    const float hh = fmaxf(h, 1e-12f);
    const float q = r / hh;
    const float pi = 3.14159265358979f;
    if (KERN == JT_SPH_CUBIC) {
        const float sigma = DIM == 2 ? 10.0f / (7.0f * pi * hh * hh) : 1.0f / (pi * hh * hh * hh);
        if (q <= 1.0f) return sigma * (1.0f - 1.5f * q * q + 0.75f * q * q * q);
        if (q <= 2.0f) {
            const float t = 2.0f - q;
            return sigma * 0.25f * t * t * t;
        }
        return 0.0f;
    } else if (KERN == JT_SPH_WENDLAND) {
        const float sigma = DIM == 2 ? 7.0f / (pi * hh * hh) : 21.0f / (2.0f * pi * hh * hh * hh);
        const float t = fmaxf(1.0f - q, 0.0f);
        const float t2 = t * t;
        return sigma * t2 * t2 * (1.0f + 4.0f * q);
    } else {
        const float ph2 = pi * hh * hh;
        const float sigma = DIM == 2 ? 1.0f / ph2 : 1.0f / (ph2 * sqrtf(ph2));
        return sigma * expf(-q * q);
    }
}

// |d| from d^2 through the hardware reciprocal square root (two instructions
// instead of the correctly rounded square root; about 2 ulp).
__device__ __forceinline__ float fast_dist(float d2) { return d2 > 0.0f ? d2 * rsqrtf(d2) : 0.0f; }

// The kernels again with the 1/h and sigma of a uniform smoothing length
// hoisted out of the pair loop (no division per pair).
template <int DIM, int KERN>
__device__ __forceinline__ float sph_sigma(float hh) {
    const float pi = 3.14159265358979f;
    if (KERN == JT_SPH_CUBIC) return DIM == 2 ? 10.0f / (7.0f * pi * hh * hh) : 1.0f / (pi * hh * hh * hh);
    if (KERN == JT_SPH_WENDLAND) return DIM == 2 ? 7.0f / (pi * hh * hh) : 21.0f / (2.0f * pi * hh * hh * hh);
    const float ph2 = pi * hh * hh;
    return DIM == 2 ? 1.0f / ph2 : 1.0f / (ph2 * sqrtf(ph2));
}

template <int KERN>
__device__ __forceinline__ float sph_shape(float q) {
    if (KERN == JT_SPH_CUBIC) {
        const float t = fmaxf(2.0f - q, 0.0f);
        const float outer = 0.25f * t * t * t;                        // 1 < q <= 2
        const float inner = fmaf(q * q, fmaf(0.75f, q, -1.5f), 1.0f);  // q <= 1
        return q <= 1.0f ? inner : outer;
    } else if (KERN == JT_SPH_WENDLAND) {
        const float t = fmaxf(1.0f - q, 0.0f);
        const float t2 = t * t;
        return t2 * t2 * fmaf(4.0f, q, 1.0f);
    }
    return expf(-q * q);
}

// sph_shape of two distances at once: the cubic spline in float32x2
// arithmetic (each lane rounds as sph_shape does), the other kernels per lane.
template <int KERN>
__device__ __forceinline__ float2 sph_shape2(float2 q) {
    if (KERN == JT_SPH_CUBIC) {
        const float2 d = __fadd2_rn(make_float2(2.0f, 2.0f), make_float2(-q.x, -q.y));
        const float2 t = make_float2(fmaxf(d.x, 0.0f), fmaxf(d.y, 0.0f));
        const float2 outer = __fmul2_rn(__fmul2_rn(__fmul2_rn(make_float2(0.25f, 0.25f), t), t), t);
        const float2 inner = __ffma2_rn(__fmul2_rn(q, q), __ffma2_rn(make_float2(0.75f, 0.75f), q,
                                                                     make_float2(-1.5f, -1.5f)),
                                        make_float2(1.0f, 1.0f));
        return make_float2(q.x <= 1.0f ? inner.x : outer.x, q.y <= 1.0f ? inner.y : outer.y);
    }
    return make_float2(sph_shape<KERN>(q.x), sph_shape<KERN>(q.y));
}

// Sum of a per-thread count over the warp, added once per warp.
__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
    const unsigned m = __activemask();
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(m, v, o);
    if ((threadIdx.x & 31) == (__ffs(m) - 1)) atomicAdd(dst, v);
}

// One particle j of the paired layout (a row's first or last particle when
// the row starts or ends mid-pair), with the scalar arithmetic of the
// {x, y, z, m} records.
template <int DIM, int KERN, bool COUNT>
__device__ __forceinline__ float sph_pair_one(const float* pairs, uint32_t j, float qx, float qy, float qz,
                                              float inv, float r2lim, float part, unsigned long long& n_in) {
    const float* f = pairs + 8 * (int64_t)(j >> 1) + (j & 1u);
    const float dx = __ldg(f) - qx, dy = __ldg(f + 2) - qy, dz = DIM == 3 ? __ldg(f + 4) - qz : 0.0f;
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (d2 <= r2lim) {
        part = fmaf(__ldg(f + 6), sph_shape<KERN>(fast_dist(d2) * inv), part);
        if (COUNT) ++n_in;
    }
    return part;
}

// COUNT: also count the candidate pairs examined and those inside the
// support (P.counters), a separate instance so the plain one keeps its loop.
template <int DIM, int KERN, bool COUNT = false>
__global__ void __launch_bounds__(kBlock) k_sph(jt_sph_params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n_queries) return;
    const float qx = P.queries[3 * (int64_t)i], qy = P.queries[3 * (int64_t)i + 1];
    const float qz = DIM == 3 ? P.queries[3 * (int64_t)i + 2] : 0.0f;
    const jt_sort_grid& g = P.grid;
    const int lim = (1 << g.bits) - 1;
    const int cx = cell_of(qx, g.origin[0], g.inv_cell[0], lim);
    const int cy = cell_of(qy, g.origin[1], g.inv_cell[1], lim);
    const int cz = DIM == 3 ? cell_of(qz, g.origin[2], g.inv_cell[2], lim) : 0;
    const float r2max = P.radius * P.radius;
    const int z0 = DIM == 3 ? max(cz - P.reach[2], 0) : 0, z1 = DIM == 3 ? min(cz + P.reach[2], lim) : 0;
    const int y0 = max(cy - P.reach[1], 0), y1 = min(cy + P.reach[1], lim);
    const int x0 = max(cx - P.reach[0], 0), x1 = min(cx + P.reach[0], lim);
    double acc = 0.0;
    unsigned long long n_cand = 0, n_in = 0;
    if (P.h == nullptr) {
        // uniform h: sigma and 1/h once; pairs beyond the kernel's support skip
        const float hh = fmaxf(P.h_const, 1e-12f), inv = 1.0f / hh, sigma = sph_sigma<DIM, KERN>(hh);
        const float sup = KERN == JT_SPH_CUBIC ? 2.0f * hh : (KERN == JT_SPH_WENDLAND ? hh : 3.4e38f);
        const float r2lim = fminf(r2max, sup >= 1.8e19f ? r2max : sup * sup);
        // rows of the cell box whose slab lies beyond the support sphere are
        // skipped and the rest trimmed in x (with a margin: only whole
        // cells that cannot hold a term are dropped)
        const float csy = 1.0f / g.inv_cell[1], csz = DIM == 3 ? 1.0f / g.inv_cell[2] : 0.0f;
        for (int z = z0; z <= z1; ++z) {
            const float dzr = DIM == 3 ? fmaxf(fmaxf(g.origin[2] + z * csz - qz, qz - (g.origin[2] + (z + 1) * csz)),
                                               0.0f)
                                       : 0.0f;
            for (int y = y0; y <= y1; ++y) {
                const float dyr = fmaxf(fmaxf(g.origin[1] + y * csy - qy, qy - (g.origin[1] + (y + 1) * csy)), 0.0f);
                const float rem = r2lim - dyr * dyr - dzr * dzr;
                if (rem < -1e-6f * r2lim) continue;
                const float rx = sqrtf(fmaxf(rem, 0.0f)) * 1.0001f + 1e-7f;
                const int xa = max(x0, cell_of(qx - rx, g.origin[0], g.inv_cell[0], lim));
                const int xb = min(x1, cell_of(qx + rx, g.origin[0], g.inv_cell[0], lim));
                if (xa > xb) continue;
                uint32_t b, e;
                row_range(P.cell_end, xa, xb, y, z, g.bits, b, e);
                float part = 0.0f;
                if (P.packed == 2) {
                    // pairs of particles (x0 x1 y0 y1 z0 z1 m0 m1): two
                    // candidates per iteration in float32x2 arithmetic, their
                    // terms added in particle order as one at a time
                    if (COUNT) n_cand += e - b;
                    const float2 nqx = make_float2(-qx, -qx), nqy = make_float2(-qy, -qy),
                                 nqz = make_float2(-qz, -qz), inv2 = make_float2(inv, inv);
                    uint32_t j = b;
                    if (j < e && (j & 1u)) {  // a row that starts on a pair's second particle
                        part = sph_pair_one<DIM, KERN, COUNT>(P.particles, j, qx, qy, qz, inv, r2lim, part, n_in);
                        ++j;
                    }
                    const float4* p4 = reinterpret_cast<const float4*>(P.particles);
#pragma unroll 2
                    for (; j + 1 < e; j += 2) {
                        const float4 u = __ldg(p4 + j), w = __ldg(p4 + j + 1);  // j even: pair j/2
                        const float2 dx = __fadd2_rn(make_float2(u.x, u.y), nqx);
                        const float2 dy = __fadd2_rn(make_float2(u.z, u.w), nqy);
                        const float2 dz = DIM == 3 ? __fadd2_rn(make_float2(w.x, w.y), nqz) : make_float2(0.0f, 0.0f);
                        const float2 d2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                        const float2 sh =
                            sph_shape2<KERN>(__fmul2_rn(make_float2(fast_dist(d2.x), fast_dist(d2.y)), inv2));
                        if (d2.x <= r2lim) {
                            part = fmaf(w.z, sh.x, part);
                            if (COUNT) ++n_in;
                        }
                        if (d2.y <= r2lim) {
                            part = fmaf(w.w, sh.y, part);
                            if (COUNT) ++n_in;
                        }
                    }
                    if (j < e)  // a row that ends on a pair's first particle
                        part = sph_pair_one<DIM, KERN, COUNT>(P.particles, j, qx, qy, qz, inv, r2lim, part, n_in);
                } else if (P.packed) {
                    // {x, y, z, m} records; FMA-contracted distance (no parity
                    // constraint on the density passes)
                    const float4* p4 = reinterpret_cast<const float4*>(P.particles);
                    if (COUNT) n_cand += e - b;
#pragma unroll 4
                    for (uint32_t j = b; j < e; ++j) {
                        const float4 r = __ldg(p4 + j);
                        const float dx = r.x - qx, dy = r.y - qy, dz = DIM == 3 ? r.z - qz : 0.0f;
                        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        if (d2 <= r2lim) {
                            part = fmaf(r.w, sph_shape<KERN>(fast_dist(d2) * inv), part);
                            if (COUNT) ++n_in;
                        }
                    }
                } else {
                    for (uint32_t j = b; j < e; ++j) {
                        const float dx = __ldg(P.particles + 3 * (int64_t)j) - qx;
                        const float dy = __ldg(P.particles + 3 * (int64_t)j + 1) - qy;
                        const float dz = DIM == 3 ? __ldg(P.particles + 3 * (int64_t)j + 2) - qz : 0.0f;
                        const float d2 = dx * dx + dy * dy + dz * dz;
                        if (d2 <= r2lim) {
                            const float m = P.masses != nullptr ? __ldg(P.masses + j) : 1.0f;
                            part += m * sph_shape<KERN>(fast_dist(d2) * inv);
                        }
                    }
                }
                acc += (double)part * (double)sigma;
            }
        }
    } else {
        for (int z = z0; z <= z1; ++z) {
            for (int y = y0; y <= y1; ++y) {
                uint32_t b, e;
                row_range(P.cell_end, x0, x1, y, z, g.bits, b, e);
                float part = 0.0f;
                for (uint32_t j = b; j < e; ++j) {
                    const float dx = __ldg(P.particles + 3 * (int64_t)j) - qx;
                    const float dy = __ldg(P.particles + 3 * (int64_t)j + 1) - qy;
                    const float dz = DIM == 3 ? __ldg(P.particles + 3 * (int64_t)j + 2) - qz : 0.0f;
                    const float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 <= r2max) {
                        const float h = __ldg(P.h + j);
                        const float m = P.masses != nullptr ? __ldg(P.masses + j) : 1.0f;
                        part += m * sph_w<DIM, KERN>(sqrtf(d2), h);
                    }
                }
                acc += (double)part;
            }
        }
    }
    P.out[i] = acc;
    if (COUNT) {
        warp_add(P.counters, n_cand);
        warp_add(P.counters + 1, n_in);
    }
}

// ---------------------------------------------------------------------------
// KDE on a grid.
constexpr int kTile3 = 8;            // 8x8x8 grid points per block
constexpr int kTile2 = 16;           // 16x16 in 2-D
constexpr int kKdeThreads = 512;     // one grid point per thread (3-D), 256 used in 2-D
// particles per shared-memory chunk: DIM*T factor rows of (chunk+1) floats
// must fit the 48 KB of static shared memory (the +1 keeps rows on distinct banks)
constexpr int kChunk3 = 480;         // 24 rows x 481 x 4 B = 46.2 KB
constexpr int kChunk2 = 352;         // 32 rows x 353 x 4 B = 45.2 KB

template <int DIM>
__global__ void __launch_bounds__(kKdeThreads) k_kde_grid(jt_kde_params P) {
    constexpr int T = DIM == 3 ? kTile3 : kTile2;
    constexpr int NT = DIM == 3 ? T * T * T : T * T;  // threads that own a grid point
    constexpr int CH = DIM == 3 ? kChunk3 : kChunk2;
    __shared__ float fac[DIM * T][CH + 1];             // factors per axis value, per particle of the chunk
    __shared__ float gcoord[3][T];
    const int t = threadIdx.x;
    const int tiles_x = (P.res[0] + T - 1) / T, tiles_y = (P.res[1] + T - 1) / T;
    const int bx = blockIdx.x % tiles_x;
    const int by = (blockIdx.x / tiles_x) % tiles_y;
    const int bz = DIM == 3 ? blockIdx.x / (tiles_x * tiles_y) : 0;
    const int base[3] = {bx * T, by * T, bz * T};
    const int cnt[3] = {min(T, P.res[0] - base[0]), min(T, P.res[1] - base[1]),
                        DIM == 3 ? min(T, P.res[2] - base[2]) : 1};
    if (t < 3 * T) {
        const int a = t / T, k = t % T;
        gcoord[a][k] = (a < DIM && k < cnt[a]) ? __ldg(P.axis[a] + base[a] + k) : 0.0f;
    }
    __syncthreads();
    // this thread's grid point inside the tile
    int pa, pb, pc;
    if (DIM == 3) { pa = t / (T * T); pb = (t / T) % T; pc = t % T; }
    else { pa = t / T; pb = t % T; pc = 0; }
    const bool owner = t < NT && pa < cnt[0] && pb < cnt[1] && pc < cnt[2];
    // cell range covering the tile widened by the radius
    const jt_sort_grid& g = P.grid;
    const int lim = (1 << g.bits) - 1;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int a = 0; a < DIM; ++a) {
        lo[a] = cell_of(gcoord[a][0] - P.radius, g.origin[a], g.inv_cell[a], lim);
        hi[a] = cell_of(gcoord[a][cnt[a] - 1] + P.radius, g.origin[a], g.inv_cell[a], lim);
    }
    double acc = 0.0;
    for (int cz = lo[2]; cz <= hi[2]; ++cz)
        for (int cy = lo[1]; cy <= hi[1]; ++cy) {
            uint32_t b, e;
            row_range(P.cell_end, lo[0], hi[0], cy, cz, g.bits, b, e);
            {
                for (uint32_t c0 = b; c0 < e; c0 += CH) {
                    const int nchunk = (int)min((uint32_t)CH, e - c0);
                    if (t < nchunk) {
                        const int64_t j = c0 + t;
                        const float p[3] = {__ldg(P.particles + 3 * j), __ldg(P.particles + 3 * j + 1),
                                            __ldg(P.particles + 3 * j + 2)};
#pragma unroll
                        for (int a = 0; a < DIM; ++a)
#pragma unroll
                            for (int k = 0; k < T; ++k) {
                                const float d = gcoord[a][k] - p[a];
                                fac[a * T + k][t] = __expf(-d * d * P.half_inv_h2);
                            }
                    }
                    __syncthreads();
                    if (owner) {
                        float part = 0.0f;
                        const float* fa = fac[pa];
                        const float* fb = fac[T + pb];
                        if (DIM == 3) {
                            const float* fc = fac[2 * T + pc];
                            for (int j = 0; j < nchunk; ++j) part = fmaf(fa[j] * fb[j], fc[j], part);
                        } else {
                            for (int j = 0; j < nchunk; ++j) part = fmaf(fa[j], fb[j], part);
                        }
                        acc += (double)part;
                    }
                    __syncthreads();
                }
            }
        }
    if (owner) {
        const int64_t gi = ((int64_t)(base[0] + pa) * P.res[1] + (base[1] + pb)) * (DIM == 3 ? P.res[2] : 1) +
                           (DIM == 3 ? base[2] + pc : 0);
        P.out[gi] = acc;
    }
}

constexpr int kKbT = 8;  // the 3-D KDE's grid tile edge

// 3-D KDE with register blocking: a block of 64 threads owns an 8^3 tile of
// grid points and each thread eight of them (two y by four z), so one particle
// costs a thread three shared loads (its x factor, two y factors in one
// 64-bit load, four z factors in one 128-bit load), one float32x2 multiply
// and four float32x2 FMAs (10 % faster than the scalar ones, same bits).  All factors are stored particle-major (32 B per particle and axis):
// a warp's loads of one particle fall in one 32-byte row per axis, one
// shared-memory wavefront each.  The tile stays 8^3 so the dilated box of
// particles each tile visits stays small.  (Four z points per thread of
// 128, with x and y factors in axis-major rows, took 3 shared loads per 4
// terms and was 12 % slower, bound by the shared-memory pipe.)
constexpr int kK8Threads = 64;
constexpr int kK8Chunk = 240;  // 3 x 240 x 32 B = 22.5 KB: eight blocks (16 warps) per SM
static_assert(kK8Threads * 8 == kKbT * kKbT * kKbT, "eight grid points per thread");

__global__ void __launch_bounds__(kK8Threads, 8) k_kde_grid3_blocked(jt_kde_params P) {
    __shared__ __align__(16) float fx[kK8Chunk][kKbT];
    __shared__ __align__(16) float fy[kK8Chunk][kKbT];
    __shared__ __align__(16) float fz[kK8Chunk][kKbT];
    __shared__ float gcoord[3][kKbT];
    const int t = threadIdx.x;
    const int tiles_a = (P.res[0] + kKbT - 1) / kKbT, tiles_b = (P.res[1] + kKbT - 1) / kKbT;
    const int ta = blockIdx.x % tiles_a, tb = (blockIdx.x / tiles_a) % tiles_b;
    const int tc = blockIdx.x / (tiles_a * tiles_b);
    const int b0 = ta * kKbT, b1 = tb * kKbT, b2 = tc * kKbT;
    const int n0 = min(kKbT, P.res[0] - b0), n1 = min(kKbT, P.res[1] - b1), n2 = min(kKbT, P.res[2] - b2);
    if (t < 3 * kKbT) {
        const int a = t / kKbT, k = t % kKbT;
        const int na = a == 0 ? n0 : (a == 1 ? n1 : n2), ba = a == 0 ? b0 : (a == 1 ? b1 : b2);
        gcoord[a][k] = k < na ? __ldg(P.axis[a] + ba + k) : 0.0f;
    }
    __syncthreads();
    // thread -> (pa, y points pb0 and pb0 + 1, z points pc0 .. pc0 + 3); z fastest
    const int pc0 = 4 * (t & 1);
    const int pb0 = 2 * ((t >> 1) & 3);
    const int pa = t >> 3;
    const jt_sort_grid& g = P.grid;
    const int lim = (1 << g.bits) - 1;
    const int lo0 = cell_of(gcoord[0][0] - P.radius, g.origin[0], g.inv_cell[0], lim);
    const int hi0 = cell_of(gcoord[0][n0 - 1] + P.radius, g.origin[0], g.inv_cell[0], lim);
    const int lo1 = cell_of(gcoord[1][0] - P.radius, g.origin[1], g.inv_cell[1], lim);
    const int hi1 = cell_of(gcoord[1][n1 - 1] + P.radius, g.origin[1], g.inv_cell[1], lim);
    const int lo2 = cell_of(gcoord[2][0] - P.radius, g.origin[2], g.inv_cell[2], lim);
    const int hi2 = cell_of(gcoord[2][n2 - 1] + P.radius, g.origin[2], g.inv_cell[2], lim);
    double acc[2][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
    unsigned long long visits = 0;
    for (int cz = lo2; cz <= hi2; ++cz)
        for (int cy = lo1; cy <= hi1; ++cy) {
            uint32_t b, e;
            row_range(P.cell_end, lo0, hi0, cy, cz, g.bits, b, e);
            visits += e - b;
            for (uint32_t c0 = b; c0 < e; c0 += kK8Chunk) {
                const int n = (int)min((uint32_t)kK8Chunk, e - c0);
                for (int j = t; j < n; j += kK8Threads) {
                    const int64_t pj = c0 + j;
                    const float px = __ldg(P.particles + 3 * pj), py = __ldg(P.particles + 3 * pj + 1);
                    const float pz = __ldg(P.particles + 3 * pj + 2);
                    float ax[kKbT], ay[kKbT], az[kKbT];
#pragma unroll
                    for (int q = 0; q < kKbT; ++q) {
                        const float dx = gcoord[0][q] - px, dy = gcoord[1][q] - py, dz = gcoord[2][q] - pz;
                        ax[q] = __expf(-dx * dx * P.half_inv_h2);
                        ay[q] = __expf(-dy * dy * P.half_inv_h2);
                        az[q] = __expf(-dz * dz * P.half_inv_h2);
                    }
#pragma unroll
                    for (int q = 0; q < kKbT; q += 4) {
                        *reinterpret_cast<float4*>(&fx[j][q]) = make_float4(ax[q], ax[q + 1], ax[q + 2], ax[q + 3]);
                        *reinterpret_cast<float4*>(&fy[j][q]) = make_float4(ay[q], ay[q + 1], ay[q + 2], ay[q + 3]);
                        *reinterpret_cast<float4*>(&fz[j][q]) = make_float4(az[q], az[q + 1], az[q + 2], az[q + 3]);
                    }
                }
                __syncthreads();
                float p[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
                // float32x2 multiplies and FMAs: each lane rounds as the scalar ones
                float2 q00 = make_float2(0.f, 0.f), q01 = q00, q10 = q00, q11 = q00;
#pragma unroll 4
                for (int j = 0; j < n; ++j) {
                    const float2 y2 = *reinterpret_cast<const float2*>(&fy[j][pb0]);
                    const float4 c = *reinterpret_cast<const float4*>(&fz[j][pc0]);
                    const float2 ab = __fmul2_rn(splat(fx[j][pa]), y2);
                    const float2 cxy = make_float2(c.x, c.y), czw = make_float2(c.z, c.w);
                    q00 = __ffma2_rn(splat(ab.x), cxy, q00);
                    q01 = __ffma2_rn(splat(ab.x), czw, q01);
                    q10 = __ffma2_rn(splat(ab.y), cxy, q10);
                    q11 = __ffma2_rn(splat(ab.y), czw, q11);
                }
                p[0][0] = q00.x; p[0][1] = q00.y; p[0][2] = q01.x; p[0][3] = q01.y;
                p[1][0] = q10.x; p[1][1] = q10.y; p[1][2] = q11.x; p[1][3] = q11.y;
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int k = 0; k < 4; ++k) acc[r][k] += (double)p[r][k];
                __syncthreads();
            }
        }
    if (P.counters != nullptr && t == 0) {
        atomicAdd(P.counters, visits);
        atomicAdd(P.counters + 1, visits * (unsigned long long)(n0 * n1 * n2));
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int pb = pb0 + r;
        if (pa < n0 && pb < n1) {
            const int64_t row = ((int64_t)(b0 + pa) * P.res[1] + (b1 + pb)) * P.res[2] + b2 + pc0;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (pc0 + k < n2) P.out[row + k] = acc[r][k];
        }
    }
}

// KDE at arbitrary points: one point per thread over the cells within radius.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_kde_points(jt_kde_params P, const float* __restrict__ pts, int m,
                                                       double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const float q[3] = {pts[3 * (int64_t)i], pts[3 * (int64_t)i + 1], DIM == 3 ? pts[3 * (int64_t)i + 2] : 0.0f};
    const jt_sort_grid& g = P.grid;
    const int lim = (1 << g.bits) - 1;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int a = 0; a < DIM; ++a) {
        lo[a] = cell_of(q[a] - P.radius, g.origin[a], g.inv_cell[a], lim);
        hi[a] = cell_of(q[a] + P.radius, g.origin[a], g.inv_cell[a], lim);
    }
    double acc = 0.0;
    for (int cz = lo[2]; cz <= hi[2]; ++cz)
        for (int cy = lo[1]; cy <= hi[1]; ++cy) {
            {
                uint32_t b, e;
                row_range(P.cell_end, lo[0], hi[0], cy, cz, g.bits, b, e);
                float part = 0.0f;
                for (uint32_t j = b; j < e; ++j) {
                    const float dx = q[0] - __ldg(P.particles + 3 * (int64_t)j);
                    const float dy = q[1] - __ldg(P.particles + 3 * (int64_t)j + 1);
                    const float dz = DIM == 3 ? q[2] - __ldg(P.particles + 3 * (int64_t)j + 2) : 0.0f;
                    part += __expf(-(dx * dx + dy * dy + dz * dz) * P.half_inv_h2);
                }
                acc += (double)part;
            }
        }
    out[i] = acc;
}

}  // namespace jt

using namespace jt;

extern "C" int jt_sph_density(const jt_sph_params* p, void* stream) {
    if (p == nullptr) return set_error(JT_ERR_INVALID, "params is NULL");
    if (p->dims != 2 && p->dims != 3) return set_error(JT_ERR_INVALID, "dims must be 2 or 3");
    if (p->kernel < JT_SPH_CUBIC || p->kernel > JT_SPH_GAUSSIAN) return set_error(JT_ERR_INVALID, "unknown SPH kernel");
    if (p->grid.bits < 1 || p->grid.bits > 7) return set_error(JT_ERR_INVALID, "grid bits must be 1..7");
    if (p->n_queries < 0 || p->n_particles < 0) return set_error(JT_ERR_INVALID, "negative size");
    if (p->n_queries == 0) return JT_OK;
    if (p->queries == nullptr || p->out == nullptr || p->cell_end == nullptr || (p->n_particles > 0 && p->particles == nullptr))
        return set_error(JT_ERR_INVALID, "queries, out, cell_end and particles are required");
    for (int a = 0; a < 3; ++a)
        if (p->reach[a] < 0 || p->reach[a] > 127) return set_error(JT_ERR_INVALID, "reach must be 0..127");
    if (p->packed < 0 || p->packed > 2) return set_error(JT_ERR_INVALID, "packed must be 0, 1 or 2");
    if (p->packed != 0 && p->h != nullptr)
        return set_error(JT_ERR_UNSUPPORTED, "packed records need a uniform smoothing length");
    const unsigned gb = grid_blocks(p->n_queries);
    cudaStream_t st = (cudaStream_t)stream;
    if (p->counters != nullptr) {
        if (p->h != nullptr || !p->packed)
            return set_error(JT_ERR_UNSUPPORTED, "SPH counters need a uniform h and packed records");
        if (p->dims == 3 && p->kernel == JT_SPH_CUBIC) k_sph<3, JT_SPH_CUBIC, true><<<gb, kBlock, 0, st>>>(*p);
        else if (p->dims == 3 && p->kernel == JT_SPH_WENDLAND) k_sph<3, JT_SPH_WENDLAND, true><<<gb, kBlock, 0, st>>>(*p);
        else if (p->dims == 3) k_sph<3, JT_SPH_GAUSSIAN, true><<<gb, kBlock, 0, st>>>(*p);
        else return set_error(JT_ERR_UNSUPPORTED, "SPH counters are for 3-D");
        return cuda_status(cudaGetLastError(), "SPH kernel launch");
    }
#define JT_SPH_LAUNCH(D, K) k_sph<D, K><<<gb, kBlock, 0, st>>>(*p)
    if (p->dims == 3) {
        if (p->kernel == JT_SPH_CUBIC) JT_SPH_LAUNCH(3, JT_SPH_CUBIC);
        else if (p->kernel == JT_SPH_WENDLAND) JT_SPH_LAUNCH(3, JT_SPH_WENDLAND);
        else JT_SPH_LAUNCH(3, JT_SPH_GAUSSIAN);
    } else {
        if (p->kernel == JT_SPH_CUBIC) JT_SPH_LAUNCH(2, JT_SPH_CUBIC);
        else if (p->kernel == JT_SPH_WENDLAND) JT_SPH_LAUNCH(2, JT_SPH_WENDLAND);
        else JT_SPH_LAUNCH(2, JT_SPH_GAUSSIAN);
    }
#undef JT_SPH_LAUNCH
    return cuda_status(cudaGetLastError(), "SPH kernel launch");
}

static int check_kde(const jt_kde_params* p) {
    if (p == nullptr) return set_error(JT_ERR_INVALID, "params is NULL");
    if (p->dims != 2 && p->dims != 3) return set_error(JT_ERR_INVALID, "dims must be 2 or 3");
    if (p->grid.bits < 1 || p->grid.bits > 7) return set_error(JT_ERR_INVALID, "grid bits must be 1..7");
    if (p->n_particles < 0) return set_error(JT_ERR_INVALID, "negative size");
    if (p->cell_end == nullptr || (p->n_particles > 0 && p->particles == nullptr))
        return set_error(JT_ERR_INVALID, "cell_end and particles are required");
    if (!(p->radius >= 0.0f) || !(p->half_inv_h2 > 0.0f)) return set_error(JT_ERR_INVALID, "bad radius or bandwidth");
    return JT_OK;
}

extern "C" int jt_kde_grid(const jt_kde_params* p, void* stream) {
    int rc;
    if ((rc = check_kde(p))) return rc;
    const int D = p->dims;
    for (int a = 0; a < D; ++a)
        if (p->res[a] < 1 || p->axis[a] == nullptr) return set_error(JT_ERR_INVALID, "grid axis %d is empty", a);
    if (D == 2 && p->res[2] != 1) return set_error(JT_ERR_INVALID, "2-D grids have res[2] == 1");
    if (p->out == nullptr) return set_error(JT_ERR_INVALID, "out is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    if (D == 3) {
        const int64_t blocks = (int64_t)((p->res[0] + kKbT - 1) / kKbT) * ((p->res[1] + kKbT - 1) / kKbT) *
                               ((p->res[2] + kKbT - 1) / kKbT);
        if (blocks > 0x7fffffff) return set_error(JT_ERR_INVALID, "grid too large");
        k_kde_grid3_blocked<<<(unsigned)blocks, kK8Threads, 0, st>>>(*p);
    } else {
        const int T = kTile2;
        const int64_t blocks = (int64_t)((p->res[0] + T - 1) / T) * ((p->res[1] + T - 1) / T);
        if (blocks > 0x7fffffff) return set_error(JT_ERR_INVALID, "grid too large");
        k_kde_grid<2><<<(unsigned)blocks, kKdeThreads, 0, st>>>(*p);
    }
    return cuda_status(cudaGetLastError(), "KDE grid kernel launch");
}

extern "C" int jt_kde_points(const jt_kde_params* p, const float* points, int32_t m, double* out, void* stream) {
    int rc;
    if ((rc = check_kde(p))) return rc;
    if (m < 0) return set_error(JT_ERR_INVALID, "m must be >= 0");
    if (m == 0) return JT_OK;
    if (points == nullptr || out == nullptr) return set_error(JT_ERR_INVALID, "points and out are required");
    cudaStream_t st = (cudaStream_t)stream;
    if (p->dims == 3) k_kde_points<3><<<grid_blocks(m), kBlock, 0, st>>>(*p, points, m, out);
    else k_kde_points<2><<<grid_blocks(m), kBlock, 0, st>>>(*p, points, m, out);
    return cuda_status(cudaGetLastError(), "KDE points kernel launch");
}
