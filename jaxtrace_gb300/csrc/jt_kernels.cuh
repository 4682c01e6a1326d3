// Kernel templates shared by the three field kinds, and the dispatch from
// the run-time (arith, integrator, storage) triple to template instances.
#pragma once

#include "jt_common.cuh"
#include "jt_internal.h"

namespace jt {

constexpr int kBlock = 256;

// Resident blocks per SM the tracking kernels are compiled for (register cap
// 65536 / (kBlock * JT_TRACK_MIN_BLOCKS)).  Measured on the precision
// configuration: 3 beats 2 by 12-15 % and 4 (heavy spills) by 5-10 %.
#ifndef JT_TRACK_MIN_BLOCKS
#define JT_TRACK_MIN_BLOCKS 3
#endif

// Persistent tracking: tracker.py:236-242 (scan body) over [step_begin, step_end).
// Blocks per SM the tracking kernel is compiled for: a field type may name its
// own (kMinBlocks, e.g. a lighter gather needs fewer registers), otherwise
// JT_TRACK_MIN_BLOCKS.
template <class F, class = void>
struct MinBlocksOf {
    static constexpr int value = JT_TRACK_MIN_BLOCKS;
};
template <class F>
struct MinBlocksOf<F, decltype(void(F::kMinBlocks))> {
    static constexpr int value = F::kMinBlocks;
};

template <bool EXACT, int INTEG, bool PATH, int BK, class Field>
__global__ void __launch_bounds__(kBlock, MinBlocksOf<Field>::value)
    k_track(Field f, jt_boundary B, InletFrame I, jt_track_params P) {
    track_body<EXACT, INTEG, PATH, BK>(f, B, I, P);
}

// Whether a field type gets an RK4 kernel specialised for the +x grid inlet
// (kInletXpos), besides the one that reads the boundary at run time.
template <class F, class = void>
struct InletXposOf {
    static constexpr bool value = false;
};
template <class F>
struct InletXposOf<F, decltype(void(F::kInletXpos))> {
    static constexpr bool value = F::kInletXpos;
};

inline bool is_inlet_xpos(const jt_boundary& B) {
    return B.inlet_mode == JT_INLET_GRID && B.inlet_axis == 0 && B.inlet_positive != 0;
}

// Field evaluation at M points with one blend: sample_at_positions(pos, t).
template <class Field>
__global__ void __launch_bounds__(kBlock) k_sample(Field f, jt_blend e, const float* __restrict__ pos,
                                                   float* __restrict__ out, int m, int32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int flags = 0;
    const V3 p{pos[3 * (int64_t)i], pos[3 * (int64_t)i + 1], pos[3 * (int64_t)i + 2]};
    const V3 v = f(p, e, flags);
    out[3 * (int64_t)i] = v.x;
    out[3 * (int64_t)i + 1] = v.y;
    out[3 * (int64_t)i + 2] = v.z;
    report_flags(status, flags);
}

struct StageBlends {
    jt_blend e[3];
};

// One integrator step without boundary (rk4_step / rk2_step / euler_step),
// scalar dt or per-particle dt (rk4.py:108-129, rk2.py:295-309, euler.py:154-157).
template <bool EXACT, int INTEG, class Field>
__global__ void __launch_bounds__(kBlock) k_step(Field f, StageBlends sb, StepConst k0,
                                                 const float* __restrict__ dt_pp,
                                                 const float* __restrict__ xin, float* __restrict__ xout,
                                                 int n, int32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    StepConst k = k0;
    if (dt_pp != nullptr) {
        const float d = dt_pp[i];
        k.dt = d;
        k.dth = __fmul_rn(0.5f, d);
        k.dt6 = __fdiv_rn(d, 6.0f);
    }
    int flags = 0;
    V3 x{xin[3 * (int64_t)i], xin[3 * (int64_t)i + 1], xin[3 * (int64_t)i + 2]};
    V3 c{0.f, 0.f, 0.f};
    integrate<EXACT, INTEG, false>(f, sb.e, k, x, c, flags);
    xout[3 * (int64_t)i] = x.x;
    xout[3 * (int64_t)i + 1] = x.y;
    xout[3 * (int64_t)i + 2] = x.z;
    report_flags(status, flags);
}

inline unsigned grid_blocks(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

// Instantiate and launch for a field template FT<EXACT, STORE>.
template <template <bool, int> class FT, class Desc, class Extra>
struct Launcher {
    template <bool EXACT, int STORE>
    static FT<EXACT, STORE> make(const Desc& d, const Extra& x) {
        return FT<EXACT, STORE>::create(d, x);
    }

    template <bool EXACT, int STORE>
    static cudaError_t track_s(const Desc& d, const Extra& x, const jt_boundary& B,
                               const jt_track_params& P, cudaStream_t st) {
        const FT<EXACT, STORE> f = make<EXACT, STORE>(d, x);
        // block_size was validated to 0, 64, 128 or 256 (<= kBlock, the launch bound)
        const int bs = P.block_size > 0 ? P.block_size : kBlock;
        const unsigned g = (unsigned)((P.n_particles + bs - 1) / bs);
        const InletFrame I = inlet_frame(B);
        if (P.path != nullptr) return launch_track<EXACT, true>(f, B, I, P, g, bs, st);
        return launch_track<EXACT, false>(f, B, I, P, g, bs, st);
    }

    template <bool EXACT, bool PATH, class FF>
    static cudaError_t launch_track(const FF& f, const jt_boundary& B, const InletFrame& I, const jt_track_params& P,
                                    unsigned g, int bs, cudaStream_t st) {
        if constexpr (InletXposOf<FF>::value && !PATH) {
            if (P.integrator == JT_RK4 && is_inlet_xpos(B)) {
                k_track<EXACT, JT_RK4, PATH, JT_BK_INLET_XPOS><<<g, bs, 0, st>>>(f, B, I, P);
                return cudaGetLastError();
            }
        }
        switch (P.integrator) {
            case JT_EULER: k_track<EXACT, JT_EULER, PATH, JT_BK_ANY><<<g, bs, 0, st>>>(f, B, I, P); break;
            case JT_RK2: k_track<EXACT, JT_RK2, PATH, JT_BK_ANY><<<g, bs, 0, st>>>(f, B, I, P); break;
            default: k_track<EXACT, JT_RK4, PATH, JT_BK_ANY><<<g, bs, 0, st>>>(f, B, I, P); break;
        }
        return cudaGetLastError();
    }

    template <bool EXACT, int STORE>
    static cudaError_t step_s(const Desc& d, const Extra& x, const StageBlends& sb, int integ,
                              StepConst k, const float* dtpp, const float* xin, float* xout, int n,
                              int32_t* status, cudaStream_t st) {
        const FT<EXACT, STORE> f = make<EXACT, STORE>(d, x);
        const unsigned g = grid_blocks(n);
        switch (integ) {
            case JT_EULER: k_step<EXACT, JT_EULER><<<g, kBlock, 0, st>>>(f, sb, k, dtpp, xin, xout, n, status); break;
            case JT_RK2: k_step<EXACT, JT_RK2><<<g, kBlock, 0, st>>>(f, sb, k, dtpp, xin, xout, n, status); break;
            default: k_step<EXACT, JT_RK4><<<g, kBlock, 0, st>>>(f, sb, k, dtpp, xin, xout, n, status); break;
        }
        return cudaGetLastError();
    }

    template <bool EXACT, int STORE>
    static cudaError_t sample_s(const Desc& d, const Extra& x, const jt_blend& e, const float* pos,
                                float* out, int m, int32_t* status, cudaStream_t st) {
        const FT<EXACT, STORE> f = make<EXACT, STORE>(d, x);
        k_sample<<<grid_blocks(m), kBlock, 0, st>>>(f, e, pos, out, m, status);
        return cudaGetLastError();
    }

    // Run-time dispatch.  Exact arithmetic is offered for float32 storage;
    // 16-bit storage runs the compensated (FMA + Kahan) arithmetic.
    static int track(const Desc& d, const Extra& x, int storage, const jt_boundary& B,
                     const jt_track_params& P, cudaStream_t st) {
        const bool exact = P.arith == JT_ARITH_EXACT;
        cudaError_t err;
        if (storage == JT_STORE_F32) {
            err = exact ? track_s<true, JT_STORE_F32>(d, x, B, P, st) : track_s<false, JT_STORE_F32>(d, x, B, P, st);
        } else if (exact) {
            return set_error(JT_ERR_UNSUPPORTED, "exact arithmetic needs float32 snapshot storage");
        } else if (storage == JT_STORE_BF16) {
            err = track_s<false, JT_STORE_BF16>(d, x, B, P, st);
        } else {
            err = track_s<false, JT_STORE_F16>(d, x, B, P, st);
        }
        return cuda_status(err, "tracking kernel launch");
    }

    static int step(const Desc& d, const Extra& x, int storage, int arith, const StageBlends& sb,
                    int integ, StepConst k, const float* dtpp, const float* xin, float* xout, int n,
                    int32_t* status, cudaStream_t st) {
        const bool exact = arith == JT_ARITH_EXACT;
        cudaError_t err;
        if (storage == JT_STORE_F32) {
            err = exact ? step_s<true, JT_STORE_F32>(d, x, sb, integ, k, dtpp, xin, xout, n, status, st)
                        : step_s<false, JT_STORE_F32>(d, x, sb, integ, k, dtpp, xin, xout, n, status, st);
        } else if (exact) {
            return set_error(JT_ERR_UNSUPPORTED, "exact arithmetic needs float32 snapshot storage");
        } else if (storage == JT_STORE_BF16) {
            err = step_s<false, JT_STORE_BF16>(d, x, sb, integ, k, dtpp, xin, xout, n, status, st);
        } else {
            err = step_s<false, JT_STORE_F16>(d, x, sb, integ, k, dtpp, xin, xout, n, status, st);
        }
        return cuda_status(err, "integrator step launch");
    }

    static int sample(const Desc& d, const Extra& x, int storage, int arith, const jt_blend& e,
                      const float* pos, float* out, int m, int32_t* status, cudaStream_t st) {
        const bool exact = arith == JT_ARITH_EXACT;
        cudaError_t err;
        if (storage == JT_STORE_F32) {
            err = exact ? sample_s<true, JT_STORE_F32>(d, x, e, pos, out, m, status, st)
                        : sample_s<false, JT_STORE_F32>(d, x, e, pos, out, m, status, st);
        } else if (exact) {
            return set_error(JT_ERR_UNSUPPORTED, "exact arithmetic needs float32 snapshot storage");
        } else if (storage == JT_STORE_BF16) {
            err = sample_s<false, JT_STORE_BF16>(d, x, e, pos, out, m, status, st);
        } else {
            err = sample_s<false, JT_STORE_F16>(d, x, e, pos, out, m, status, st);
        }
        return cuda_status(err, "field sample launch");
    }
};

}  // namespace jt
