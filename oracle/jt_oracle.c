/*
 * jt_oracle.c -- CPU restatement of JAXTrace's tracking hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker of the GPU library:
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 * The product never links, calls or falls back to it.
 *
 * Two arithmetic modes:
 *   ORC_F32: the float32 operation order and rounding of the reference's
 *            NumPy path, one rounding per operation, no FMA contraction
 *            (build with -ffp-contract=off).  Bit-identical results to the
 *            reference are expected.
 *   ORC_F64: the same algorithm in float64 (snapshot data, times and dt
 *            taken as their float32 values), the "FP64 oracle" that error
 *            figures are measured against.
 *
 * Every routine names the reference lines it restates (paths inside the
 * JAXTrace project).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_F32 0
#define ORC_F64 1

enum { GRID_CLAMP = 0, GRID_ZERO = 1, GRID_NAN = 2, GRID_PERIODIC = 3 };
enum { EX_CONSTANT = 0, EX_LINEAR = 1, EX_ZERO = 2, EX_NAN = 3 };
enum { IN_EULER = 0, IN_RK2 = 1, IN_RK4 = 2 };
enum { BC_NONE = 0, BC_PERIODIC = 1, BC_REFLECTIVE = 2, BC_CLAMP = 3, BC_ABSORBING = 4 };
enum { FIELD_GRID = 1, FIELD_MESH = 2, FIELD_FEM = 4 };
enum { SEM_NUMPY = 0, SEM_JAX = 1 };

typedef struct {
    /* time series (time_series.py:82) */
    int n_snap;
    const float* snap_times;  /* (n_snap)                       */
    const float* data;        /* (n_snap, n_nodes, 3)           */
    int n_nodes;
    int extrapolation;        /* EX_*                           */
    int semantics;            /* SEM_NUMPY or SEM_JAX time blend */
    int kind;                 /* FIELD_GRID or FIELD_MESH       */
    /* grid (structured.py:65) */
    int nx, ny, nz, bounds_mode;
    const float* gx; const float* gy; const float* gz;
    /* mesh (octree_fem_interpolator_optimized.py:18) in the reference layout */
    const float* points;      /* (n_nodes,3) */
    const int32_t* conn;      /* (n_tets,4)  */
    int n_tets;
    const float* elem_bounds; /* (n_tets,2,3) */
    const float* nodes_min;   /* (K,3) */
    const float* nodes_max;   /* (K,3) */
    const int32_t* nodes_elements; /* (K,maxE) -1 padded */
    int max_elems;
    const int32_t* nodes_children; /* (K,8) */
    const uint8_t* nodes_is_leaf;  /* (K) */
    int max_depth;
    /* hash grid (fem_interpolator.py:18-143) in the reference layout */
    int fem_grid_size[3];
    float fem_grid_min[3];
    float fem_cell_size[3];            /* float32 copy used by the lookup */
    const int32_t* fem_cell_elements;  /* (cells, fem_max_per_cell) -1 padded */
    int fem_max_per_cell;
} orc_field;

typedef struct {
    int axis_kind[3];
    int absorbing_joint;
    float lo[3], hi[3];
    float outside_value;
    int inlet_axis;          /* -1: no inlet */
    int inlet_positive;
    int inlet_res[2];
    const float* lattice[2]; /* float32 linspace lattices of the two other axes */
} orc_boundary;

typedef struct {
    int precision;           /* ORC_F32 / ORC_F64 */
    int integrator;          /* IN_* */
    const float* step_times; /* (T) float32 linspace (tracker.py:347) */
    int n_times;
    double dt;               /* Python float dt (tracker.py:348-351) */
    int n_threads;
    int64_t fallback_count;  /* out: octree fallback lookups */
    int64_t wrapped_count;   /* out: periodic index == N events */
    uint64_t* cell_sig;      /* optional out (n), float64 mode, grid fields:
                                a hash of the sequence of cells every field
                                evaluation of the particle falls in (equal
                                for two runs that visit the same cells) */
    int32_t* reseed;         /* optional out (n,3): the last continuous-inlet
                                replacement of each particle -- its step and
                                the lattice indices it snapped to; -1 if none */
} orc_run;

/* ------------------------------------------------------------------------ */
/* NumPy float remainder (np.mod): fmod, then the sign of the divisor.     */
static float mod_f(float a, float b) {
    float m = fmodf(a, b);
    if (m != 0.0f) {
        if ((b < 0.0f) != (m < 0.0f)) m = m + b;
    } else {
        m = copysignf(0.0f, b);
    }
    return m;
}
static double mod_d(double a, double b) {
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0.0) != (m < 0.0)) m = m + b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}

/* ------------------------------------------------------------------------ */
/* Time blend.  Returns snapshot indices il, ir and weights w0, w1 such that
 * the value is w0*V[il] + w1*V[ir] (form 0), or V[il] + w1*(V[ir]-V[il])
 * (form 1), or V[ir] + w1*(V[ir]-V[il]) (form 2).                          */
typedef struct { int il, ir, form; float w0f, w1f; double w0d, w1d; } blend_t;

/* time_series.py:314-367, the NumPy path; t is the Python float value. */
static blend_t blend_numpy(const orc_field* F, double t) {
    blend_t b = {0, 0, 0, 1.0f, 0.0f, 1.0, 0.0};
    const float* ts = F->snap_times;
    const int T = F->n_snap;
    int ir = 0;
    while (ir < T && (double)ts[ir] <= t) ++ir;  /* searchsorted right, in float64 */
    int il = ir - 1 > 0 ? ir - 1 : 0;
    const float tf = (float)t;                    /* t < times[0]: t rounded to float32 */
    if (tf < ts[0] || tf > ts[T - 1]) {
        const int left = tf < ts[0];
        if (F->extrapolation == EX_LINEAR && T > 1) {
            /* alpha = (t - times[k]) / max(times[.]-times[.], 1e-12): float32 */
            const float d = left ? ts[1] - ts[0] : ts[T - 1] - ts[T - 2];
            const float dd = d > 1e-12f ? d : 1e-12f;
            const float num = tf - (left ? ts[0] : ts[T - 1]);
            const float alpha = num / dd;
            b.il = left ? 0 : T - 2; b.ir = left ? 1 : T - 1; b.form = left ? 1 : 2;
            b.w1f = alpha; b.w1d = (double)alpha;
            return b;
        }
        if (F->extrapolation == EX_ZERO) { b.w0f = 0; b.w0d = 0; return b; }
        if (F->extrapolation == EX_NAN) { b.w0f = NAN; b.w0d = NAN; b.w1f = NAN; b.w1d = NAN; return b; }
        b.il = b.ir = left ? 0 : T - 1;
        return b;
    }
    ir = ir < T - 1 ? ir : T - 1;
    il = il < 0 ? 0 : (il > T - 1 ? T - 1 : il);
    const double t0 = ts[il], t1 = ts[ir];
    const double dt = (t1 - t0) > 1e-12 ? (t1 - t0) : 1e-12;
    const double alpha = (t - t0) / dt;
    b.il = il; b.ir = ir;
    b.w0f = (float)(1.0 - alpha); b.w1f = (float)alpha;
    b.w0d = 1.0 - alpha; b.w1d = alpha;
    return b;
}

/* time_series.py:155-245, the JAX path (float32 throughout). */
static blend_t blend_jax(const orc_field* F, float t) {
    blend_t b = {0, 0, 0, 1.0f, 0.0f, 1.0, 0.0};
    const float* ts = F->snap_times;
    const int T = F->n_snap;
    int ir = 0;
    while (ir < T && ts[ir] <= t) ++ir;
    int il = ir - 1; il = il < 0 ? 0 : (il > T - 1 ? T - 1 : il);
    if (t < ts[0] || t > ts[T - 1]) {
        const int left = t < ts[0];
        if (F->extrapolation == EX_LINEAR && T > 1) {
            float d = left ? ts[1] - ts[0] : ts[T - 1] - ts[T - 2];
            d = d > 1e-12f ? d : 1e-12f;
            float alpha = (t - (left ? ts[0] : ts[T - 1])) / d;
            b.il = left ? 0 : T - 2; b.ir = left ? 1 : T - 1; b.form = left ? 1 : 2;
            b.w1f = alpha; b.w1d = alpha;
            return b;
        }
        if (F->extrapolation == EX_ZERO) { b.w0f = 0; b.w0d = 0; return b; }
        if (F->extrapolation == EX_NAN) { b.w0f = NAN; b.w0d = NAN; b.w1f = NAN; b.w1d = NAN; return b; }
        b.il = b.ir = left ? 0 : T - 1;
        return b;
    }
    const int irc = ir < T - 1 ? ir : T - 1;
    const float t0 = ts[il], t1 = ts[irc];
    float d = t1 - t0; d = d > 1e-12f ? d : 1e-12f;
    float alpha = (t - t0) / d;
    alpha = alpha < 0.0f ? 0.0f : (alpha > 1.0f ? 1.0f : alpha);
    b.il = il; b.ir = irc;
    b.w0f = 1.0f - alpha; b.w1f = alpha;
    b.w0d = 1.0 - (double)alpha; b.w1d = alpha;
    return b;
}

static void node_f(const orc_field* F, const blend_t* b, int node, float* v) {
    const float* A = F->data + ((size_t)b->il * F->n_nodes + node) * 3;
    const float* B = F->data + ((size_t)b->ir * F->n_nodes + node) * 3;
    for (int c = 0; c < 3; ++c) {
        if (b->form == 0) { float p = b->w0f * A[c]; float q = b->w1f * B[c]; v[c] = p + q; }
        else if (b->form == 1) { float d = B[c] - A[c]; float q = b->w1f * d; v[c] = A[c] + q; }
        else { float d = B[c] - A[c]; float q = b->w1f * d; v[c] = B[c] + q; }
    }
}
static void node_d(const orc_field* F, const blend_t* b, int node, double* v) {
    const float* A = F->data + ((size_t)b->il * F->n_nodes + node) * 3;
    const float* B = F->data + ((size_t)b->ir * F->n_nodes + node) * 3;
    for (int c = 0; c < 3; ++c) {
        if (b->form == 0) v[c] = b->w0d * A[c] + b->w1d * B[c];
        else if (b->form == 1) v[c] = A[c] + b->w1d * ((double)B[c] - A[c]);
        else v[c] = B[c] + b->w1d * ((double)B[c] - A[c]);
    }
}

/* ------------------------------------------------------------------------ */
/* Trilinear sampler, structured.py:284-349 (NumPy path).                  */
static void grid_axis_f(const orc_field* F, int a, float x, int* i0, int* i1, float* w, int* valid, int64_t* wrapped) {
    const float* g = a == 0 ? F->gx : (a == 1 ? F->gy : F->gz);
    const int n = a == 0 ? F->nx : (a == 1 ? F->ny : F->nz);
    const float org = g[0];
    const float d = n > 1 ? (float)(g[1] - g[0]) : 1.0f;
    float f = (x - org) / d;
    if (F->bounds_mode == GRID_PERIODIC) {
        const int nn = n > 1 ? n : 1;
        f = mod_f(f, (float)nn);
        const float fl = floorf(f);
        int i = (int)fl;
        *w = f - fl;
        if (i >= nn) { i -= nn; if (wrapped) (*wrapped)++; }
        if (i < 0) i = 0;
        *i0 = i; *i1 = (i + 1) % nn; *valid = 1;
    } else {
        const double vhi_d = (double)org + (double)(n - 1) * (double)d;
        const float vhi = (float)vhi_d;
        *valid = (x >= org) && (x <= vhi);
        const float hi = (float)(n > 1 ? n - 1 : 0);
        if (f < 0.0f) f = 0.0f;
        if (f > hi) f = hi;
        const float fl = floorf(f);
        int i = (int)fl;
        if (i < 0) i = 0;
        if (i > n - 1) i = n - 1;
        *w = f - fl;
        *i0 = i; *i1 = (i + 1 > n - 1) ? n - 1 : i + 1;
    }
}

static void grid_axis_d(const orc_field* F, int a, double x, int* i0, int* i1, double* w, int* valid) {
    const float* g = a == 0 ? F->gx : (a == 1 ? F->gy : F->gz);
    const int n = a == 0 ? F->nx : (a == 1 ? F->ny : F->nz);
    const double org = g[0];
    const double d = n > 1 ? (double)(float)(g[1] - g[0]) : 1.0;
    double f = (x - org) / d;
    if (F->bounds_mode == GRID_PERIODIC) {
        const int nn = n > 1 ? n : 1;
        f = mod_d(f, (double)nn);
        const double fl = floor(f);
        int i = (int)fl;
        *w = f - fl;
        if (i >= nn) i -= nn;
        if (i < 0) i = 0;
        *i0 = i; *i1 = (i + 1) % nn; *valid = 1;
    } else {
        *valid = (x >= org) && (x <= org + (double)(n - 1) * d);
        const double hi = (double)(n > 1 ? n - 1 : 0);
        if (f < 0.0) f = 0.0;
        if (f > hi) f = hi;
        const double fl = floor(f);
        int i = (int)fl;
        if (i < 0) i = 0;
        if (i > n - 1) i = n - 1;
        *w = f - fl;
        *i0 = i; *i1 = (i + 1 > n - 1) ? n - 1 : i + 1;
    }
}

static void grid_eval_f(const orc_field* F, const blend_t* b, const float* p, float* out, int64_t* wrapped) {
    int i0, i1, j0, j1, k0, k1, vx, vy, vz;
    float wx, wy, wz;
    grid_axis_f(F, 0, p[0], &i0, &i1, &wx, &vx, wrapped);
    grid_axis_f(F, 1, p[1], &j0, &j1, &wy, &vy, wrapped);
    grid_axis_f(F, 2, p[2], &k0, &k1, &wz, &vz, wrapped);
    const int ny = F->ny, nz = F->nz;
#define NID(i, j, k) (((i) * ny + (j)) * nz + (k))
    float v000[3], v100[3], v010[3], v110[3], v001[3], v101[3], v011[3], v111[3];
    node_f(F, b, NID(i0, j0, k0), v000); node_f(F, b, NID(i1, j0, k0), v100);
    node_f(F, b, NID(i0, j1, k0), v010); node_f(F, b, NID(i1, j1, k0), v110);
    node_f(F, b, NID(i0, j0, k1), v001); node_f(F, b, NID(i1, j0, k1), v101);
    node_f(F, b, NID(i0, j1, k1), v011); node_f(F, b, NID(i1, j1, k1), v111);
#undef NID
    const float ox = 1.0f - wx, oy = 1.0f - wy, oz = 1.0f - wz;
    for (int c = 0; c < 3; ++c) {
        float c00 = v000[c] * ox; c00 = c00 + v100[c] * wx;
        float c10 = v010[c] * ox; c10 = c10 + v110[c] * wx;
        float c01 = v001[c] * ox; c01 = c01 + v101[c] * wx;
        float c11 = v011[c] * ox; c11 = c11 + v111[c] * wx;
        float c0 = c00 * oy; c0 = c0 + c10 * wy;
        float c1 = c01 * oy; c1 = c1 + c11 * wy;
        float r = c0 * oz; r = r + c1 * wz;
        out[c] = r;
    }
    if ((F->bounds_mode == GRID_ZERO || F->bounds_mode == GRID_NAN) && !(vx && vy && vz)) {
        const float o = F->bounds_mode == GRID_ZERO ? 0.0f : NAN;
        out[0] = out[1] = out[2] = o;
    }
}

static void grid_eval_d(const orc_field* F, const blend_t* b, const double* p, double* out) {
    int i0, i1, j0, j1, k0, k1, vx, vy, vz;
    double wx, wy, wz;
    grid_axis_d(F, 0, p[0], &i0, &i1, &wx, &vx);
    grid_axis_d(F, 1, p[1], &j0, &j1, &wy, &vy);
    grid_axis_d(F, 2, p[2], &k0, &k1, &wz, &vz);
    const int ny = F->ny, nz = F->nz;
#define NID(i, j, k) (((i) * ny + (j)) * nz + (k))
    double v[8][3];
    node_d(F, b, NID(i0, j0, k0), v[0]); node_d(F, b, NID(i1, j0, k0), v[1]);
    node_d(F, b, NID(i0, j1, k0), v[2]); node_d(F, b, NID(i1, j1, k0), v[3]);
    node_d(F, b, NID(i0, j0, k1), v[4]); node_d(F, b, NID(i1, j0, k1), v[5]);
    node_d(F, b, NID(i0, j1, k1), v[6]); node_d(F, b, NID(i1, j1, k1), v[7]);
#undef NID
    for (int c = 0; c < 3; ++c) {
        double c00 = v[0][c] * (1 - wx) + v[1][c] * wx, c10 = v[2][c] * (1 - wx) + v[3][c] * wx;
        double c01 = v[4][c] * (1 - wx) + v[5][c] * wx, c11 = v[6][c] * (1 - wx) + v[7][c] * wx;
        double c0 = c00 * (1 - wy) + c10 * wy, c1 = c01 * (1 - wy) + c11 * wy;
        out[c] = c0 * (1 - wz) + c1 * wz;
    }
    if ((F->bounds_mode == GRID_ZERO || F->bounds_mode == GRID_NAN) && !(vx && vy && vz)) {
        const double o = F->bounds_mode == GRID_ZERO ? 0.0 : NAN;
        out[0] = out[1] = out[2] = o;
    }
}

/* ------------------------------------------------------------------------ */
/* Octree lookup + P1, octree_fem_interpolator_optimized.py:218-380.        */
/* jnp.linalg.det of a 3x3 matrix: six triple products summed in order.    */
static float det3_f(const float* c0, const float* c1, const float* c2) {
    const float a00 = c0[0], a01 = c1[0], a02 = c2[0];
    const float a10 = c0[1], a11 = c1[1], a12 = c2[1];
    const float a20 = c0[2], a21 = c1[2], a22 = c2[2];
    float t1 = a00 * a11; t1 = t1 * a22;
    float t2 = a01 * a12; t2 = t2 * a20;
    float t3 = a02 * a10; t3 = t3 * a21;
    float t4 = a02 * a11; t4 = t4 * a20;
    float t5 = a00 * a12; t5 = t5 * a21;
    float t6 = a01 * a10; t6 = t6 * a22;
    float s = t1 + t2; s = s + t3; s = s - t4; s = s - t5; s = s - t6;
    return s;
}
static double det3_d(const double* c0, const double* c1, const double* c2) {
    return c0[0] * c1[1] * c2[2] + c1[0] * c2[1] * c0[2] + c2[0] * c0[1] * c1[2] - c2[0] * c1[1] * c0[2] -
           c0[0] * c2[1] * c1[2] - c1[0] * c0[1] * c2[2];
}

static int octree_leaf(const orc_field* F, double qx, double qy, double qz, int f32) {
    int node = 0;
    for (int d = 0; d < F->max_depth; ++d) {
        if (F->nodes_is_leaf[node]) break;
        float c[3];
        for (int a = 0; a < 3; ++a) {
            float s = F->nodes_min[3 * node + a] + F->nodes_max[3 * node + a];
            c[a] = s / 2.0f;
        }
        int oct = 0;
        if (f32) {
            if ((float)qx >= c[0]) oct += 1;
            if ((float)qy >= c[1]) oct += 2;
            if ((float)qz >= c[2]) oct += 4;
        } else {
            if (qx >= c[0]) oct += 1;
            if (qy >= c[1]) oct += 2;
            if (qz >= c[2]) oct += 4;
        }
        int ch = F->nodes_children[8 * node + oct];
        if (ch < 0) break;
        node = ch;
    }
    return node;
}

static void mesh_eval_f(const orc_field* F, const blend_t* b, const float* q, float* out, int64_t* fb) {
    const int node = octree_leaf(F, q[0], q[1], q[2], 1);
    const int32_t* cand = F->nodes_elements + (size_t)node * F->max_elems;
    for (int s = 0; s < F->max_elems; ++s) {
        const int e = cand[s];
        if (e < 0) continue;
        const float* eb = F->elem_bounds + 6 * (size_t)e;
        if (!(q[0] >= eb[0] && q[1] >= eb[1] && q[2] >= eb[2] && q[0] <= eb[3] && q[1] <= eb[4] && q[2] <= eb[5]))
            continue;
        const int32_t* cv = F->conn + 4 * (size_t)e;
        const float* v0 = F->points + 3 * (size_t)cv[0];
        float v0p[3], v01[3], v02[3], v03[3];
        for (int a = 0; a < 3; ++a) {
            v0p[a] = q[a] - v0[a];
            v01[a] = F->points[3 * (size_t)cv[1] + a] - v0[a];
            v02[a] = F->points[3 * (size_t)cv[2] + a] - v0[a];
            v03[a] = F->points[3 * (size_t)cv[3] + a] - v0[a];
        }
        float det = det3_f(v01, v02, v03);
        if (fabsf(det) < 1e-10f) det = 1.0f;
        const float b1 = det3_f(v0p, v02, v03) / det;
        const float b2 = det3_f(v01, v0p, v03) / det;
        const float b3 = det3_f(v01, v02, v0p) / det;
        float b0 = 1.0f - b1; b0 = b0 - b2; b0 = b0 - b3;
        const float lo = -1e-6f, hi = 0.999999f;
        if (!(b0 >= lo && b1 >= lo && b2 >= lo && b3 >= lo && b0 <= hi && b1 <= hi && b2 <= hi && b3 <= hi)) continue;
        float n[4][3];
        for (int k = 0; k < 4; ++k) node_f(F, b, cv[k], n[k]);
        for (int c = 0; c < 3; ++c) {
            float r = b0 * n[0][c];
            r = r + b1 * n[1][c];
            r = r + b2 * n[2][c];
            r = r + b3 * n[3][c];
            out[c] = r;
        }
        return;
    }
    if (fb) (*fb)++;
    int first = cand[0];
    if (first < 0) first += F->n_tets;
    const int32_t* cv = F->conn + 4 * (size_t)first;
    int best = cv[0];
    float bd = 0.0f;
    for (int k = 0; k < 4; ++k) {
        const float* p = F->points + 3 * (size_t)cv[k];
        float dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
        float d = dx * dx; d = d + dy * dy; d = d + dz * dz;
        if (k == 0 || d < bd) { bd = d; best = cv[k]; }
    }
    node_f(F, b, best, out);
}

static void mesh_eval_d(const orc_field* F, const blend_t* b, const double* q, double* out, int64_t* fb) {
    const int node = octree_leaf(F, q[0], q[1], q[2], 0);
    const int32_t* cand = F->nodes_elements + (size_t)node * F->max_elems;
    for (int s = 0; s < F->max_elems; ++s) {
        const int e = cand[s];
        if (e < 0) continue;
        const float* eb = F->elem_bounds + 6 * (size_t)e;
        if (!(q[0] >= eb[0] && q[1] >= eb[1] && q[2] >= eb[2] && q[0] <= eb[3] && q[1] <= eb[4] && q[2] <= eb[5]))
            continue;
        const int32_t* cv = F->conn + 4 * (size_t)e;
        double v0p[3], v01[3], v02[3], v03[3];
        for (int a = 0; a < 3; ++a) {
            const double v0 = F->points[3 * (size_t)cv[0] + a];
            v0p[a] = q[a] - v0;
            v01[a] = F->points[3 * (size_t)cv[1] + a] - v0;
            v02[a] = F->points[3 * (size_t)cv[2] + a] - v0;
            v03[a] = F->points[3 * (size_t)cv[3] + a] - v0;
        }
        double det = det3_d(v01, v02, v03);
        if (fabs(det) < 1e-10) det = 1.0;
        const double b1 = det3_d(v0p, v02, v03) / det, b2 = det3_d(v01, v0p, v03) / det;
        const double b3 = det3_d(v01, v02, v0p) / det, b0 = 1.0 - b1 - b2 - b3;
        const double lo = -1e-6, hi = 1.0 - 1e-6;
        if (!(b0 >= lo && b1 >= lo && b2 >= lo && b3 >= lo && b0 <= hi && b1 <= hi && b2 <= hi && b3 <= hi)) continue;
        double n[4][3];
        for (int k = 0; k < 4; ++k) node_d(F, b, cv[k], n[k]);
        for (int c = 0; c < 3; ++c) out[c] = b0 * n[0][c] + b1 * n[1][c] + b2 * n[2][c] + b3 * n[3][c];
        return;
    }
    if (fb) (*fb)++;
    int first = cand[0];
    if (first < 0) first += F->n_tets;
    const int32_t* cv = F->conn + 4 * (size_t)first;
    int best = cv[0];
    double bd = 0.0;
    for (int k = 0; k < 4; ++k) {
        const float* p = F->points + 3 * (size_t)cv[k];
        double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
        double d = dx * dx + dy * dy + dz * dz;
        if (k == 0 || d < bd) { bd = d; best = cv[k]; }
    }
    node_d(F, b, best, out);
}

/* ------------------------------------------------------------------------ */
/* Hash-grid lookup + P1, fem_interpolator.py:146-328.                      */
static int nearest_node(const orc_field* F, const float* q);

/* floor(v).astype(int32) then clip(0, n-1), with XLA's saturating float ->
 * int conversion (NaN -> 0). */
static int fem_cell_coord(float v, int n) {
    float f = floorf(v);
    if (f != f) return 0;
    if (f < 0.0f) return 0;
    if (f > (float)(n - 1)) return n - 1;
    return (int)f;
}

static int fem_cell(const orc_field* F, const float* q) {
    int c[3];
    for (int a = 0; a < 3; ++a) {
        const float u = q[a] - F->fem_grid_min[a];
        c[a] = fem_cell_coord(u / F->fem_cell_size[a], F->fem_grid_size[a]);
    }
    return (c[0] * F->fem_grid_size[1] + c[1]) * F->fem_grid_size[2] + c[2];
}

static void fem_eval_f(const orc_field* F, const blend_t* b, const float* q, float* out, int64_t* fb) {
    const int32_t* cand = F->fem_cell_elements + (size_t)fem_cell(F, q) * F->fem_max_per_cell;
    /* lax.scan over the padded row keeps the first element found */
    for (int s = 0; s < F->fem_max_per_cell; ++s) {
        const int e = cand[s];
        if (e < 0) continue;
        const float* eb = F->elem_bounds + 6 * (size_t)e;
        if (!(q[0] >= eb[0] && q[1] >= eb[1] && q[2] >= eb[2] && q[0] <= eb[3] && q[1] <= eb[4] && q[2] <= eb[5]))
            continue;
        const int32_t* cv = F->conn + 4 * (size_t)e;
        const float* v0 = F->points + 3 * (size_t)cv[0];
        float v0p[3], v01[3], v02[3], v03[3];
        for (int a = 0; a < 3; ++a) {
            v0p[a] = q[a] - v0[a];
            v01[a] = F->points[3 * (size_t)cv[1] + a] - v0[a];
            v02[a] = F->points[3 * (size_t)cv[2] + a] - v0[a];
            v03[a] = F->points[3 * (size_t)cv[3] + a] - v0[a];
        }
        float det = det3_f(v01, v02, v03);
        if (fabsf(det) < 1e-10f) det = 1.0f;
        const float b1 = det3_f(v0p, v02, v03) / det;
        const float b2 = det3_f(v01, v0p, v03) / det;
        const float b3 = det3_f(v01, v02, v0p) / det;
        float b0 = 1.0f - b1; b0 = b0 - b2; b0 = b0 - b3;
        const float lo = -1e-6f, hi = 0.999999f;
        if (!(b0 >= lo && b1 >= lo && b2 >= lo && b3 >= lo && b0 <= hi && b1 <= hi && b2 <= hi && b3 <= hi)) continue;
        float n[4][3];
        for (int k = 0; k < 4; ++k) node_f(F, b, cv[k], n[k]);
        for (int c = 0; c < 3; ++c) {
            float r = b0 * n[0][c];
            r = r + b1 * n[1][c];
            r = r + b2 * n[2][c];
            r = r + b3 * n[3][c];
            out[c] = r;
        }
        return;
    }
    /* not found: the nearest node of the whole mesh (fem_interpolator.py:311-316) */
    if (fb) (*fb)++;
    node_f(F, b, nearest_node(F, q), out);
}

static void fem_eval_d(const orc_field* F, const blend_t* b, const double* q, double* out, int64_t* fb) {
    const float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
    const int32_t* cand = F->fem_cell_elements + (size_t)fem_cell(F, qf) * F->fem_max_per_cell;
    for (int s = 0; s < F->fem_max_per_cell; ++s) {
        const int e = cand[s];
        if (e < 0) continue;
        const float* eb = F->elem_bounds + 6 * (size_t)e;
        if (!(q[0] >= eb[0] && q[1] >= eb[1] && q[2] >= eb[2] && q[0] <= eb[3] && q[1] <= eb[4] && q[2] <= eb[5]))
            continue;
        const int32_t* cv = F->conn + 4 * (size_t)e;
        double v0p[3], v01[3], v02[3], v03[3];
        for (int a = 0; a < 3; ++a) {
            const double v0 = F->points[3 * (size_t)cv[0] + a];
            v0p[a] = q[a] - v0;
            v01[a] = F->points[3 * (size_t)cv[1] + a] - v0;
            v02[a] = F->points[3 * (size_t)cv[2] + a] - v0;
            v03[a] = F->points[3 * (size_t)cv[3] + a] - v0;
        }
        double det = det3_d(v01, v02, v03);
        if (fabs(det) < 1e-10) det = 1.0;
        const double b1 = det3_d(v0p, v02, v03) / det, b2 = det3_d(v01, v0p, v03) / det;
        const double b3 = det3_d(v01, v02, v0p) / det, b0 = 1.0 - b1 - b2 - b3;
        const double lo = -1e-6, hi = 1.0 - 1e-6;
        if (!(b0 >= lo && b1 >= lo && b2 >= lo && b3 >= lo && b0 <= hi && b1 <= hi && b2 <= hi && b3 <= hi)) continue;
        double n[4][3];
        for (int k = 0; k < 4; ++k) node_d(F, b, cv[k], n[k]);
        for (int c = 0; c < 3; ++c) out[c] = b0 * n[0][c] + b1 * n[1][c] + b2 * n[2][c] + b3 * n[3][c];
        return;
    }
    if (fb) (*fb)++;
    node_d(F, b, nearest_node(F, qf), out);
}

/* ------------------------------------------------------------------------ */
/* Boundaries, boundary.py:101-210, :377-438, :1517-1599.                  */
static float bc_axis_f(int kind, float x, float lo, float hi, float outside) {
    float width = hi - lo; width = width > 0.0f ? width : 0.0f;
    const float ws = width > 0.0f ? width : 1.0f;
    switch (kind) {
        case BC_PERIODIC: return lo + mod_f(x - lo, ws);
        case BC_REFLECTIVE: {
            float y = mod_f(x - lo, 2.0f * ws);
            float yr = (y <= width) ? y : (2.0f * width - y);
            return lo + yr;
        }
        case BC_CLAMP: x = x < lo ? lo : x; x = x > hi ? hi : x; return x;
        case BC_ABSORBING: return (x < lo || x > hi) ? outside : x;
        default: return x;
    }
}
static double bc_axis_d(int kind, double x, double lo, double hi, double outside) {
    double width = hi - lo; width = width > 0.0 ? width : 0.0;
    const double ws = width > 0.0 ? width : 1.0;
    switch (kind) {
        case BC_PERIODIC: return lo + mod_d(x - lo, ws);
        case BC_REFLECTIVE: {
            double y = mod_d(x - lo, 2.0 * ws);
            return lo + ((y <= width) ? y : (2.0 * width - y));
        }
        case BC_CLAMP: x = x < lo ? lo : x; x = x > hi ? hi : x; return x;
        case BC_ABSORBING: return (x < lo || x > hi) ? outside : x;
        default: return x;
    }
}

/* argmin |coords - c| over the float32 lattice, first index on ties (boundary.py:1309) */
static int lattice_index_f(int res, float c, const float* lat) {
    int best = 0;
    float bd = fabsf(lat[0] - c);
    for (int j = 1; j < res; ++j) {
        const float d = fabsf(lat[j] - c);
        if (d < bd) { bd = d; best = j; }
    }
    return best;
}

/* ev (may be NULL): set to the snapped lattice indices when the inlet
 * replaced the particle in this call */
static void boundary_f(const orc_boundary* B, const float* lat0, const float* lat1, float* r, int* ev) {
    if (B->inlet_axis >= 0) {
        const int a = B->inlet_axis, o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
        const float amin = B->lo[a], amax = B->hi[a];
        const int exited = B->inlet_positive ? r[a] > amax : r[a] < amin;
        if (exited) {
            const int j0 = lattice_index_f(B->inlet_res[0], r[o0], lat0);
            const int j1 = lattice_index_f(B->inlet_res[1], r[o1], lat1);
            r[a] = B->inlet_positive ? amin : amax;
            r[o0] = lat0[j0]; r[o1] = lat1[j1];
            if (ev) { ev[0] = j0; ev[1] = j1; }
        }
        if (B->inlet_positive) {
            if (r[a] < amin) { float w = amax - amin; float s = 0.001f * w; r[a] = amin + s; }
        } else {
            if (r[a] > amax) { float w = amax - amin; float s = 0.001f * w; r[a] = amax - s; }
        }
        const int os[2] = {o0, o1};
        for (int q = 0; q < 2; ++q) {
            const int o = os[q];
            if (r[o] < B->lo[o]) r[o] = 2.0f * B->lo[o] - r[o];
            else if (r[o] > B->hi[o]) r[o] = 2.0f * B->hi[o] - r[o];
        }
        return;
    }
    if (B->absorbing_joint) {
        int out = 0;
        for (int a = 0; a < 3; ++a) out |= (r[a] < B->lo[a]) || (r[a] > B->hi[a]);
        if (out) r[0] = r[1] = r[2] = B->outside_value;
        return;
    }
    for (int a = 0; a < 3; ++a) r[a] = bc_axis_f(B->axis_kind[a], r[a], B->lo[a], B->hi[a], B->outside_value);
}

static void boundary_d(const orc_boundary* B, const float* lat0, const float* lat1, double* r, int* ev) {
    if (B->inlet_axis >= 0) {
        const int a = B->inlet_axis, o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
        const double amin = B->lo[a], amax = B->hi[a];
        const int exited = B->inlet_positive ? r[a] > amax : r[a] < amin;
        if (exited) {
            const int res[2] = {B->inlet_res[0], B->inlet_res[1]};
            const float* lats[2] = {lat0, lat1};
            const int os[2] = {o0, o1};
            double g[2];
            for (int q = 0; q < 2; ++q) {
                int best = 0;
                double bd = fabs(lats[q][0] - r[os[q]]);
                for (int j = 1; j < res[q]; ++j) {
                    const double d = fabs(lats[q][j] - r[os[q]]);
                    if (d < bd) { bd = d; best = j; }
                }
                g[q] = lats[q][best];
                if (ev) ev[q] = best;
            }
            r[a] = B->inlet_positive ? amin : amax;
            r[o0] = g[0]; r[o1] = g[1];
        }
        if (B->inlet_positive) { if (r[a] < amin) r[a] = amin + 0.001 * (amax - amin); }
        else { if (r[a] > amax) r[a] = amax - 0.001 * (amax - amin); }
        const int os[2] = {o0, o1};
        for (int q = 0; q < 2; ++q) {
            const int o = os[q];
            if (r[o] < B->lo[o]) r[o] = 2.0 * B->lo[o] - r[o];
            else if (r[o] > B->hi[o]) r[o] = 2.0 * B->hi[o] - r[o];
        }
        return;
    }
    if (B->absorbing_joint) {
        int out = 0;
        for (int a = 0; a < 3; ++a) out |= (r[a] < B->lo[a]) || (r[a] > B->hi[a]);
        if (out) r[0] = r[1] = r[2] = B->outside_value;
        return;
    }
    for (int a = 0; a < 3; ++a) r[a] = bc_axis_d(B->axis_kind[a], r[a], B->lo[a], B->hi[a], B->outside_value);
}

/* ------------------------------------------------------------------------ */
/* Field call at a stage time.  tf: the time as the integrator passes it.   */
typedef struct { double t; int is_f32; } stime;

static blend_t blend_at(const orc_field* F, stime s) {
    if (F->semantics == SEM_JAX) return blend_jax(F, (float)s.t);
    return blend_numpy(F, s.t);
}

/* Nearest node by brute force: argmin over nodes of the float32
 * sum((q - p)^2), first index on ties (time_series.py:249-259). */
static int nearest_node(const orc_field* F, const float* q) {
    int best = 0;
    float bd = 0.0f;
    for (int i = 0; i < F->n_nodes; ++i) {
        const float* p = F->points + 3 * (size_t)i;
        float dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
        float d = dx * dx; d = d + dy * dy; d = d + dz * dz;
        if (i == 0 || d < bd) { bd = d; best = i; }
    }
    return best;
}

static void field_f(const orc_field* F, stime s, const float* p, float* v, int64_t* fb, int64_t* wr) {
    const blend_t b = blend_at(F, s);
    if (F->kind == FIELD_GRID) grid_eval_f(F, &b, p, v, wr);
    else if (F->kind == FIELD_MESH) mesh_eval_f(F, &b, p, v, fb);
    else if (F->kind == FIELD_FEM) fem_eval_f(F, &b, p, v, fb);
    else node_f(F, &b, nearest_node(F, p), v);
}
static void field_d(const orc_field* F, stime s, const double* p, double* v, int64_t* fb) {
    blend_t b;
    if (F->semantics == SEM_JAX) b = blend_jax(F, (float)s.t);
    else b = blend_numpy(F, s.t);
    if (F->kind == FIELD_GRID) grid_eval_d(F, &b, p, v);
    else if (F->kind == FIELD_MESH) mesh_eval_d(F, &b, p, v, fb);
    else if (F->kind == FIELD_FEM) fem_eval_d(F, &b, p, v, fb);
    else {
        const float pf[3] = {(float)p[0], (float)p[1], (float)p[2]};
        node_d(F, &b, nearest_node(F, pf), v);
    }
}

/* All node values at one time: TimeSeriesField.sample_at_time (time_series.py:306). */
int orc_blend_nodes(const orc_field* F, double t, int t_is_f32, float* out) {
    const stime s = {t, t_is_f32};
    const blend_t b = blend_at(F, s);
    for (int i = 0; i < F->n_nodes; ++i) node_f(F, &b, i, out + 3 * (size_t)i);
    return 0;
}

/* One step; rk4.py:82-106, rk2.py:283-309, euler.py:146-157. */
static void step_f(const orc_field* F, const orc_run* R, int s, float* x, int64_t* fb, int64_t* wr) {
    const float tj = R->step_times[s];
    const float dtj = (float)R->dt;
    float k1[3], k2[3], k3[3], k4[3], xs[3];
    if (R->integrator == IN_RK4) {
        const float dth = 0.5f * dtj;
        const float th = tj + dth, tfull = tj + dtj;
        const stime s0 = {tj, 1}, sh = {th, 1}, sf = {tfull, 1};
        field_f(F, s0, x, k1, fb, wr);
        for (int a = 0; a < 3; ++a) { float q = dth * k1[a]; xs[a] = x[a] + q; }
        field_f(F, sh, xs, k2, fb, wr);
        for (int a = 0; a < 3; ++a) { float q = dth * k2[a]; xs[a] = x[a] + q; }
        field_f(F, sh, xs, k3, fb, wr);
        for (int a = 0; a < 3; ++a) { float q = dtj * k3[a]; xs[a] = x[a] + q; }
        field_f(F, sf, xs, k4, fb, wr);
        const float dt6 = dtj / 6.0f;
        for (int a = 0; a < 3; ++a) {
            float sm = k1[a] + 2.0f * k2[a];
            sm = sm + 2.0f * k3[a];
            sm = sm + k4[a];
            float q = dt6 * sm;
            x[a] = x[a] + q;
        }
    } else if (R->integrator == IN_RK2) {
        const float dth = dtj * 0.5f;
        const double tmid = (double)tj + (double)dth;   /* Python float sum */
        const stime s0 = {tj, 0}, sm = {tmid, 0};
        field_f(F, s0, x, k1, fb, wr);
        for (int a = 0; a < 3; ++a) { float q = dth * k1[a]; xs[a] = x[a] + q; }
        field_f(F, sm, xs, k2, fb, wr);
        for (int a = 0; a < 3; ++a) { float q = dtj * k2[a]; x[a] = x[a] + q; }
    } else {
        const stime s0 = {tj, 0};
        field_f(F, s0, x, k1, fb, wr);
        for (int a = 0; a < 3; ++a) { float q = dtj * k1[a]; x[a] = x[a] + q; }
    }
}

/* Fold the grid cell of p into a running signature (grid fields only). */
static void cell_sig_d(const orc_field* F, const double* p, uint64_t* sig) {
    if (sig == NULL || F->kind != FIELD_GRID) return;
    int i0, i1, j0, j1, k0, k1, v;
    double w;
    grid_axis_d(F, 0, p[0], &i0, &i1, &w, &v);
    grid_axis_d(F, 1, p[1], &j0, &j1, &w, &v);
    grid_axis_d(F, 2, p[2], &k0, &k1, &w, &v);
    const uint64_t c = ((uint64_t)(uint32_t)i0 << 42) ^ ((uint64_t)(uint32_t)j0 << 21) ^ (uint64_t)(uint32_t)k0;
    *sig ^= c + 0x9e3779b97f4a7c15ULL + (*sig << 6) + (*sig >> 2);
}

static void step_d(const orc_field* F, const orc_run* R, int s, double* x, int64_t* fb, uint64_t* sig) {
    const double tj = R->step_times[s];
    const double dt = (double)(float)R->dt;
    double k1[3], k2[3], k3[3], k4[3], xs[3];
    if (R->integrator == IN_RK4) {
        const stime s0 = {tj, 1}, sh = {tj + 0.5 * dt, 1}, sf = {tj + dt, 1};
        cell_sig_d(F, x, sig);
        field_d(F, s0, x, k1, fb);
        for (int a = 0; a < 3; ++a) xs[a] = x[a] + 0.5 * dt * k1[a];
        cell_sig_d(F, xs, sig);
        field_d(F, sh, xs, k2, fb);
        for (int a = 0; a < 3; ++a) xs[a] = x[a] + 0.5 * dt * k2[a];
        cell_sig_d(F, xs, sig);
        field_d(F, sh, xs, k3, fb);
        for (int a = 0; a < 3; ++a) xs[a] = x[a] + dt * k3[a];
        cell_sig_d(F, xs, sig);
        field_d(F, sf, xs, k4, fb);
        for (int a = 0; a < 3; ++a) x[a] += dt / 6.0 * (k1[a] + 2.0 * k2[a] + 2.0 * k3[a] + k4[a]);
    } else if (R->integrator == IN_RK2) {
        const stime s0 = {tj, 0}, sm = {tj + 0.5 * dt, 0};
        cell_sig_d(F, x, sig);
        field_d(F, s0, x, k1, fb);
        for (int a = 0; a < 3; ++a) xs[a] = x[a] + 0.5 * dt * k1[a];
        cell_sig_d(F, xs, sig);
        field_d(F, sm, xs, k2, fb);
        for (int a = 0; a < 3; ++a) x[a] += dt * k2[a];
    } else {
        const stime s0 = {tj, 0};
        cell_sig_d(F, x, sig);
        field_d(F, s0, x, k1, fb);
        for (int a = 0; a < 3; ++a) x[a] += dt * k1[a];
    }
}

/* Track n particles through all steps (tracker.py:441-446).  x0: (n,3)
 * float32.  out_f32 (n,3) in ORC_F32 mode or out_f64 (n,3) in ORC_F64 mode.
 * traj (T,n,3) float32 may be NULL; when given every step is recorded. */
/* x0_f64 (optional, float64 mode): float64 initial positions, so finite
 * differences can use steps below float32 resolution. */
int orc_track(const orc_field* F, const orc_boundary* B, orc_run* R, int n, const float* x0,
              float* out_f32, double* out_f64, float* traj, const double* x0_f64) {
    if (F == NULL || B == NULL || R == NULL || n < 0 || (x0 == NULL && x0_f64 == NULL)) return -1;
    if (x0 == NULL && R->precision == ORC_F32) return -1;
    const float* lat[2] = {B->lattice[0], B->lattice[1]};
    if (B->inlet_axis >= 0 && (lat[0] == NULL || lat[1] == NULL)) return -1;
    int64_t fb = 0, wr = 0;
    const int T = R->n_times;
#ifdef _OPENMP
    if (R->n_threads > 0) omp_set_num_threads(R->n_threads);
#endif
#pragma omp parallel for schedule(static) reduction(+ : fb, wr)
    for (int i = 0; i < n; ++i) {
        int32_t last[3] = {-1, -1, -1};
        if (R->precision == ORC_F32) {
            float x[3] = {x0[3 * (size_t)i], x0[3 * (size_t)i + 1], x0[3 * (size_t)i + 2]};
            if (traj) memcpy(traj + 3 * (size_t)i, x, sizeof x);
            for (int s = 0; s + 1 < T; ++s) {
                int ev[2] = {-1, -1};
                step_f(F, R, s, x, &fb, &wr);
                boundary_f(B, lat[0], lat[1], x, ev);
                if (ev[0] >= 0) { last[0] = s; last[1] = ev[0]; last[2] = ev[1]; }
                if (traj) memcpy(traj + ((size_t)(s + 1) * n + i) * 3, x, sizeof x);
            }
            memcpy(out_f32 + 3 * (size_t)i, x, sizeof x);
        } else {
            double x[3];
            for (int a = 0; a < 3; ++a) x[a] = x0_f64 ? x0_f64[3 * (size_t)i + a] : (double)x0[3 * (size_t)i + a];
            uint64_t sig = 0;
            for (int s = 0; s + 1 < T; ++s) {
                int ev[2] = {-1, -1};
                step_d(F, R, s, x, &fb, R->cell_sig ? &sig : NULL);
                boundary_d(B, lat[0], lat[1], x, ev);
                if (ev[0] >= 0) { last[0] = s; last[1] = ev[0]; last[2] = ev[1]; }
            }
            out_f64[3 * (size_t)i] = x[0]; out_f64[3 * (size_t)i + 1] = x[1]; out_f64[3 * (size_t)i + 2] = x[2];
            if (R->cell_sig) R->cell_sig[i] = sig;
        }
        if (R->reseed) memcpy(R->reseed + 3 * (size_t)i, last, sizeof last);
    }
    R->fallback_count = fb;
    R->wrapped_count = wr;
    return 0;
}

/* Field evaluation at m points and one time (sample_at_positions). */
int orc_sample(const orc_field* F, double t, int t_is_f32, int precision, int m, const float* pos,
               float* out_f32, double* out_f64) {
    const stime s = {t, t_is_f32};
    int64_t fb = 0, wr = 0;
    for (int i = 0; i < m; ++i) {
        if (precision == ORC_F32) {
            field_f(F, s, pos + 3 * (size_t)i, out_f32 + 3 * (size_t)i, &fb, &wr);
        } else {
            double p[3] = {pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2]};
            field_d(F, s, p, out_f64 + 3 * (size_t)i, &fb);
        }
    }
    return (int)fb;
}

/* Apply a boundary to m float32 points in place. */
int orc_boundary_apply(const orc_boundary* B, int m, float* pos) {
    if (B->inlet_axis >= 0 && (B->lattice[0] == NULL || B->lattice[1] == NULL)) return -1;
    for (int i = 0; i < m; ++i) boundary_f(B, B->lattice[0], B->lattice[1], pos + 3 * (size_t)i, NULL);
    return 0;
}

int orc_sizes(int64_t* out) {
    out[0] = sizeof(orc_field);
    out[1] = sizeof(orc_boundary);
    out[2] = sizeof(orc_run);
    return 3;
}
