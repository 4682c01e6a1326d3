/*
 * jaxtrace_gb300.h -- C ABI of the GB300 Lagrangian-tracking library.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns 0 (JT_OK) or a negative JT_ERR_* code; the reason of the last
 * failure on the calling thread is returned by jt_last_error().
 *
 * Ownership: every device buffer is allocated and owned by the caller.
 * Pointers documented "device" must point to memory of the current CUDA
 * device; pointers documented "host" to ordinary host memory.  `stream`
 * is a cudaStream_t passed as void* (NULL = legacy default stream); all
 * device work of a call is enqueued on it and the call does not
 * synchronise unless stated.  Kernels report runtime anomalies through an
 * optional device status word (bit flags JT_STATUS_*), never by trapping.
 *
 * Reference interfaces replaced (paths are inside the JAXTrace project):
 *   jaxtrace/tracking/tracker.py      ParticleTracker.track_particles, lax.scan body
 *   jaxtrace/integrators/rk4.py, rk2.py, euler.py   rk4_step / rk2_step / euler_step
 *   jaxtrace/fields/time_series.py    TimeSeriesField time blend + nearest-node sampling
 *   jaxtrace/fields/structured.py     StructuredGridSampler trilinear sampling
 *   jaxtrace/fields/octree_fem_interpolator_optimized.py   octree build + P1 lookup
 *   jaxtrace/tracking/boundary.py     periodic / reflective / clamping / absorbing /
 *                                     mixed / continuous-inlet boundary callables
 *   jaxtrace/density/kde.py, sph.py, neighbors.py          density passes
 */
#ifndef JAXTRACE_GB300_H
#define JAXTRACE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JT_ABI_VERSION 5

/* ---- return codes ------------------------------------------------------ */
#define JT_OK 0
#define JT_ERR_INVALID (-1)     /* bad argument: shape, size, enum, null   */
#define JT_ERR_UNSUPPORTED (-2) /* combination not implemented             */
#define JT_ERR_CUDA (-3)        /* a CUDA runtime call failed              */
#define JT_ERR_NOMEM (-4)       /* caller-provided workspace too small     */
#define JT_ERR_STATUS (-5)      /* device status word reported an error    */

/* ---- device status bits (OR-ed by kernels into *status) --------------- */
#define JT_STATUS_INDEX_WRAPPED 0x1 /* periodic cell index hit N (the reference raises IndexError there) */
#define JT_STATUS_NONFINITE 0x2     /* a non-finite position was produced          */
#define JT_STATUS_OCTREE_FALLBACK 0x4 /* at least one mesh lookup found no containing tet and used
                                         the nearest-vertex / nearest-node fallback */

/* ---- enums ------------------------------------------------------------- */
/* snapshot value storage */
#define JT_STORE_F32 0  /* float32 x,y,z                                   */
#define JT_STORE_BF16 1 /* bfloat16 x,y,z with a per-snapshot float32 scale */
#define JT_STORE_F16 2  /* float16  x,y,z with a per-snapshot float32 scale */
/* Pre-blended stage fields of a regular grid (jt_stage_fields), tracking only
 * (no velocity recording: JT_ERR_UNSUPPORTED when vel is set): one time level
 * per schedule entry, entry.pair = the field slot. */
#define JT_STORE_STAGE_F32 3 /* float32 {x,y,z,0} per node (16 B)               */
#define JT_STORE_STAGE_F16 4 /* offset float16 yz-quads per node (32 B) of the
                                values divided by the power-of-two scale held
                                in entry.wa: the values of nodes (j,k),
                                (j,k1), (j1,k), (j1,k1) are o + r with float16
                                residuals r -- words 0-3 their (rx,ry), words
                                4-5 their rz in pairs -- and a per-quad offset
                                o: word 6 ox as float32, word 7 a float32
                                whose value is oy and whose low 16 bits are oz
                                as float16                                  */
#define JT_STORE_STAGE_F32Q 8 /* float32 yz-quads per node (48 B): the (x,y) of
                                nodes (j,k), (j,k1), (j1,k), (j1,k1) in a
                                32 B part A; their z in a 16 B part B stored
                                after the part-A records of the slot.  A
                                slot holds S = nodes rounded up to even
                                records (S * 48 B; pair_stride = S), so each
                                starts 32-byte aligned                       */
/* Affine-tile snapshots of a regular grid (input of jt_stage_tile_fields).
 * The grid's cells are cut into tiles of JT_TILE^3 cells; tile (tx,ty,tz)
 * covers cells [JT_TILE*t, JT_TILE*t + JT_TILE) per axis and its
 * (JT_TILE+1)^3 nodes.  Local node l (0..JT_TILE) of axis a is grid node
 * min(JT_TILE*t + l, n-1) (clamp, zero, nan) or (JT_TILE*t + l) mod n
 * (periodic), at continuous index coordinate min(JT_TILE*t + l, n-1) or
 * JT_TILE*t + l.  Per snapshot and tile a float32 affine base
 * b(f) = o + Gx*fx + Gy*fy + Gz*fz in the continuous index coordinates f is
 * stored as 16 floats {ox, oy, Gx.x, Gx.y, Gy.x, Gy.y, Gz.x, Gz.y, oz, Gx.z,
 * Gy.z, Gz.z, 0, 0, 0, 0}, and every tile node holds the 16-bit residual
 * v - b at its coordinate: 4 halves {x, y, z, 0} (8 B), nodes in order
 * (lx*(JT_TILE+1) + ly)*(JT_TILE+1) + lz. */
#define JT_STORE_TILE_BF16 5 /* bfloat16 residuals                            */
#define JT_STORE_TILE_F16 6  /* float16 residuals                             */
#define JT_TILE 4
#define JT_TILE_NODES 125 /* (JT_TILE+1)^3 residual nodes per snapshot tile   */

/* grid sampler bounds handling: fields/structured.py:89 */
#define JT_GRID_CLAMP 0
#define JT_GRID_ZERO 1
#define JT_GRID_NAN 2
#define JT_GRID_PERIODIC 3

/* time-blend forms (fields/time_series.py:326-367 and :155-245)
 *   WEIGHTED : v = wa*A + wb*B                 (in-bounds linear, constant,
 *                                               zero and nan extrapolation)
 *   LERP_FWD : v = A + wb*(B - A)              (linear extrapolation left)
 *   LERP_BWD : v = B + wb*(B - A)              (linear extrapolation right)
 *   SAME_A   : v = wa*A + wb*A                 (both bracket indices equal:
 *   SAME_B   : v = wa*B + wb*B                  a time that rounds onto an end)
 * A and B are snapshots `pair` and `pair+1`; for 16-bit storage they are
 * decoded as value*scale where sa/sb are the snapshots' scales (for the
 * WEIGHTED and SAME forms the host folds the scales into wa/wb and sets
 * sa=sb=1). */
#define JT_BLEND_WEIGHTED 0
#define JT_BLEND_LERP_FWD 1
#define JT_BLEND_LERP_BWD 2
#define JT_BLEND_SAME_A 3
#define JT_BLEND_SAME_B 4

typedef struct {
    int32_t pair;
    int32_t form;
    float wa, wb;
    float sa, sb;
    int32_t pad0, pad1;
} jt_blend; /* 32 bytes */

/* integrators: integrators/euler.py:111, rk2.py:246, rk4.py:62 */
#define JT_EULER 0
#define JT_RK2 1
#define JT_RK4 2

/* per-axis box boundary kinds: tracking/boundary.py:101-210 */
#define JT_BC_NONE 0
#define JT_BC_PERIODIC 1
#define JT_BC_REFLECTIVE 2
#define JT_BC_CLAMP 3
#define JT_BC_ABSORBING 4

/* continuous-inlet replacement distributions: boundary.py:1444-1601 */
#define JT_INLET_OFF 0
#define JT_INLET_GRID 1

/* arithmetic mode of the tracking kernels */
#define JT_ARITH_EXACT 0       /* float32, round-to-nearest, no contraction:
                                  bit-identical to the NumPy reference path */
#define JT_ARITH_COMPENSATED 1 /* float32 with FMA and Kahan-compensated
                                  position accumulation                     */

/* ---- field descriptors ------------------------------------------------- */

/* Regular grid field: StructuredGridSampler (fields/structured.py:65) whose
 * node values come from a time series of snapshots (time_series.py:82).
 * Node (i,j,k) of an (nx,ny,nz) grid has index (i*ny + j)*nz + k, the
 * reference's ij layout.  Values are stored as snapshot PAIRS: record n of
 * pair p holds snapshot p and p+1 of node n side by side:
 *   F32 : 8 floats  {Ax,Ay,Bx,By, Az,Bz,0,0}        (32 B, one sector)
 *   BF16/F16 (grid field): 24 halves, the yz-QUAD of node (i,j,k): nodes
 *         (i,j,k), (i,j,k1), (i,j1,k), (i,j1,k1) with k1 = (k+1) mod nz for
 *         periodic bounds and min(k+1, nz-1) otherwise (j1 alike), six
 *         halves {Ax,Ay,Bx,By,Az,Bz} each in that order.  Halves 0-15 form a
 *         32 B part A; halves 16-23 a 16 B part B stored after the part-A
 *         records of all pairs (at pairs + 32 B * n_pairs * pair_stride).
 *   BF16/F16 (mesh, nearest fields): 8 halves {Ax,Ay,Bx,By,Az,Bz,0,0} (16 B)
 * so aligned 256-bit (and 128-bit) loads return both bracketing snapshots of
 * a node (or of a yz-quad of nodes), x,y components in register pairs. */
typedef struct {
    int32_t nx, ny, nz;
    int32_t bounds_mode;   /* JT_GRID_*                                       */
    float origin[3];       /* grid_x[0], grid_y[0], grid_z[0]                 */
    float spacing[3];      /* float32(grid[1]-grid[0]), 1 when n == 1         */
    float inv_spacing[3];  /* 1/spacing (used by the non-exact modes only)    */
    float valid_hi[3];     /* float32(min + (n-1)*d), the zero/nan validity edge */
    int32_t storage;       /* JT_STORE_*                                      */
    int32_t n_pairs;       /* number of snapshot pairs (>= 1)                  */
    int64_t pair_stride;   /* records per pair (= nx*ny*nz)                    */
    const void* pairs;     /* device                                          */
    /* affine-tile snapshots (JT_STORE_TILE_*) only: pairs holds the residual
     * nodes of n_pairs+1 snapshots, pair_stride = tiles*JT_TILE_NODES records
     * (8 B) per snapshot, and tile_base the (n_pairs+1) x tiles base records,
     * where tiles = tiles[0]*tiles[1]*tiles[2], tiles[a] = (n_a + JT_TILE - 1)
     * / JT_TILE, tile (tx,ty,tz) at (tx*tiles[1] + ty)*tiles[2] + tz.  Unused
     * (NULL, 0) by the other storages. */
    const float* tile_base; /* device                                         */
    int32_t tiles[3];
    int32_t pad_tiles;
} jt_grid_field;

/* Tetrahedral mesh field with the octree point location of
 * fields/octree_fem_interpolator_optimized.py.  Arrays are produced by
 * jt_octree_build and uploaded by the caller. */
typedef struct {
    float cx, cy, cz;      /* float32 (min+max)/2 of the node box             */
    int32_t is_leaf;
    int32_t children[8];   /* -1 where the octant is empty                    */
    int32_t elem_offset;   /* into the element list                            */
    int32_t elem_count;
    int32_t pad0, pad1;
} jt_octree_node; /* 64 bytes */

typedef struct {
    int32_t n_points, n_tets;
    int32_t n_nodes;        /* octree nodes                                   */
    int32_t max_depth;      /* traversal iterations (reference default 12)   */
    int32_t storage;        /* JT_STORE_* of the node values                  */
    int32_t n_pairs;
    int32_t near_degenerate; /* nonzero: tet_box flags some tetrahedra (jt_mark_near_degenerate) */
    int32_t pad;
    int64_t pair_stride;    /* records per pair (= n_points)                  */
    const float* points;    /* device (n_points,4): x,y,z,0                   */
    const float* tet_box;   /* device (n_tets,8): min xyz,flag, max xyz,0 (flag: jt_mark_near_degenerate) */
    const float* tet_geom;  /* device (n_tets,16): v0, v1-v0, v2-v0, v3-v0 (xyz each), conn as int32 bits */
    const jt_octree_node* nodes; /* device (n_nodes)                        */
    const int32_t* elems;   /* device element lists                           */
    const void* pairs;      /* device value pairs, layout as jt_grid_field   */
    /* Optional compact copy of the tree for the descent (NULL: descend on
     * nodes).  Nodes in breadth-first order, the root first and the present
     * children of a node consecutive in octant order: desc (n_nodes,4) holds
     * the centre's float32 bits and mask | first << 8, mask the present
     * octants (0 for a leaf) and first the breadth-first index of the first
     * child (< 2^24); dtab (n_nodes,2) holds the node's elem_offset and
     * elem_count.  One 16-byte load per level instead of two dependent
     * loads, the same moves as the node records. */
    const int32_t* desc;
    const int32_t* dtab;
} jt_mesh_field;

/* Nearest-node field: TimeSeriesField spatial sampling (time_series.py:391)
 * over scattered nodes, accelerated by a uniform cell list. */
typedef struct {
    int32_t n_points;
    int32_t cells[3];       /* cell-list resolution                          */
    float origin[3];
    float inv_cell[3];
    int32_t storage;
    int32_t n_pairs;
    int64_t pair_stride;    /* = n_points                                     */
    const float* points;    /* device (n_points,4) sorted by cell            */
    const int32_t* point_ids; /* device (n_points) original node index of sorted slot */
    const int32_t* cell_start; /* device (cells+1) CSR offsets                 */
    const void* pairs;      /* device value pairs indexed by ORIGINAL node id */
} jt_nearest_field;

/* Tetrahedral mesh field with the hash-grid point location of
 * FEMTimeSeriesField (fields/fem_time_series.py:16-110,
 * fields/fem_interpolator.py:36-328): the query's cell of a uniform grid
 * over the node bounding box (float32 (q - grid_min) / cell_size, floored,
 * clipped), the cell's elements in ascending order, the first whose box and
 * barycentric test hold the query gives P1; otherwise the nearest node of
 * the whole mesh (searched through the embedded nearest-node cell list). */
typedef struct {
    jt_nearest_field nearest; /* nodes, nearest-node cell list and the
                                 snapshot value pairs (indexed by node id)  */
    int32_t n_tets;
    int32_t grid_size[3];   /* hash cells per axis; cell id (i*gy + j)*gz + k */
    float grid_min[3];      /* float32 node bounding-box minimum              */
    float cell_size[3];     /* float32 cell edges of the lookup               */
    const float* tet_box;   /* device (n_tets,8): min xyz,flag, max xyz,0 (flag: jt_mark_near_degenerate) */
    const float* tet_geom;  /* device (n_tets,16) as jt_mesh_field            */
    const int32_t* cell_start; /* device (cells+1) CSR offsets                 */
    const int32_t* cell_elems; /* device element ids, ascending within a cell */
    /* Optional refinement that keeps the result: each hash cell split into
     * sub_div^3 sub-cells, each listing (ascending) the cell's elements whose
     * box, widened slightly, meets the sub-cell.  The element the cell scan
     * would pick holds the query in its box, so it is on the query's
     * sub-cell list, and every element before it there is before it in the
     * cell list too.  sub_div 0: scan the cell lists. */
    int32_t sub_div;
    int32_t near_degenerate; /* nonzero: tet_box flags some tetrahedra (jt_mark_near_degenerate) */
    const int32_t* sub_start;  /* device (cells*sub_div^3 + 1) CSR offsets     */
    const int32_t* sub_elems;  /* device element ids                          */
} jt_fem_field;

#define JT_FIELD_GRID 1
#define JT_FIELD_MESH 2
#define JT_FIELD_NEAREST 3
#define JT_FIELD_FEM 4

typedef struct {
    int32_t kind;           /* JT_FIELD_*                                     */
    int32_t pad;
    const jt_grid_field* grid;
    const jt_mesh_field* mesh;
    const jt_nearest_field* nearest;
    const jt_fem_field* fem;
} jt_field;

/* ---- boundary descriptor ------------------------------------------------ */
typedef struct {
    int32_t axis_kind[3];   /* JT_BC_* per axis                               */
    int32_t absorbing_joint;/* 1: absorbing_boundary_factory semantics -- a
                               particle outside on any axis gets outside_value
                               on all three (boundary.py:175-210)           */
    float lo[3], hi[3];     /* per-axis bounds                                */
    float outside_value;
    /* continuous inlet, boundary.py:1517-1599 (replaces axis_kind when on)  */
    int32_t inlet_mode;     /* JT_INLET_*                                     */
    int32_t inlet_axis;     /* 0,1,2                                          */
    int32_t inlet_positive; /* 1: flow toward max, 0: toward min              */
    int32_t inlet_res[2];   /* lattice sizes of the two other axes (ascending axis order) */
    float inlet_nudge;      /* float32 axis_min + 0.001f*(axis_max-axis_min) (or mirror) */
    const float* inlet_coords[2]; /* device float32 linspace lattices         */
} jt_boundary;

/* ---- tracking ---------------------------------------------------------- */
typedef struct {
    int32_t integrator;     /* JT_EULER / JT_RK2 / JT_RK4                     */
    int32_t arith;          /* JT_ARITH_*                                     */
    int32_t n_particles;
    int32_t step_begin;     /* global index of the first step of this launch  */
    int32_t step_end;       /* one past the last                              */
    float dt;               /* float32 dt                                     */
    float dt_half;          /* float32 0.5*dt                                 */
    float dt_sixth;         /* float32 dt/6                                   */
    const jt_blend* schedule;  /* device, 4 entries per step s:
                                  [4s+0] time of stage 1 (t_s),
                                  [4s+1] t_s + dt/2 (RK2 / RK4 mid stages),
                                  [4s+2] t_s + dt   (RK4 last stage),
                                  [4s+3] times[s+1] (velocity recording)     */
    int64_t schedule_stride;/* entries between ensembles (0: one schedule)    */
    const int32_t* ens_offsets; /* device (n_ens+1) particle offsets or NULL:
                                   particles [ens_offsets[e], ens_offsets[e+1])
                                   use schedule + e*schedule_stride; the
                                   particle of slot i is ids[i] when ids is
                                   set (after a locality sort), else i     */
    int32_t n_ens;
    int32_t block_size;     /* threads per block of the tracking launch:
                               0 (256), 64, 128 or 256                     */
    float* pos;             /* device (N,3) in/out                            */
    float* comp;            /* device (N,3) Kahan compensation (COMPENSATED) or NULL */
    float* traj;            /* device (rows,N,3) or NULL                      */
    float* vel;             /* device (rows,N,3) or NULL (record_velocities)  */
    int32_t record_every;   /* step count c=s+1 is recorded when c % record_every == 0 */
    int32_t record_compact; /* row = c/record_every (1) or row = c (0)       */
    int32_t row_base;       /* row of traj[0] for this launch                 */
    int32_t n_rows;         /* rows held by traj/vel for this launch          */
    int32_t* status;        /* device status word or NULL                     */
    const int32_t* ids;     /* device (N): particle index of slot i, used as the
                               row index of traj/vel writes after a locality
                               sort, or NULL (slot i is particle i)           */
    float* path;            /* device (N) float32 per-particle path length or
                               NULL: each step adds |x_after - x_before| (the
                               positions after the boundary, float32
                               sqrt((dx*dx + dy*dy) + dz*dz)) in step order,
                               the sum Trajectory.compute_path_length forms
                               over rows recorded every step
                               (tracking/particles.py:296-313); indexed by
                               particle (through ids after a sort), carried
                               across launches                              */
} jt_track_params;

/* ABI / diagnostics */
int jt_abi_version(void);

/* Device memory for the library's own scratch: the device builds
 * (jt_octree_build_device, jt_fem_grid_build_device) and the arrays their
 * handles hold until the matching _free_device, and the count of
 * jt_mark_near_degenerate.  Every other entry point works in caller buffers.
 * By default that scratch comes from cudaMallocAsync / cudaFreeAsync on the
 * call's stream; a caller that owns the device's memory (a framework's pool)
 * installs its own pair here and the library allocates nothing itself.
 * alloc(bytes, stream, ctx) returns a device pointer usable in stream order
 * on `stream`, or NULL (the call then fails with JT_ERR_CUDA); free(ptr,
 * stream, ctx) releases it in stream order.  Both NULL restore the default.
 * Install before the calls that allocate, not while one runs, and release
 * handles with the allocator that made them. */
typedef void* (*jt_alloc_fn)(size_t bytes, void* stream, void* ctx);
typedef void (*jt_free_fn)(void* ptr, void* stream, void* ctx);
int jt_set_allocator(jt_alloc_fn alloc, jt_free_fn free_fn, void* ctx);
const char* jt_last_error(void);
/* sizes of the public structs, in the order: jt_blend, jt_grid_field,
 * jt_octree_node, jt_mesh_field, jt_nearest_field, jt_field, jt_boundary,
 * jt_track_params.  Lets a binding check its mirror of the layouts.        */
int jt_struct_sizes(int64_t* out, int32_t n);

/* Advance particles through steps [step_begin, step_end) of the schedule,
 * fusing integrator stages, field evaluation and boundary into one kernel
 * with the time loop held in registers.  Replaces the lax.scan body
 * tracker.py:236-242 (and the step loop :441-446), rk4.py:62-106,
 * rk2.py:246-309, euler.py:111-157 and the boundary callables. */
int jt_track(const jt_field* field, const jt_boundary* bc,
             const jt_track_params* params, void* stream);

/* Evaluate a field at M positions with one blend entry: the
 * sample_at_positions(positions, t) protocol (fields/base.py:106-122,
 * time_series.py:391, structured.py:258, octree_fem_time_series_optimized.py:87).
 * pos, out: device (M,3) float32. */
int jt_field_sample(const jt_field* field, const jt_blend* blend, int32_t arith,
                    const float* pos, float* out, int32_t m,
                    int32_t* status, void* stream);

/* Apply a boundary in place to (N,3) device positions: the callables
 * returned by periodic_boundary / reflective_boundary / clamping_boundary /
 * absorbing_boundary_factory / mixed_boundary /
 * continuous_inlet_boundary_factory (boundary.py:215-438, :1444-1601). */
int jt_boundary_apply(const jt_boundary* bc, float* pos, int32_t n, void* stream);

/* One integrator step without boundary: rk4_step / rk2_step / euler_step
 * (x, t, dt, field_fn) with a scalar or per-particle dt.  stage blends: the
 * three entries of jt_track_params.schedule for this step (host memory,
 * copied by value).  dt_per_particle: device (N) float32 or NULL. */
int jt_integrator_step(const jt_field* field, const jt_blend* stage_blends,
                       int32_t integrator, int32_t arith, float dt,
                       const float* dt_per_particle, const float* x_in,
                       float* x_out, int32_t n, int32_t* status, void* stream);

/* ---- pre-blended stage fields --------------------------------------------- */
/* No reference counterpart as an entry point: TimeSeriesField.sample_at_time
 * (time_series.py:306-389) blends every node at the query time before
 * StructuredGridSampler interpolates; this does that once per schedule entry
 * of a time chunk so the tracking kernel gathers one time level.
 * field: a regular-grid field (F32 or 16-bit pair storage).
 * entries: device (n) schedule entries (their pair and blend); out_scales:
 * device (n) power-of-two scales for JT_STORE_STAGE_F16 (NULL for F32).
 * out_storage: JT_STORE_STAGE_F32 / _F32Q (from float32 snapshots, exact
 * blend) or JT_STORE_STAGE_F16 (from 16-bit snapshots).
 * out: device (32-byte aligned; so must the field's pairs be), n fields of
 * S records of out_storage, field j at out + j * S * record_bytes (16, 48 or
 * 32 B), S = nodes, or nodes rounded up to even for F32Q.  The tracking
 * launch then takes a jt_grid_field with storage = out_storage, pairs = out,
 * n_pairs = n, pair_stride = S and entries whose pair is the slot j (and,
 * for F16, wa = out_scales[j]). */
int jt_stage_fields(const jt_field* field, const jt_blend* entries, const float* out_scales, int32_t n,
                    int32_t out_storage, void* out, void* stream);

/* The same for affine-tile snapshots (JT_STORE_TILE_BF16 / _F16), always
 * into JT_STORE_STAGE_F16 fields: each node's quad values are the tile base
 * at the nodes' coordinates plus their residuals, blended per the entry
 * (sa = sb = 1: tile snapshots carry no per-snapshot scale).  out_scales:
 * device (n) power-of-two bounds of the blended values (the entries' wa in
 * the tracking launch); out: device, field j at out + j * nodes * 32 B. */
int jt_stage_tile_fields(const jt_field* field, const jt_blend* entries, const float* out_scales, int32_t n,
                         void* out, void* stream);

/* ---- adjoint ------------------------------------------------------------- */
/* No reference counterpart: JAXTrace has no gradients (no jax.grad on this
 * path).  Reverse-mode RK4 for loss gradients with respect to the initial
 * positions and the snapshot values, one checkpoint segment per call. */
#define JT_ADJOINT_MAX_SEGMENT 64
typedef struct {
    int32_t n_particles;
    int32_t step_begin, step_end;  /* the segment, at most JT_ADJOINT_MAX_SEGMENT steps */
    float dt, dt_half, dt_sixth;   /* as jt_track_params                    */
    int32_t pad;
    const jt_blend* schedule;      /* as jt_track_params.schedule          */
    const float* ckpt;             /* device (N,3): positions at step_begin (forward checkpoint) */
    float* lambda;                 /* device (N,3): dL/dx at step_end on entry, at step_begin on exit */
    float* grad;                   /* device, the field's pair-record layout in float32
                                      (n_pairs, nodes, 8): += dL/dA in slots 0,1,4 and dL/dB
                                      in slots 2,3,5 (A = snapshot p, B = snapshot p+1);
                                      NULL: dL/dx only                          */
    void* work;                    /* device workspace (16-byte aligned) of at least
                                      jt_adjoint_workspace_bytes(nodes, steps) bytes when
                                      grad is set; zeroed by the call           */
    int64_t work_bytes;
    const float* stage;            /* device float32 stage fields of the segment
                                      (jt_stage_fields with JT_STORE_STAGE_F32 over its
                                      3 * steps schedule entries, slot 3*s + k), or NULL to
                                      blend the pair records                     */
} jt_adjoint_params;

/* Workspace of one backward segment of n_steps steps over n_nodes grid
 * nodes: three float4 snapshot-gradient accumulators per step and node. */
size_t jt_adjoint_workspace_bytes(int64_t n_nodes, int32_t n_steps);

/* One backward segment over a float32 regular-grid field with per-axis box
 * boundaries: recomputes the segment from its checkpoint with the forward
 * (exact) arithmetic, keeping every step's stage positions, then propagates
 * lambda back step by step.  The snapshot gradient of each stage time is
 * accumulated per node (vector atomics into the workspace) and folded into
 * grad with the stage's blend coefficients by a second kernel. */
int jt_adjoint_rk4(const jt_field* field, const jt_boundary* bc, const jt_adjoint_params* p, void* stream);

/* ---- locality sort ------------------------------------------------------ */
/* Cell grid of the sort: cell = clamp(floor((x-origin)*inv_cell), 0, 2^bits-1)
 * per axis; cells ordered by Morton key (tracking locality) or row-major
 * with x fastest (density passes: an x-run of cells is one particle range). */
#define JT_ORDER_MORTON 0
#define JT_ORDER_LINEAR 1
typedef struct {
    float origin[3];
    float inv_cell[3];
    int32_t bits;            /* 1..7 bits per axis                           */
    int32_t order;           /* JT_ORDER_*                                   */
} jt_sort_grid;

/* Bytes of device workspace jt_cell_sort needs (0 for invalid arguments). */
size_t jt_cell_sort_workspace_bytes(int32_t n, int32_t bits);

/* Reorder particles by Morton cell (counting sort) so that warps gather from
 * few cache lines.  No reference counterpart changes meaning: the reference
 * keeps particles in input order (tracker.py:428-446); particle results do
 * not depend on their slot, and ids_out (slot -> original particle) lets
 * jt_unpermute restore the input order.  pos_in/pos_out: device (N,3);
 * comp_in/comp_out: optional Kahan terms; ids_in: device (N) or NULL for the
 * identity; workspace: caller-allocated device memory of at least
 * jt_cell_sort_workspace_bytes(n, bits).  Not in place. */
int jt_cell_sort(const jt_sort_grid* g, int32_t n, const float* pos_in, const float* comp_in,
                 const int32_t* ids_in, float* pos_out, float* comp_out, int32_t* ids_out,
                 void* workspace, size_t workspace_bytes, void* stream);

/* Allocation-free jt_cell_sort.  No counterpart in the reference.
 * For callers that cannot allocate device memory when they call in (an
 * application that owns every device allocation through its own pool, or a
 * time-critical loop where cudaMalloc/cudaFree and their device-wide
 * synchronisation are not allowed): the scratch is a fixed array in the
 * library's own device memory, so the call allocates nothing.
 *   limits: n <= JT_NOALLOC_SORT_MAX_PARTICLES, bits <= JT_NOALLOC_SORT_MAX_BITS
 *           (larger sizes return JT_ERR_INVALID); the array (about 9 MiB) is
 *           held on every GPU that loads the library until the process exits.
 *   set-up: the first call on a device looks up the array's device address
 *           (cudaGetSymbolAddress) with that device current; make that first
 *           call before any stream capture.  A device reset (cudaDeviceReset)
 *           ends the context the address belongs to: the next call notices
 *           the new context and looks the address up again, so the first
 *           call after a reset must also come before any stream capture.
 *   sharing: every call uses the same array, which keeps the last call's
 *           contents (the call clears what it accumulates into); calls whose
 *           work overlaps on the GPU race -- serialise them on one stream.
 * Arguments as jt_cell_sort without the workspace. */
#define JT_NOALLOC_SORT_MAX_PARTICLES (1 << 21)
#define JT_NOALLOC_SORT_MAX_BITS 6
int jt_cell_sort_noalloc(const jt_sort_grid* g, int32_t n, const float* pos_in, const float* comp_in,
                         const int32_t* ids_in, float* pos_out, float* comp_out, int32_t* ids_out,
                         void* stream);

/* pos_out[ids[i]] = pos_sorted[i]: back to the caller's particle order. */
int jt_unpermute(int32_t n, const float* pos_sorted, const int32_t* ids, float* pos_out, void* stream);

/* Counting sort of particles by Morton cell that also returns the cell list:
 * cell_end[key] = one past the last sorted particle of Morton cell `key`
 * (device, 2^(3*bits) entries; the cell starts at cell_end[key-1], or 0).
 * Replaces HashGridNeighbors.__post_init__ (density/neighbors.py:61-104):
 * cell keys, argsort, unique starts/counts.  Other arguments as jt_cell_sort. */
int jt_cell_list(const jt_sort_grid* g, int32_t n, const float* pos_in, float* pos_out, int32_t* ids_out,
                 uint32_t* cell_end, void* workspace, size_t workspace_bytes, void* stream);

/* ---- density passes ------------------------------------------------------ */
#define JT_SPH_CUBIC 0    /* sph.py:227-236 */
#define JT_SPH_WENDLAND 1 /* sph.py:238-246 */
#define JT_SPH_GAUSSIAN 2 /* sph.py:248-255 */

typedef struct {
    int32_t dims;              /* 2 or 3 (2-D: z of particles and queries is 0) */
    int32_t kernel;            /* JT_SPH_*                                    */
    int32_t n_particles;
    int32_t n_queries;
    float radius;              /* neighbour cutoff (the NumPy path uses 3*mean(h), sph.py:284-285) */
    float h_const;             /* smoothing length when h == NULL            */
    jt_sort_grid grid;         /* cell grid of the particle cell list        */
    int32_t reach[3];          /* cells searched on each side, per axis      */
    int32_t packed;            /* 0: particles (N,3) and masses apart; 1:
                                  particles (N,4) {x,y,z,mass} in one 16-byte
                                  record; 2: particle pairs (ceil(N/2),8)
                                  {x0,x1,y0,y1,z0,z1,mass0,mass1} (16-byte
                                  aligned; an odd N pads the last pair).  1
                                  and 2 leave masses unused and need h NULL */
    const float* particles;    /* device (N,3) or (N,4) in cell order        */
    const float* masses;       /* device (N) in cell order, or NULL (unit masses) */
    const float* h;            /* device (N) in cell order, or NULL (h_const) */
    const uint32_t* cell_end;  /* device, from jt_cell_list                  */
    const float* queries;      /* device (M,3)                               */
    double* out;               /* device (M): sum_j m_j W(|q - p_j|, h_j)    */
    unsigned long long* counters; /* device [2] or NULL: when set, the call adds
                                  the candidate pairs it examined and the
                                  pairs inside the kernel's support (uniform
                                  h, packed records only; a counting
                                  instance of the kernel, for measurement) */
} jt_sph_params;

/* SPH density at M query points: _evaluate_density (density/sph.py:269-292)
 * summed exactly over every particle within `radius` (the NumPy brute-force
 * semantics; no per-cell cap or nearest-512 truncation).  Each cell's terms
 * are summed in float32 and the cells in float64.  Normalisation by N/volume
 * (sph.py:365-378) is left to the caller. */
int jt_sph_density(const jt_sph_params* p, void* stream);

typedef struct {
    int32_t dims;              /* 2 or 3                                      */
    int32_t n_particles;
    int32_t res[3];            /* grid points per axis (x, y, z; z = 1 in 2-D) */
    float half_inv_h2;         /* 0.5 / h^2                                   */
    float radius;              /* particles farther than this along an axis from every grid point of a tile are skipped */
    jt_sort_grid grid;         /* cell grid of the particle cell list         */
    const float* axis[3];      /* device float32 grid coordinates per axis    */
    const float* particles;    /* device (N,3) in cell order                  */
    const uint32_t* cell_end;  /* device, from jt_cell_list                   */
    double* out;               /* device: grid (x index i, y index j, z index k) at (i*res_y + j)*res_z + k */
    unsigned long long* counters; /* device [2] or NULL (3-D grids): when set,
                                  the call adds the (particle, tile) visits of
                                  its 8^3 tiles and the (grid point,
                                  particle) kernel terms they sum          */
} jt_kde_params;

/* Gaussian KDE on a tensor grid: out = sum_j exp(-|g - p_j|^2 h^-2 / 2) at
 * every grid point g (the float32 JAX / pure-NumPy formula of
 * density/kde.py:249-282 without its constant factors, which the grid
 * normalisation of kde.py:229-239 removes).  Separable per 8^3 (3-D) or
 * 16^2 (2-D) tile; per-tile float32 chunks accumulated in float64. */
int jt_kde_grid(const jt_kde_params* p, void* stream);

/* The same sum at M arbitrary points (KDEEstimator.evaluate, kde.py:123-169):
 * points device (M,3), out device (M).  p->axis and p->res are unused. */
int jt_kde_points(const jt_kde_params* p, const float* points, int32_t m, double* out, void* stream);

/* ---- octree build (host) ------------------------------------------------ */
typedef struct {
    int32_t n_nodes;         /* octree nodes                                   */
    int32_t n_elem_entries;  /* length of the concatenated leaf element lists  */
    int32_t max_elems;       /* longest list (the reference's padded width)    */
    int32_t max_tree_depth;  /* deepest node                                   */
    int32_t n_leaves;
    int32_t pad;
} jt_octree_info;

/* Build the octree of a tetrahedral mesh on the host: replaces
 * build_octree_mesh_optimized (fields/octree_fem_interpolator_optimized.py:41-215)
 * with identical node numbering, octant assignment and leaf rule.
 * points: host (n_points,3) float32; conn: host (n_tets,4) int32.
 * On success *handle_out owns the result until jt_octree_free. */
int jt_octree_build(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                    int32_t max_elements_per_leaf, int32_t max_depth, void** handle_out,
                    jt_octree_info* info);

/* Copy a built octree into caller host buffers (any may be NULL):
 * nodes (n_nodes) [pad0 holds the node depth], elems (n_elem_entries),
 * tet_box (n_tets,8), tet_geom (n_tets,16), node_bounds (n_nodes,6 = min xyz,
 * max xyz; the reference's nodes_min/nodes_max). */
int jt_octree_fetch(void* handle, jt_octree_node* nodes, int32_t* elems, float* tet_box,
                    float* tet_geom, float* node_bounds);

void jt_octree_free(void* handle);

/* The same octree built on the device (identical arrays to jt_octree_build):
 * points device (n_points,3) float32, conn device (n_tets,4) int32; elems
 * (n_tets int32, every element lands in exactly one leaf) and, if not NULL,
 * tet_box (n_tets,8) and tet_geom (n_tets,16) are caller device buffers
 * filled on `stream`.  Node records and node bounds, whose count is known
 * only after the build (info->n_nodes), stay in *handle_out (device memory)
 * until jt_octree_fetch_device copies them and jt_octree_free_device
 * releases them.  Returns after the build has finished on `stream`. */
int jt_octree_build_device(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                           int32_t max_elements_per_leaf, int32_t max_depth, int32_t* elems,
                           float* tet_box, float* tet_geom, void* stream, void** handle_out,
                           jt_octree_info* info);

/* Flag near-degenerate tetrahedra for the compensated arithmetic: sets the
 * pad slot after the box minimum (tet_box[8t+3]) to 1 where |det| of
 * (v1-v0, v2-v0, v3-v0) is below 1e-2 |v1-v0| |v2-v0| |v3-v0| (float32, from
 * tet_geom), else 0.  jt_track / jt_field_sample in JT_ARITH_COMPENSATED
 * re-solve the barycentric weights of a flagged tetrahedron in float64;
 * JT_ARITH_EXACT ignores the flag.  Device buffers; *count_out (host, may be
 * NULL) receives the number flagged.  Returns after the pass has finished. */
int jt_mark_near_degenerate(float* tet_box, const float* tet_geom, int32_t n_tets, int32_t* count_out,
                            void* stream);

/* Copy the device build's nodes (n_nodes) and node_bounds (n_nodes,6) into
 * caller buffers (device or host; either may be NULL), ordered on `stream`. */
int jt_octree_fetch_device(void* handle, jt_octree_node* nodes, float* node_bounds, void* stream);

void jt_octree_free_device(void* handle, void* stream);

/* ---- FEM hash grid build (host) ----------------------------------------- */
typedef struct {
    int64_t n_cells;        /* grid_size[0]*grid_size[1]*grid_size[2]         */
    int64_t n_entries;      /* length of the concatenated cell lists         */
    int64_t n_sub_cells;    /* n_cells * sub_div^3 (0 without sub-cells)      */
    int64_t n_sub_entries;  /* length of the concatenated sub-cell lists     */
    int32_t max_per_cell;   /* the reference's padded table width            */
    int32_t pad;
} jt_fem_grid_info;

/* Build the hash grid of build_tetrahedral_mesh
 * (fields/fem_interpolator.py:36-143) on the host: every element in every
 * cell its float32 box overlaps (float32 box minus float32 grid_min, divided
 * by the float64 cell_edge, floored, clipped), elements ascending per cell;
 * with sub_div > 0, the sub-cell lists of jt_fem_field (each cell split into
 * sub_div^3, boxes widened by eps[axis], float64 sub-cell index).
 * points: host (n_points,3) float32; conn: host (n_tets,4) int32;
 * grid_size, grid_min (float32), cell_edge (float64), eps (float64): 3 each.
 * On success *handle_out owns the lists until jt_fem_grid_free. */
int jt_fem_grid_build(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                      const int32_t* grid_size, const float* grid_min, const double* cell_edge, int32_t sub_div,
                      const double* eps, void** handle_out, jt_fem_grid_info* info);

/* Copy the lists into caller host buffers (any may be NULL): cell_start
 * (n_cells+1), cell_elems (n_entries), sub_start (n_sub_cells+1; one 0 without
 * sub-cells), sub_elems (n_sub_entries). */
int jt_fem_grid_fetch(void* handle, int32_t* cell_start, int32_t* cell_elems, int32_t* sub_start,
                      int32_t* sub_elems);

void jt_fem_grid_free(void* handle);

/* The same lists built on the device (identical arrays to jt_fem_grid_build):
 * points device (n_points,3), conn device (n_tets,4); grid_size, grid_min,
 * cell_edge and eps are host arrays of 3.  tet_box (n_tets,8, required) and
 * tet_geom (n_tets,16, or NULL) are caller device buffers filled with the
 * box (min xyz,0,max xyz,0) and geometry (v0, v1-v0, v2-v0, v3-v0, vertex
 * ids) records.  The lists stay in *handle_out (device memory) until
 * jt_fem_grid_fetch_device copies them and jt_fem_grid_free_device releases
 * them.  JT_ERR_UNSUPPORTED when the grid has more than 4,194,303 cells or
 * sub-cells or a cell lists more than 4096 elements (the host builder covers
 * those).  Returns after the build has finished on `stream`. */
int jt_fem_grid_build_device(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                             const int32_t* grid_size, const float* grid_min, const double* cell_edge,
                             int32_t sub_div, const double* eps, float* tet_box, float* tet_geom,
                             void* stream, void** handle_out, jt_fem_grid_info* info);

/* Copy the device build's lists into caller buffers (device or host; any may
 * be NULL), ordered on `stream`. */
int jt_fem_grid_fetch_device(void* handle, int32_t* cell_start, int32_t* cell_elems, int32_t* sub_start,
                             int32_t* sub_elems, void* stream);

void jt_fem_grid_free_device(void* handle, void* stream);

/* ---- trajectory analytics ------------------------------------------------- */
/* The pair term of compute_mixing_metrics (tracking/analysis.py:297-312):
 * over every ordered pair (i, j) whose float32 initial distance
 * d0 = |x0_i - x0_j| (sqrt((dx*dx + dy*dy) + dz*dz), each operation rounded)
 * satisfies 0 < d0 < rmax, *out_sum receives the float64 sum of
 * logf(d1 / d0) with d1 = |x1_i - x1_j|, and *out_count the number of such
 * pairs.  x0, x1: device (n,3) float32 (the first and last recorded rows);
 * out_sum, out_count: device scalars, overwritten. */
int jt_pair_log_ratio(const float* x0, const float* x1, int32_t n, float rmax, double* out_sum,
                      unsigned long long* out_count, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* JAXTRACE_GB300_H */
