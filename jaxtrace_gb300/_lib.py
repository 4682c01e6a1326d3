"""ctypes binding of ``libjaxtrace_gb300.so`` (the C ABI in include/jaxtrace_gb300.h).

The library is required: there is no CPU fallback.  Importing this module
never needs a GPU; calls that launch kernels need a CUDA device.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _build

i32, i64, f32, vp = C.c_int32, C.c_int64, C.c_float, C.c_void_p

# ---- constants (mirror of the header) ------------------------------------
ABI_VERSION = 5
JT_OK, JT_ERR_INVALID, JT_ERR_UNSUPPORTED, JT_ERR_CUDA, JT_ERR_NOMEM, JT_ERR_STATUS = 0, -1, -2, -3, -4, -5
JT_STATUS_INDEX_WRAPPED, JT_STATUS_NONFINITE, JT_STATUS_OCTREE_FALLBACK = 0x1, 0x2, 0x4
JT_STORE_F32, JT_STORE_BF16, JT_STORE_F16 = 0, 1, 2
JT_STORE_STAGE_F32, JT_STORE_STAGE_F16 = 3, 4
JT_STORE_TILE_BF16, JT_STORE_TILE_F16, JT_STORE_STAGE_F32Q = 5, 6, 8
JT_TILE, JT_TILE_NODES = 4, 125
JT_GRID_CLAMP, JT_GRID_ZERO, JT_GRID_NAN, JT_GRID_PERIODIC = 0, 1, 2, 3
JT_BLEND_WEIGHTED, JT_BLEND_LERP_FWD, JT_BLEND_LERP_BWD, JT_BLEND_SAME_A, JT_BLEND_SAME_B = 0, 1, 2, 3, 4
JT_EULER, JT_RK2, JT_RK4 = 0, 1, 2
JT_BC_NONE, JT_BC_PERIODIC, JT_BC_REFLECTIVE, JT_BC_CLAMP, JT_BC_ABSORBING = 0, 1, 2, 3, 4
JT_INLET_OFF, JT_INLET_GRID = 0, 1
JT_ARITH_EXACT, JT_ARITH_COMPENSATED = 0, 1
JT_FIELD_GRID, JT_FIELD_MESH, JT_FIELD_NEAREST, JT_FIELD_FEM = 1, 2, 3, 4

STORAGE_CODES = {"f32": JT_STORE_F32, "float32": JT_STORE_F32, "bf16": JT_STORE_BF16,
                 "bfloat16": JT_STORE_BF16, "f16": JT_STORE_F16, "float16": JT_STORE_F16}


# ---- struct mirrors --------------------------------------------------------
class Blend(C.Structure):
    _fields_ = [("pair", i32), ("form", i32), ("wa", f32), ("wb", f32), ("sa", f32), ("sb", f32),
                ("pad0", i32), ("pad1", i32)]


BLEND_DTYPE = np.dtype([("pair", "<i4"), ("form", "<i4"), ("wa", "<f4"), ("wb", "<f4"),
                        ("sa", "<f4"), ("sb", "<f4"), ("pad0", "<i4"), ("pad1", "<i4")])


class GridField(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("bounds_mode", i32),
                ("origin", f32 * 3), ("spacing", f32 * 3), ("inv_spacing", f32 * 3), ("valid_hi", f32 * 3),
                ("storage", i32), ("n_pairs", i32), ("pair_stride", i64), ("pairs", vp),
                ("tile_base", vp), ("tiles", i32 * 3), ("pad_tiles", i32)]


class OctreeNode(C.Structure):
    _fields_ = [("cx", f32), ("cy", f32), ("cz", f32), ("is_leaf", i32), ("children", i32 * 8),
                ("elem_offset", i32), ("elem_count", i32), ("pad0", i32), ("pad1", i32)]


OCTREE_NODE_DTYPE = np.dtype([("c", "<f4", (3,)), ("is_leaf", "<i4"), ("children", "<i4", (8,)),
                              ("elem_offset", "<i4"), ("elem_count", "<i4"), ("pad", "<i4", (2,))])


class MeshField(C.Structure):
    _fields_ = [("n_points", i32), ("n_tets", i32), ("n_nodes", i32), ("max_depth", i32),
                ("storage", i32), ("n_pairs", i32), ("near_degenerate", i32), ("pad", i32), ("pair_stride", i64),
                ("points", vp), ("tet_box", vp), ("tet_geom", vp), ("nodes", vp), ("elems", vp),
                ("pairs", vp), ("desc", vp), ("dtab", vp)]


class NearestField(C.Structure):
    _fields_ = [("n_points", i32), ("cells", i32 * 3), ("origin", f32 * 3), ("inv_cell", f32 * 3),
                ("storage", i32), ("n_pairs", i32), ("pair_stride", i64),
                ("points", vp), ("point_ids", vp), ("cell_start", vp), ("pairs", vp)]


class FemField(C.Structure):
    _fields_ = [("nearest", NearestField), ("n_tets", i32), ("grid_size", i32 * 3), ("grid_min", f32 * 3),
                ("cell_size", f32 * 3), ("tet_box", vp), ("tet_geom", vp), ("cell_start", vp), ("cell_elems", vp),
                ("sub_div", i32), ("near_degenerate", i32), ("sub_start", vp), ("sub_elems", vp)]


class Field(C.Structure):
    _fields_ = [("kind", i32), ("pad", i32), ("grid", C.POINTER(GridField)),
                ("mesh", C.POINTER(MeshField)), ("nearest", C.POINTER(NearestField)), ("fem", C.POINTER(FemField))]


class Boundary(C.Structure):
    _fields_ = [("axis_kind", i32 * 3), ("absorbing_joint", i32), ("lo", f32 * 3), ("hi", f32 * 3),
                ("outside_value", f32), ("inlet_mode", i32), ("inlet_axis", i32),
                ("inlet_positive", i32), ("inlet_res", i32 * 2), ("inlet_nudge", f32),
                ("inlet_coords", vp * 2)]


class TrackParams(C.Structure):
    _fields_ = [("integrator", i32), ("arith", i32), ("n_particles", i32), ("step_begin", i32),
                ("step_end", i32), ("dt", f32), ("dt_half", f32), ("dt_sixth", f32),
                ("schedule", vp), ("schedule_stride", i64), ("ens_offsets", vp), ("n_ens", i32),
                ("block_size", i32), ("pos", vp), ("comp", vp), ("traj", vp), ("vel", vp),
                ("record_every", i32), ("record_compact", i32), ("row_base", i32), ("n_rows", i32),
                ("status", vp), ("ids", vp), ("path", vp)]


class SortGrid(C.Structure):
    _fields_ = [("origin", f32 * 3), ("inv_cell", f32 * 3), ("bits", i32), ("order", i32)]


class AdjointParams(C.Structure):
    _fields_ = [("n_particles", i32), ("step_begin", i32), ("step_end", i32), ("dt", f32), ("dt_half", f32),
                ("dt_sixth", f32), ("pad", i32), ("schedule", vp), ("ckpt", vp), ("lambda_", vp), ("grad", vp),
                ("work", vp), ("work_bytes", i64), ("stage", vp)]


JT_ORDER_MORTON, JT_ORDER_LINEAR = 0, 1
JT_SPH_CUBIC, JT_SPH_WENDLAND, JT_SPH_GAUSSIAN = 0, 1, 2


class SphParams(C.Structure):
    _fields_ = [("dims", i32), ("kernel", i32), ("n_particles", i32), ("n_queries", i32), ("radius", f32),
                ("h_const", f32), ("grid", SortGrid), ("reach", i32 * 3), ("packed", i32), ("particles", vp),
                ("masses", vp), ("h", vp), ("cell_end", vp), ("queries", vp), ("out", vp), ("counters", vp)]


class KdeParams(C.Structure):
    _fields_ = [("dims", i32), ("n_particles", i32), ("res", i32 * 3), ("half_inv_h2", f32), ("radius", f32),
                ("grid", SortGrid), ("axis", vp * 3), ("particles", vp), ("cell_end", vp), ("out", vp),
                ("counters", vp)]


class FemGridInfo(C.Structure):
    _fields_ = [("n_cells", i64), ("n_entries", i64), ("n_sub_cells", i64), ("n_sub_entries", i64),
                ("max_per_cell", i32), ("pad", i32)]


class OctreeInfo(C.Structure):
    _fields_ = [("n_nodes", i32), ("n_elem_entries", i32), ("max_elems", i32), ("max_tree_depth", i32),
                ("n_leaves", i32), ("pad", i32)]


STRUCTS = [Blend, GridField, OctreeNode, MeshField, NearestField, Field, Boundary, TrackParams, SortGrid, SphParams,
           KdeParams, AdjointParams, OctreeInfo, FemField]


class JTError(RuntimeError):
    """A device-side failure reported by the native library."""


_lib = None


def library_path() -> Path:
    """The in-tree library, or the file named by JAXTRACE_GB300_LIB (a tuning
    variant built by ``_build.build(defines=..., out=...)``)."""
    alt = os.environ.get("JAXTRACE_GB300_LIB")
    return Path(alt) if alt else _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load the native library (building it in-tree on first use)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        if not build_if_missing or os.environ.get("JAXTRACE_GB300_NO_BUILD"):
            raise ImportError(f"native library {path} is missing; run jaxtrace_gb300._build.build()")
        _build.build()
    lib = C.CDLL(str(path))
    P = C.POINTER
    sig = {
        "jt_abi_version": (i32, []),
        "jt_last_error": (C.c_char_p, []),
        "jt_struct_sizes": (i32, [P(i64), i32]),
        "jt_track": (i32, [P(Field), P(Boundary), P(TrackParams), vp]),
        "jt_field_sample": (i32, [P(Field), P(Blend), i32, vp, vp, i32, vp, vp]),
        "jt_boundary_apply": (i32, [P(Boundary), vp, i32, vp]),
        "jt_integrator_step": (i32, [P(Field), P(Blend), i32, i32, f32, vp, vp, vp, i32, vp, vp]),
        "jt_octree_build": (i32, [vp, i32, vp, i32, i32, i32, P(vp), P(OctreeInfo)]),
        "jt_octree_fetch": (i32, [vp, vp, vp, vp, vp, vp]),
        "jt_octree_build_device": (i32, [vp, i32, vp, i32, i32, i32, vp, vp, vp, vp, P(vp), P(OctreeInfo)]),
        "jt_octree_fetch_device": (i32, [vp, vp, vp, vp]),
        "jt_octree_free_device": (None, [vp, vp]),
        "jt_mark_near_degenerate": (i32, [vp, vp, i32, P(i32), vp]),
        "jt_pair_log_ratio": (i32, [vp, vp, i32, f32, vp, vp, vp]),
        "jt_fem_grid_build": (i32, [vp, i32, vp, i32, vp, vp, vp, i32, vp, P(vp), P(FemGridInfo)]),
        "jt_fem_grid_fetch": (i32, [vp, vp, vp, vp, vp]),
        "jt_fem_grid_free": (None, [vp]),
        "jt_fem_grid_build_device": (i32, [vp, i32, vp, i32, vp, vp, vp, i32, vp, vp, vp, vp, P(vp), P(FemGridInfo)]),
        "jt_fem_grid_fetch_device": (i32, [vp, vp, vp, vp, vp, vp]),
        "jt_fem_grid_free_device": (None, [vp, vp]),
        "jt_octree_free": (None, [vp]),
        "jt_cell_sort_workspace_bytes": (C.c_size_t, [i32, i32]),
        "jt_cell_sort": (i32, [P(SortGrid), i32, vp, vp, vp, vp, vp, vp, vp, C.c_size_t, vp]),
        "jt_unpermute": (i32, [i32, vp, vp, vp, vp]),
        "jt_cell_sort_noalloc": (i32, [P(SortGrid), i32, vp, vp, vp, vp, vp, vp, vp]),
        "jt_cell_list": (i32, [P(SortGrid), i32, vp, vp, vp, vp, vp, C.c_size_t, vp]),
        "jt_sph_density": (i32, [P(SphParams), vp]),
        "jt_kde_grid": (i32, [P(KdeParams), vp]),
        "jt_kde_points": (i32, [P(KdeParams), vp, i32, vp, vp]),
        "jt_adjoint_rk4": (i32, [P(Field), P(Boundary), P(AdjointParams), vp]),
        "jt_adjoint_workspace_bytes": (C.c_size_t, [i64, i32]),
        "jt_stage_fields": (i32, [P(Field), vp, vp, i32, i32, vp, vp]),
        "jt_stage_tile_fields": (i32, [P(Field), vp, vp, i32, vp, vp]),
        "jt_set_allocator": (i32, [ALLOC_FN, FREE_FN, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.jt_abi_version() != ABI_VERSION:
        raise ImportError("jaxtrace_gb300 native library ABI mismatch")
    # every descriptor this module hands the library must have the C layout's
    # size: a shorter mirror would let the library read past it
    out = (i64 * 16)()
    n = lib.jt_struct_sizes(out, 16)
    want = [C.sizeof(st) for st in STRUCTS]
    if n != len(want) or [int(out[k]) for k in range(n)] != want:
        raise ImportError(f"jaxtrace_gb300 struct layouts differ from the library's: {list(out)[:max(n, 0)]} vs {want}")
    _lib = lib
    use_torch_allocator(lib)
    return lib


# jt_set_allocator callback types: alloc(bytes, stream, ctx) -> ptr, free(ptr, stream, ctx)
ALLOC_FN = C.CFUNCTYPE(vp, C.c_size_t, vp, vp)
FREE_FN = C.CFUNCTYPE(None, vp, vp, vp)
_ALLOCATOR = []       # the installed callbacks, kept alive while the library holds them


def _torch_alloc(nbytes, stream, ctx):
    try:
        import torch
        return torch.cuda.caching_allocator_alloc(max(int(nbytes), 1), stream=int(stream or 0))
    except Exception:      # noqa: BLE001 -- NULL is the allocator's failure value; the call reports it
        return None


def _torch_free(ptr, stream, ctx):
    if ptr:
        import torch
        torch.cuda.caching_allocator_delete(int(ptr))


def use_torch_allocator(lib=None) -> bool:
    """Route the library's own device scratch (the device octree and hash-grid
    builds, the near-degenerate count) through torch's caching allocator, so
    that all device memory the library touches belongs to the caller's pool
    (jt_set_allocator).  Done on load when CUDA is visible; returns whether it
    was installed."""
    import torch
    if not torch.cuda.is_available():
        return False
    lib = lib or load()
    if not _ALLOCATOR:
        _ALLOCATOR.extend([ALLOC_FN(_torch_alloc), FREE_FN(_torch_free)])
    check(lib.jt_set_allocator(_ALLOCATOR[0], _ALLOCATOR[1], None))
    return True


def check(rc: int) -> int:
    """Map a JT_* return code to the reference's exception types."""
    if rc >= 0:
        return rc
    msg = load().jt_last_error().decode(errors="replace")
    if rc == JT_ERR_INVALID:
        raise ValueError(msg)
    if rc == JT_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == JT_ERR_NOMEM:
        raise MemoryError(msg)
    raise JTError(msg)


def struct_sizes() -> list[int]:
    out = (i64 * 16)()
    n = check(load().jt_struct_sizes(out, 16))
    return [int(out[i]) for i in range(n)]


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def ptr(t) -> C.c_void_p:
    """Device pointer of a torch tensor (or None)."""
    if t is None:
        return C.c_void_p(None)
    return C.c_void_p(t.data_ptr())
