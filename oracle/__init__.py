"""CPU oracle of the tracking path -- TEST INFRASTRUCTURE ONLY.

This package checks the GPU library; it is imported by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` and by
nothing in ``jaxtrace_gb300``.  It holds:

* ``jt_oracle.c`` -- a C restatement of the reference arithmetic (float32
  mode bit-compatible with JAXTrace's NumPy path, float64 mode for error
  figures), compiled by ``build()`` with gcc (no FMA contraction, OpenMP);
* ``jaxshim/`` -- a NumPy stand-in for ``jax`` so the reference's octree
  modules (which import jax unconditionally) can run in this container
  when golden fixtures are regenerated;
* ``reference.py`` -- helpers that run the reference itself (only where
  its sources are present) to produce golden fixtures.

Parity status: the float32 restatement is pinned to golden vectors produced
by running the reference (tests/golden/make_golden.py); the reference's own
test suite pins no numeric result on this path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "jt_oracle.c"

ORC_F32, ORC_F64 = 0, 1
EX = {"constant": 0, "linear": 1, "zero": 2, "nan": 3}
GRID = {"clamp": 0, "zero": 1, "nan": 2, "periodic": 3}
INTEG = {"euler": 0, "rk2": 1, "rk4": 2}
BC = {"none": 0, "periodic": 1, "reflective": 2, "clamping": 3, "clamp": 3, "absorbing": 4}
FIELD_GRID, FIELD_MESH, FIELD_FEM = 1, 2, 4
SEM = {"numpy": 0, "jax": 1}

vp, i32, i64, f32, f64 = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_double


class OrcField(C.Structure):
    _fields_ = [("n_snap", i32), ("snap_times", vp), ("data", vp), ("n_nodes", i32), ("extrapolation", i32),
                ("semantics", i32), ("kind", i32), ("nx", i32), ("ny", i32), ("nz", i32), ("bounds_mode", i32),
                ("gx", vp), ("gy", vp), ("gz", vp), ("points", vp), ("conn", vp), ("n_tets", i32),
                ("elem_bounds", vp), ("nodes_min", vp), ("nodes_max", vp), ("nodes_elements", vp),
                ("max_elems", i32), ("nodes_children", vp), ("nodes_is_leaf", vp), ("max_depth", i32),
                ("fem_grid_size", i32 * 3), ("fem_grid_min", f32 * 3), ("fem_cell_size", f32 * 3),
                ("fem_cell_elements", vp), ("fem_max_per_cell", i32)]


class OrcBoundary(C.Structure):
    _fields_ = [("axis_kind", i32 * 3), ("absorbing_joint", i32), ("lo", f32 * 3), ("hi", f32 * 3),
                ("outside_value", f32), ("inlet_axis", i32), ("inlet_positive", i32), ("inlet_res", i32 * 2),
                ("lattice", vp * 2)]


class OrcRun(C.Structure):
    _fields_ = [("precision", i32), ("integrator", i32), ("step_times", vp), ("n_times", i32), ("dt", f64),
                ("n_threads", i32), ("fallback_count", i64), ("wrapped_count", i64), ("cell_sig", vp), ("reseed", vp)]


def build(force: bool = False) -> Path:
    """Compile jt_oracle.c with gcc: -O2, no FMA contraction, OpenMP."""
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-o", str(tmp), str(SRC), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.orc_track.argtypes = [C.POINTER(OrcField), C.POINTER(OrcBoundary), C.POINTER(OrcRun), i32, vp, vp, vp, vp,
                                  vp]
        lib.orc_track.restype = i32
        lib.orc_sample.argtypes = [C.POINTER(OrcField), f64, i32, i32, i32, vp, vp, vp]
        lib.orc_sample.restype = i32
        lib.orc_boundary_apply.argtypes = [C.POINTER(OrcBoundary), i32, vp]
        lib.orc_boundary_apply.restype = i32
        lib.orc_blend_nodes.argtypes = [C.POINTER(OrcField), f64, i32, vp]
        lib.orc_blend_nodes.restype = i32
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


class GridSpec:
    """Structured time-series field for the oracle (keeps arrays alive)."""

    def __init__(self, data, times, gx, gy, gz, bounds_handling="clamp", extrapolation="constant",
                 semantics="numpy"):
        gx, gy, gz = (np.ascontiguousarray(np.asarray(g, np.float32)) for g in (gx, gy, gz))
        data = np.ascontiguousarray(np.asarray(data, np.float32).reshape(len(times), -1, 3))
        self.keep = [data, np.ascontiguousarray(np.asarray(times, np.float32)), gx, gy, gz]
        f = OrcField()
        f.n_snap = len(times)
        f.snap_times = _p(self.keep[1])
        f.data = _p(data)
        f.n_nodes = data.shape[1]
        f.extrapolation = EX[extrapolation]
        f.semantics = SEM[semantics]
        f.kind = FIELD_GRID
        f.nx, f.ny, f.nz = len(gx), len(gy), len(gz)
        f.bounds_mode = GRID[bounds_handling]
        f.gx, f.gy, f.gz = _p(gx), _p(gy), _p(gz)
        self.c = f


class MeshSpec:
    """Octree/P1 time-series field in the reference array layout."""

    def __init__(self, data, times, points, conn, elem_bounds, nodes_min, nodes_max, nodes_elements,
                 nodes_children, nodes_is_leaf, max_depth=12, extrapolation="constant"):
        arrs = dict(
            data=np.ascontiguousarray(np.asarray(data, np.float32).reshape(len(times), -1, 3)),
            times=np.ascontiguousarray(np.asarray(times, np.float32)),
            points=np.ascontiguousarray(np.asarray(points, np.float32)),
            conn=np.ascontiguousarray(np.asarray(conn, np.int32)),
            eb=np.ascontiguousarray(np.asarray(elem_bounds, np.float32)),
            nmin=np.ascontiguousarray(np.asarray(nodes_min, np.float32)),
            nmax=np.ascontiguousarray(np.asarray(nodes_max, np.float32)),
            nel=np.ascontiguousarray(np.asarray(nodes_elements, np.int32)),
            nch=np.ascontiguousarray(np.asarray(nodes_children, np.int32)),
            nleaf=np.ascontiguousarray(np.asarray(nodes_is_leaf, np.uint8)))
        self.keep = arrs
        f = OrcField()
        f.n_snap = len(times)
        f.snap_times, f.data = _p(arrs["times"]), _p(arrs["data"])
        f.n_nodes = arrs["points"].shape[0]
        f.extrapolation = EX[extrapolation]
        f.semantics = SEM["jax"]
        f.kind = FIELD_MESH
        f.points, f.conn, f.n_tets = _p(arrs["points"]), _p(arrs["conn"]), arrs["conn"].shape[0]
        f.elem_bounds, f.nodes_min, f.nodes_max = _p(arrs["eb"]), _p(arrs["nmin"]), _p(arrs["nmax"])
        f.nodes_elements, f.max_elems = _p(arrs["nel"]), arrs["nel"].shape[1]
        f.nodes_children, f.nodes_is_leaf, f.max_depth = _p(arrs["nch"]), _p(arrs["nleaf"]), int(max_depth)
        self.c = f


class NearestSpec:
    """Scattered nodes sampled by nearest node (TimeSeriesField)."""

    def __init__(self, data, times, points, extrapolation="constant", semantics="numpy"):
        arrs = dict(data=np.ascontiguousarray(np.asarray(data, np.float32).reshape(len(times), -1, 3)),
                    times=np.ascontiguousarray(np.asarray(times, np.float32)),
                    points=np.ascontiguousarray(np.asarray(points, np.float32)))
        self.keep = arrs
        f = OrcField()
        f.n_snap = len(times)
        f.snap_times, f.data = _p(arrs["times"]), _p(arrs["data"])
        f.n_nodes = arrs["points"].shape[0]
        f.extrapolation = EX[extrapolation]
        f.semantics = SEM[semantics]
        f.kind = 3
        f.points = _p(arrs["points"])
        self.c = f


def blend_nodes(field, t, t_is_f32=False):
    out = np.zeros((field.c.n_nodes, 3), np.float32)
    load().orc_blend_nodes(C.byref(field.c), float(t), int(t_is_f32), out.ctypes.data)
    return out


class BoundarySpec:
    def __init__(self, kinds=("none", "none", "none"), bounds=((0, 0, 0), (1, 1, 1)), absorbing_joint=False,
                 outside_value=np.nan, inlet_axis=-1, inlet_positive=True, lattices=None):
        b = OrcBoundary()
        b.axis_kind[:] = [BC[k] for k in kinds]
        b.absorbing_joint = int(absorbing_joint)
        bb = np.asarray(bounds, np.float32)
        b.lo[:] = [float(v) for v in bb[0]]
        b.hi[:] = [float(v) for v in bb[1]]
        b.outside_value = float(outside_value)
        b.inlet_axis = int(inlet_axis)
        b.inlet_positive = int(inlet_positive)
        self.keep = []
        if inlet_axis >= 0:
            for q in range(2):
                lat = np.ascontiguousarray(np.asarray(lattices[q], np.float32))
                self.keep.append(lat)
                b.lattice[q] = lat.ctypes.data
                b.inlet_res[q] = len(lat)
        self.c = b


class FemSpec:
    """Hash-grid FEM time-series field (fem_time_series.py:16-110) in the
    reference layout: grid_size, grid_min, float32 grid_cell_size, the
    (cells, max_per_cell) -1-padded cell_to_elements table and element_bounds
    as build_tetrahedral_mesh returns them."""

    def __init__(self, data, times, points, conn, grid_size, grid_min, grid_cell_size, cell_to_elements,
                 element_bounds, extrapolation="constant"):
        arrs = dict(
            data=np.ascontiguousarray(np.asarray(data, np.float32).reshape(len(times), -1, 3)),
            times=np.ascontiguousarray(np.asarray(times, np.float32)),
            points=np.ascontiguousarray(np.asarray(points, np.float32)),
            conn=np.ascontiguousarray(np.asarray(conn, np.int32)),
            eb=np.ascontiguousarray(np.asarray(element_bounds, np.float32)),
            cells=np.ascontiguousarray(np.asarray(cell_to_elements, np.int32)))
        self.keep = arrs
        f = OrcField()
        f.n_snap = len(times)
        f.snap_times, f.data = _p(arrs["times"]), _p(arrs["data"])
        f.n_nodes = arrs["points"].shape[0]
        f.extrapolation = EX[extrapolation]
        f.semantics = SEM["jax"]
        f.kind = FIELD_FEM
        f.points, f.conn, f.n_tets = _p(arrs["points"]), _p(arrs["conn"]), arrs["conn"].shape[0]
        f.elem_bounds = _p(arrs["eb"])
        f.fem_grid_size[:] = [int(v) for v in grid_size]
        f.fem_grid_min[:] = [float(v) for v in np.asarray(grid_min, np.float32)]
        f.fem_cell_size[:] = [float(v) for v in np.asarray(grid_cell_size, np.float32)]
        f.fem_cell_elements = _p(arrs["cells"])
        f.fem_max_per_cell = arrs["cells"].shape[1]
        self.c = f


def track(field, boundary, x0, step_times, dt, integrator="rk4", precision=ORC_F32, n_threads=0,
          record=False, reseed=False, cell_sig=False):
    """Run the oracle; returns (final positions, trajectory or None, run info).
    In float64 mode a float64 ``x0`` is used as given (no float32 rounding).
    With ``reseed`` the info holds ``"reseed"``: (n,3) int32, each particle's
    last continuous-inlet replacement (step, lattice index 0, lattice index 1),
    -1 where the inlet never replaced it.  With ``cell_sig`` (float64 mode,
    grid fields) the info holds ``"cell_sig"``: (n,) uint64, a hash of the
    cells every field evaluation fell in (a difference quotient whose two
    runs share it never straddles a cell face)."""
    lib = load()
    x64 = None
    if precision == ORC_F64 and np.asarray(x0).dtype == np.float64:
        x64 = np.ascontiguousarray(np.asarray(x0, np.float64).reshape(-1, 3))
    x0 = np.ascontiguousarray(np.asarray(x0, np.float32).reshape(-1, 3))
    st = np.ascontiguousarray(np.asarray(step_times, np.float32))
    n = x0.shape[0]
    r = OrcRun(precision=precision, integrator=INTEG[integrator], step_times=st.ctypes.data, n_times=len(st),
               dt=float(dt), n_threads=int(n_threads))
    out32 = np.zeros((n, 3), np.float32) if precision == ORC_F32 else None
    out64 = np.zeros((n, 3), np.float64) if precision == ORC_F64 else None
    traj = np.zeros((len(st), n, 3), np.float32) if (record and precision == ORC_F32) else None
    ev = np.full((n, 3), -1, np.int32) if reseed else None
    r.reseed = _p(ev)
    sig = np.zeros(n, np.uint64) if (cell_sig and precision == ORC_F64) else None
    r.cell_sig = _p(sig)
    rc = lib.orc_track(C.byref(field.c), C.byref(boundary.c), C.byref(r), n, x0.ctypes.data, _p(out32), _p(out64),
                       _p(traj), _p(x64))
    if rc != 0:
        raise RuntimeError("oracle rejected its arguments")
    out = out32 if precision == ORC_F32 else out64
    info = {"fallback_count": int(r.fallback_count), "wrapped_count": int(r.wrapped_count)}
    if reseed:
        info["reseed"] = ev
    if sig is not None:
        info["cell_sig"] = sig
    return out, traj, info


def sample(field, pos, t, t_is_f32=True, precision=ORC_F32):
    lib = load()
    pos = np.ascontiguousarray(np.asarray(pos, np.float32).reshape(-1, 3))
    m = pos.shape[0]
    o32 = np.zeros((m, 3), np.float32)
    o64 = np.zeros((m, 3), np.float64)
    fb = lib.orc_sample(C.byref(field.c), float(t), int(t_is_f32), precision, m, pos.ctypes.data, o32.ctypes.data,
                        o64.ctypes.data)
    return (o32 if precision == ORC_F32 else o64), fb


def boundary_apply(boundary, pos):
    lib = load()
    p = np.ascontiguousarray(np.asarray(pos, np.float32).reshape(-1, 3)).copy()
    if lib.orc_boundary_apply(C.byref(boundary.c), p.shape[0], p.ctypes.data) != 0:
        raise RuntimeError("oracle rejected its arguments")
    return p
