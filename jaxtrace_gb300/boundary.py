"""Boundary conditions of the GPU path (tracking/boundary.py of JAXTrace).

The factories keep the reference names and signatures and return callable
descriptor objects: calling one applies the boundary to (N,3) positions on
the GPU; ``create_tracker`` fuses the same descriptor into the tracking
kernel's per-step epilogue.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import _lib as L

F32 = np.float32


def _ensure_bounds_shape(bounds) -> np.ndarray:
    """Bounds in any accepted form -> (2,3) float32 (boundary.py:39-86)."""
    b = np.asarray(bounds, dtype=F32)
    if b.ndim == 1:
        if len(b) == 4:
            b = np.array([[b[0], b[2], 0.0], [b[1], b[3], 0.0]], dtype=F32)
        elif len(b) == 6:
            b = np.array([[b[0], b[2], b[4]], [b[1], b[3], b[5]]], dtype=F32)
        else:
            raise ValueError(f"1D bounds must have 4 or 6 elements, got {len(b)}")
    elif b.ndim == 2:
        if b.shape == (2, 2):
            b = np.array([[b[0, 0], b[1, 0], 0.0], [b[0, 1], b[1, 1], 0.0]], dtype=F32)
        elif b.shape == (2, 3):
            pass
        elif b.shape == (3, 2):
            b = b.T
        else:
            raise ValueError(f"2D bounds must have shape (2,2), (2,3), or (3,2), got {b.shape}")
    else:
        raise ValueError(f"Bounds must be 1D or 2D array, got {b.ndim}D")
    if not np.all(b[0] < b[1]):
        raise ValueError(f"Invalid bounds: min {b[0]} >= max {b[1]}")
    return np.ascontiguousarray(b.astype(F32))


class BoundaryDescriptor:
    """A boundary callable backed by the jt_boundary descriptor."""

    def __init__(self, name: str, bounds: np.ndarray, axis_kind=(0, 0, 0), absorbing_joint=False,
                 outside_value=np.nan, inlet=None):
        self.__name__ = name
        self.bounds = bounds
        self.axis_kind = tuple(int(k) for k in axis_kind)
        self.absorbing_joint = bool(absorbing_joint)
        self.outside_value = F32(outside_value)
        self.inlet = inlet
        self._dev = None

    def jt_boundary(self):
        if self._dev is not None:
            return self._dev[0]
        b = L.Boundary()
        b.axis_kind[:] = list(self.axis_kind)
        b.absorbing_joint = int(self.absorbing_joint)
        b.lo[:] = [float(v) for v in self.bounds[0]]
        b.hi[:] = [float(v) for v in self.bounds[1]]
        b.outside_value = float(self.outside_value)
        keep = []
        if self.inlet is not None:
            import torch
            if not torch.cuda.is_available():
                raise RuntimeError("jaxtrace_gb300 boundaries run on a CUDA GPU; none is visible")
            inl = self.inlet
            b.inlet_mode = L.JT_INLET_GRID
            b.inlet_axis = inl["axis"]
            b.inlet_positive = int(inl["positive"])
            b.inlet_res[:] = [len(inl["coords"][0]), len(inl["coords"][1])]
            b.inlet_nudge = float(inl["nudge"])
            for q in range(2):
                t = torch.from_numpy(inl["coords"][q]).cuda()
                keep.append(t)
                b.inlet_coords[q] = t.data_ptr()
        self._dev = (b, keep)
        return b

    def __call__(self, positions):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("jaxtrace_gb300 boundaries run on a CUDA GPU; none is visible")
        is_tensor = isinstance(positions, torch.Tensor)
        if is_tensor:
            x = positions.to(device="cuda", dtype=torch.float32).contiguous().clone()
        else:
            x = torch.from_numpy(np.ascontiguousarray(np.asarray(positions, dtype=F32).reshape(-1, 3))).cuda()
        b = self.jt_boundary()
        L.check(L.load().jt_boundary_apply(C.byref(b), L.ptr(x), x.shape[0], L.stream_ptr()))
        return x if is_tensor else x.cpu().numpy()

    def __repr__(self):
        return f"<{self.__name__} bounds={self.bounds.tolist()}>"


def periodic_boundary(bounds) -> BoundaryDescriptor:
    """boundary.py:215-242: lo + mod(x - lo, width) on every axis."""
    b = _ensure_bounds_shape(bounds)
    return BoundaryDescriptor("_periodic_bc", b, (L.JT_BC_PERIODIC,) * 3)


def reflective_boundary(bounds) -> BoundaryDescriptor:
    """boundary.py:245-272: sawtooth reflection with period 2*width."""
    b = _ensure_bounds_shape(bounds)
    return BoundaryDescriptor("_reflective_bc", b, (L.JT_BC_REFLECTIVE,) * 3)


def clamping_boundary(bounds) -> BoundaryDescriptor:
    """boundary.py:275-302: clip to [lo, hi]."""
    b = _ensure_bounds_shape(bounds)
    return BoundaryDescriptor("_clamping_bc", b, (L.JT_BC_CLAMP,) * 3)


def absorbing_boundary_factory(bounds, outside_value: float = np.nan) -> BoundaryDescriptor:
    """boundary.py:305-337: particles outside on any axis become outside_value."""
    b = _ensure_bounds_shape(bounds)
    return BoundaryDescriptor("_absorbing_bc", b, (L.JT_BC_ABSORBING,) * 3, absorbing_joint=True,
                              outside_value=outside_value)


_MIXED_KINDS = {"periodic": L.JT_BC_PERIODIC, "reflective": L.JT_BC_REFLECTIVE,
                "clamping": L.JT_BC_CLAMP, "absorbing": L.JT_BC_ABSORBING}


def mixed_boundary(bounds, conditions: Dict[str, str]) -> BoundaryDescriptor:
    """boundary.py:377-438: one condition per axis (missing axes: periodic)."""
    b = _ensure_bounds_shape(bounds)
    kinds = []
    for axis in ("x", "y", "z"):
        c = conditions.get(axis, "periodic")
        if c not in _MIXED_KINDS:
            raise ValueError(f"Unknown condition type: {c}")
        kinds.append(_MIXED_KINDS[c])
    return BoundaryDescriptor("_mixed_bc", b, kinds, outside_value=np.nan)


def no_boundary() -> BoundaryDescriptor:
    """boundary.py:941-946: identity."""
    return BoundaryDescriptor("_no_bc", np.array([[0, 0, 0], [1, 1, 1]], dtype=F32), (L.JT_BC_NONE,) * 3)


def unit_box_periodic() -> BoundaryDescriptor:
    return periodic_boundary([[0, 0, 0], [1, 1, 1]])


def unit_box_reflective() -> BoundaryDescriptor:
    return reflective_boundary([[0, 0, 0], [1, 1, 1]])


def continuous_inlet_boundary_factory(bounds, flow_axis: str = "x", flow_direction: str = "positive",
                                      inlet_distribution: str = "uniform",
                                      concentrations: Optional[Dict[str, int]] = None) -> BoundaryDescriptor:
    """boundary.py:1444-1601: exited particles re-enter at the inlet.

    The grid-preserving replacement (``inlet_distribution='grid'`` with
    ``concentrations``) snaps each exited particle to the nearest point of the
    float32 ``linspace`` lattice of the two other axes (ties to the lower
    index), puts it on the inlet plane, nudges backward crossers 0.1 % inside
    and mirrors the other axes once.  The random 'uniform'/'gaussian'
    replacements of the reference draw from NumPy's global generator and are
    not offered on the GPU path.
    """
    b = _ensure_bounds_shape(bounds)
    axis_map = {"x": 0, "y": 1, "z": 2}
    if flow_axis not in axis_map:
        raise ValueError(f"flow_axis must be 'x', 'y', or 'z', got {flow_axis}")
    a = axis_map[flow_axis]
    if not (inlet_distribution == "grid" and concentrations is not None):
        raise NotImplementedError(
            "continuous inlet on the GPU path needs inlet_distribution='grid' with concentrations; "
            "the reference's random replacement uses NumPy's global RNG")
    names = ["x", "y", "z"]
    others = [i for i in range(3) if i != a]
    coords = []
    for i in others:
        res = max(1, int(concentrations[names[i]]))
        coords.append(np.linspace(b[0, i], b[1, i], res, dtype=F32))   # boundary.py:1295
    positive = flow_direction == "positive"
    amin, amax = b[0, a], b[1, a]
    # boundary.py:1583/:1587 in float32: axis_min + 0.001*(axis_max-axis_min)
    nudge = (amin + 0.001 * (amax - amin)) if positive else (amax - 0.001 * (amax - amin))
    inlet = {"axis": a, "positive": positive, "coords": coords, "nudge": F32(nudge)}
    d = BoundaryDescriptor("_continuous_inlet_bc", b, (L.JT_BC_NONE,) * 3, inlet=inlet)
    d.flow_axis, d.flow_direction = flow_axis, flow_direction
    d.inlet_distribution, d.concentrations = inlet_distribution, dict(concentrations)
    return d


__all__ = ["periodic_boundary", "reflective_boundary", "clamping_boundary", "absorbing_boundary_factory",
           "mixed_boundary", "continuous_inlet_boundary_factory", "no_boundary", "unit_box_periodic",
           "unit_box_reflective", "BoundaryDescriptor"]


def clamp_to_bounds(x, bounds):
    """Positions clipped to [lo, hi] per axis (boundary.py:127-144), on the
    device through the clamping boundary kernel."""
    return clamping_boundary(bounds)(x)


def reflect_boundary(x, bounds):
    """Sawtooth reflection into [lo, hi] per axis (boundary.py:147-172), on
    the device through the reflective boundary kernel (the same mapping)."""
    return reflective_boundary(bounds)(x)
