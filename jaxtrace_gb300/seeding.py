"""Seed generators used to build tracking inputs (tracking/seeding.py:140-247).

These are one-off host array constructions with the reference's NumPy
semantics (the NumPy branch of ``random_seeds``).
"""
from __future__ import annotations

import numpy as np

from .boundary import _ensure_bounds_shape

F32 = np.float32


def random_seeds(n: int, bounds, rng_seed: int = 0, dtype=np.float32) -> np.ndarray:
    """seeding.py:140-182 (NumPy branch): lo + U[0,1) * (hi - lo) in float32."""
    if n <= 0:
        return np.zeros((0, 3), dtype=F32)
    b = _ensure_bounds_shape(bounds)
    np.random.seed(rng_seed)
    u = np.random.uniform(0, 1, size=(n, 3)).astype(F32)
    return (b[0] + u * (b[1] - b[0])).astype(F32)


def uniform_grid_seeds(resolution, bounds, include_boundaries: bool = True) -> np.ndarray:
    """seeding.py:185-247: ij meshgrid of float32 linspace axes."""
    b = _ensure_bounds_shape(bounds)
    if isinstance(resolution, int):
        nx = ny = nz = resolution
    elif len(resolution) == 2:
        (nx, ny), nz = resolution, 1
    elif len(resolution) == 3:
        nx, ny, nz = resolution
    else:
        raise ValueError(f"Resolution must be int or tuple of 2-3 ints, got {resolution}")
    x_min, y_min, z_min = b[0]
    x_max, y_max, z_max = b[1]
    if include_boundaries:
        xs = np.linspace(x_min, x_max, nx, dtype=F32)
        ys = np.linspace(y_min, y_max, ny, dtype=F32)
        zs = np.linspace(z_min, z_max, nz, dtype=F32) if nz > 1 else np.array([z_min], dtype=F32)
    else:
        dx = (x_max - x_min) / (nx + 1)
        dy = (y_max - y_min) / (ny + 1)
        dz = (z_max - z_min) / (nz + 1) if nz > 1 else 0.0
        xs = np.linspace(x_min + dx, x_max - dx, nx, dtype=F32)
        ys = np.linspace(y_min + dy, y_max - dy, ny, dtype=F32)
        zs = np.linspace(z_min + dz, z_max - dz, nz, dtype=F32) if nz > 1 else np.array([z_min], dtype=F32)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    return np.column_stack([X.ravel(), Y.ravel(), Z.ravel()]).astype(F32)
