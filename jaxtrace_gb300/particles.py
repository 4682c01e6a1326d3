"""Trajectory container with the reference layout (tracking/particles.py:82-129):
positions (T,N,3) float32, times (T,) float32, optional velocities (T,N,3).

The statistics follow Trajectory.compute_* and compute_trajectory_statistics
(tracking/particles.py:279-340, :401-416, :862-924) in the same float32
NumPy arithmetic.  ``path_length`` (optional) is the per-particle path length
the tracking kernel accumulates over every step when the tracker was created
with ``record_path_length=True``: the value compute_path_length gives on a
trajectory recorded at every step, available without recording one."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, Optional, Tuple

import numpy as np

F32 = np.float32


def _ensure_trajectory_shape(a) -> np.ndarray:
    a = np.asarray(a, dtype=F32)
    if a.ndim == 2:
        a = a[None]
    if a.ndim != 3:
        raise ValueError(f"Trajectory arrays must be (T,N,3), got {a.shape}")
    if a.shape[2] == 2:
        a = np.concatenate([a, np.zeros(a.shape[:2] + (1,), dtype=F32)], axis=2)
    return a


@dataclass
class Trajectory:
    positions: np.ndarray
    times: np.ndarray
    velocities: Optional[np.ndarray] = None
    metadata: Dict[str, Any] = field(default_factory=dict)
    path_length: Optional[np.ndarray] = None

    def __post_init__(self):
        self.positions = _ensure_trajectory_shape(self.positions)
        self.times = np.asarray(self.times, dtype=F32)
        self.T, self.N, self.D = self.positions.shape
        if self.D != 3:
            raise ValueError("Positions must have 3 spatial dimensions after processing")
        if self.times.shape != (self.T,):
            raise ValueError(f"Times shape {self.times.shape} doesn't match trajectory length {self.T}")
        if self.velocities is not None:
            self.velocities = _ensure_trajectory_shape(self.velocities)
            if self.velocities.shape != (self.T, self.N, 3):
                raise ValueError(f"Velocities shape {self.velocities.shape} doesn't match positions shape "
                                 f"{self.positions.shape}")
        self.metadata.setdefault("format_version", "1.0")
        self.metadata.setdefault("dtype", "float32")
        self.metadata.setdefault("coordinate_system", "cartesian")

    def __len__(self) -> int:
        return self.T

    @property
    def num_particles(self) -> int:
        return self.N

    @property
    def num_timesteps(self) -> int:
        return self.T

    @property
    def duration(self) -> float:
        return float(self.times[-1] - self.times[0]) if self.T > 1 else 0.0

    @property
    def dt_mean(self) -> float:
        return float(np.mean(np.diff(self.times))) if self.T > 1 else 0.0

    def get_positions_at_time(self, t: float) -> np.ndarray:
        return self.positions[int(np.argmin(np.abs(self.times - t)))]

    def get_particle_trajectory(self, particle_idx: int) -> np.ndarray:
        return self.positions[:, particle_idx, :]

    def get_final_positions(self) -> np.ndarray:
        return self.positions[-1]

    def get_initial_positions(self) -> np.ndarray:
        return self.positions[0]

    def memory_usage_mb(self) -> float:
        n = self.positions.nbytes + self.times.nbytes
        if self.velocities is not None:
            n += self.velocities.nbytes
        return n / 1024 ** 2

    def compute_displacement(self) -> np.ndarray:
        """|x_T - x_0| per particle, float32 (particles.py:279-294)."""
        if self.T < 2:
            return np.zeros(self.N, dtype=F32)
        return np.linalg.norm(self.positions[-1] - self.positions[0], axis=1).astype(F32)

    def compute_path_length(self) -> np.ndarray:
        """Sum over recorded rows of |x_{t+1} - x_t|, float32 (particles.py:296-313)."""
        if self.T < 2:
            return np.zeros(self.N, dtype=F32)
        steps = np.linalg.norm(np.diff(self.positions, axis=0), axis=2)
        return np.sum(steps, axis=0).astype(F32)

    def compute_speeds(self) -> np.ndarray:
        """(T-1, N) speeds: |v| of the stored velocities without the last row,
        or |dx/dt| of consecutive rows (particles.py:315-340)."""
        if self.T < 2:
            return np.zeros((0, self.N), dtype=F32)
        if self.velocities is not None:
            return np.linalg.norm(self.velocities, axis=2)[:-1].astype(F32)
        rates = np.diff(self.positions, axis=0) / np.diff(self.times)[:, None, None]
        return np.linalg.norm(rates, axis=2).astype(F32)

    def get_bounds(self) -> Tuple[np.ndarray, np.ndarray]:
        """Per-axis minimum and maximum over every row (particles.py:401-416)."""
        flat = self.positions.reshape(-1, 3)
        return np.min(flat, axis=0), np.max(flat, axis=0)

    def export_to_vtk(self, filename: str, time_indices=None, encoding: str = "appended") -> None:
        """Write the selected rows as one .vtu of vertex cells
        (particles.py:448-539): points in row-major (row, particle) order,
        point arrays Velocity (stored, or the float32 difference quotient to
        the previous row, zero on row 0), Time, ParticleID and Speed.
        Written by ``vtk_io.write_vtu``; no VTK library needed."""
        from .vtk_io import write_vtu
        idx = np.arange(self.T) if time_indices is None else np.asarray(list(time_indices), dtype=np.int64)
        pos = self.positions[idx].reshape(-1, 3)
        if self.velocities is not None:
            vel = self.velocities[idx]
        else:
            vel = np.zeros((len(idx), self.N, 3), dtype=F32)
            later = idx > 0
            if later.any():
                t = idx[later]
                dt = (self.times[t] - self.times[t - 1]).astype(F32)
                vel[later] = (self.positions[t] - self.positions[t - 1]) / dt[:, None, None]
        vel = vel.reshape(-1, 3).astype(F32)
        times = np.repeat(self.times[idx], self.N).astype(F32)
        ids = np.tile(np.arange(self.N, dtype=np.int32), len(idx))
        speed = np.linalg.norm(vel, axis=1).astype(F32)
        write_vtu(filename, pos, point_data={"Velocity": vel, "Time": times, "ParticleID": ids, "Speed": speed},
                  encoding=encoding, vertices=True)

    def subsample_time(self, step: int = 2) -> "Trajectory":
        return Trajectory(positions=self.positions[::step], times=self.times[::step],
                          velocities=self.velocities[::step] if self.velocities is not None else None,
                          metadata={**self.metadata, "subsampled": step})


def _summary(a: np.ndarray) -> Dict[str, float]:
    return {"mean": float(np.mean(a)), "std": float(np.std(a)), "min": float(np.min(a)), "max": float(np.max(a))}


def compute_trajectory_statistics(trajectory: Trajectory) -> Dict[str, Any]:
    """Basic sizes, displacement / path-length / speed summaries and bounds
    (particles.py:862-924)."""
    tr = trajectory
    stats: Dict[str, Any] = {"basic": {"num_particles": tr.N, "num_timesteps": tr.T, "duration": tr.duration,
                                       "dt_mean": tr.dt_mean, "memory_mb": tr.memory_usage_mb()}}
    if tr.T > 1:
        stats["displacement"] = _summary(tr.compute_displacement())
        stats["path_length"] = _summary(tr.compute_path_length())
        speeds = tr.compute_speeds()
        if speeds.size > 0:
            stats["speed"] = _summary(speeds)
        lo, hi = tr.get_bounds()
        stats["bounds"] = {"min": lo.tolist(), "max": hi.tolist(), "extent": (hi - lo).tolist()}
    return stats
