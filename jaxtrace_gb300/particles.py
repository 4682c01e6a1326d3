"""Trajectory container with the reference layout (tracking/particles.py:82-129):
positions (T,N,3) float32, times (T,) float32, optional velocities (T,N,3)."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, Optional

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
    def duration(self) -> float:
        return float(self.times[-1] - self.times[0]) if self.T > 1 else 0.0

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
        return np.linalg.norm(self.positions[-1] - self.positions[0], axis=1)
