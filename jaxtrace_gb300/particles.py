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
import warnings
from typing import Any, Dict, List, Optional, Tuple, Union

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

    def __getitem__(self, key: Union[int, slice, tuple]) -> "Trajectory":
        """Rows (an int keeps the 3-D shape), a row slice, or (rows,
        particles) (particles.py:137-164)."""
        vel = self.velocities
        if isinstance(key, (int, np.integer)):
            k = int(key)
            return Trajectory(positions=self.positions[k:k + 1], times=self.times[k:k + 1],
                              velocities=vel[k:k + 1] if vel is not None else None, metadata=self.metadata.copy())
        if isinstance(key, slice):
            return Trajectory(positions=self.positions[key], times=self.times[key],
                              velocities=vel[key] if vel is not None else None, metadata=self.metadata.copy())
        if isinstance(key, tuple) and len(key) == 2:
            t_key, p_key = key
            return Trajectory(positions=self.positions[t_key, p_key], times=self.times[t_key],
                              velocities=vel[t_key, p_key] if vel is not None else None,
                              metadata=self.metadata.copy())
        raise TypeError(f"Invalid key type for Trajectory indexing: {type(key)}")

    def __repr__(self) -> str:
        return f"Trajectory(T={self.T}, N={self.N}, duration={self.duration:.3f}, memory={self.memory_usage_mb():.1f}MB)"

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

    def get_positions_at_time(self, t_idx: int) -> np.ndarray:
        """(N,3) copy of row t_idx (particles.py:189-206)."""
        if not 0 <= t_idx < self.T:
            raise IndexError(f"Time index {t_idx} out of range [0, {self.T})")
        return self.positions[t_idx].copy()

    def get_particle_trajectory(self, p_idx: int) -> Tuple[np.ndarray, np.ndarray]:
        """((T,3) positions, (T,) times) of particle p_idx (particles.py:208-227)."""
        if not 0 <= p_idx < self.N:
            raise IndexError(f"Particle index {p_idx} out of range [0, {self.N})")
        return self.positions[:, p_idx].copy(), self.times.copy()

    def extract_2d_slice(self, plane: str = "xy") -> "Trajectory":
        """The trajectory with the axis normal to ``plane`` zeroed, still
        (T,N,3) (particles.py:229-277)."""
        plane = plane.lower()
        axis = {"xy": 2, "xz": 1, "yz": 0}.get(plane)
        if axis is None:
            raise ValueError("plane must be 'xy', 'xz', or 'yz'")
        pos = self.positions.copy()
        pos[:, :, axis] = 0.0
        vel = None
        if self.velocities is not None:
            vel = self.velocities.copy()
            vel[:, :, axis] = 0.0
        return Trajectory(positions=pos, times=self.times.copy(), velocities=vel,
                          metadata={**self.metadata, "extracted_plane": plane})

    def to_jax(self) -> "Trajectory":
        """A float32 copy (particles.py:343-359; JAX is not used here, as in
        the reference without JAX)."""
        warnings.warn("JAX not available, returning copy with NumPy arrays")
        return self.to_numpy()

    def to_numpy(self) -> "Trajectory":
        return Trajectory(positions=np.array(self.positions, dtype=F32), times=np.array(self.times, dtype=F32),
                          velocities=np.array(self.velocities, dtype=F32) if self.velocities is not None else None,
                          metadata=self.metadata.copy())

    def analyze_convergence(self) -> Dict[str, Any]:
        """Displacement-from-start summaries (particles.py:418-446)."""
        if self.T < 10:
            return {"status": "insufficient_data", "num_timesteps": self.T}
        disp = np.linalg.norm(self.positions - self.positions[0][None, :, :], axis=2)
        final, peak = disp[-1], np.max(disp, axis=0)
        return {"status": "success", "num_timesteps": self.T, "num_particles": self.N, "duration": self.duration,
                "mean_final_displacement": float(np.mean(final)), "max_final_displacement": float(np.max(final)),
                "mean_max_displacement": float(np.mean(peak)), "trajectory_bounds": self.get_bounds(),
                "memory_usage_mb": self.memory_usage_mb()}

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


def create_trajectory_from_positions(positions: np.ndarray, times: Optional[np.ndarray] = None,
                                     velocities: Optional[np.ndarray] = None, **metadata) -> Trajectory:
    """particles.py:637-686: times default to 0, 1, ..., T-1."""
    positions = _ensure_trajectory_shape(positions)
    T, N, _ = positions.shape
    if times is None:
        times = np.arange(T, dtype=F32)
    else:
        times = np.asarray(times, dtype=F32)
        if times.shape != (T,):
            raise ValueError(f"Times shape {times.shape} doesn't match trajectory length {T}")
    if velocities is not None:
        velocities = _ensure_trajectory_shape(velocities)
        if velocities.shape != (T, N, 3):
            raise ValueError(f"Velocities shape {velocities.shape} doesn't match positions {(T, N, 3)}")
    return Trajectory(positions=positions, times=times, velocities=velocities, metadata=metadata)


def create_single_particle_trajectory(positions: np.ndarray, times: Optional[np.ndarray] = None,
                                      velocities: Optional[np.ndarray] = None, **metadata) -> Trajectory:
    """particles.py:688-753: (T,2|3) positions of one particle."""
    positions = np.asarray(positions, dtype=F32)
    if positions.ndim != 2:
        raise ValueError(f"Single particle positions must be 2D (T, D), got {positions.ndim}D")
    T, D = positions.shape
    if D == 2:
        positions = np.concatenate([positions, np.zeros((T, 1), F32)], axis=1)
    elif D != 3:
        raise ValueError(f"Positions must have 2 or 3 spatial dimensions, got {D}")
    if velocities is not None:
        velocities = np.asarray(velocities, dtype=F32)
        if velocities.ndim != 2 or velocities.shape[0] != T:
            raise ValueError(f"Velocities shape {velocities.shape} doesn't match positions time dimension {T}")
        if velocities.shape[1] == 2:
            velocities = np.concatenate([velocities, np.zeros((T, 1), F32)], axis=1)
        velocities = velocities[:, None, :]
    times = np.arange(T, dtype=F32) if times is None else np.asarray(times, dtype=F32)
    return Trajectory(positions=positions[:, None, :], times=times, velocities=velocities,
                      metadata={**metadata, "particle_type": "single"})


def create_empty_trajectory(num_particles: int, num_timesteps: int) -> Trajectory:
    """particles.py:755-779."""
    return Trajectory(positions=np.zeros((num_timesteps, num_particles, 3), dtype=F32),
                      times=np.zeros(num_timesteps, dtype=F32), metadata={"status": "empty", "initialized": True})


def merge_trajectories(trajectories: List[Trajectory], axis: str = "time") -> Trajectory:
    """Concatenate along time (same N) or particles (same T; the first
    trajectory's times) (particles.py:781-860)."""
    if not trajectories:
        raise ValueError("No trajectories provided for merging")
    if len(trajectories) == 1:
        return trajectories[0]
    vels = [t.velocities for t in trajectories]
    if axis == "time":
        ns = [t.N for t in trajectories]
        if len(set(ns)) != 1:
            raise ValueError(f"All trajectories must have same number of particles for time merge: {ns}")
        positions = np.concatenate([t.positions for t in trajectories], axis=0)
        times = np.concatenate([t.times for t in trajectories], axis=0)
        velocities = np.concatenate(vels, axis=0) if all(v is not None for v in vels) else None
    elif axis == "particles":
        ts = [t.T for t in trajectories]
        if len(set(ts)) != 1:
            raise ValueError(f"All trajectories must have same number of timesteps for particle merge: {ts}")
        ref = trajectories[0].times
        for i, t in enumerate(trajectories[1:], 1):
            if not np.allclose(t.times, ref, atol=1e-6):
                warnings.warn(f"Trajectory {i} has different time points - using first trajectory's times")
        positions = np.concatenate([t.positions for t in trajectories], axis=1)
        times = ref.copy()
        velocities = np.concatenate(vels, axis=1) if all(v is not None for v in vels) else None
    else:
        raise ValueError(f"Unknown merge axis: {axis}. Use 'time' or 'particles'.")
    metadata = {**trajectories[0].metadata, "merged_axis": axis, "merged_count": len(trajectories)}
    return Trajectory(positions=positions, times=times, velocities=velocities, metadata=metadata)


def validate_trajectory_data(trajectory: Trajectory, strict: bool = False) -> Dict[str, Any]:
    """Shape, dtype, finiteness and time-order checks (particles.py:927-994)."""
    tr = trajectory
    res: Dict[str, Any] = {"valid": True, "warnings": [], "errors": []}

    def error(msg):
        res["errors"].append(msg)
        res["valid"] = False

    if tr.positions.shape != (tr.T, tr.N, 3):
        error(f"Position shape {tr.positions.shape} doesn't match (T,N,3) = ({tr.T},{tr.N},3)")
    if tr.times.shape != (tr.T,):
        error(f"Times shape {tr.times.shape} doesn't match (T,) = ({tr.T},)")
    if tr.positions.dtype != np.float32:
        if strict:
            error(f"Positions dtype {tr.positions.dtype} is not float32")
        else:
            res["warnings"].append(f"Positions dtype {tr.positions.dtype} is not optimal float32")
    if not np.all(np.isfinite(tr.positions)):
        error("Positions contain non-finite values (NaN/inf)")
    if not np.all(np.isfinite(tr.times)):
        error("Times contain non-finite values (NaN/inf)")
    if tr.T > 1:
        d = np.diff(tr.times)
        if not np.all(d >= 0):
            error("Time array is not monotonically non-decreasing")
        if np.min(d) < 1e-10:
            res["warnings"].append(f"Very small minimum time step: {np.min(d)}")
    if tr.velocities is not None:
        if tr.velocities.shape != (tr.T, tr.N, 3):
            error(f"Velocities shape {tr.velocities.shape} doesn't match positions")
        if not np.all(np.isfinite(tr.velocities)):
            error("Velocities contain non-finite values")
    mem = tr.memory_usage_mb()
    if mem > 1000:
        res["warnings"].append(f"Large memory usage: {mem:.1f} MB")
    return res
