"""Mixing metrics of a trajectory (tracking/analysis.py:257-320).

Variance growth and the return ratio are float32 NumPy reductions over the
recorded rows, as in the reference.  The Lyapunov-like term compares every
pair of particles: the reference builds two N x N distance matrices on the
host; here the pairs run on the device (``jt_pair_log_ratio``) with the same
float32 distances and cutoff, summing the logs in float64.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict

import numpy as np

from . import _lib as L

F32 = np.float32


def pair_log_ratio(x0, x1, rmax: float = 0.1):
    """(sum of log(|x1_i - x1_j| / |x0_i - x0_j|), pair count) over ordered
    pairs with 0 < |x0_i - x0_j| < rmax (float32 distances)."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the pair term runs on a CUDA GPU; none is visible")
    a = torch.as_tensor(np.ascontiguousarray(x0, dtype=F32)).reshape(-1, 3).cuda()
    b = torch.as_tensor(np.ascontiguousarray(x1, dtype=F32)).reshape(-1, 3).cuda()
    if a.shape != b.shape:
        raise ValueError(f"x0 {tuple(a.shape)} and x1 {tuple(b.shape)} differ")
    out_sum = torch.zeros(1, dtype=torch.float64, device="cuda")
    out_cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    L.check(L.load().jt_pair_log_ratio(L.ptr(a), L.ptr(b), int(a.shape[0]), float(F32(rmax)), L.ptr(out_sum),
                                       L.ptr(out_cnt), L.stream_ptr()))
    return float(out_sum.item()), int(out_cnt.item())


def mixing_host_terms(trajectory) -> Dict[str, float]:
    """The row reductions of compute_mixing_metrics (analysis.py:271-295):
    variance growth rate, final variance and return ratio, in the
    reference's float32 NumPy arithmetic."""
    positions = np.asarray(trajectory.positions)
    total_variance = np.sum(np.var(positions, axis=1), axis=1)
    T, N = positions.shape[0], positions.shape[1]
    growth = (total_variance[-1] - total_variance[0]) / trajectory.duration if T > 1 else 0.0
    returns = 0.0
    if positions.shape[2] >= 2:
        first, last = positions[0], positions[-1]
        dist = np.linalg.norm(last - first, axis=1)
        threshold = 0.1 * np.mean(np.std(first, axis=0))
        returns = np.sum(dist < threshold) / N
    return {"variance_growth_rate": growth, "final_variance": total_variance[-1], "poincare_return_ratio": returns}


def compute_mixing_metrics(trajectory) -> Dict[str, float]:
    """Variance growth rate, final variance, return ratio, Lyapunov-like
    exponent and mixing efficiency (analysis.py:257-320)."""
    out = mixing_host_terms(trajectory)
    positions = np.asarray(trajectory.positions)
    T, N = positions.shape[0], positions.shape[1]
    lyap = 0.0
    if T > 2:
        s, n = pair_log_ratio(positions[0], positions[-1], 0.1)
        if n > 0:
            lyap = (s / n) / trajectory.duration
    out["lyapunov_approximation"] = lyap
    out["mixing_efficiency"] = out["variance_growth_rate"] / (N * trajectory.duration)
    return out


def analyze_trajectory_results(trajectory, strategy_info=None, verbose: bool = True):
    """(statistics, validation) of a trajectory with the spatial spread
    summary (tracking/analysis.py:13-105)."""
    from .particles import compute_trajectory_statistics, validate_trajectory_data
    validation = validate_trajectory_data(trajectory)
    try:
        stats = compute_trajectory_statistics(trajectory)
        s0 = np.std(trajectory.positions[0], axis=0)
        s1 = np.std(trajectory.positions[-1], axis=0)
        with np.errstate(divide="ignore", invalid="ignore"):
            change = np.where(s0 > 0, (s1 / s0 - 1) * 100, np.inf)
        disp = stats.get("displacement", {})
        eff = (float(np.sum(disp["values"])) / (trajectory.duration * trajectory.N)
               if "values" in disp else 0.0)
        stats["spatial"] = {"initial_spread": s0, "final_spread": s1, "spread_change_percent": change,
                            "mixing_efficiency": eff}
        if verbose:
            print(f"Trajectory {trajectory.positions.shape} (T,N,3), duration {trajectory.duration:.2f}, "
                  f"validation {'PASSED' if validation['valid'] else 'FAILED'}")
    except Exception as e:  # noqa: BLE001 -- the reference reports and returns None
        if verbose:
            print(f"Statistics failed: {e}")
        stats = None
    return stats, validation
