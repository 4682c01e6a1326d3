"""Time-blend schedules: the per-stage snapshot weights of a tracking run.

The reference blends two bracketing snapshots at every field call.  The
weights depend only on the call's time, which is the same for every
particle, so they are computed here once per integrator stage with the
reference's own scalar arithmetic, and the kernels apply them per node.

Two semantics exist in the reference and both are kept:

* ``"numpy"`` -- ``TimeSeriesField.sample_at_time`` without JAX
  (jaxtrace/fields/time_series.py:314-367): ``searchsorted`` in float64, the
  bound tests against float32 times, ``alpha`` in float64 and the two weights
  rounded to float32 when they multiply the float32 snapshots.
* ``"jax"`` -- ``_sample_all_nodes_at_time_jax`` (time_series.py:155-245),
  float32 throughout with ``alpha`` clipped to [0, 1]; this is what the octree
  field always uses (octree_fem_time_series_optimized.py:108).

Stage times follow the integrators: RK4 evaluates at float32 ``t``,
``t + 0.5*dt`` and ``t + dt`` (integrators/rk4.py:89-92); RK2 at ``t`` and the
Python-float sum ``float(t) + float(0.5*dt)`` (rk2.py:284-294); Euler at
``float(t)`` (euler.py:150).  Step start times are
``np.linspace(t0, t1, T, dtype=float32)`` (tracking/tracker.py:347).
"""
from __future__ import annotations

import numpy as np

from ._lib import (BLEND_DTYPE, JT_BLEND_LERP_BWD, JT_BLEND_LERP_FWD, JT_BLEND_SAME_A, JT_BLEND_SAME_B,
                   JT_BLEND_WEIGHTED,
                   JT_EULER, JT_RK2, JT_RK4)

F32 = np.float32


def _entry(pair, form, wa, wb, sa=1.0, sb=1.0):
    return (int(pair), int(form), F32(wa), F32(wb), F32(sa), F32(sb), 0, 0)


def blend_numpy(times: np.ndarray, t, interpolation: str = "linear", extrapolation: str = "constant"):
    """Blend entry for ``TimeSeriesField.sample_at_time(t)`` on the NumPy path.

    Mirrors time_series.py:314-367 expression by expression (the reference
    computes the blended snapshot; the same scalars are returned here).
    """
    times = np.asarray(times, dtype=F32)
    T = len(times)
    interp = interpolation.lower()
    extra = extrapolation.lower()
    t = float(t)
    if interp == "nearest":
        idx = int(np.argmin(np.abs(times - t)))
        return _slot(idx, T, F32(1.0))
    if interp != "linear":
        raise NotImplementedError(f"time interpolation {interpolation!r} is not available on the GPU path")
    ir = int(np.searchsorted(times, t, side="right"))
    il = max(ir - 1, 0)
    if t < times[0]:
        if extra == "linear" and T > 1:
            dt = max(times[1] - times[0], 1e-12)
            alpha = (t - times[0]) / dt
            return _entry(0, JT_BLEND_LERP_FWD, 0.0, np.asarray(alpha, dtype=F32))
        if extra == "zero":
            return _entry(0, JT_BLEND_WEIGHTED, 0.0, 0.0)
        if extra == "nan":
            return _entry(0, JT_BLEND_WEIGHTED, np.nan, np.nan)
        return _slot(0, T, F32(1.0))
    if t > times[-1]:
        if extra == "linear" and T > 1:
            dt = max(times[-1] - times[-2], 1e-12)
            alpha = (t - times[-1]) / dt
            return _entry(T - 2, JT_BLEND_LERP_BWD, 0.0, np.asarray(alpha, dtype=F32))
        if extra == "zero":
            return _entry(0, JT_BLEND_WEIGHTED, 0.0, 0.0)
        if extra == "nan":
            return _entry(0, JT_BLEND_WEIGHTED, np.nan, np.nan)
        return _slot(T - 1, T, F32(1.0))
    ir = min(ir, T - 1)
    il = min(max(il, 0), T - 1)
    t0, t1 = float(times[il]), float(times[ir])
    dt = max(t1 - t0, 1e-12)
    alpha = (t - t0) / dt
    w0, w1 = F32(1.0 - alpha), F32(alpha)
    return _two(il, ir, w0, w1, T)


def blend_jax(times: np.ndarray, t, interpolation: str = "linear", extrapolation: str = "constant"):
    """Blend entry for ``_sample_all_nodes_at_time_jax(t)`` (time_series.py:155-245)."""
    times = np.asarray(times, dtype=F32)
    T = len(times)
    t = F32(t)
    interp = interpolation.lower()
    extra = extrapolation.lower()
    if interp == "nearest":
        idx = int(np.argmin(np.abs(times - t)))
        return _slot(idx, T, F32(1.0))
    if interp != "linear":
        raise NotImplementedError("cubic interpolation not supported with JAX")
    ir = int(np.searchsorted(times, t, side="right"))
    ir = min(max(ir, 0), T)
    il = min(max(ir - 1, 0), T - 1)
    if t < times[0]:
        if extra == "linear":
            t0, t1 = times[0], times[min(1, T - 1)]
            dt = np.maximum(t1 - t0, F32(1e-12))
            alpha = (t - t0) / dt
            if T > 1:
                return _entry(0, JT_BLEND_LERP_FWD, 0.0, alpha)
            return _slot(0, T, F32(1.0))
        if extra == "zero":
            return _entry(0, JT_BLEND_WEIGHTED, 0.0, 0.0)
        if extra == "nan":
            return _entry(0, JT_BLEND_WEIGHTED, np.nan, np.nan)
        return _slot(0, T, F32(1.0))
    if t > times[-1]:
        if extra == "linear":
            t0, t1 = times[max(T - 2, 0)], times[T - 1]
            dt = np.maximum(t1 - t0, F32(1e-12))
            alpha = (t - t1) / dt
            if T > 1:
                return _entry(T - 2, JT_BLEND_LERP_BWD, 0.0, alpha)
            return _slot(T - 1, T, F32(1.0))
        if extra == "zero":
            return _entry(0, JT_BLEND_WEIGHTED, 0.0, 0.0)
        if extra == "nan":
            return _entry(0, JT_BLEND_WEIGHTED, np.nan, np.nan)
        return _slot(T - 1, T, F32(1.0))
    irc = min(max(ir, 0), T - 1)
    t0, t1 = times[il], times[irc]
    dt = np.maximum(t1 - t0, F32(1e-12))
    alpha = np.clip((t - t0) / dt, F32(0.0), F32(1.0)).astype(F32)
    return _two(il, irc, F32(F32(1.0) - alpha), alpha, T)


def _slot(idx: int, T: int, w: np.float32):
    """w * V[idx] (w is 1 for a plain copy)."""
    if T == 1:
        return _entry(0, JT_BLEND_WEIGHTED, w, 0.0)
    if idx >= T - 1:
        return _entry(T - 2, JT_BLEND_WEIGHTED, 0.0, w)
    return _entry(idx, JT_BLEND_WEIGHTED, w, 0.0)


def _two(il: int, ir: int, w0, w1, T: int):
    """w0*V[il] + w1*V[ir] for il+1 == ir, or both weights on one snapshot when
    il == ir (a Python-float time that rounds onto an end snapshot)."""
    if T == 1:
        return _entry(0, JT_BLEND_SAME_A, w0, w1)
    if ir == il + 1:
        return _entry(il, JT_BLEND_WEIGHTED, w0, w1)
    if il >= T - 1:
        return _entry(T - 2, JT_BLEND_SAME_B, w0, w1)
    return _entry(il, JT_BLEND_SAME_A, w0, w1)


BLENDERS = {"numpy": blend_numpy, "jax": blend_jax}


def stage_times(integrator: int, t_start, dt):
    """Times of the field calls of one step starting at ``t_start``.

    Returns three objects (stage 0, mid, full); unused slots repeat stage 0.
    """
    if integrator == JT_RK4:
        t_j = np.asarray(t_start, dtype=F32)        # rk4.py:29
        dt_j = np.asarray(dt, dtype=F32)            # rk4.py:30
        dt_half = 0.5 * dt_j                        # rk4.py:90
        return t_j, t_j + dt_half, t_j + dt_j       # rk4.py:91-92
    t_arr = np.asarray(t_start, dtype=F32)
    t_float = float(t_arr)                          # rk2.py:284, euler.py:150
    if integrator == JT_RK2:
        dt_arr = np.asarray(dt, dtype=F32)
        dt_half = dt_arr * 0.5                      # rk2.py:292
        return t_float, t_float + float(dt_half), t_float   # rk2.py:294
    if integrator == JT_EULER:
        return t_float, t_float, t_float
    raise ValueError(f"unknown integrator code {integrator}")


def step_constants(dt):
    """float32 dt, dt/2 and dt/6 as the integrators round them (rk4.py:90, :44)."""
    dt_j = np.asarray(dt, dtype=F32)
    return F32(dt_j), F32(0.5 * dt_j), F32(dt_j / 6.0)


def build_schedule(times_steps: np.ndarray, dt, integrator: int, snap_times: np.ndarray,
                   semantics: str = "numpy", interpolation: str = "linear",
                   extrapolation: str = "constant", scales: np.ndarray | None = None) -> np.ndarray:
    """Schedule of a run: 4 entries per step (stage 0, mid, full, record time).

    ``times_steps`` is the float32 time grid of the run (T values); step s
    starts at ``times_steps[s]`` and its recording entry is for
    ``times_steps[s+1]`` (tracker.py:441-449).  Returns a structured array
    with the jt_blend layout, length 4*(T-1).
    """
    blend = BLENDERS[semantics]
    times_steps = np.asarray(times_steps, dtype=F32)
    n_steps = max(len(times_steps) - 1, 0)
    out = np.zeros(4 * n_steps, dtype=BLEND_DTYPE)
    cache = {}

    def get(t):
        key = (type(t).__name__, float(t))
        e = cache.get(key)
        if e is None:
            e = blend(snap_times, t, interpolation, extrapolation)
            cache[key] = e
        return e

    for s in range(n_steps):
        t0, tm, tf = stage_times(integrator, times_steps[s], dt)
        out[4 * s + 0] = get(t0)
        out[4 * s + 1] = get(tm)
        out[4 * s + 2] = get(tf)
        out[4 * s + 3] = get(times_steps[s + 1])
    if scales is not None:
        apply_scales(out, scales)
    return out


def apply_scales(entries: np.ndarray, scales: np.ndarray) -> None:
    """Fold per-snapshot decode scales of 16-bit storage into the entries."""
    scales = np.asarray(scales, dtype=F32)
    n = len(scales)
    pa = entries["pair"]
    sa = scales[np.clip(pa, 0, n - 1)]
    sb = scales[np.clip(pa + 1, 0, n - 1)] if n > 1 else sa
    form = entries["form"]
    folded = (form == JT_BLEND_WEIGHTED) | (form == JT_BLEND_SAME_A) | (form == JT_BLEND_SAME_B)
    fa = np.where(form == JT_BLEND_SAME_B, sb, sa)   # scale under the wa term
    fb = np.where(form == JT_BLEND_SAME_A, sa, sb)   # scale under the wb term
    entries["wa"] = np.where(folded, entries["wa"] * fa, entries["wa"])
    entries["wb"] = np.where(folded, entries["wb"] * fb, entries["wb"])
    entries["sa"] = np.where(folded, F32(1.0), sa)
    entries["sb"] = np.where(folded, F32(1.0), sb)


def single_blend(snap_times, t, semantics="numpy", interpolation="linear", extrapolation="constant",
                 scales=None) -> np.ndarray:
    e = np.zeros(1, dtype=BLEND_DTYPE)
    e[0] = BLENDERS[semantics](snap_times, t, interpolation, extrapolation)
    if scales is not None:
        apply_scales(e, scales)
    return e


def blend_nodes(entry, pairs_a: np.ndarray, pairs_b: np.ndarray) -> np.ndarray:
    """NumPy evaluation of one entry on node arrays (test helper mirroring the kernel)."""
    wa, wb = F32(entry["wa"]), F32(entry["wb"])
    form = int(entry["form"])
    lerp = form in (JT_BLEND_LERP_FWD, JT_BLEND_LERP_BWD)
    a = np.asarray(pairs_a, dtype=F32) * F32(entry["sa"]) if lerp else np.asarray(pairs_a, F32)
    b = np.asarray(pairs_b, dtype=F32) * F32(entry["sb"]) if lerp else np.asarray(pairs_b, F32)
    if form == JT_BLEND_WEIGHTED:
        return (wa * a + wb * b).astype(F32)
    if form == JT_BLEND_SAME_A:
        return (wa * a + wb * a).astype(F32)
    if form == JT_BLEND_SAME_B:
        return (wa * b + wb * b).astype(F32)
    if form == JT_BLEND_LERP_FWD:
        return (a + wb * (b - a)).astype(F32)
    return (b + wb * (b - a)).astype(F32)
