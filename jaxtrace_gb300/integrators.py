"""Integrator step functions with the reference protocol
``step(x, t, dt, field_fn) -> x_next`` (jaxtrace/integrators/base.py:42-76).

``field_fn`` must be a GPU field of this package (or its bound
``sample_at_positions``); the step then runs as one CUDA kernel.  Opaque
Python callables are rejected with TypeError: there is no CPU path.
``dt`` may be a scalar or a per-particle (N,) array (rk4.py:108-129).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .schedule import single_blend, stage_times

F32 = np.float32


def resolve_field(field_fn):
    """The GPU field behind ``field_fn`` or TypeError."""
    from .fields import _DeviceField
    if isinstance(field_fn, _DeviceField):
        return field_fn
    owner = getattr(field_fn, "__self__", None)
    if isinstance(owner, _DeviceField):
        return owner
    gpu = getattr(field_fn, "_jt_gpu_field", None)
    if isinstance(gpu, _DeviceField):
        return gpu
    raise TypeError("unsupported field for the GPU path: pass a jaxtrace_gb300 field "
                    "(TimeSeriesField, StructuredTimeSeriesField, StructuredGridSampler, "
                    "OctreeFEMTimeSeriesFieldOptimized)")


def _step(code: int, x, t, dt, field_fn):
    import torch
    field = resolve_field(field_fn)
    is_tensor = isinstance(x, torch.Tensor)
    if is_tensor:
        xin = x.to(device="cuda", dtype=torch.float32).reshape(-1, 3).contiguous()
    else:
        xa = np.asarray(x, dtype=F32)
        if xa.ndim == 1:
            xa = xa.reshape(1, -1)
        if xa.ndim != 2 or xa.shape[1] != 3:
            raise ValueError(f"Positions must have shape (N,3), got {xa.shape}")
        xin = torch.from_numpy(np.ascontiguousarray(xa)).cuda()
    n = xin.shape[0]
    dt_arr = np.asarray(dt, dtype=F32)
    dtpp = None
    if dt_arr.ndim == 0:
        t_stages = stage_times(code, t, dt_arr)
    else:
        dt_arr = dt_arr.reshape(-1)
        if dt_arr.shape[0] != n:
            raise ValueError("per-particle dt must have one entry per particle")
        dtpp = torch.from_numpy(np.ascontiguousarray(dt_arr)).cuda()
        t_j = np.asarray(t, dtype=F32)
        if code == L.JT_RK4:   # rk4.py:114-116: stage times from the mean step
            dt_mean = np.mean(dt_arr)
            t_stages = (t_j, t_j + 0.5 * dt_mean, t_j + dt_mean)
        elif code == L.JT_RK2:  # rk2.py:299: float(t) + float(mean(dt/2))
            tf = float(t_j)
            t_stages = (tf, tf + float(np.mean(dt_arr * 0.5)), tf)
        else:
            tf = float(t_j)
            t_stages = (tf, tf, tf)
    args = field._blend_args()
    blends = np.concatenate([single_blend(field.times, ts, **args) for ts in t_stages])
    arr = (L.Blend * 3).from_buffer_copy(blends.tobytes())
    out = torch.empty_like(xin)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.check(L.load().jt_integrator_step(C.byref(field.jt_field()), arr, code, field._default_arith(),
                                        float(F32(dt_arr.mean()) if dt_arr.ndim else dt_arr), L.ptr(dtpp),
                                        L.ptr(xin), L.ptr(out), n, L.ptr(status), L.stream_ptr()))
    return out if is_tensor else out.cpu().numpy()


def euler_step(x, t, dt, field_fn):
    """x + dt * v(x, t) (integrators/euler.py:111-157)."""
    return _step(L.JT_EULER, x, t, dt, field_fn)


def rk2_step(x, t, dt, field_fn):
    """Midpoint rule x + dt * v(x + dt/2 v(x,t), t + dt/2) (integrators/rk2.py:246-309)."""
    return _step(L.JT_RK2, x, t, dt, field_fn)


def rk4_step(x, t, dt, field_fn):
    """Classic RK4, x + dt/6 (k1 + 2k2 + 2k3 + k4) (integrators/rk4.py:62-129)."""
    return _step(L.JT_RK4, x, t, dt, field_fn)


euler_step._jt_code = L.JT_EULER
rk2_step._jt_code = L.JT_RK2
rk4_step._jt_code = L.JT_RK4

INTEGRATORS = {"euler": euler_step, "rk2": rk2_step, "rk4": rk4_step}

__all__ = ["euler_step", "rk2_step", "rk4_step", "INTEGRATORS", "resolve_field"]
