"""Differentiable RK4 tracking on a regular-grid time-series field.

``AdjointRK4`` maps initial positions ``x0`` (N,3) and snapshot values ``U``
(T, Nx, Ny, Nz, 3) to the final positions ``x_T`` as a
``torch.autograd.Function``: the forward pass runs the tracking kernel and
keeps positions every ``checkpoint_every`` steps; the backward pass runs the
hand-written adjoint kernel segment by segment (recomputing each segment from
its checkpoint) and returns dL/dx0 and dL/dU.  dL/dx0 of a loss of the final
positions is the flow-map Jacobian transpose applied to dL/dx_T, the
building block of FTLE fields.

JAXTrace itself has no gradients on this path; the adjoint is checked against
central finite differences of the float64 oracle.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L
from .boundary import BoundaryDescriptor, no_boundary
from .fields import A_SLOTS, B_SLOTS
from .schedule import build_schedule, step_constants

F32 = np.float32


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the adjoint runs on a CUDA GPU; none is visible")
    return torch


class AdjointRK4:
    """Differentiable RK4 over a trilinear, linear-in-time grid field.

    times: snapshot times (T,); grid_x/y/z: node coordinates; bounds_handling
    as StructuredGridSampler; boundary: a per-axis box boundary descriptor.
    """

    def __init__(self, times, grid_x, grid_y, grid_z, bounds_handling: str = "periodic",
                 boundary: Optional[BoundaryDescriptor] = None, checkpoint_every: int = 50,
                 time_semantics: str = "numpy"):
        from .fields import StructuredTimeSeriesField
        self.times = np.asarray(times, dtype=F32)
        self.gx, self.gy, self.gz = (np.asarray(g, dtype=F32) for g in (grid_x, grid_y, grid_z))
        self.nodes = len(self.gx) * len(self.gy) * len(self.gz)
        # a host-side template for the grid descriptor (no snapshot data needed)
        self._tmpl = StructuredTimeSeriesField(np.zeros((len(self.times), self.nodes, 3), F32), self.times,
                                               self.gx, self.gy, self.gz, bounds_handling,
                                               time_semantics=time_semantics)
        self.bc = boundary if boundary is not None else no_boundary()
        if self.bc.inlet is not None or self.bc.absorbing_joint:
            raise NotImplementedError("the adjoint supports the per-axis box boundaries")
        k = int(checkpoint_every)
        if not 1 <= k <= 64:
            raise ValueError("checkpoint_every must be in 1..64")
        self.k = k

    def _field(self, pairs):
        t = self._tmpl
        g = L.GridField()
        g.nx, g.ny, g.nz = t.Nx, t.Ny, t.Nz
        g.bounds_mode = t._mode
        g.origin[:] = [F32(t.x_min), F32(t.y_min), F32(t.z_min)]
        g.spacing[:] = [F32(t.dx), F32(t.dy), F32(t.dz)]
        g.inv_spacing[:] = [float(F32(1.0) / F32(v)) for v in (t.dx, t.dy, t.dz)]
        g.valid_hi[:] = [F32(t.x_min + (t.Nx - 1) * t.dx), F32(t.y_min + (t.Ny - 1) * t.dy),
                         F32(t.z_min + (t.Nz - 1) * t.dz)]
        g.storage = L.JT_STORE_F32
        g.n_pairs = pairs.shape[0]
        g.pair_stride = self.nodes
        g.pairs = pairs.data_ptr()
        return g, L.Field(kind=L.JT_FIELD_GRID, grid=C.pointer(g))

    def pairs_from(self, U):
        torch = _torch()
        T = U.shape[0]
        V = U.reshape(T, self.nodes, 3).float()
        P = max(T - 1, 1)
        pairs = torch.zeros((P, self.nodes, 8), dtype=torch.float32, device=U.device)
        a = torch.tensor(A_SLOTS, device=U.device)
        b = torch.tensor(B_SLOTS, device=U.device)
        pairs.index_copy_(2, a, V[:P])
        pairs.index_copy_(2, b, V[1:] if T > 1 else V[:1])
        return pairs

    def pairs_grad_to_U(self, G, T):
        torch = _torch()
        P = G.shape[0]
        dU = torch.zeros((T, self.nodes, 3), dtype=torch.float32, device=G.device)
        dU[:P] += G[:, :, A_SLOTS]
        if T > 1:
            dU[1:] += G[:, :, B_SLOTS]
        else:
            dU[:1] += G[:, :, B_SLOTS]
        return dU

    def __call__(self, x0, U, time_span, n_timesteps: int, dt: Optional[float] = None):
        torch = _torch()
        steps = np.linspace(float(time_span[0]), float(time_span[1]), int(n_timesteps), dtype=np.float32)
        dt = float(steps[1] - steps[0]) if dt is None else float(dt)
        sched = build_schedule(steps, dt, L.JT_RK4, self.times, semantics=self._tmpl._semantics,
                               interpolation=self._tmpl.interpolation, extrapolation=self._tmpl.extrapolation)
        sched_dev = torch.from_numpy(sched.view(np.int32).reshape(-1, 8)).to(x0.device)
        return _function().apply(x0, U, self, sched_dev, len(steps) - 1, dt)


def _make_function():
    import torch

    class AdjointFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x0, U, solver, sched_dev, n_steps, dt):
            lib = L.load()
            pairs = solver.pairs_from(U.detach())
            gfield, field = solver._field(pairs)
            bc = solver.bc.jt_boundary()
            pos = x0.detach().float().contiguous().clone()
            n = pos.shape[0]
            k = solver.k
            n_seg = (n_steps + k - 1) // k
            ckpt = torch.empty((max(n_seg, 1), n, 3), dtype=torch.float32, device=pos.device)
            status = torch.zeros(1, dtype=torch.int32, device=pos.device)
            p = L.TrackParams()
            p.integrator, p.arith, p.n_particles = L.JT_RK4, L.JT_ARITH_EXACT, n
            dtf, dth, dt6 = step_constants(dt)
            p.dt, p.dt_half, p.dt_sixth = float(dtf), float(dth), float(dt6)
            p.schedule, p.pos, p.status, p.record_every = sched_dev.data_ptr(), pos.data_ptr(), status.data_ptr(), 1
            stream = L.stream_ptr()
            for sgi in range(n_seg):
                ckpt[sgi].copy_(pos)
                p.step_begin, p.step_end = sgi * k, min((sgi + 1) * k, n_steps)
                L.check(lib.jt_track(C.byref(field), C.byref(bc), C.byref(p), stream))
            ctx.solver, ctx.sched, ctx.n_steps, ctx.dt = solver, sched_dev, n_steps, dt
            ctx.T = U.shape[0]
            ctx.save_for_backward(ckpt, pairs)
            ctx.keep = (gfield, field, bc)
            return pos

        @staticmethod
        def backward(ctx, g_xT):
            ckpt, pairs = ctx.saved_tensors
            solver, k = ctx.solver, ctx.solver.k
            lib = L.load()
            gfield, field, bc = ctx.keep
            lam = g_xT.detach().float().contiguous().clone()
            grad = torch.zeros_like(pairs)
            n = lam.shape[0]
            a = L.AdjointParams()
            a.n_particles = n
            dtf, dth, dt6 = step_constants(ctx.dt)
            a.dt, a.dt_half, a.dt_sixth = float(dtf), float(dth), float(dt6)
            a.schedule, a.lambda_, a.grad = ctx.sched.data_ptr(), lam.data_ptr(), grad.data_ptr()
            stream = L.stream_ptr()
            n_seg = ckpt.shape[0]
            for sgi in reversed(range(n_seg)):
                a.step_begin, a.step_end = sgi * k, min((sgi + 1) * k, ctx.n_steps)
                a.ckpt = ckpt[sgi].data_ptr()
                L.check(lib.jt_adjoint_rk4(C.byref(field), C.byref(bc), C.byref(a), stream))
            dU = solver.pairs_grad_to_U(grad, ctx.T)
            shape = (ctx.T,) + tuple(len(g) for g in (solver.gx, solver.gy, solver.gz)) + (3,)
            return lam, dU.reshape(shape), None, None, None, None

    return AdjointFunction


_FUNCTION = []


def _function():
    """The autograd.Function class, created on first use (torch imported lazily)."""
    if not _FUNCTION:
        _FUNCTION.append(_make_function())
    return _FUNCTION[0]


__all__ = ["AdjointRK4"]
