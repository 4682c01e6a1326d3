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
                 time_semantics: str = "numpy", sort_bits: int = 6, sort_min_particles: int = 1 << 16,
                 stage_fields: bool = True):
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
        # particles are re-sorted by cell (2^sort_bits per axis over the grid)
        # at every checkpoint for gather and scatter locality; 0 disables it
        if not 0 <= int(sort_bits) <= 7:
            raise ValueError("sort_bits must be in 0..7")
        self.sort_bits = int(sort_bits)
        self.sort_min_particles = int(sort_min_particles)
        # the backward gathers pre-blended float32 stage fields of each segment
        # (bit-identical recompute, half the bytes of the pair records)
        self.stage_fields = bool(stage_fields)

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
            n = x0.shape[0]
            k = solver.k
            n_seg = (n_steps + k - 1) // k
            dev = x0.device
            ckpt = torch.empty((max(n_seg, 1), n, 3), dtype=torch.float32, device=dev)
            status = torch.zeros(1, dtype=torch.int32, device=dev)
            stream = L.stream_ptr()
            sort = solver.sort_bits > 0 and n >= solver.sort_min_particles
            pos = x0.detach().float().contiguous().clone()
            ids_all = None
            if sort:
                grid = solver._tmpl.sort_grid(bits=solver.sort_bits)
                ids_all = torch.empty((max(n_seg, 1), n), dtype=torch.int32, device=dev)
                ws = torch.empty(int(lib.jt_cell_sort_workspace_bytes(n, grid.bits)), dtype=torch.uint8, device=dev)
            p = L.TrackParams()
            p.integrator, p.arith, p.n_particles = L.JT_RK4, L.JT_ARITH_EXACT, n
            dtf, dth, dt6 = step_constants(dt)
            p.dt, p.dt_half, p.dt_sixth = float(dtf), float(dth), float(dt6)
            p.schedule, p.pos, p.status, p.record_every = sched_dev.data_ptr(), pos.data_ptr(), status.data_ptr(), 1
            for sgi in range(n_seg):
                if sort:
                    # particles in cell order at every checkpoint: ids_all[s][j] is the
                    # particle in slot j during segment s
                    src_ids = ids_all[sgi - 1] if sgi > 0 else None
                    L.check(lib.jt_cell_sort(C.byref(grid), n, L.ptr(pos), None, L.ptr(src_ids), L.ptr(ckpt[sgi]),
                                             None, L.ptr(ids_all[sgi]), L.ptr(ws), ws.numel(), stream))
                    pos.copy_(ckpt[sgi])
                else:
                    ckpt[sgi].copy_(pos)
                p.step_begin, p.step_end = sgi * k, min((sgi + 1) * k, n_steps)
                L.check(lib.jt_track(C.byref(field), C.byref(bc), C.byref(p), stream))
            out = pos
            if sort and n_seg > 0:
                out = torch.empty_like(pos)
                L.check(lib.jt_unpermute(n, L.ptr(pos), L.ptr(ids_all[n_seg - 1]), L.ptr(out), stream))
            ctx.solver, ctx.sched, ctx.n_steps, ctx.dt = solver, sched_dev, n_steps, dt
            ctx.T = U.shape[0]
            ctx.save_for_backward(ckpt, pairs, ids_all)
            ctx.keep = (gfield, field, bc)
            ctx.status = status
            return out

        @staticmethod
        def backward(ctx, g_xT):
            ckpt, pairs, ids_all = ctx.saved_tensors
            solver, k = ctx.solver, ctx.solver.k
            lib = L.load()
            gfield, field, bc = ctx.keep
            lam = g_xT.detach().float().contiguous().clone()          # particle order
            want_u = ctx.needs_input_grad[1]
            grad = torch.zeros_like(pairs) if want_u else None
            n = lam.shape[0]
            n_seg = ckpt.shape[0]
            a = L.AdjointParams()
            a.n_particles = n
            dtf, dth, dt6 = step_constants(ctx.dt)
            a.dt, a.dt_half, a.dt_sixth = float(dtf), float(dth), float(dt6)
            a.schedule = ctx.sched.data_ptr()
            a.grad = grad.data_ptr() if grad is not None else None
            work = None
            if want_u:
                wb = int(lib.jt_adjoint_workspace_bytes(solver.nodes, k))
                work = torch.empty(wb // 4, dtype=torch.float32, device=lam.device)
                a.work, a.work_bytes = work.data_ptr(), wb
            stream = L.stream_ptr()
            stage = src = None
            if solver.stage_fields:
                # 3 schedule entries (stage times) per step, and room for one segment's fields
                src = ctx.sched.view(-1, 4, 8)[:, :3].contiguous().view(-1, 8)
                stage = torch.empty((3 * k * solver.nodes, 4), dtype=torch.float32, device=lam.device)
            for sgi in reversed(range(n_seg)):
                a.step_begin, a.step_end = sgi * k, min((sgi + 1) * k, ctx.n_steps)
                a.ckpt = ckpt[sgi].data_ptr()
                if stage is not None:
                    ns = a.step_end - a.step_begin
                    L.check(lib.jt_stage_fields(C.byref(field), C.c_void_p(src.data_ptr() + 3 * a.step_begin * 32),
                                                None, 3 * ns, L.JT_STORE_STAGE_F32, C.c_void_p(stage.data_ptr()),
                                                stream))
                    a.stage = stage.data_ptr()
                if ids_all is not None:
                    idx = ids_all[sgi].long()
                    lam_s = lam.index_select(0, idx).contiguous()    # slot order of the segment
                    a.lambda_ = lam_s.data_ptr()
                    L.check(lib.jt_adjoint_rk4(C.byref(field), C.byref(bc), C.byref(a), stream))
                    lam.index_copy_(0, idx, lam_s)
                else:
                    a.lambda_ = lam.data_ptr()
                    L.check(lib.jt_adjoint_rk4(C.byref(field), C.byref(bc), C.byref(a), stream))
            dU = None
            if want_u:
                dU = solver.pairs_grad_to_U(grad, ctx.T)
                shape = (ctx.T,) + tuple(len(g) for g in (solver.gx, solver.gy, solver.gz)) + (3,)
                dU = dU.reshape(shape)
            return lam, dU, None, None, None, None

    return AdjointFunction


_FUNCTION = []


def _function():
    """The autograd.Function class, created on first use (torch imported lazily)."""
    if not _FUNCTION:
        _FUNCTION.append(_make_function())
    return _FUNCTION[0]


__all__ = ["AdjointRK4"]
