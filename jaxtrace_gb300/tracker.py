"""Particle tracker with the JAXTrace API (tracking/tracker.py:107-855).

``create_tracker(integrator_name, field, boundary_condition, **options)``
returns a ``ParticleTracker`` whose ``track_particles`` runs the whole time
loop in one persistent CUDA kernel per time chunk: integrator stages, field
evaluation and boundary fused, positions held in registers, recorded rows
written straight into a device trajectory slab that streams to the host.
"""
from __future__ import annotations

import collections

import ctypes as C
from dataclasses import dataclass, field as dc_field
from typing import Any, Callable, Dict, List, Optional, Tuple

import numpy as np

from . import _lib as L
from .boundary import BoundaryDescriptor
from .fields import ensure_positions_shape, ensure_positions_tensor
from .integrators import INTEGRATORS, resolve_field
from .particles import Trajectory
from .schedule import build_schedule, step_constants

F32 = np.float32


def _estimate_memory_usage(n_particles: int, n_timesteps: int, has_velocities: bool = False) -> float:
    """tracker.py:89-101 (GB of host trajectory storage)."""
    pos_size = n_timesteps * n_particles * 3 * 4
    time_size = n_timesteps * 4
    vel_size = pos_size if has_velocities else 0
    workspace_size = n_particles * 3 * 4 * 4
    return (pos_size + time_size + vel_size + workspace_size) / (1024 ** 3)


@dataclass
class TrackerOptions:
    """tracker.py:107-153, extended.  The reference fields are all accepted
    and keep their meaning where it applies to a GPU run; new fields:

    record_every       record every k-th step into a compact trajectory
                       (rows 0, k, 2k, ...; None keeps the reference layout)
    record_final_only  keep only the initial and final positions
    precision          'exact' (float32, bit-compatible with the NumPy
                       reference) or 'compensated' (FMA + Kahan sums); 16-bit
                       snapshot storage always runs 'compensated'
    device_memory_gb   device budget of one trajectory slab
    time_chunk         steps per kernel launch (None: as many as fit)
    sort_every         re-sort particles by cell every k steps for gather
                       locality (None: from 2^18 particles up, 100 for float32
                       snapshots and 200 for 16-bit ones; 0: never)
    sort_bits          cells per axis of that sort, as a power of two
                       (None: 2^7)
    block_size         threads per block of the tracking kernel (0: 256)
    autotune           pick sort_every / sort_bits / block_size by timing a
                       short sample of the run (``autotune.Autotuner``)
    cuda_graph         capture the whole tracking pass of ``track_ensembles``
                       in a CUDA graph and replay it
    stage_fields       regular grids: blend every node once per stage time
                       of a chunk of ``stage_chunk`` steps before the tracking
                       launch, so it gathers one time level (the reference's
                       own order of operations; float32 stays bit-identical)
    stage_overlap      blend the next chunk's stage fields on a side stream
                       while the current chunk is tracked (a ring twice as deep)
    record_path_length accumulate each particle's path length over every step
                       in the tracking kernel (Trajectory.path_length; what
                       compute_path_length gives on an every-step recording)
    row_sink           callable(first_row, positions, velocities, row_times)
                       handed every row of the trajectory once, in order, on a
                       writer thread as soon as the row is in host memory
                       (e.g. ``vtk_io.VTKTrajectorySeries``); recorded slabs
                       are copied to the host on a side stream while the next
                       time chunk runs, so with ``time_chunk`` set the export
                       overlaps the tracking
    """
    max_memory_gb: float = 8.0
    batch_size: Optional[int] = None
    oom_recovery: bool = True
    use_jax_jit: bool = True
    static_compilation: bool = True
    use_scan_jit: bool = True
    device_put_inputs: bool = True
    record_on_device: bool = True
    max_batch_size: int = 100_000
    min_batch_size: int = 100
    record_velocities: bool = False
    recording_interval: int = 1
    progress_callback: Optional[Callable[[float], None]] = None
    progress_style: str = "auto"
    progress_desc: str = "Tracking"
    progress_update_every: float = 0.05
    adaptive_dt: bool = False
    error_tolerance: float = 1e-6
    # GPU-path additions
    record_every: Optional[int] = None
    record_final_only: bool = False
    precision: str = "exact"
    device_memory_gb: float = 32.0
    time_chunk: Optional[int] = None
    sort_every: Optional[int] = None
    sort_bits: Optional[int] = None
    block_size: int = 0
    autotune: bool = False
    cuda_graph: bool = False
    stage_fields: bool = True
    stage_chunk: int = 32
    stage_overlap: bool = True
    row_sink: Optional[Callable[[int, np.ndarray, Optional[np.ndarray], np.ndarray], None]] = None
    record_path_length: bool = False

    def estimate_batch_size(self, n_particles: int, n_timesteps: int) -> int:
        """tracker.py:142-153."""
        if self.batch_size is not None:
            return min(self.batch_size, self.max_batch_size)
        batch_size = min(n_particles, self.max_batch_size)
        while batch_size >= self.min_batch_size:
            if _estimate_memory_usage(batch_size, n_timesteps, self.record_velocities) <= self.max_memory_gb:
                break
            batch_size = max(batch_size // 2, self.min_batch_size)
        return max(batch_size, self.min_batch_size)


def _integrator_code(integrator) -> int:
    code = getattr(integrator, "_jt_code", None)
    if code is None:
        raise TypeError("unsupported integrator for the GPU path: use euler_step, rk2_step or rk4_step")
    return int(code)


def _boundary_descriptor(bc) -> BoundaryDescriptor:
    if isinstance(bc, BoundaryDescriptor):
        return bc
    raise TypeError("unsupported boundary for the GPU path: use a jaxtrace_gb300.boundary factory")


@dataclass
class ParticleTracker:
    """tracker.py:159-804 with the GPU engine behind ``track_particles``."""
    integrator: Callable
    field_fn: Callable
    boundary_fn: Callable
    options: TrackerOptions = dc_field(default_factory=TrackerOptions)

    def __post_init__(self):
        if not callable(self.integrator):
            raise ValueError("integrator must be callable")
        if not callable(self.field_fn):
            raise ValueError("field_fn must be callable")
        if not callable(self.boundary_fn):
            raise ValueError("boundary_fn must be callable")
        self._code = _integrator_code(self.integrator)
        self._field = resolve_field(self.field_fn)
        self._bc = _boundary_descriptor(self.boundary_fn)
        if self.options.precision not in ("exact", "compensated"):
            raise ValueError("precision must be 'exact' or 'compensated'")
        self.last_status = 0

    # ------------------------------------------------------------------
    def _arith(self) -> int:
        if self._field._storage != L.JT_STORE_F32 or self.options.precision == "compensated":
            return L.JT_ARITH_COMPENSATED
        return L.JT_ARITH_EXACT

    def _schedule(self, times: np.ndarray, dt: float) -> np.ndarray:
        """The run's blend schedule, cached per (time grid, dt): building it
        replays the reference's scalar arithmetic step by step on the host."""
        cache = self.__dict__.setdefault("_sched_cache", {})
        key = (np.asarray(times, dtype=np.float32).tobytes(), float(dt))
        hit = cache.get(key)
        if hit is None:
            hit = build_schedule(times, dt, self._code, self._field.times, **self._field._blend_args())
            if len(cache) >= 8:
                cache.pop(next(iter(cache)))
            cache[key] = hit
        return hit

    def _record_plan(self, n_timesteps: int):
        """(record_every, compact, n_rows, row_times_index) of the output."""
        o = self.options
        T = n_timesteps
        if o.record_final_only:
            k = max(T - 1, 1)
            idx = np.array([0, T - 1] if T > 1 else [0])
            return k, True, idx
        if o.record_every is not None:
            k = int(o.record_every)
            if k < 1:
                raise ValueError("record_every must be >= 1")
            idx = np.arange(0, T, k)
            return k, True, idx
        k = int(o.recording_interval)
        if k < 1:
            raise ValueError("recording_interval must be >= 1")
        return k, False, np.arange(T)

    def track_particles(self, initial_positions, time_span: Tuple[float, float], n_timesteps: int,
                        dt: Optional[float] = None, return_device: bool = False, **kwargs):
        """tracker.py:320-358: T = n_timesteps rows from linspace(t0, t1, T).

        ``initial_positions`` may also be a float32 (N, 3) torch tensor: on the
        host (pinned memory: one DMA) or already on the device (no copy in).
        ``return_device=True`` (with ``record_final_only``) returns the final
        positions as a (N, 3) CUDA tensor instead of a host ``Trajectory``,
        for callers that keep the particles on the device."""
        import torch
        src = dev_in = None
        if isinstance(initial_positions, torch.Tensor) and initial_positions.is_cuda:
            dev_in = ensure_positions_tensor(initial_positions)
            x0 = None
            n = dev_in.shape[0]
        elif isinstance(initial_positions, torch.Tensor) and initial_positions.device.type == "cpu" \
                and initial_positions.dtype == torch.float32 and initial_positions.ndim == 2 \
                and initial_positions.shape[1] == 3 and initial_positions.is_contiguous():
            src = initial_positions          # e.g. pinned host memory: one DMA to the device
            x0 = src.numpy()
        else:
            x0 = ensure_positions_shape(initial_positions)
        if x0 is not None:
            n = x0.shape[0]
        if return_device:
            if int(n_timesteps) > 1 and not self.options.record_final_only:
                raise ValueError("return_device=True returns the final positions: use record_final_only=True")
            if self.options.record_velocities or self.options.row_sink is not None:
                raise ValueError("return_device=True records no rows (no velocities, no row sink)")
            return self._track_on_device(dev_in if dev_in is not None else
                                         (src if src is not None else torch.from_numpy(x0)),
                                         time_span, n_timesteps, dt)
        t_start, t_end = time_span
        times = np.linspace(float(t_start), float(t_end), int(n_timesteps), dtype=np.float32)
        if dt is None:
            dt = float(times[1] - times[0]) if n_timesteps > 1 else 0.0
        else:
            dt = float(dt)
        T = len(times)
        batch_size = self.options.estimate_batch_size(n, T)
        k, compact, row_idx = self._record_plan(T)
        n_rows = len(row_idx)
        # compact layouts write every row; the reference layout with a
        # recording interval leaves unrecorded rows at zero
        positions = _host_rows((n_rows, n, 3), zero=not compact)
        velocities = _host_rows((n_rows, n, 3), zero=not compact) if self.options.record_velocities else None
        if n == 0 or T == 0:
            return self._trajectory(positions, times[row_idx], velocities, n, T, dt, batch_size, 0)
        if dev_in is not None:
            pos = dev_in.clone()               # the caller's tensor stays as it is
            host0 = pos.cpu()
        else:
            host0 = src if src is not None else torch.from_numpy(x0)
            pos = host0.to("cuda", non_blocking=src is not None)
        if velocities is not None:
            torch.from_numpy(velocities[0]).copy_(self._field.sample_at_positions(pos, times[0], arith=self._arith()))
        # row 0 is a host copy of the input: made on a helper thread while
        # the device tracks (torch releases the GIL inside copy_)
        import threading
        failed = []

        def copy_row0():
            try:
                torch.from_numpy(positions[0]).copy_(host0)
            except BaseException as exc:   # re-raised on the caller's thread
                failed.append(exc)

        row0 = threading.Thread(target=copy_row0)
        row0.start()
        rows_out = None
        if self.options.row_sink is not None:
            rows_out = _RowStream(self.options.row_sink, positions, velocities, times[row_idx])
            rows_out.put(0, 1, row0)
        ran = False
        try:
            n_chunks = self._run(pos, times, dt, k, compact, n_rows, positions, velocities, rows_out)
            ran = True
        finally:
            row0.join()
            if rows_out is not None and (failed or not ran):
                rows_out.close(raise_error=False)
        if failed:
            raise failed[0]
        if compact and self.options.record_final_only and T > 1:
            torch.from_numpy(positions[-1]).copy_(pos)        # device -> final row, no staging array
            if velocities is not None:
                torch.from_numpy(velocities[-1]).copy_(self._field.sample_at_positions(pos, times[-1], arith=self._arith()))
            if rows_out is not None:
                rows_out.put(n_rows - 1, 1)
        if rows_out is not None:
            rows_out.close()
        traj = self._trajectory(positions, times[row_idx], velocities, n, T, dt, batch_size, n_chunks)
        if self.options.record_path_length:
            traj.path_length = getattr(self, "_last_path_length", None)
            if traj.path_length is None:       # no step ran
                traj.path_length = np.zeros(n, dtype=F32)
        return traj

    def _track_on_device(self, x0, time_span, n_timesteps: int, dt: Optional[float]):
        """track_particles for return_device=True: the final positions as a
        CUDA tensor, no host rows."""
        import torch
        times = np.linspace(float(time_span[0]), float(time_span[1]), int(n_timesteps), dtype=np.float32)
        if dt is None:
            dt = float(times[1] - times[0]) if len(times) > 1 else 0.0
        pos = x0.to("cuda", non_blocking=True).to(torch.float32).reshape(-1, 3).clone()
        if pos.shape[0] and len(times) > 1:
            self._run(pos, times, float(dt), 1, True, 2, None, None)
        return pos

    def _trajectory(self, positions, times, velocities, n, T, dt, batch_size, n_chunks):
        meta = {
            "integrator": str(self.integrator),
            "batch_processing": "single_batch" if batch_size >= n else "multi_batch",
            "n_particles": n,
            "n_timesteps": T,
            "dt": dt,
            "jax_compiled": False,
            "jit_scan": False,
            "backend": "gb300",
            "kernel": f"jt_track/{type(self._field).__name__}",
            "storage": self._field.storage,
            "arith": "exact" if self._arith() == L.JT_ARITH_EXACT else "compensated",
            "precision": "exact" if self._arith() == L.JT_ARITH_EXACT else "compensated",
            "time_chunks": n_chunks,
            "device_status": self.last_status,
        }
        if batch_size < n:
            meta["batch_size"] = batch_size
            meta["n_batches"] = (n + batch_size - 1) // batch_size
        return Trajectory(positions=positions, times=np.asarray(times, dtype=F32), velocities=velocities,
                          metadata=meta)

    # ------------------------------------------------------------------
    def make_params(self, pos, dt, n_steps_total, sched_dev, status, comp=None) -> L.TrackParams:
        p = L.TrackParams()
        p.integrator = self._code
        p.arith = self._arith()
        p.n_particles = pos.shape[0]
        dtf, dth, dt6 = step_constants(dt)
        p.dt, p.dt_half, p.dt_sixth = float(dtf), float(dth), float(dt6)
        p.schedule = sched_dev.data_ptr()
        p.pos = pos.data_ptr()
        p.comp = comp.data_ptr() if comp is not None else None
        p.status = status.data_ptr()
        p.record_every = 1
        p.block_size = int(self.options.block_size)
        return p

    def _sort_every(self, n: int) -> int:
        """Locality re-sort interval: measured best at 100 steps for float32
        snapshots and 200 for 16-bit ones (whose launches are shorter, so the
        sort is a larger share) on the 16.8M-particle precision workload of a
        regular grid; 32 on tetrahedral meshes, whose lookups lose locality
        sooner (FEM configuration, octree: 5.28e9 particle-steps/s at 25, 5.27e9
        at 50, 5.11e9 at 100, 5.15e9 at 10)."""
        se = self.options.sort_every
        if se is None:
            if n < (1 << 18):
                return 0
            from .fields import FEMTimeSeriesField, OctreeFEMTimeSeriesFieldOptimized
            if isinstance(self._field, (OctreeFEMTimeSeriesFieldOptimized, FEMTimeSeriesField)):
                return 32
            return 100 if self._field._storage == L.JT_STORE_F32 else 200
        return max(int(se), 0)

    def _sort_bits(self) -> int:
        b = self.options.sort_bits
        return 7 if b is None else int(b)

    def _engine(self, pos, times, dt, sched_dev=None, status=None, comp=None, ens=None):
        import torch
        if sched_dev is None:
            sched_dev = torch.from_numpy(self._schedule(times, dt).view(np.int32).reshape(-1, 8)).cuda()
        if status is None:
            status = torch.zeros(1, dtype=torch.int32, device="cuda")
        if comp is None and self._arith() == L.JT_ARITH_COMPENSATED:
            comp = torch.zeros_like(pos)
        return _Engine(self, pos, len(times) - 1, dt, sched_dev, status, comp, self._sort_every(pos.shape[0]),
                       ens=ens)

    def _run(self, pos, times, dt, k, compact, n_rows, positions, velocities, rows_out=None) -> int:
        """Advance ``pos`` (device, (N,3)) through all steps, filling rows 1..
        of the outputs.  Each recorded slab is copied to the host on a side
        stream while the next chunk runs; at most two slabs are alive."""
        import torch
        n = pos.shape[0]
        n_steps = len(times) - 1
        if n_steps <= 0:
            return 0
        eng = self._engine(pos, times, dt)
        record = n_rows > 1 and not self.options.record_final_only
        row_bytes = n * 12 * (2 if velocities is not None else 1)
        budget_rows = max(1, int(self.options.device_memory_gb * 1024 ** 3 // max(row_bytes, 1)))
        chunk = n_steps
        if record:  # steps per launch bounded by the rows that fit in one slab
            chunk = max(1, min(budget_rows * (k if compact else 1), n_steps))
        if self.options.time_chunk:
            chunk = max(1, min(chunk, int(self.options.time_chunk)))
        cb = self.options.progress_callback
        copy_stream = torch.cuda.Stream() if record else None
        inflight = collections.deque()       # (copy-done event or None, end step)

        def land(ev, end):
            if ev is not None:
                ev.synchronize()
            if cb is not None:
                cb(end / n_steps)

        s = 0
        try:
            while s < n_steps:
                e = min(s + chunk, n_steps)
                slab = vslab = None
                rec = None
                if record:
                    # rows written by steps s..e-1 are the counts c in (s, e]
                    r0, r1 = (s // k + 1, e // k) if compact else (s + 1, e)
                    nr = max(r1 - r0 + 1, 0)
                    if nr > 0:
                        slab = torch.zeros((nr, n, 3), dtype=torch.float32, device="cuda")
                        if velocities is not None:
                            vslab = torch.zeros_like(slab)
                    rec = (slab, vslab, k, compact, r0, nr)
                eng.advance(s, e, rec)
                ev = None
                if slab is not None:
                    ev = _copy_rows_async(slab, vslab, positions, velocities, r0, copy_stream)
                    if rows_out is not None:
                        rows_out.put(r0, nr, ev)
                inflight.append((ev, e))
                while len(inflight) > 1:
                    land(*inflight.popleft())
                s = e
            while inflight:
                land(*inflight.popleft())
        finally:
            if copy_stream is not None:
                copy_stream.synchronize()
        eng.finish()
        self.last_status = int(eng.status.item())
        self._last_path_length = eng.path.cpu().numpy() if eng.path is not None else None
        return eng.launches

    def track_device(self, pos, times, dt, status=None, comp=None, sched_dev=None, timers=None):
        """Advance device positions (N,3) in place through every step of the
        float32 time grid ``times`` without recording (benchmark and ensemble
        entry).  ``timers``: a list that receives a (start, end) CUDA-event
        pair around every tracking-kernel launch.  Returns the number of
        tracking launches and of all kernels this library launched."""
        eng = self._engine(pos, times, dt, sched_dev, status, comp)
        eng.timers = timers
        eng.advance(0, len(times) - 1, None)
        eng.finish()
        out = {"track_launches": eng.launches, "kernels": eng.kernels}
        if eng.stage is not None:
            # distinct pre-blended fields of the run and the bytes of one
            # (what a tracking launch must read at least once)
            out["stage_fields"] = eng.stage.n_fields
            out["stage_field_bytes"] = eng.stage.field_bytes
        return out

    def ensemble_batch(self, ensembles, release_times, n_timesteps: int, dt: Optional[float] = None,
                       duration: Optional[float] = None) -> "EnsembleBatch":
        """Device buffers and per-ensemble schedules of a batched run (see
        ``EnsembleBatch``); ``run()`` advances it, ``capture()`` records it
        in a CUDA graph."""
        return EnsembleBatch(self, ensembles, release_times, n_timesteps, dt, duration)

    def track_ensembles(self, ensembles, release_times, n_timesteps: int, dt: Optional[float] = None,
                        duration: Optional[float] = None, return_device: bool = False):
        """Final positions of many ensembles of uneven size and release time,
        advanced together.  Ensemble e gives what
        ``track_particles(x_e, (t_e, t_e + duration), n_timesteps, dt=dt)``
        gives in its last row (``duration`` defaults to (n_timesteps-1)*dt).
        Returns a list of (n_e, 3) float32 arrays, or the concatenated device
        tensor with ``return_device=True``."""
        b = self.ensemble_batch(ensembles, release_times, n_timesteps, dt, duration)
        if self.options.autotune:
            from .autotune import Autotuner
            Autotuner.shared().tune_batch(b)
        if self.options.cuda_graph:
            b.capture()
        b.run()
        return b.pos if return_device else b.finals()

    # ------------------------------------------------------------------
    def validate_configuration(self) -> Dict[str, Any]:
        """tracker.py:720-787 on a one-particle probe."""
        res = {"valid": True, "warnings": [], "errors": [], "configuration": {}}
        test_pos = np.array([[0.0, 0.0, 0.0]], dtype=F32)
        try:
            v = np.asarray(self._field.sample_at_positions(test_pos, 0.0), dtype=F32)
            if v.shape != (1, 3):
                res["errors"].append(f"field_fn returned wrong shape: {v.shape}, expected (1, 3)")
                res["valid"] = False
            if not np.all(np.isfinite(v)):
                res["warnings"].append("field_fn returned non-finite values")
        except Exception as e:  # noqa: BLE001 -- report, as the reference does
            res["errors"].append(f"field_fn test failed: {e}")
            res["valid"] = False
        try:
            b = np.asarray(self._bc(test_pos), dtype=F32)
            if b.shape != test_pos.shape:
                res["errors"].append(f"boundary_fn changed shape: {b.shape} != {test_pos.shape}")
                res["valid"] = False
        except Exception as e:  # noqa: BLE001
            res["errors"].append(f"boundary_fn test failed: {e}")
            res["valid"] = False
        res["configuration"] = {"backend": "gb300", "integrator": self._code,
                                "max_memory_gb": self.options.max_memory_gb,
                                "record_velocities": self.options.record_velocities}
        return res

    def benchmark_performance(self, test_sizes=(100, 500, 1000, 5000), n_timesteps: int = 100) -> Dict[str, Any]:
        """Wall time of track_particles at each size, particle-steps/s, the
        trajectory's size and the fitted scaling exponent (tracker.py:590-657)."""
        import math
        import time
        res: Dict[str, Any] = {"test_sizes": list(test_sizes), "n_timesteps": int(n_timesteps), "timing_results": {},
                               "memory_usage": {}, "throughput": {}, "scalability": {}}
        for n in test_sizes:
            x0 = np.random.uniform(-1, 1, size=(n, 3)).astype(F32)
            t0 = time.time()
            try:
                traj = self.track_particles(x0, (0.0, 1.0), n_timesteps)
                el = time.time() - t0
                res["timing_results"][n] = el
                res["memory_usage"][n] = traj.memory_usage_mb()
                res["throughput"][n] = n * n_timesteps / max(el, 1e-9)
            except Exception:  # noqa: BLE001 -- recorded as a failed size, as the reference does
                res["timing_results"][n] = res["memory_usage"][n] = res["throughput"][n] = None
        ok = [s for s in test_sizes if res["timing_results"][s] is not None]
        if len(ok) >= 2:
            xs = [math.log(ok[i + 1] / ok[i]) for i in range(len(ok) - 1)]
            tr = [res["timing_results"][ok[i + 1]] / res["timing_results"][ok[i]] for i in range(len(ok) - 1)]
            if all(r > 0 for r in tr):
                ys = [math.log(r) for r in tr]
                mx, my = sum(xs) / len(xs), sum(ys) / len(ys)
                den = sum((x - mx) ** 2 for x in xs)
                if den > 0:
                    k = sum((x - mx) * (y - my) for x, y in zip(xs, ys)) / den
                    res["scalability"] = {"scaling_exponent": k, "complexity": f"O(N^{k:.2f})"}
        return res

    def analyze_field_sampling(self, test_positions, time_points) -> Dict[str, Any]:
        """Sampling time per call and velocity statistics of the field at the
        given positions and times (tracker.py:659-718)."""
        import time
        q = ensure_positions_shape(test_positions)
        tp = np.asarray(time_points, dtype=F32)
        res: Dict[str, Any] = {"num_positions": q.shape[0], "num_times": len(tp), "sampling_stats": {},
                               "performance": {}, "field_properties": {}}
        vels, secs = [], []
        for t in tp:
            t0 = time.time()
            try:
                v = np.asarray(self._field.sample_at_positions(q, float(t)), dtype=F32)
            except Exception as e:  # noqa: BLE001
                res["field_properties"]["sampling_error"] = str(e)
                return res
            secs.append(time.time() - t0)
            vels.append(v)
        if secs:
            m = float(np.mean(secs))
            res["performance"] = {"mean_sampling_time": m, "sampling_rate_per_second": q.shape[0] / max(m, 1e-9),
                                  "total_samples": q.shape[0] * len(tp)}
            a = np.concatenate(vels, axis=0)
            mags = np.linalg.norm(a, axis=1)
            res["field_properties"] = {
                "velocity_magnitude": {"mean": float(np.mean(mags)), "std": float(np.std(mags)),
                                       "min": float(np.min(mags)), "max": float(np.max(mags))},
                "velocity_components": {ax: {"mean": float(np.mean(a[:, k])), "std": float(np.std(a[:, k]))}
                                        for k, ax in enumerate("xyz")},
                "finite_values": int(np.sum(np.isfinite(a).all(axis=1))),
                "infinite_values": int(np.sum(np.isinf(a).any(axis=1))),
                "nan_values": int(np.sum(np.isnan(a).any(axis=1)))}
        return res

    def get_memory_info(self) -> Dict[str, Any]:
        """Host memory of this process (tracker.py:789-805), plus the GPU's
        free and total memory."""
        out: Dict[str, Any]
        try:
            import psutil
            proc = psutil.Process()
            mem = proc.memory_info()
            vm = psutil.virtual_memory()
            out = {"available": True, "rss_mb": mem.rss / 1024 ** 2, "vms_mb": mem.vms / 1024 ** 2,
                   "percent": proc.memory_percent(), "system_available_mb": vm.available / 1024 ** 2,
                   "system_total_mb": vm.total / 1024 ** 2}
        except Exception:  # noqa: BLE001
            out = {"available": False, "message": "psutil not available"}
        try:
            import torch
            if torch.cuda.is_available():
                free, total = torch.cuda.mem_get_info()
                out["device_free_mb"], out["device_total_mb"] = free / 1024 ** 2, total / 1024 ** 2
        except Exception:  # noqa: BLE001
            pass
        return out

    def estimate_runtime(self, n_particles: int, n_timesteps: int, calibration_particles: int = 1000,
                         calibration_steps: int = 10) -> Dict[str, Any]:
        """tracker.py:538-588 with a GPU calibration run."""
        import time
        x = np.random.uniform(-1, 1, size=(calibration_particles, 3)).astype(F32)
        t0 = time.time()
        try:
            self.track_particles(x, (0.0, 1.0), calibration_steps)
        except Exception as e:  # noqa: BLE001
            return {"success": False, "error": str(e), "error_type": type(e).__name__}
        el = time.time() - t0
        per = el / max(calibration_particles * calibration_steps, 1)
        est = n_particles * n_timesteps * per
        return {"success": True, "estimated_runtime_seconds": est, "time_per_particle_step": per,
                "calibration_time": el, "calibration_particles": calibration_particles}


class _Engine:
    """Buffers of one run: positions in slot order, optional Kahan terms, the
    slot -> particle map of the locality sort and the sort workspace."""

    def __init__(self, tracker, pos, n_steps, dt, sched_dev, status, comp, sort_every, ens=None):
        import torch
        self.t, self.out, self.n_steps = tracker, pos, n_steps
        self.status, self.sched = status, sched_dev
        self.n = pos.shape[0]
        self.sort_every = sort_every
        self.launches = 0      # tracking-kernel launches
        self.kernels = 0       # every kernel of this library
        self.timers = None
        self.field = tracker._field
        self.field_c = None    # the gathering descriptor, built when a launch needs it
        self.bc_c = tracker._bc.jt_boundary()
        self.lib = L.load()
        self.stream = L.stream_ptr()
        self.pos, self.comp, self.ids = pos, comp, None
        if sort_every > 0 and self.n > 0:
            self.grid = tracker._field.sort_grid(bits=tracker._sort_bits())
            self.pos = torch.empty_like(pos)
            self.pos_alt = torch.empty_like(pos)
            self.comp_alt = torch.empty_like(comp) if comp is not None else None
            self.ids = torch.empty(self.n, dtype=torch.int32, device=pos.device)
            self.ids_alt = torch.empty_like(self.ids)
            ws = int(self.lib.jt_cell_sort_workspace_bytes(self.n, self.grid.bits))
            self.ws = torch.empty(ws, dtype=torch.uint8, device=pos.device)
            self._sort(first=True)
        self.p = tracker.make_params(self.pos, dt, n_steps, sched_dev, status, self.comp)
        # per-particle path length (indexed by particle, so the sort leaves it be)
        self.path = None
        if ens is None and tracker.options.record_path_length and self.n > 0:
            self.path = torch.zeros(self.n, dtype=torch.float32, device=pos.device)
            self.p.path = self.path.data_ptr()
        if ens is not None:       # (device offsets (E+1,) int32, E, schedule entries per ensemble)
            self.ens = ens
            self.p.ens_offsets, self.p.n_ens, self.p.schedule_stride = ens[0].data_ptr(), ens[1], ens[2]
        self.stage = None
        if ens is None and tracker.options.stage_fields and n_steps > 0 and self.n > 0:
            from .fields import StructuredTimeSeriesField
            if isinstance(tracker._field, StructuredTimeSeriesField):
                f = tracker._field
                overlap = bool(tracker.options.stage_overlap)
                rec_bytes = _stage_node_bytes(f) * (2 if overlap else 1)
                free = torch.cuda.mem_get_info(pos.device)[0]
                chunk = _stage_chunk(int(tracker.options.stage_chunk), n_steps, len(f.grid_x) * len(f.grid_y) * len(f.grid_z),
                                     rec_bytes, free)
                if chunk > 0:
                    self.stage = _StageFields(f, sched_dev, n_steps, chunk, overlap=overlap)

    def _sort(self, first=False):
        src_pos = self.out if first else self.pos
        dst_pos = self.pos if first else self.pos_alt
        src_ids = None if first else self.ids
        dst_ids = self.ids if first else self.ids_alt
        comp_dst = None
        if self.comp is not None:
            comp_dst = self.comp_alt
        L.check(self.lib.jt_cell_sort(C.byref(self.grid), self.n, L.ptr(src_pos), L.ptr(self.comp), L.ptr(src_ids),
                                      L.ptr(dst_pos), L.ptr(comp_dst), L.ptr(dst_ids), L.ptr(self.ws),
                                      self.ws.numel(), self.stream))
        self.kernels += 5      # keys, two scan levels, scan add, scatter
        if not first:
            self.pos, self.pos_alt = self.pos_alt, self.pos
            self.ids, self.ids_alt = self.ids_alt, self.ids
        if self.comp is not None:
            self.comp, self.comp_alt = self.comp_alt, self.comp

    def _stop(self, s, e, staged):
        """End of the launch that starts at step s: the next re-sort, the
        stage-field chunk, or e."""
        stop = e
        if self.sort_every > 0:
            stop = min(e, (s // self.sort_every + 1) * self.sort_every)
        if staged:
            stop = min(stop, s + self.stage.chunk)
        return stop

    def advance(self, s, e, rec):
        """Steps [s, e) with optional recording (slab, vslab, k, compact, row0, rows)."""
        p = self.p
        staged = self.stage is not None and not (rec is not None and rec[1] is not None)
        while s < e:
            if self.sort_every > 0 and s > 0 and s % self.sort_every == 0:
                self._sort()
            stop = self._stop(s, e, staged)
            if staged:
                self.kernels += self.stage.prepare(s, stop)
                field_c = self.stage.field_c
                p.schedule = self.stage.sched.data_ptr()
            else:
                if self.field_c is None:
                    self.field_c = self.field.jt_field()
                field_c = self.field_c
                p.schedule = self.sched.data_ptr()
            p.pos = self.pos.data_ptr()
            p.comp = self.comp.data_ptr() if self.comp is not None else None
            p.ids = self.ids.data_ptr() if self.ids is not None else None
            p.step_begin, p.step_end = s, stop
            if rec is not None:
                slab, vslab, k, compact, r0, nr = rec
                p.traj = slab.data_ptr() if slab is not None else None
                p.vel = vslab.data_ptr() if vslab is not None else None
                p.record_every, p.record_compact, p.row_base, p.n_rows = k, int(compact), r0, nr
            else:
                p.traj = p.vel = None
            if self.timers is not None:
                import torch
                ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                ev[0].record()
            L.check(self.lib.jt_track(C.byref(field_c), C.byref(self.bc_c), C.byref(p), self.stream))
            if self.timers is not None:
                ev[1].record()
                self.timers.append(ev)
            self.launches += 1
            self.kernels += 1
            if staged and stop < e:
                self.kernels += self.stage.prefetch(stop, self._stop(stop, e, staged))
            s = stop

    def finish(self):
        if self.ids is not None:
            L.check(self.lib.jt_unpermute(self.n, L.ptr(self.pos), L.ptr(self.ids), L.ptr(self.out), self.stream))
            self.kernels += 1


class EnsembleBatch:
    """Ensembles of uneven size and release time in one tracking pass.

    All ensembles take the same number of steps; ensemble e steps on its own
    float32 time grid ``linspace(t_e, t_e + duration, n_timesteps)`` (the
    grid ``track_particles`` builds for time_span (t_e, t_e + duration)).
    The particles of all ensembles sit in one (sum n_e, 3) device array in
    ensemble order; one tracking launch per time chunk advances them all,
    each thread reading its ensemble's row of a stacked schedule through the
    (E+1) offset table.  ``capture()`` records the whole pass (initial copy,
    locality sorts, tracking launches, unpermute) in a CUDA graph that
    ``run()`` then replays.
    """

    def __init__(self, tracker: ParticleTracker, ensembles, release_times, n_timesteps: int,
                 dt: Optional[float] = None, duration: Optional[float] = None):
        import torch
        self.tracker = tracker
        xs = [ensure_positions_shape(x) for x in ensembles]
        rel = np.asarray(release_times, dtype=np.float64).reshape(-1)
        if len(xs) != len(rel):
            raise ValueError(f"{len(xs)} ensembles but {len(rel)} release times")
        if len(xs) == 0:
            raise ValueError("no ensembles")
        T = int(n_timesteps)
        if T < 2:
            raise ValueError("n_timesteps must be >= 2")
        if duration is None:
            if dt is None:
                raise ValueError("give dt or duration")
            duration = (T - 1) * float(dt)
        self.times = [np.linspace(float(t), float(t) + float(duration), T, dtype=np.float32) for t in rel]
        if dt is None:
            steps = {float(tm[1] - tm[0]) for tm in self.times}
            if len(steps) != 1:
                raise ValueError("with dt=None every ensemble's float32 step must agree; pass dt")
            dt = steps.pop()
        self.dt = float(dt)
        self.n_steps = T - 1
        self.sizes = np.array([len(x) for x in xs], dtype=np.int64)
        off = np.zeros(len(xs) + 1, dtype=np.int64)
        np.cumsum(self.sizes, out=off[1:])
        if off[-1] >= 2 ** 31:
            raise ValueError("at most 2^31-1 particles per batch")
        self.offsets = off
        self.n = int(off[-1])
        if not torch.cuda.is_available():
            raise RuntimeError("ensemble tracking runs on a CUDA GPU; none is visible")
        host = torch.empty((self.n, 3), dtype=torch.float32).pin_memory()
        hv = host.numpy()
        for x, a in zip(xs, off[:-1]):
            hv[a:a + len(x)] = x
        self.x0 = host.to("cuda", non_blocking=True)
        self.pos = torch.empty_like(self.x0)
        sched = np.stack([tracker._schedule(tm, self.dt) for tm in self.times])
        self.stride = sched.shape[1]
        self.sched_dev = torch.from_numpy(sched.view(np.int32).reshape(-1, 8)).cuda()
        self.off_dev = torch.from_numpy(off.astype(np.int32)).cuda()
        self.status = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.comp = torch.zeros_like(self.pos) if tracker._arith() == L.JT_ARITH_COMPENSATED else None
        self.graph = None
        self._graph_engine = None
        self.launches = 0
        self.kernels = 0

    def _pass(self):
        """One tracking pass on the current stream: x0 -> pos."""
        self.pos.copy_(self.x0)
        if self.comp is not None:
            self.comp.zero_()
        eng = self.tracker._engine(self.pos, self.times[0], self.dt, self.sched_dev, self.status, self.comp,
                                   ens=(self.off_dev, len(self.sizes), self.stride))
        eng.advance(0, self.n_steps, None)
        eng.finish()
        self.launches, self.kernels = eng.launches, eng.kernels
        return eng

    def capture(self):
        """Record one pass in a CUDA graph (after one eager pass that loads
        the library and sets kernel attributes outside the capture)."""
        import torch
        self._pass()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._graph_engine = self._pass()
        self.graph = g
        return self

    def run(self):
        """Advance every ensemble from its initial positions to its last step."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._pass()
        return self

    def check_status(self) -> int:
        st = int(self.status.item())
        self.tracker.last_status = st
        return st

    def finals(self) -> List[np.ndarray]:
        out = self.pos.cpu().numpy()
        self.check_status()
        return [out[a:b] for a, b in zip(self.offsets[:-1], self.offsets[1:])]


class _StageFields:
    """Pre-blended stage fields of a regular-grid run (jt_stage_fields).

    The stage entries of the run (step s, stage k: 0 at t, 1 at t + h/2,
    2 at t + h) are numbered in order, and an entry equal to the one before it
    (the t + h entry of a step and the t entry of the next, when the float32
    times agree) takes the same number u.  Entry u lives in ring slot
    u mod R; the entries of a launch of at most ``chunk`` steps span at most
    3 * chunk numbers, so ``prepare`` finds room for all of them with
    R = 3 * chunk.  Float32 snapshots give float32 yz-quads blended with the
    exact arithmetic; 16-bit snapshots (per-snapshot scale or affine tiles)
    give offset float16 yz-quads of the blend divided by a power-of-two bound
    of it.

    Overlap (R = 6 * chunk): ``prefetch`` blends the next launch's fields on a
    side stream while the current launch tracks.  Its writes go to the slots
    of numbers below the current launch's first (two launches span at most
    6 * chunk numbers), after the launches before the current one are done
    (an event recorded just before the current launch).
    """

    def __init__(self, field, sched_dev, n_steps: int, chunk: int, overlap: bool = False):
        import torch
        from .schedule import BLEND_DTYPE
        self.lib = L.load()
        self.chunk = max(1, min(int(chunk), n_steps))
        self.overlap = bool(overlap)
        host = np.ascontiguousarray(sched_dev.cpu().numpy()).view(BLEND_DTYPE).reshape(-1)
        n_ent = 4 * n_steps
        host = host[:n_ent].copy()
        every = host.reshape(n_steps, 4)[:, :3].reshape(-1).copy()        # 3 entries per step
        self.uid = _stage_numbers(every)
        first = np.ones(len(every), dtype=bool)
        first[1:] = self.uid[1:] != self.uid[:-1]
        src = every[first]                                                  # one entry per number
        self.slots = (6 if self.overlap else 3) * self.chunk
        self.ready = -1                                                     # last number blended
        self.tile = getattr(field, "encoding", "snapshot") == "tile"
        self.f32 = field._storage == L.JT_STORE_F32
        self.out_storage = L.JT_STORE_STAGE_F32Q if self.f32 else L.JT_STORE_STAGE_F16
        scales = np.ones(len(src), dtype=F32)
        if self.tile:
            field.tile_field()
            scales = _tile_stage_scales(src, field._tiles["amax"])
        elif not self.f32:
            scales = _stage_scales(src)
        # the tracking schedule: pair -> slot, weights -> the slot's scale
        stage = host.copy().reshape(n_steps, 4)
        uid = self.uid.reshape(n_steps, 3)
        for k in range(3):
            stage[:, k]["pair"] = uid[:, k] % self.slots
            stage[:, k]["form"] = L.JT_BLEND_WEIGHTED
            stage[:, k]["wa"] = scales[uid[:, k]]
            stage[:, k]["wb"] = 0.0
        dev = sched_dev.device
        self.sched = torch.from_numpy(stage.reshape(-1).view(np.int32).reshape(-1, 8).copy()).to(dev)
        self.src = torch.from_numpy(src.view(np.int32).reshape(-1, 8).copy()).to(dev)
        self.scales = torch.from_numpy(scales).to(dev)
        if self.tile:
            self.src_field = field.tile_field()
            g0 = field._tiles["grid"]
        else:
            field._device()
            g0 = field._cgrid
            self.src_field = field.jt_field()
        nodes = len(field.grid_x) * len(field.grid_y) * len(field.grid_z)
        rec = 12 if self.f32 else 8                                          # float32 words per node
        # float32-quad slots hold an even number of node records, so that
        # every slot starts on a 32-byte boundary (jt_stage_fields)
        stride = nodes + (nodes & 1) if self.f32 else nodes
        self.buf = torch.empty(self.slots * stride * rec, dtype=torch.float32, device=dev)
        self.nodes, self.rec, self.stride = nodes, rec, stride
        self.n_fields = int(self.uid[-1]) + 1 if len(self.uid) else 0
        self.field_bytes = stride * rec * 4
        self.side = self.before = self.pending = None
        if self.overlap:
            self.side = torch.cuda.Stream(device=dev, priority=-1)
            self.buf.record_stream(self.side)
        g = L.GridField()
        C.memmove(C.byref(g), C.byref(g0), C.sizeof(L.GridField))            # copy the descriptor
        g.storage = self.out_storage
        g.n_pairs = self.slots
        g.pair_stride = stride
        g.pairs = self.buf.data_ptr()
        g.tile_base = None
        g.tiles[:] = [0, 0, 0]
        self.grid = g
        self.field_c = L.Field(kind=L.JT_FIELD_GRID, grid=C.pointer(g))

    def prepare(self, s: int, stop: int) -> int:
        """Put the fields of steps [s, stop) in their slots before the launch
        that tracks them: wait for a prefetch, blend what is missing on the
        current stream.  Returns the number of kernels launched."""
        import torch
        cur = torch.cuda.current_stream()
        if self.pending is not None:
            cur.wait_event(self.pending)
            self.pending = None
        n = self._blend(s, stop, L.stream_ptr())
        if self.overlap:
            self.before = torch.cuda.Event()
            self.before.record(cur)
        return n

    def prefetch(self, s: int, stop: int) -> int:
        """Blend the fields of the next launch, steps [s, stop), on the side
        stream once the launches before the current one are done."""
        import torch
        if not self.overlap:
            return 0
        self.side.wait_event(self.before)
        n = self._blend(s, stop, L.stream_ptr(self.side))
        self.pending = torch.cuda.Event()
        self.pending.record(self.side)
        return n

    def _blend(self, s: int, stop: int, stream) -> int:
        runs, self.ready = _stage_plan(self.uid, s, stop, self.ready, self.slots)
        for lo, run in runs:
            ent = self.src.data_ptr() + lo * 32
            sc = self.scales.data_ptr() + lo * 4
            out = self.buf.data_ptr() + (lo % self.slots) * self.stride * self.rec * 4
            if self.tile:
                L.check(self.lib.jt_stage_tile_fields(C.byref(self.src_field), C.c_void_p(ent), C.c_void_p(sc),
                                                      run, C.c_void_p(out), stream))
                continue
            L.check(self.lib.jt_stage_fields(C.byref(self.src_field), C.c_void_p(ent),
                                             C.c_void_p(None if self.f32 else sc), run, self.out_storage,
                                             C.c_void_p(out), stream))
        return len(runs)


def _stage_numbers(entries) -> np.ndarray:
    """Run-ordered numbers of blend entries: an entry whose bytes equal the
    previous entry's takes its number, any other the next one."""
    raw = np.ascontiguousarray(entries).view(np.uint8).reshape(len(entries), -1)
    new = np.ones(len(entries), dtype=np.int64)
    if len(entries) > 1:
        new[1:] = np.any(raw[1:] != raw[:-1], axis=1)
    new[0] = 0
    return np.cumsum(new)


def _stage_node_bytes(field) -> int:
    """Device bytes per grid node of one pre-blended stage field: float32
    yz-quads (48 B) or offset float16 yz-quads (32 B)."""
    return 48 if field._storage == L.JT_STORE_F32 else 32


def _stage_chunk(chunk: int, n_steps: int, nodes: int, rec_bytes: int, free_bytes: int) -> int:
    """Steps per stage-field chunk: the requested chunk, shortened so that the
    ring (3 fields per step, ``rec_bytes`` per node) takes at most a quarter
    of the free device memory; 0 (gather snapshot pairs instead) when the
    memory shortens it below 4 steps."""
    want = max(1, min(int(chunk), int(n_steps)))
    fit = int((free_bytes // 4) // max(1, 3 * nodes * rec_bytes))
    if fit >= want:
        return want
    return fit if fit >= 4 else 0


def _stage_plan(uid: np.ndarray, s: int, stop: int, ready: int, slots: int):
    """Blend launches that put every field of steps [s, stop) in its slot.

    Returns ([(first number, count), ...], new ``ready``).  Numbers up to
    ``ready`` were blended by earlier launches in order; the last ``slots`` of
    them are still in the ring, so a range that starts at or before ``ready``
    only needs the numbers after it.  A range that wraps the ring is split.
    """
    lo, hi = int(uid[3 * s]), int(uid[3 * stop - 1]) + 1
    if hi - lo > slots:
        raise ValueError("a tracking launch spans more stage fields than the ring holds")
    if lo <= ready < hi:
        lo = ready + 1
    runs = []
    while lo < hi:
        run = min(hi - lo, slots - lo % slots)
        runs.append((lo, run))
        lo += run
    return runs, hi - 1


def _tile_stage_scales(src, amax) -> np.ndarray:
    """Power-of-two bounds of |blend| for affine-tile snapshots, whose
    entries carry plain weights: the larger of the pair's max |v| times
    |wa| + |wb| (folded forms) or 1 + 2 |wb| (lerp forms)."""
    n = len(amax)
    p = np.clip(src["pair"].astype(np.int64), 0, n - 2)
    m = np.maximum(amax[p], amax[p + 1])
    wa = np.abs(src["wa"].astype(np.float64))
    wb = np.abs(src["wb"].astype(np.float64))
    lerp = (src["form"] == L.JT_BLEND_LERP_FWD) | (src["form"] == L.JT_BLEND_LERP_BWD)
    bound = m * np.where(lerp, 1.0 + 2.0 * wb, wa + wb)
    bound = np.where(np.isfinite(bound) & (bound > 0), bound, 1.0)
    return np.exp2(np.ceil(np.log2(bound))).astype(F32)


def _stage_scales(src) -> np.ndarray:
    """Power-of-two bounds of |blend| on raw 16-bit values (|raw| <= 1):
    |wa| + |wb| for the folded forms, (sa + sb)(1 + |w|) for the lerps."""
    wa = np.abs(src["wa"].astype(np.float64))
    wb = np.abs(src["wb"].astype(np.float64))
    sa = np.abs(src["sa"].astype(np.float64))
    sb = np.abs(src["sb"].astype(np.float64))
    lerp = (src["form"] == L.JT_BLEND_LERP_FWD) | (src["form"] == L.JT_BLEND_LERP_BWD)
    bound = np.where(lerp, (sa + sb) * (1.0 + wb), wa + wb)
    bound = np.where(bound > 0, bound, 1.0)
    return np.exp2(np.ceil(np.log2(bound))).astype(F32)


def _copy_rows_async(slab, vslab, positions, velocities, r0: int, copy_stream):
    """Copy a recorded slab into host rows r0.. on ``copy_stream`` once the
    current stream has written it; returns the copy's completion event."""
    import torch
    written = torch.cuda.Event()
    written.record()
    copy_stream.wait_event(written)
    nr = slab.shape[0]
    with torch.cuda.stream(copy_stream):
        torch.from_numpy(positions[r0:r0 + nr]).copy_(slab, non_blocking=True)
        slab.record_stream(copy_stream)
        if vslab is not None:
            torch.from_numpy(velocities[r0:r0 + nr]).copy_(vslab, non_blocking=True)
            vslab.record_stream(copy_stream)
    done = torch.cuda.Event()
    done.record(copy_stream)
    return done


class _RowStream:
    """Hands trajectory rows to ``TrackerOptions.row_sink`` on a writer
    thread, in the order they are put, each once its copy has landed (a CUDA
    event, or the thread that writes it)."""

    def __init__(self, sink, positions, velocities, row_times):
        import queue
        import threading
        self.sink, self.pos, self.vel, self.times = sink, positions, velocities, np.asarray(row_times, dtype=F32)
        self.q = queue.Queue()
        self.error = None
        self.thread = threading.Thread(target=self._work, daemon=True)
        self.thread.start()

    def put(self, r0: int, nr: int, ready=None) -> None:
        self.q.put((r0, nr, ready))

    def _work(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            r0, nr, ready = item
            try:
                if ready is not None:
                    ready.join() if hasattr(ready, "join") else ready.synchronize()
                if self.error is None:
                    self.sink(r0, self.pos[r0:r0 + nr], None if self.vel is None else self.vel[r0:r0 + nr],
                              self.times[r0:r0 + nr])
            except BaseException as exc:       # re-raised by close() on the caller's thread
                if self.error is None:
                    self.error = exc

    def close(self, raise_error: bool = True) -> None:
        self.q.put(None)
        self.thread.join()
        if raise_error and self.error is not None:
            raise self.error


# Trajectory arrays up to this size live in pinned host memory: device
# copies reach them at full speed, and torch's pinned-block cache hands the
# pages of a dropped trajectory to the next call, so no run pays for first
# touches of freshly mapped memory.  Larger arrays are plain NumPy memory.
PINNED_TRAJECTORY_BYTES = 1 << 30


def _host_rows(shape, zero: bool) -> np.ndarray:
    """A float32 host array for trajectory rows (pinned when small enough)."""
    nbytes = 4 * int(np.prod(shape))
    if 0 < nbytes <= PINNED_TRAJECTORY_BYTES:
        import torch
        if torch.cuda.is_available():
            t = torch.empty(shape, dtype=torch.float32, pin_memory=True)
            if zero:
                t.zero_()
            return t.numpy()
    return np.zeros(shape, dtype=F32) if zero else np.empty(shape, dtype=F32)


def create_tracker(integrator_name: str, field, boundary_condition, **options) -> ParticleTracker:
    """tracker.py:810-855."""
    if integrator_name not in INTEGRATORS:
        raise ValueError(f"Unknown integrator: {integrator_name}. Available: {list(INTEGRATORS.keys())}")
    integrator = INTEGRATORS[integrator_name]
    if hasattr(field, "sample_at_positions"):
        field_fn = field
    elif hasattr(field, "sample"):
        field_fn = field
    elif callable(field):
        field_fn = field
    else:
        raise TypeError("field must be BaseField-like or a callable: field(positions, t) -> velocities")
    if not callable(boundary_condition):
        raise TypeError("boundary_condition must be callable")
    tracker_options = TrackerOptions(**options)
    return ParticleTracker(integrator=integrator, field_fn=field_fn, boundary_fn=boundary_condition,
                           options=tracker_options)


def track_particles_simple(initial_positions, velocity_field, time_span, n_timesteps, integrator: str = "rk4",
                           boundary_condition=None, dt: Optional[float] = None, **tracker_options) -> Trajectory:
    """tracker.py:857-880."""
    if boundary_condition is None:
        from .boundary import no_boundary
        boundary_condition = no_boundary()
    tr = create_tracker(integrator, velocity_field, boundary_condition, **tracker_options)
    return tr.track_particles(initial_positions, time_span, n_timesteps, dt=dt)


__all__ = ["TrackerOptions", "ParticleTracker", "create_tracker", "track_particles_simple"]


def compare_integrators(initial_positions, velocity_field, time_span: Tuple[float, float], n_timesteps: int,
                        integrators=("euler", "rk2", "rk4"), dt: Optional[float] = None, **options) -> Dict[str, Any]:
    """Each integrator over the same run without boundaries: trajectories,
    wall times and final-position differences against the first
    (tracker.py:882-951)."""
    import time
    from .boundary import no_boundary
    res: Dict[str, Any] = {"integrators": list(integrators), "trajectories": {}, "timing": {}, "comparison": {}}
    for name in integrators:
        try:
            tr = create_tracker(name, velocity_field, no_boundary(), **options)
            t0 = time.time()
            traj = tr.track_particles(initial_positions, time_span, n_timesteps, dt=dt)
            res["trajectories"][name], res["timing"][name] = traj, time.time() - t0
        except Exception:  # noqa: BLE001 -- recorded as a failed integrator, as the reference does
            res["trajectories"][name] = res["timing"][name] = None
    ok = {k: v for k, v in res["trajectories"].items() if v is not None}
    if len(ok) >= 2:
        names = list(ok)
        ref = ok[names[0]].positions[-1]
        for name in names[1:]:
            d = np.linalg.norm(ok[name].positions[-1] - ref, axis=1)
            res["comparison"][f"{name}_vs_{names[0]}"] = {"mean_difference": float(np.mean(d)),
                                                          "max_difference": float(np.max(d)),
                                                          "std_difference": float(np.std(d))}
    return res
