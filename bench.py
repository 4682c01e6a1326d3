#!/usr/bin/env python
"""Benchmark of the tracking hot path on one GB300 (or N, one rank per GPU).

Workload (the precision configuration): 128^3 clamp grid, 64 snapshots over
[0,2] of ABC flow + (1,0,0) + N(0, 0.01^2) noise, 16,777,216 particles on a
256^3 lattice, continuous inlet at x=0 with grid-preserving replacement on a
256x256 lattice, RK4 dt=0.002, 1000 steps.  One bench step = one full
1000-step pass over all particles.

value      : particle-steps/s of the BF16-storage path, inputs resident in HBM
variants   : the same for FP32 (exact, bit-compatible) and FP16 storage
e2e        : the same metric through the public API (create_tracker(...)
             .track_particles) from pinned host positions to host results
error      : relative position error vs the FP64 CPU oracle on every 256th
             particle (the inlet keeps particles independent)
--impl reference : the CPU restatement of the reference on all host cores
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RK4 particle-steps/s on 1 GB300: BF16/adjoint vs plain FP32 at stated FP64 error"
UNIT = "particle-steps/s"
# algorithmic bytes per RK4 particle-step of k_track (cache-oblivious): 4 field
# evaluations x 8 corners x 3 values of one pre-blended time level (float32 or
# float16 stage fields) + 24 B of position read/write
BYTES_PER_PSTEP = {"f32": 4 * 8 * 12 + 24, "bf16": 4 * 8 * 6 + 24, "f16": 4 * 8 * 6 + 24}


def profile_figure(key, storage):
    """A figure of the committed ncu summary of k_track
    (profiles/k_track_precision.md, line '<key> <storage> <value>')."""
    f = ROOT / "profiles" / "k_track_precision.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = line.replace("|", " ").split()
        if len(parts) >= 3 and parts[0] == key and parts[1] == storage:
            try:
                return float(parts[2])
            except ValueError:
                return None
    return None


def traffic_per_pstep(storage):
    """DRAM bytes per particle-step of k_track (ncu, full size)."""
    return profile_figure("dram_bytes_per_particle_step", storage)


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--variants", default="bf16,f32,f16")
    p.add_argument("--seeds", type=int, default=256, help="lattice seeds per axis (256 -> 16,777,216)")
    p.add_argument("--n-steps", type=int, default=1000)
    p.add_argument("--dt", type=float, default=0.002)
    p.add_argument("--sort-every", type=int, default=None, help="locality re-sort interval (default: automatic)")
    p.add_argument("--sort-bits", type=int, default=None, help="cells per axis of the re-sort as 2^bits (default 7)")
    p.add_argument("--block-size", type=int, default=0, help="tracking kernel threads per block (0: 256)")
    p.add_argument("--stage-chunk", type=int, default=32, help="steps per stage-field chunk")
    p.add_argument("--no-stage-overlap", action="store_true",
                   help="blend each chunk's stage fields before its launch instead of during the previous one")
    p.add_argument("--grid", type=int, default=128)
    p.add_argument("--no-error", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-fem", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--fem-steps", type=int, default=1000)
    p.add_argument("--adj-lattice", default="256,256,64", help="seed lattice of the adjoint leg")
    p.add_argument("--adj-steps", type=int, default=500)
    p.add_argument("--density-particles", type=int, default=16_000_000)
    p.add_argument("--leg", default=None, choices=["fem", "fem_hash", "batch", "adjoint", "density"],
                   help="run one configuration leg alone and print its JSON (with --profile: the leg's timed "
                        "region bracketed by cudaProfilerStart/Stop)")
    p.add_argument("--profile", action="store_true",
                   help="first variant only, no error/e2e/CPU legs; the timed region is bracketed by "
                        "cudaProfilerStart/Stop for ncu --profile-from-start off")
    return p.parse_args()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = np.array([float(r[1]) for r in rows if r[1].replace(".", "").isdigit()])
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        load = sm[sm > 0.5 * smax] if len(sm) else sm
        return {"sm_mhz": float(np.median(load if len(load) else sm)), "sm_max_mhz": smax,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def oracle_subset_run(case, idx, precision, n_threads=0):
    import oracle
    g = case["grid"][0]
    spec = oracle.GridSpec(case["data"], case["times"], g, g, g, "clamp")
    lat = np.linspace(np.float32(0), np.float32(1), case["concentrations"]["y"], dtype=np.float32)
    bc = oracle.BoundarySpec(inlet_axis=0, inlet_positive=True, lattices=[lat, lat])
    times = np.linspace(case["time_span"][0], case["time_span"][1], case["n_timesteps"], dtype=np.float32)
    t0 = time.perf_counter()
    out, _, _ = oracle.track(spec, bc, case["x0"][idx], times, case["dt"], "rk4", precision=precision,
                             n_threads=n_threads)
    return out, time.perf_counter() - t0


def run_reference(a, world, rank):
    """CPU restatement of the reference on all host cores (oracle port)."""
    if rank != 0:
        return
    from jaxtrace_gb300 import workloads as W
    import oracle
    case = W.precision_case(n=a.grid, seeds=(a.seeds,) * 3, lattice=a.seeds, n_steps=a.n_steps, dt=a.dt)
    cores = os.cpu_count() or 1
    n = len(case["x0"])
    sample = min(n, 4096)
    idx = np.linspace(0, n - 1, sample).astype(np.int64)
    oracle.build()
    for _ in range(a.warmup):
        oracle_subset_run(case, idx[:256], oracle.ORC_F32, cores)
    times = []
    for _ in range(a.steps):
        _, dt = oracle_subset_run(case, idx, oracle.ORC_F32, cores)
        times.append(dt)
    ms = float(np.mean(times)) * 1e3
    val = sample * a.n_steps / (ms / 1e3)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(a), "sample_particles": sample},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sample} of the {n} particles x {a.n_steps} RK4 steps per bench step, "
                                       f"float32 C restatement of the NumPy reference path, OpenMP"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def adjoint_leg(a, profile=False):
    """Differentiation configuration: plain ABC field at 64^3 (16 snapshots,
    periodic), 256x256x64 lattice seeds, RK4 dt=0.01, 500 steps, checkpoint
    every 50; loss = sum |x_T - y|^2 with y ~ U[0,1)^3 (default_rng(3)).
    Times the forward pass (with checkpoints) and the backward pass, and
    checks dL/dx0 against float64 central differences on sampled particles."""
    import torch

    import jaxtrace_gb300 as jt
    import oracle
    from jaxtrace_gb300 import workloads as W
    from jaxtrace_gb300.adjoint import AdjointRK4
    c = W.plain_rk4(n_particles=1, n=64, n_snap=16)
    g = c["grid"][0]
    lattice = tuple(int(v) for v in a.adj_lattice.split(","))
    x0 = jt.uniform_grid_seeds(lattice, W.UNIT)
    n = len(x0)
    y = np.random.default_rng(3).uniform(size=(n, 3)).astype(np.float32)
    solver = AdjointRK4(c["times"], g, g, g, "periodic", jt.periodic_boundary(W.UNIT), checkpoint_every=50)
    x0_t = torch.tensor(x0, device="cuda", requires_grad=True)
    U_t = torch.tensor(c["data"].reshape(16, 64, 64, 64, 3), device="cuda", requires_grad=True)
    y_t = torch.tensor(y, device="cuda")
    n_steps, dt = a.adj_steps, 0.01
    if profile:
        # one untimed pass, then one pass inside cudaProfilerStart/Stop
        for k in range(2):
            if k == 1:
                torch.cuda.synchronize()
                torch.cuda.profiler.start()
            xT = solver(x0_t, U_t, (0.0, n_steps * dt), n_steps + 1, dt=dt)
            ((xT - y_t) ** 2).sum().backward()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        return {}
    fwd_ms, bwd_ms = [], []
    for it in range(a.warmup + a.steps):
        x0_t.grad = None
        U_t.grad = None
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record()
        xT = solver(x0_t, U_t, (0.0, n_steps * dt), n_steps + 1, dt=dt)
        e[1].record()
        loss = ((xT - y_t) ** 2).sum()
        loss.backward()
        e[2].record()
        torch.cuda.synchronize()
        if it >= a.warmup:
            fwd_ms.append(e[0].elapsed_time(e[1]))
            bwd_ms.append(e[1].elapsed_time(e[2]))
    gx = x0_t.grad.cpu().numpy().astype(np.float64)
    # float64 central differences of single particles (each particle's loss term is its own)
    spec = oracle.GridSpec(c["data"], c["times"], g, g, g, "periodic")
    obc = oracle.BoundarySpec(kinds=("periodic",) * 3)
    rng = np.random.default_rng(17)
    fd_stats = {}
    for horizon in sorted({min(50, n_steps), n_steps}):
        if horizon != n_steps:
            # a shorter horizon needs its own adjoint
            xs = torch.tensor(x0[:4096], device="cuda", requires_grad=True)
            xh = solver(xs, U_t.detach(), (0.0, horizon * dt), horizon + 1, dt=dt)
            ((xh - y_t[:4096]) ** 2).sum().backward()
            gref = xs.grad.cpu().numpy().astype(np.float64)
            pool = 4096
        else:
            gref, pool = gx, n
        times = np.linspace(0.0, horizon * dt, horizon + 1, dtype=np.float32)
        picks = list(zip(rng.integers(0, pool, 96), rng.integers(0, 3, 96)))
        for h in (1e-3, 1e-5, 1e-7):
            ad, fd = [], []
            for i, ax in picks:
                if h < 1e-6:
                    # below float32 resolution: float64 start points straddle fewer cell faces
                    pair = np.repeat(x0[i:i + 1].astype(np.float64), 2, axis=0)
                    xp, xm = float(x0[i, ax]) + h, float(x0[i, ax]) - h
                else:
                    pair = np.repeat(x0[i:i + 1], 2, axis=0)
                    xp, xm = np.float32(float(x0[i, ax]) + h), np.float32(float(x0[i, ax]) - h)
                pair[0, ax], pair[1, ax] = xp, xm
                out, _, _ = oracle.track(spec, obc, pair, times, dt, precision=oracle.ORC_F64)
                fd.append((np.sum((out[0] - y[i]) ** 2) - np.sum((out[1] - y[i]) ** 2)) / (float(xp) - float(xm)))
                ad.append(gref[i, ax])
            ad, fd = np.array(ad), np.array(fd)
            rel = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
            fd_stats[f"{horizon}_steps_h{h:g}"] = {"frac_within_1e-3": float(np.mean(rel < 1e-3)),
                                                  "median_rel": float(np.median(rel)), "samples": int(len(rel))}
    # dL/dU of a 2048-particle subset's loss against float64 central differences
    # (h = 1e-3 on one snapshot value; each difference reruns the subset in the oracle)
    m = 2048
    fd_U = {}
    for horizon in sorted({min(50, n_steps), n_steps}):
        xs = torch.tensor(x0[:m], device="cuda")
        Us = U_t.detach().clone().requires_grad_(True)
        xh = solver(xs, Us, (0.0, horizon * dt), horizon + 1, dt=dt)
        ((xh - y_t[:m]) ** 2).sum().backward()
        gU = Us.grad.cpu().numpy().reshape(16, -1, 3).astype(np.float64)
        nz = np.argwhere(gU != 0.0)
        times = np.linspace(0.0, horizon * dt, horizon + 1, dtype=np.float32)

        def sub_loss(d):
            s = oracle.GridSpec(d, c["times"], g, g, g, "periodic")
            o, _, _ = oracle.track(s, obc, x0[:m], times, dt, precision=oracle.ORC_F64)
            return float(np.sum((o - y[:m]) ** 2))

        ad, fd = [], []
        for t, nd, cc in nz[rng.choice(len(nz), size=min(24, len(nz)), replace=False)]:
            dp, dm = c["data"].copy(), c["data"].copy()
            dp[t, nd, cc] += np.float32(1e-3)
            dm[t, nd, cc] -= np.float32(1e-3)
            fd.append((sub_loss(dp) - sub_loss(dm)) / (float(dp[t, nd, cc]) - float(dm[t, nd, cc])))
            ad.append(gU[t, nd, cc])
        ad, fd = np.array(ad), np.array(fd)
        rel = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
        fd_U[f"{horizon}_steps_h0.001"] = {"frac_within_1e-3": float(np.mean(rel < 1e-3)),
                                           "median_rel": float(np.median(rel)), "samples": int(len(rel)),
                                           "subset_particles": m}
    f, b = float(np.mean(fwd_ms)), float(np.mean(bwd_ms))
    return {"fd_check_dL_dU": fd_U,
            "workload": f"differentiation: 64^3 periodic ABC, 16 snapshots, {n:,} lattice seeds, RK4 dt=0.01, "
                        f"{n_steps} steps, checkpoint every 50, loss sum|x_T - y|^2",
            "forward_ms": f, "backward_ms": b, "backward_over_forward": b / f,
            "forward_particle_steps_per_s": n * n_steps / (f / 1e3),
            "adjoint_particle_steps_per_s": n * n_steps / (b / 1e3),
            "fd_check_dL_dx0": fd_stats,
            "fd_note": "float64 central differences of single particles at h=1e-3, 1e-5 (float32 start points) "
                       "and 1e-7 (float64 start points) on x0; trilinear cell faces make the exact derivative "
                       "jump, so the wider steps and the longer horizon have more samples whose difference "
                       "straddles a face"}


def _mesh_oracle_spec(c, f):
    import oracle
    m = f.octree_mesh
    return oracle.MeshSpec(c["data"], c["times"], c["points"], c["tets"], m.element_bounds, m.nodes_min,
                           m.nodes_max, m.nodes_elements, m.nodes_children, m.nodes_is_leaf,
                           max_depth=m.max_depth)


def _timed(fn, reps):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def fem_leg(a, profile=False):
    """Unstructured FEM configuration: 64^3 hexes split into 6 jittered Kuhn
    tets (1,572,864 tets), 32 FP32 snapshots, octree location + P1, 1M
    particles, x/z periodic and y reflective, RK4 dt=0.005, 1000 steps.
    Parity: every 1000th particle against the float32 oracle (bit-exact
    count) and the float64 oracle (relative error)."""
    import torch

    import jaxtrace_gb300 as jt
    import oracle
    from jaxtrace_gb300 import _lib as L
    from jaxtrace_gb300 import workloads as W
    n_steps = a.fem_steps
    c = W.fem_case(n_steps=n_steps)
    f = jt.OctreeFEMTimeSeriesFieldOptimized(c["data"], c["times"], c["points"], c["tets"])
    bc = jt.mixed_boundary(W.UNIT, c["conditions"])
    tr = jt.create_tracker("rk4", f, bc, record_final_only=True)
    times = np.linspace(c["time_span"][0], c["time_span"][1], c["n_timesteps"], dtype=np.float32)
    x0 = torch.from_numpy(c["x0"]).cuda()
    pos = torch.empty_like(x0)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    sched = torch.from_numpy(tr._schedule(times, c["dt"]).view(np.int32).reshape(-1, 8)).cuda()
    timers = []

    def one(t=None):
        pos.copy_(x0)
        return tr.track_device(pos, times, c["dt"], status, None, sched, timers=t)

    for _ in range(1 if profile else 2):
        one()
    torch.cuda.synchronize()
    if profile:
        torch.cuda.profiler.start()
    ms = _timed(lambda: one(timers), 1 if profile else 2)
    if profile:
        torch.cuda.profiler.stop()
        return {}
    n = len(c["x0"])
    launch_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in timers]))
    n_launch = len(timers) / 2
    bpp = 4 * (16 + 4 * 12 + 2 * 4 * 12) + 24      # connectivity + vertices + two snapshots' values
    units = n * n_steps / n_launch
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    final = pos.cpu().numpy()
    sub = np.arange(0, n, 1000)
    spec = _mesh_oracle_spec(c, f)
    obc = oracle.BoundarySpec(kinds=("periodic", "reflective", "periodic"))
    t0 = time.perf_counter()
    o32, _, info = oracle.track(spec, obc, c["x0"][sub], times, c["dt"])
    cpu_s = time.perf_counter() - t0
    o64, _, _ = oracle.track(spec, obc, c["x0"][sub], times, c["dt"], precision=oracle.ORC_F64)
    same = np.all(final[sub].view(np.uint32) == o32.view(np.uint32), axis=1)
    rel = np.linalg.norm(final[sub] - o64, axis=1) / np.maximum(np.linalg.norm(o64, axis=1), 1e-30)
    hash_grid = {} if profile else fem_hash_grid_variant(c, bc, times, x0, n_steps, sub, obc)
    return {"octree_build": octree_build_times(c),
            "workload": "unstructured FEM: 64^3 hexes x 6 jittered tets (1,572,864), 32 FP32 snapshots, octree + "
                        f"P1, 1,000,000 particles, x/z periodic y reflective, RK4 dt=0.005, {n_steps} steps",
            "hash_grid_variant": hash_grid,
            "value": n * n_steps / (ms / 1e3), "unit": UNIT, "ms_per_pass": ms, "status": int(status.item()),
            "roofline": {"bound": "hbm", "achieved": units * bpp / (launch_ms / 1e3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": units * bpp / (launch_ms / 1e3) / 1e9 / peak,
                         "kernel": "k_track (RK4, octree mesh field, f32)", "bytes_per_particle_step": bpp,
                         "note": "P1 bytes exclude the octree search"},
            "parity_f32_oracle": {"bit_exact_fraction": float(np.mean(same)), "particles": len(sub),
                                  "oracle_fallbacks": info["fallback_count"]},
            "error_vs_fp64": {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),
                              "max": float(rel.max())},
            "cpu_baseline": {"value": len(sub) * n_steps / cpu_s, "unit": UNIT, "cores": os.cpu_count() or 1,
                             "kind": "port", "sample": f"{len(sub)} particles (every 1000th) x {n_steps} steps, "
                                                       "float32 C restatement of the octree/P1 path, OpenMP"}}


def octree_build_times(c):
    """Octree build of the FEM mesh from host arrays: the host builder and the
    device builder (host->device copy of points and connectivity included),
    and whether their arrays agree bit for bit."""
    import torch

    import jaxtrace_gb300 as jt
    t = time.perf_counter()
    h = jt.OctreeMesh(c["points"], c["tets"], build="host")
    host_s = time.perf_counter() - t
    jt.OctreeMesh(c["points"], c["tets"], build="device")
    torch.cuda.synchronize()
    t = time.perf_counter()
    d = jt.OctreeMesh(c["points"], c["tets"], build="device")
    torch.cuda.synchronize()
    dev_s = time.perf_counter() - t
    same = bool(np.array_equal(d.nodes.view(np.int32), h.nodes.view(np.int32)) and
                np.array_equal(d.elems, h.elems) and np.array_equal(d.tet_geom, h.tet_geom))
    return {"host_ms": host_s * 1e3, "device_ms": dev_s * 1e3, "nodes": int(h.info.n_nodes),
            "leaves": int(h.info.n_leaves), "depth": int(h.info.max_tree_depth), "same_arrays": same}


def fem_hash_leg(a, profile=False):
    """The unstructured FEM configuration through the hash-grid field alone
    (FEMTimeSeriesField, 32^3 cells, 4^3 sub-cells): one timed pass of
    ``--fem-steps`` steps (with --profile bracketed by cudaProfilerStart/Stop)."""
    import torch

    import jaxtrace_gb300 as jt
    from jaxtrace_gb300 import workloads as W
    c = W.fem_case(n_steps=a.fem_steps)
    f = jt.FEMTimeSeriesField(c["data"], c["times"], c["points"], c["tets"])
    bc = jt.mixed_boundary(W.UNIT, c["conditions"])
    tr = jt.create_tracker("rk4", f, bc, record_final_only=True)
    times = np.linspace(c["time_span"][0], c["time_span"][1], c["n_timesteps"], dtype=np.float32)
    x0 = torch.from_numpy(c["x0"]).cuda()
    pos = torch.empty_like(x0)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    sched = torch.from_numpy(tr._schedule(times, c["dt"]).view(np.int32).reshape(-1, 8)).cuda()

    def one():
        pos.copy_(x0)
        return tr.track_device(pos, times, c["dt"], status, None, sched)

    one()
    torch.cuda.synchronize()
    if profile:
        torch.cuda.profiler.start()
    ms = _timed(one, 1)
    if profile:
        torch.cuda.profiler.stop()
    n = len(c["x0"])
    return {"value": n * a.fem_steps / (ms / 1e3), "unit": UNIT, "ms_per_pass": ms, "steps": a.fem_steps,
            "status": int(status.item())}


def fem_grid_build_times(c):
    """Hash grid (32^3 cells, 4^3 sub-cells each) of the FEM mesh from host
    arrays: the host builder with its NumPy element records, and the device
    builder (host->device copy of points and connectivity included)."""
    import torch

    import jaxtrace_gb300 as jt
    t = time.perf_counter()
    h = jt.FemHashGrid(c["points"], c["tets"], build="host")
    host_s = time.perf_counter() - t
    jt.FemHashGrid(c["points"], c["tets"], build="device")
    torch.cuda.synchronize()
    t = time.perf_counter()
    d = jt.FemHashGrid(c["points"], c["tets"], build="device")
    torch.cuda.synchronize()
    dev_s = time.perf_counter() - t
    same = bool(all(np.array_equal(getattr(d, k), getattr(h, k))
                    for k in ("cell_start", "cell_elems", "sub_start", "sub_elems", "tet_geom")))
    return {"host_ms": host_s * 1e3, "device_ms": dev_s * 1e3, "cell_entries": int(len(h.cell_elems)),
            "sub_cell_entries": int(len(h.sub_elems)), "same_arrays": same}


def fem_hash_grid_variant(c, bc, times, x0, n_steps, sub, obc):
    """The same run through the hash-grid FEM field (FEMTimeSeriesField,
    32^3 cells, global nearest-node fallback)."""
    import torch

    import jaxtrace_gb300 as jt
    import oracle
    f = jt.FEMTimeSeriesField(c["data"], c["times"], c["points"], c["tets"])
    tr = jt.create_tracker("rk4", f, bc, record_final_only=True)
    pos = torch.empty_like(x0)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    sched = torch.from_numpy(tr._schedule(times, c["dt"]).view(np.int32).reshape(-1, 8)).cuda()

    def one():
        pos.copy_(x0)
        tr.track_device(pos, times, c["dt"], status, None, sched)

    one()
    ms = _timed(one, 2)
    n = x0.shape[0]
    final = pos.cpu().numpy()
    h = f.fem_mesh
    spec = oracle.FemSpec(c["data"], c["times"], c["points"], c["tets"], h.grid_size, h.grid_min, h.grid_cell_size,
                          h.cell_to_elements(), h.element_bounds)
    o32, _, info = oracle.track(spec, obc, c["x0"][sub], times, c["dt"])
    same = np.all(final[sub].view(np.uint32) == o32.view(np.uint32), axis=1)
    return {"value": n * n_steps / (ms / 1e3), "unit": UNIT, "ms_per_pass": ms, "status": int(status.item()),
            "grid_build": fem_grid_build_times(c),
            "hash_grid": list(h.grid_size), "max_elements_per_cell": h.max_elems_per_cell,
            "parity_f32_oracle": {"bit_exact_fraction": float(np.mean(same)), "particles": len(sub),
                                  "oracle_fallbacks": info["fallback_count"]}}


def batch_leg(a, profile=False, part="track"):
    """Batching + density configuration: 256 ensembles of round(10^U(3,6))
    particles (default_rng(7); 36,800,084 in all) released at U(0,0.5) on the
    FEM mesh, 400 RK4 steps of dt=0.005 each from its own release time, in
    one tracking pass (autotuned, captured in a CUDA graph); then cubic-spline
    SPH (h=0.02, 3-D) at, and a Scott-bandwidth Gaussian KDE on the 100^3
    grid of, the first 16,000,000 final positions."""
    import torch

    import jaxtrace_gb300 as jt
    import oracle
    from jaxtrace_gb300 import workloads as W
    c = W.fem_case(n_particles=1)
    f = jt.OctreeFEMTimeSeriesFieldOptimized(c["data"], c["times"], c["points"], c["tets"])
    bc = jt.mixed_boundary(W.UNIT, c["conditions"])
    sizes, release, xs = W.ensembles()
    tr = jt.create_tracker("rk4", f, bc, record_final_only=True)
    b = tr.ensemble_batch(xs, release, 401, dt=0.005)
    if part == "density":
        # positions only: one untimed pass, then the density passes alone
        b.run()
        return density_part(b.pos[: a.density_particles].contiguous(), profile)
    tune = jt.Autotuner(cache_path="").tune_batch(b)
    b.capture()
    b.run()
    torch.cuda.synchronize()
    if profile:
        torch.cuda.profiler.start()
    ms = _timed(b.run, 1 if profile else 2)
    if profile:
        torch.cuda.profiler.stop()
        return {}
    n = b.n
    status = b.check_status()
    # eager pass for comparison: the graph saves the host launch overhead only
    eager = tr.ensemble_batch(xs, release, 401, dt=0.005)
    eager.run()
    ms_eager = _timed(eager.run, 1)
    # parity: a few ensembles' first particles against the float32 oracle
    spec = _mesh_oracle_spec(c, f)
    obc = oracle.BoundarySpec(kinds=("periodic", "reflective", "periodic"))
    fin = b.pos.cpu().numpy()
    del eager
    exact, tot = 0, 0
    for e in range(0, 256, 16):
        lo = int(b.offsets[e])
        k = min(64, int(sizes[e]))
        o, _, _ = oracle.track(spec, obc, xs[e][:k], b.times[e], b.dt)
        exact += int(np.sum(np.all(fin[lo:lo + k].view(np.uint32) == o.view(np.uint32), axis=1)))
        tot += k
    out = {"workload": "batching: 256 ensembles (sizes round(10^U(3,6)), default_rng(7)), "
                       f"{n:,} particles, release U(0,0.5), FEM mesh, 400 RK4 steps dt=0.005 each",
           "value": n * 400 / (ms / 1e3), "unit": UNIT, "ms_per_pass": ms, "ms_per_pass_eager": ms_eager,
           "cuda_graph": True, "status": status,
           "autotune": {"block_size": tune.block_size, "sort_every": tune.sort_every, "sort_bits": tune.sort_bits,
                        "trials": len(tune.trials)},
           "parity_f32_oracle": {"bit_exact_fraction": exact / max(tot, 1), "particles": tot}}
    # density passes on the first 16,000,000 final positions
    P = b.pos[: a.density_particles].contiguous()
    del b
    torch.cuda.empty_cache()
    out["density"] = density_part(P, False)
    return out


def density_part(P, profile):
    """Cubic-spline SPH (h = 0.02, 3-D) at every position and a Scott KDE on
    the 100^3 grid; with ``profile`` both run once inside
    cudaProfilerStart/Stop and nothing is returned."""
    import torch

    from jaxtrace_gb300.density import KDEEstimator, SPHDensityEstimator
    sph = SPHDensityEstimator(P, dimensions="3d", smoothing_length=0.02, kernel_type="cubic_spline")
    sph.evaluate(P[:1024])
    kde = KDEEstimator(P, bandwidth_rule="scott")
    kde.evaluate_3d()
    torch.cuda.synchronize()
    if profile:
        torch.cuda.profiler.start()
        sph._density_sum(P)
        kde.evaluate_3d()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        return {}
    sph_ms = _timed(lambda: sph._density_sum(P), 1)
    kde_ms = _timed(kde.evaluate_3d, 1)
    n = int(P.shape[0])
    return {"particles": n, "sph_ms": sph_ms, "sph_queries_per_s": n / (sph_ms / 1e3),
            "kde_ms": kde_ms, "kde_bandwidth": kde.h, "kde_grid": "100^3", "kde_particles_per_s": n / (kde_ms / 1e3)}


def analytics_part(a, case, g, bc, x0_dev, times, plain_ms, storage):
    """Trajectory analytics on the device: one pass of the headline run with
    the per-particle path length fused into the tracking kernel (its cost
    against the plain pass), and the pair term of the mixing metrics over
    100,000 particles (10^10 ordered pairs)."""
    import torch

    import jaxtrace_gb300 as jt
    from jaxtrace_gb300.analysis import pair_log_ratio
    field = jt.StructuredTimeSeriesField(case["data"], case["times"], g, g, g, "clamp", storage=storage)
    tr = jt.create_tracker("rk4", field, bc, record_final_only=True, record_path_length=True)
    sched = torch.from_numpy(tr._schedule(times, case["dt"]).view(np.int32).reshape(-1, 8)).cuda()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    comp = torch.zeros_like(x0_dev) if tr._arith() == 1 else None
    pos = torch.empty_like(x0_dev)

    def one():
        pos.copy_(x0_dev)
        if comp is not None:
            comp.zero_()
        tr.track_device(pos, times, case["dt"], status, comp, sched)

    one()
    path_ms = _timed(one, 1)
    rng = np.random.default_rng(5)
    p0 = rng.random((100_000, 3)).astype(np.float32)
    p1 = (p0 + rng.normal(0, 0.01, p0.shape)).astype(np.float32)
    pair_log_ratio(p0[:1000], p1[:1000])
    torch.cuda.synchronize()
    t = time.perf_counter()
    s, cnt = pair_log_ratio(p0, p1, 0.1)
    pair_ms = (time.perf_counter() - t) * 1e3
    return {"path_length_pass_ms": path_ms, "plain_pass_ms": plain_ms,
            "path_length_overhead": path_ms / plain_ms - 1.0,
            "pair_term_ms": pair_ms, "pair_term_particles": 100_000, "pair_term_pairs_in_cutoff": cnt,
            "pair_term_pairs_per_s": 100_000 * 99_999 / (pair_ms / 1e3)}


def recording_part(case, bc, storage, every=100, chunk=100):
    """Recorded trajectories through track_particles (pinned host x0 in, the
    Trajectory out) on a quarter of the headline particles, every
    ``every``-th step recorded: the final-only pass, one recorded slab copied
    after the pass, ``chunk``-step slabs copied on a side stream while the
    next chunk runs, and the same with a row sink receiving each slab."""
    import torch

    import jaxtrace_gb300 as jt
    g = case["grid"][0]
    field = jt.StructuredTimeSeriesField(case["data"], case["times"], g, g, g, "clamp", storage=storage)
    x0 = torch.from_numpy(np.ascontiguousarray(case["x0"][: len(case["x0"]) // 4])).pin_memory()
    handed = []

    def run(**kw):
        tr = jt.create_tracker("rk4", field, bc, **kw)
        tr.track_particles(x0, case["time_span"], case["n_timesteps"], dt=case["dt"])
        torch.cuda.synchronize()
        handed.clear()
        t = time.perf_counter()
        traj = tr.track_particles(x0, case["time_span"], case["n_timesteps"], dt=case["dt"])
        torch.cuda.synchronize()
        return (time.perf_counter() - t) * 1e3, traj

    out = {"particles": int(x0.shape[0]), "record_every": every, "time_chunk": chunk}
    out["final_only_ms"], _ = run(record_final_only=True)
    out["one_slab_ms"], t1 = run(record_every=every)
    out["chunked_ms"], t2 = run(record_every=every, time_chunk=chunk)
    out["chunked_sink_ms"], t3 = run(record_every=every, time_chunk=chunk,
                                     row_sink=lambda r0, p, v, t: handed.append(len(p)))
    out["rows"] = int(t1.T)
    out["recorded_bytes"] = int(t1.positions.nbytes)
    out["rows_handed_to_sink"] = int(sum(handed))
    out["same_bits"] = bool(np.array_equal(t1.positions, t2.positions) and np.array_equal(t1.positions, t3.positions))
    return out


def workload_name(a):
    return (f"precision: {a.grid}^3 clamp grid, 64 snapshots ABC+(1,0,0)+N(0,0.01^2) over [0,2], "
            f"{a.seeds ** 3} lattice seeds, continuous inlet x (lattice {a.seeds}x{a.seeds}), "
            f"RK4 dt={a.dt}, {a.n_steps} steps")


def main():
    a = args_parse()
    world, rank, local = dist_setup()
    if a.impl == "reference":
        run_reference(a, world, rank)
        return
    import torch
    if a.leg is not None:
        # one configuration leg alone (rank 0 of a single process)
        from jaxtrace_gb300 import _lib as L
        L.load()
        if a.leg == "adjoint":
            out = adjoint_leg(a, profile=a.profile)
        else:
            out = {"fem": fem_leg, "fem_hash": fem_hash_leg, "batch": batch_leg,
                   "density": lambda a, profile: batch_leg(a, profile, part="density")}[a.leg](a, profile=a.profile)
        if rank == 0:
            print(json.dumps({"leg": a.leg} | out), flush=True)
        return

    import jaxtrace_gb300 as jt
    from jaxtrace_gb300 import _lib as L
    from jaxtrace_gb300 import workloads as W

    L.load()
    dt = a.dt
    case = W.precision_case(n=a.grid, seeds=(a.seeds,) * 3, lattice=a.seeds, n_steps=a.n_steps, dt=dt)
    x0 = case["x0"]
    n = len(x0)
    g = case["grid"][0]
    bc = jt.continuous_inlet_boundary_factory(W.UNIT, "x", "positive", "grid", case["concentrations"])
    times = np.linspace(case["time_span"][0], case["time_span"][1], case["n_timesteps"], dtype=np.float32)
    x0_dev = torch.from_numpy(x0).cuda()
    variants = [v.strip() for v in a.variants.split(",") if v.strip()]
    results, finals, trackers = {}, {}, {}
    launches = 0
    stream = torch.cuda.current_stream()
    clk = Clocks(local)
    for v in variants:
        field = jt.StructuredTimeSeriesField(case["data"], case["times"], g, g, g, "clamp", storage=v)
        tr = jt.create_tracker("rk4", field, bc, record_final_only=True, sort_every=a.sort_every,
                               sort_bits=a.sort_bits, block_size=a.block_size, stage_chunk=a.stage_chunk,
                               stage_overlap=not a.no_stage_overlap)
        trackers[v] = tr
        sched = torch.from_numpy(tr._schedule(times, case["dt"]).view(np.int32).reshape(-1, 8)).cuda()
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        comp = torch.zeros_like(x0_dev) if tr._arith() == L.JT_ARITH_COMPENSATED else None
        pos = torch.empty_like(x0_dev)

        def one(timers=None):
            pos.copy_(x0_dev)
            if comp is not None:
                comp.zero_()
            return tr.track_device(pos, times, case["dt"], status, comp, sched, timers=timers)

        for _ in range(a.warmup):
            one()
        torch.cuda.synchronize()
        barrier(world)
        timers = []
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        headline = v == variants[0]
        if headline:
            clk.__enter__()
        torch.cuda.synchronize()
        t0.record(stream)
        if a.profile:
            torch.cuda.profiler.start()
        counts = [one(timers) for _ in range(a.steps)]
        if a.profile:
            torch.cuda.profiler.stop()
        t1.record(stream)
        torch.cuda.synchronize()
        if headline:
            clk.__exit__()
        barrier(world)
        ms_total = max_over_ranks(world, t0.elapsed_time(t1))
        launch_ms = [e[0].elapsed_time(e[1]) for e in timers]
        per_launch_ms = float(np.mean(launch_ms))
        n_track = sum(c["track_launches"] for c in counts)
        if headline:
            launches = sum(c["kernels"] for c in counts)
        psteps = n * a.n_steps
        results[v] = {"value": world * psteps * a.steps / (ms_total / 1e3), "ms_per_step": ms_total / a.steps,
                      "track_kernel_ms_per_step": float(np.sum(launch_ms)) / a.steps, "status": int(status.item())}
        bpp = BYTES_PER_PSTEP[v]
        from_peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        peak = float(from_peaks.get("hbm_gbs", 6800.0))
        units_per_launch = psteps * a.steps / n_track          # particle-steps per k_track launch
        achieved = units_per_launch * bpp / (per_launch_ms / 1e3) / 1e9
        tb = traffic_per_pstep(v)
        results[v]["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                  "frac": achieved / peak,
                                  "traffic": (tb * units_per_launch if tb is not None else None),
                                  "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if from_peaks else "fallback",
                                  "kernel": "k_track (RK4, grid field, %s)" % v,
                                  "launch_ms": per_launch_ms, "particle_steps_per_launch": units_per_launch,
                                  "bytes_per_particle_step": bpp}
        wi = profile_figure("warp_inst_per_warp_step", v)
        if wi is not None:
            # instruction issue: the ncu count of warp instructions per particle-step
            # against one warp instruction per cycle on each of the SMs' schedulers
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            results[v]["roofline"]["issue"] = {
                "warp_inst_per_particle_step": wi / 32.0,
                "achieved": units_per_launch * wi / 32.0 / (per_launch_ms / 1e3),
                "peak_per_mhz": sms * 4 * 1e6, "unit": "warp-inst/s", "schedulers": sms * 4}
        finals[v] = pos.cpu().numpy()
        del field
        if a.profile:
            break

    head = variants[0]
    line = {"metric": METRIC, "value": results[head]["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": results[head]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(a), "storage": head, "particles": n,
                       "steps_per_pass": a.n_steps,
                       "l2": f"inputs larger than L2 (positions {n * 12 / 1e6:.0f} MB, snapshot pairs "
                             f"{(len(case['times']) - 1) * g.size ** 3 * (32 if head == 'f32' else 48) / 1e9:.2f} GB)"},
            "variants": {v: {k: r[k] for k in ("value", "ms_per_step", "track_kernel_ms_per_step", "status")} |
                         {"roofline_frac": r["roofline"]["frac"]} for v, r in results.items()},
            "roofline": results[head]["roofline"], "gpu_launches": launches}
    if not a.profile and rank == 0:
        import oracle
        oracle.build()
        sub = np.arange(0, n, 256)
        if not a.no_error:
            ref64, _ = oracle_subset_run(case, sub, oracle.ORC_F64, os.cpu_count() or 1)
            err = {}
            for v, fin in finals.items():
                d = np.linalg.norm(fin[sub].astype(np.float64) - ref64, axis=1)
                rel = d / np.maximum(np.linalg.norm(ref64, axis=1), 1e-30)
                err[v] = {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),
                          "max": float(rel.max()), "frac_above_1e-4": float(np.mean(rel > 1e-4))}
            line["error_vs_fp64"] = err
            line["error_sample"] = f"every 256th particle ({len(sub)}) vs the float64 oracle, relative |dx|/|x|"
        if not a.no_cpu:
            cores = os.cpu_count() or 1
            csub = sub[: min(len(sub), 16384)]
            _, sec = oracle_subset_run(case, csub, oracle.ORC_F32, cores)
            line["cpu_baseline"] = {"value": len(csub) * a.n_steps / sec, "unit": UNIT, "cores": cores,
                                    "kind": "port",
                                    "sample": f"{len(csub)} particles (every 256th) x {a.n_steps} RK4 steps, float32 "
                                              f"C restatement of the reference NumPy path, OpenMP"}
    if not a.profile and not a.no_e2e:
        tr = trackers[head]
        x0_pin = torch.from_numpy(x0).pin_memory()
        traj = None
        for _ in range(max(2, a.warmup - 1)):   # the timed loop's pattern: the last result stays alive
            traj = tr.track_particles(x0_pin, case["time_span"], case["n_timesteps"], dt=case["dt"])
        torch.cuda.synchronize()
        barrier(world)
        t = time.perf_counter()
        for _ in range(a.steps):
            traj = tr.track_particles(x0_pin, case["time_span"], case["n_timesteps"], dt=case["dt"])
        torch.cuda.synchronize()
        el = max_over_ranks(world, time.perf_counter() - t)
        line["e2e"] = {"value": world * n * a.n_steps * a.steps / el, "unit": UNIT,
                       "h2d_bytes_per_step": int(n * 12), "d2h_bytes_per_step": int(n * 12),
                       "ms_per_step": el * 1e3 / a.steps,
                       "api": "create_tracker('rk4', field, continuous_inlet, record_final_only=True)"
                              ".track_particles(pinned host x0)"}
    line["clocks"] = clk.summary()
    if not a.profile and rank == 0:
        line["analytics"] = analytics_part(a, case, g, bc, x0_dev, times, results[head]["ms_per_step"], head)
        line["recording"] = recording_part(case, bc, head)
    iss = line.get("roofline", {}).get("issue")
    if iss is not None:
        mhz = line["clocks"].get("sm_mhz") or 2070.0
        iss["peak"] = iss.pop("peak_per_mhz") * mhz
        iss["frac"] = iss["achieved"] / iss["peak"]
        iss["clock_mhz"] = mhz
    if not a.profile and rank == 0:
        del trackers
        torch.cuda.empty_cache()
        if not a.no_adjoint:
            line["adjoint"] = adjoint_leg(a)
        if not a.no_fem:
            line["fem"] = fem_leg(a)
        if not a.no_batch:
            line["batching"] = batch_leg(a)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
