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
# algorithmic bytes per RK4 particle-step (cache-oblivious): 4 field evaluations
# x 2 snapshots x 8 corners x 3 values + 24 B of position read/write
BYTES_PER_PSTEP = {"f32": 4 * 2 * 8 * 12 + 24, "bf16": 4 * 2 * 8 * 6 + 24, "f16": 4 * 2 * 8 * 6 + 24}


def traffic_per_pstep(storage):
    """DRAM bytes per particle-step of k_track from the committed ncu summary
    (profiles/k_track_precision.md, line 'dram_bytes_per_particle_step <storage> <value>')."""
    f = ROOT / "profiles" / "k_track_precision.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = line.replace("|", " ").split()
        if len(parts) >= 3 and parts[0] == "dram_bytes_per_particle_step" and parts[1] == storage:
            try:
                return float(parts[2])
            except ValueError:
                return None
    return None


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
    p.add_argument("--grid", type=int, default=128)
    p.add_argument("--no-error", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
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
        tr = jt.create_tracker("rk4", field, bc, record_final_only=True, sort_every=a.sort_every)
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
                             f"{(len(case['times']) - 1) * g.size ** 3 * (32 if head == 'f32' else 16) / 1e9:.2f} GB)"},
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
        for _ in range(max(1, a.warmup - 1)):
            tr.track_particles(x0_pin, case["time_span"], case["n_timesteps"], dt=case["dt"])
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
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
