"""Time the JAXTrace reference's own NumPy path on the precision
configuration -- TEST INFRASTRUCTURE ONLY (a measurement of the reference,
never imported by the package).

Run from the repository root in a checkout that has the reference sources:
    python oracle/reference_timing.py /path/to/JAXTrace [--particles P] [--steps S] [--procs N]
(or with the path in the JAXTRACE_REFERENCE environment variable).  The
reference is imported as-is (no jax installed, so every module takes its
NumPy path) and driven through its public API the way its own examples
compose a regular-grid time series: ``TimeSeriesField.sample_at_time`` blends
every node at the stage time, ``StructuredGridSampler(...).sample`` does the
trilinear lookup (fields/time_series.py:306-389, fields/structured.py:274-349),
and ``create_tracker('rk4', field, continuous_inlet_boundary_factory(...))
.track_particles`` steps (tracking/tracker.py:320-469, boundary.py:1444-1601).

The sample is every k-th seed of the 256^3 inlet lattice, split over N
spawned processes (one NumPy process per core: the reference's step loop is
single-threaded), each timed over S steps after one untimed step.  The
result is written to oracle/reference_timing.json with the host's CPU model
and core count; it is a figure of the machine that ran the script.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import platform
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
F32 = np.float32


def _cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def _worker(ref, data_path, x0, steps, dt, q):
    sys.path.insert(0, ref)
    import warnings
    warnings.simplefilter("ignore")
    from jaxtrace.fields.structured import StructuredGridSampler
    from jaxtrace.fields.time_series import TimeSeriesField
    from jaxtrace.tracking import boundary as bnd
    from jaxtrace.tracking.tracker import create_tracker
    from jaxtrace.utils.jax_utils import JAX_AVAILABLE
    assert not JAX_AVAILABLE, "the timing runs the reference's NumPy path (no jax installed)"
    z = np.load(data_path)
    data, times, g = z["data"], z["times"], z["g"]
    n = len(g)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(F32)
    ts = TimeSeriesField(data=data, times=times, positions=nodes)

    def field(p, t):
        V = np.asarray(ts.sample_at_time(t)).reshape(n, n, n, 3)
        return StructuredGridSampler(V, g, g, g, bounds_handling="clamp").sample(p)

    bc = bnd.continuous_inlet_boundary_factory(((0, 0, 0), (1, 1, 1)), "x", "positive", "grid",
                                               {"x": 256, "y": 256, "z": 256})
    tr = create_tracker("rk4", field, bc, progress_style="none")
    tr.track_particles(x0, (0.0, dt), 2, dt=dt)                  # untimed: first touch of every array
    t0 = time.perf_counter()
    traj = tr.track_particles(x0, (0.0, steps * dt), steps + 1, dt=dt)
    q.put((time.perf_counter() - t0, int(np.isfinite(traj.positions[-1]).all())))


def run(ref: str, particles: int, steps: int, procs: int, dt: float = 0.002) -> dict:
    sys.path.insert(0, str(REPO))
    from jaxtrace_gb300 import workloads as W
    c = W.precision_case()
    x0 = c["x0"]
    stride = max(1, len(x0) // particles)
    x0 = np.ascontiguousarray(x0[::stride][:particles])
    shards = np.array_split(x0, procs)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "field.npz")
        np.savez(path, data=c["data"], times=c["times"], g=c["grid"][0])
        ctx = mp.get_context("spawn")
        q = ctx.Queue()
        ps = [ctx.Process(target=_worker, args=(ref, path, s, steps, dt, q)) for s in shards]
        t0 = time.perf_counter()
        for p in ps:
            p.start()
        res = [q.get() for _ in ps]
        for p in ps:
            p.join()
        wall = time.perf_counter() - t0
    assert all(ok for _, ok in res), "non-finite positions"
    longest = max(t for t, _ in res)
    return {"value": len(x0) * steps / longest, "unit": "particle-steps/s", "particles": len(x0),
            "steps": steps, "processes": procs, "seconds": longest, "wall_with_setup_s": wall,
            "sample": f"{'every' if stride == 1 else f'every {stride}th'} seed of the 256^3 lattice "
                      f"({len(x0)} particles) x {steps} RK4 steps "
                      f"after one untimed step, {procs} NumPy process(es), max over processes",
            "cpu": _cpu_model(), "host_cores": os.cpu_count(), "machine": platform.machine()}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("ref", nargs="?", default=os.environ.get("JAXTRACE_REFERENCE"))
    ap.add_argument("--particles", type=int, default=1 << 24)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--procs", type=int, nargs="+", default=[1, os.cpu_count()])
    ap.add_argument("--out", default=str(HERE / "reference_timing.json"))
    a = ap.parse_args(argv)
    if not a.ref:
        ap.error("give the JAXTrace checkout as an argument or in JAXTRACE_REFERENCE")
    rows = []
    for n in a.procs:
        r = run(a.ref, a.particles, a.steps, n)
        print(json.dumps(r), flush=True)
        rows.append(r)
    Path(a.out).write_text(json.dumps({"reference_numpy": rows}, indent=1) + "\n")


if __name__ == "__main__":
    main()
