"""Time the JAXTrace reference's own NumPy path on the benchmark
configurations -- TEST INFRASTRUCTURE ONLY (a measurement of the reference,
never imported by the package).

Run from the repository root in a checkout that has the reference sources:
    python oracle/reference_timing.py /path/to/JAXTrace [--legs ...] [--procs 1 8]
(or with the path in the JAXTRACE_REFERENCE environment variable).  The
reference is imported as-is (no jax installed, so every module takes its
NumPy path; the octree modules import jax unconditionally and run under the
NumPy stand-in oracle/jaxshim) and driven through its public API:

- grid legs: ``TimeSeriesField.sample_at_time`` blends every node at the
  stage time, ``StructuredGridSampler(...).sample`` interpolates
  (fields/time_series.py:306-389, fields/structured.py:274-349), and
  ``create_tracker('rk4', field, boundary).track_particles`` steps
  (tracking/tracker.py:320-469);
- ``fem_octree``: ``OctreeFEMTimeSeriesFieldOptimized`` (its octree build is
  setup, not timed) with the mixed periodic/reflective boundary;
- ``density``: ``SPHDensityEstimator.evaluate`` (cubic spline, h = 0.02) at
  the points, and ``KDEEstimator.evaluate`` (Scott bandwidth) at the nodes of
  a 32^3 grid through SciPy and through the pure-NumPy formula
  (density/sph.py, density/kde.py).

Each leg runs as one process and as N spawned processes over shards of its
particles (or query points), which are independent: the reference's step
loop is single-threaded.  Setup (field construction, octree build, input
generation) is outside the timed region; each timing is the median of the
given number of repeats, the longest process of a run counting.  The result
is written to oracle/reference_timing.json with the host's CPU model and core
count; it is a figure of the machine that ran the script.
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
UNIT = ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))


def _cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


# ---------------------------------------------------------------------------
# Workloads: (inputs saved by the parent, shard runner in the child)
def _grid_case(leg: str) -> dict:
    sys.path.insert(0, str(REPO))
    from jaxtrace_gb300 import workloads as W
    if leg.startswith("precision"):
        c = W.precision_case()
        return dict(data=c["data"], times=c["times"], g=c["grid"][0], x0=c["x0"], mode="clamp", inlet=256,
                    dt=0.002)
    if leg == "plain":
        c = W.plain_rk4()
        return dict(data=c["data"], times=c["times"], g=c["grid"][0], x0=c["x0"], mode="periodic", inlet=0,
                    dt=0.01)
    if leg == "differentiation_forward":
        from jaxtrace_gb300.seeding import uniform_grid_seeds
        c = W.plain_rk4(n=64)
        x0 = uniform_grid_seeds((256, 256, 64), UNIT)
        return dict(data=c["data"], times=c["times"], g=c["grid"][0], x0=x0, mode="periodic", inlet=0, dt=0.01)
    raise ValueError(leg)


def _run_grid(ref, case, x0, steps):
    from jaxtrace.fields.structured import StructuredGridSampler
    from jaxtrace.fields.time_series import TimeSeriesField
    from jaxtrace.tracking import boundary as bnd
    from jaxtrace.tracking.tracker import create_tracker
    data, times, g, dt = case["data"], case["times"], case["g"], float(case["dt"])
    n = len(g)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(F32)
    ts = TimeSeriesField(data=data, times=times, positions=nodes)
    mode = str(case["mode"])

    def field(p, t):
        V = np.asarray(ts.sample_at_time(t)).reshape(n, n, n, 3)
        if mode == "periodic":
            # a stage point in (-4e-8, 0) makes np.mod(fx, N) round up to N and
            # the reference index out of bounds (structured.py:294, :325); the
            # seed-42 particles of the plain case meet it, so stage points are
            # wrapped into [0, 1) first (one comparison per coordinate)
            p = np.where(p < 0, p + F32(1), p)
        return StructuredGridSampler(V, g, g, g, bounds_handling=mode).sample(p)

    lat = int(case["inlet"])
    bc = (bnd.continuous_inlet_boundary_factory(UNIT, "x", "positive", "grid", {"x": lat, "y": lat, "z": lat})
          if lat else bnd.periodic_boundary(UNIT))
    tr = create_tracker("rk4", field, bc, progress_style="none")
    tr.track_particles(x0, (0.0, dt), 2, dt=dt)                  # untimed: first touch of every array
    t0 = time.perf_counter()
    traj = tr.track_particles(x0, (0.0, steps * dt), steps + 1, dt=dt)
    sec = time.perf_counter() - t0
    assert np.isfinite(traj.positions[-1]).all()
    return sec, len(x0) * steps


def _run_octree(ref, case, x0, steps):
    import contextlib
    import io
    from jaxtrace.fields.octree_fem_time_series_optimized import OctreeFEMTimeSeriesFieldOptimized
    from jaxtrace.tracking import boundary as bnd
    from jaxtrace.tracking.tracker import create_tracker
    with contextlib.redirect_stdout(io.StringIO()):
        f = OctreeFEMTimeSeriesFieldOptimized(case["data"], case["times"], case["P"], case["T"],
                                              max_elements_per_leaf=32, max_depth=12)
    bc = bnd.mixed_boundary(UNIT, {"x": "periodic", "y": "reflective", "z": "periodic"})
    tr = create_tracker("rk4", f, bc, use_jax_jit=False, progress_style="none")
    dt = float(case["dt"])
    t0 = time.perf_counter()
    traj = tr.track_particles(x0, (0.0, steps * dt), steps + 1, dt=dt)
    sec = time.perf_counter() - t0
    assert np.isfinite(traj.positions[-1]).all()
    return sec, len(x0) * steps


def _run_density(ref, case, q, what):
    from jaxtrace.density import kde as kde_mod
    from jaxtrace.density.kde import KDEEstimator
    from jaxtrace.density.sph import SPHDensityEstimator
    P = case["P"]
    if what == "sph":
        s = SPHDensityEstimator(P, dimensions="3d", smoothing_length=0.02, kernel_type="cubic_spline")
        t0 = time.perf_counter()
        s.evaluate(q)
        return time.perf_counter() - t0, len(q) * len(P)
    kde_mod.SCIPY_AVAILABLE = what == "kde_scipy"
    k = KDEEstimator(P, bandwidth_rule="scott", resolution=int(case["res"]))
    t0 = time.perf_counter()
    k.evaluate(q)
    return time.perf_counter() - t0, len(q) * len(P)


def _worker(ref, leg, path, lo, hi, steps, what, q):
    try:
        _work(ref, leg, path, lo, hi, steps, what, q)
    except BaseException as e:  # noqa: BLE001 -- reported to the parent, which raises
        import traceback
        q.put(("error", f"{type(e).__name__}: {e}\n{traceback.format_exc()}"))


def _work(ref, leg, path, lo, hi, steps, what, q):
    if leg == "fem_octree":
        sys.path.insert(0, str(HERE / "jaxshim"))
    sys.path.insert(1, ref)
    import warnings
    warnings.simplefilter("ignore")
    from jaxtrace.utils.jax_utils import JAX_AVAILABLE
    assert leg == "fem_octree" or not JAX_AVAILABLE, "the timing runs the reference's NumPy path"
    z = dict(np.load(path))
    if leg == "fem_octree":
        res = _run_octree(ref, z, z["x0"][lo:hi], steps)
    elif leg == "density":
        res = _run_density(ref, z, z["q"][lo:hi], what)
    else:
        res = _run_grid(ref, z, z["x0"][lo:hi], steps)
    q.put(res)


def _inputs(leg: str, particles: int) -> tuple[dict, str]:
    """Inputs of a leg, the particles (or queries) sampled evenly."""
    sys.path.insert(0, str(REPO))
    from jaxtrace_gb300 import workloads as W
    if leg == "fem_octree":
        P, T = W.kuhn_mesh(64, 0.2, 1)
        times = np.linspace(0.0, 1.0, 32).astype(F32)
        x0 = np.random.default_rng(42).uniform(size=(1_000_000, 3)).astype(F32)
        sel = np.linspace(0, len(x0) - 1, particles).astype(np.int64)
        return (dict(P=P, T=T, data=W.abc_snapshots(P, times), times=times, x0=x0[sel], dt=0.005),
                f"{particles} of the 1,000,000 particles (evenly spaced), 64^3 x 6 jittered Kuhn tets, 32 snapshots")
    if leg == "density":
        pts = np.random.default_rng(0).random((particles, 3)).astype(F32)
        res = 32
        g = np.linspace(0.0, 1.0, res, dtype=F32)
        X, Y, Z = np.meshgrid(g, g, g, indexing="xy")
        grid = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(F32)
        return (dict(P=pts, q=pts, grid=grid, res=res),
                f"{particles} uniform points; SPH queries at the points, KDE at a {res}^3 grid")
    c = _grid_case(leg)
    x0 = c["x0"]
    stride = max(1, len(x0) // particles)
    c["x0"] = np.ascontiguousarray(x0[::stride][:particles])
    what = "every" if stride == 1 else f"every {stride}th"
    return c, f"{what} particle of {len(x0)} ({len(c['x0'])} particles)"


def run(ref: str, leg: str, particles: int, steps: int, procs: int, repeats: int, what: str = "") -> dict:
    case, sample = _inputs(leg, particles)
    if leg == "density" and what.startswith("kde"):
        case["q"] = case["grid"]
    n_units = len(case["q"]) if leg == "density" else len(case["x0"])
    bounds = np.linspace(0, n_units, procs + 1).astype(np.int64)
    times = []
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "case.npz")
        np.savez(path, **case)
        ctx = mp.get_context("spawn")
        for _ in range(repeats):
            q = ctx.Queue()
            ps = [ctx.Process(target=_worker, args=(ref, leg, path, int(bounds[i]), int(bounds[i + 1]), steps,
                                                    what, q)) for i in range(procs)]
            for p in ps:
                p.start()
            res = [q.get() for _ in ps]
            for p in ps:
                p.join()
            for r in res:
                if r[0] == "error":
                    raise RuntimeError(f"{leg} worker failed: {r[1]}")
            times.append((max(s for s, _ in res), sum(u for _, u in res)))
    sec = float(np.median([s for s, _ in times]))
    units = times[0][1]
    unit = {"density": "pairs/s" if what == "sph" else "terms/s"}.get(leg, "particle-steps/s")
    steps_txt = "" if leg == "density" else f" x {steps} RK4 steps after one untimed step"
    return {"leg": leg + (f"_{what}" if what else ""), "value": units / sec, "unit": unit, "processes": procs,
            "units_per_run": int(units), "seconds": sec, "repeats": repeats,
            "sample": sample + steps_txt + f", {procs} process(es), median of {repeats}",
            "cpu": _cpu_model(), "host_cores": os.cpu_count(), "machine": platform.machine()}


# leg: (particles or points, steps, repeats, variants)
LEGS = {
    "precision": (1 << 24, 3, 1, [""]),
    "precision_subset": (65536, 20, 3, [""]),
    "plain": (10_000, 100, 3, [""]),
    "differentiation_forward": (65536, 20, 3, [""]),
    "fem_octree": (2000, 5, 1, [""]),
    "density": (20_000, 0, 1, ["sph", "kde_scipy", "kde_numpy"]),
}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("ref", nargs="?", default=os.environ.get("JAXTRACE_REFERENCE"))
    ap.add_argument("--legs", nargs="+", default=list(LEGS))
    ap.add_argument("--procs", type=int, nargs="+", default=[1, os.cpu_count()])
    ap.add_argument("--out", default=str(HERE / "reference_timing.json"))
    a = ap.parse_args(argv)
    if not a.ref:
        ap.error("give the JAXTrace checkout as an argument or in JAXTRACE_REFERENCE")
    out = {}
    if Path(a.out).exists():
        out = json.loads(Path(a.out).read_text()).get("legs", {})
    for leg in a.legs:
        particles, steps, repeats, variants = LEGS[leg]
        for what in variants:
            rows = []
            for n in a.procs:
                r = run(a.ref, leg, particles, steps, n, repeats, what)
                print(json.dumps(r), flush=True)
                rows.append(r)
            out[rows[0]["leg"]] = rows
    Path(a.out).write_text(json.dumps({"legs": out}, indent=1) + "\n")


if __name__ == "__main__":
    main()
