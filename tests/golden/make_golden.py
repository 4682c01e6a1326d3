"""Regenerate the golden fixtures by running the JAXTrace reference itself.

Run from the repository root in a checkout that has the reference sources:
    python tests/golden/make_golden.py /path/to/JAXTrace
(or with the path in the JAXTRACE_REFERENCE environment variable).
Phase ``numpy`` imports the reference as-is (no jax installed, so every
module takes its NumPy path).  Phase ``octree`` puts the NumPy stand-in for
jax (oracle/jaxshim) first on sys.path so the octree modules, which import
jax unconditionally, can run.  Each phase runs in its own process.

Fixtures hold both the inputs and the reference outputs, so the tests need
only the .npz files.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
F32 = np.float32


def abc(points01: np.ndarray, t: float, A=1.0, B=0.7, C=0.43) -> np.ndarray:
    """ABC flow at points in [0,1]^3 (coordinates scaled to [0,2pi]), float64."""
    x, y, z = (2 * np.pi * points01[..., k].astype(np.float64) for k in range(3))
    s = 1.0 + 0.1 * np.sin(2 * np.pi * t)
    return np.stack([A * np.sin(z) + C * np.cos(y), B * np.sin(x) + A * np.cos(z),
                     C * np.sin(y) + B * np.cos(x)], axis=-1) * s


def grid_nodes(gx, gy, gz):
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(F32)


def kuhn_mesh(n: int, jitter: float, seed: int):
    """(n+1)^3 nodes on [0,1]^3, interior jittered by U(-j,j)/n; 6 tets per hex."""
    g = np.linspace(0, 1, n + 1)
    P = grid_nodes(g, g, g).astype(np.float64)
    idx = np.arange((n + 1) ** 3).reshape(n + 1, n + 1, n + 1)
    interior = np.all((P > 0) & (P < 1), axis=1)
    rng = np.random.default_rng(seed)
    P[interior] += rng.uniform(-jitter, jitter, (interior.sum(), 3)) / n
    tets = []
    local = [(0, 1, 3, 7), (0, 1, 5, 7), (0, 2, 3, 7), (0, 2, 6, 7), (0, 4, 5, 7), (0, 4, 6, 7)]
    for i in range(n):
        for j in range(n):
            for k in range(n):
                v = [idx[i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1)] for c in range(8)]
                for t in local:
                    tets.append([v[q] for q in t])
    return P.astype(F32), np.asarray(tets, dtype=np.int32)


# ---------------------------------------------------------------------------
def phase_numpy(ref: str):
    sys.path.insert(0, ref)
    import warnings
    warnings.simplefilter("ignore")
    from jaxtrace.fields.structured import StructuredGridSampler
    from jaxtrace.fields.time_series import TimeSeriesField
    from jaxtrace.tracking import boundary as bnd
    from jaxtrace.tracking.tracker import create_tracker
    from jaxtrace.utils.jax_utils import JAX_AVAILABLE
    assert not JAX_AVAILABLE, "phase numpy must run without jax"
    rng = np.random.default_rng(1234)

    # A1: time blend, every extrapolation mode, f32 and python-float times
    data = rng.standard_normal((5, 7, 3)).astype(F32)
    times = np.array([0.0, 0.25, 0.5, 0.5, 1.0], dtype=F32)
    pos = rng.random((7, 3)).astype(F32)
    tq = np.concatenate([np.linspace(-0.3, 1.3, 33), times.astype(np.float64), [0.5 - 1e-9, 1.0 + 1e-12, -1e-13],
                         np.float32(np.linspace(0.01, 0.99, 7)).astype(np.float64)])
    out = {}
    for ex in ("constant", "linear", "zero", "nan"):
        ts = TimeSeriesField(data=data, times=times, positions=pos, extrapolation=ex)
        out[ex] = np.stack([np.asarray(ts.sample_at_time(float(t)), dtype=F32) for t in tq])
    np.savez_compressed(HERE / "time_blend.npz", data=data, times=times, tq=tq, **{f"out_{k}": v for k, v in out.items()})

    # A2: structured sampler, all bounds modes
    res = {}
    for mode in ("clamp", "zero", "nan", "periodic"):
        nx, ny, nz = 5, 6, 7
        if mode == "periodic":
            gx, gy, gz = (np.arange(n, dtype=np.float64) / n for n in (nx, ny, nz))
        else:
            gx, gy, gz = np.linspace(-0.5, 1.0, nx), np.linspace(0, 2, ny), np.linspace(0.25, 0.75, nz)
        gx, gy, gz = (g.astype(F32) for g in (gx, gy, gz))
        V = rng.standard_normal((nx, ny, nz, 3)).astype(F32)
        q = np.concatenate([rng.uniform(-1.5, 2.5, (400, 3)), grid_nodes(gx, gy, gz)[:60],
                            np.array([[gx[-1], gy[-1], gz[-1]], [gx[0], gy[0], gz[0]]])]).astype(F32)
        s = StructuredGridSampler(V, gx, gy, gz, bounds_handling=mode)
        res[mode] = dict(V=V, gx=gx, gy=gy, gz=gz, q=q, out=np.asarray(s.sample(q), dtype=F32))
    np.savez_compressed(HERE / "structured.npz", **{f"{m}_{k}": v for m, d in res.items() for k, v in d.items()})

    # A3: boundary callables
    B = np.array([[-1.0, 0.0, 0.5], [1.0, 2.0, 1.5]], dtype=F32)
    P = np.concatenate([rng.uniform(-4, 5, (600, 3)), np.array([[-1.0, 0.0, 0.5], [1.0, 2.0, 1.5], [0, 1, 1]])]).astype(F32)
    bres = {"P": P, "B": B}
    bres["periodic"] = bnd.periodic_boundary(B)(P)
    bres["reflective"] = bnd.reflective_boundary(B)(P)
    bres["clamping"] = bnd.clamping_boundary(B)(P)
    bres["absorbing"] = bnd.absorbing_boundary_factory(B)(P)
    bres["absorbing_m7"] = bnd.absorbing_boundary_factory(B, outside_value=-7.0)(P)
    bres["mixed_prc"] = bnd.mixed_boundary(B, {"x": "periodic", "y": "reflective", "z": "clamping"})(P)
    bres["mixed_ab"] = bnd.mixed_boundary(B, {"x": "absorbing", "z": "reflective"})(P)
    # continuous inlet: particles mostly near the faces so that many exit
    Pin = np.concatenate([rng.uniform(-1.3, 1.3, (300, 3)) * np.array([1, 1.2, 0.6]) + np.array([0, 1, 1]),
                          rng.uniform(0.9, 1.1, (100, 3)) * np.array([1, 2, 1.5])]).astype(F32)
    bres["Pin"] = Pin
    conc = {"x": 9, "y": 17, "z": 5}
    bres["inlet_xpos"] = bnd.continuous_inlet_boundary_factory(B, "x", "positive", "grid", conc)(Pin)
    bres["inlet_yneg"] = bnd.continuous_inlet_boundary_factory(B, "y", "negative", "grid", conc)(Pin)
    bres["inlet_zpos"] = bnd.continuous_inlet_boundary_factory(B, "z", "positive", "grid", conc)(Pin)
    np.savez_compressed(HERE / "boundary.npz", **bres)

    # A4: config-0 style tracking (trilinear + linear time + periodic), all integrators
    n = 12
    g = (np.arange(n) / n).astype(F32)
    nodes = grid_nodes(g, g, g)
    st = np.linspace(0, 1, 8).astype(F32)
    D = np.stack([abc(nodes, float(t)) for t in st]).astype(F32)
    ts = TimeSeriesField(data=D, times=st, positions=nodes)

    def field(p, t):
        V = np.asarray(ts.sample_at_time(t)).reshape(n, n, n, 3)
        return StructuredGridSampler(V, g, g, g, bounds_handling="periodic").sample(p)

    # A stage position in (-4e-8, 0) makes np.mod(fx, N) round up to N and the
    # reference raise IndexError (structured.py:294, :325); seeds whose runs
    # never hit that are kept (the GPU path wraps the index instead).
    for seed in range(42, 200):
        np.random.seed(seed)
        x0 = np.random.uniform(0, 1, (300, 3)).astype(F32)
        trk = {"D": D, "st": st, "g": g, "x0": x0, "seed": np.int64(seed)}
        try:
            for integ, T in (("rk4", 31), ("rk2", 21), ("euler", 21)):
                tr = create_tracker(integ, field, bnd.periodic_boundary(((0, 0, 0), (1, 1, 1))),
                                    progress_style="none")
                traj = tr.track_particles(x0, (0.0, 0.3 if integ == "rk4" else 0.2), T, dt=0.01)
                trk[f"{integ}_traj"] = traj.positions
            break
        except IndexError:
            continue
    # record_velocities + recording_interval semantics of the step loop
    tr = create_tracker("rk4", field, bnd.periodic_boundary(((0, 0, 0), (1, 1, 1))), progress_style="none",
                        record_velocities=True, recording_interval=3)
    traj = tr.track_particles(x0[:50], (0.0, 0.1), 11, dt=0.01)
    trk["rec_pos"], trk["rec_vel"] = traj.positions, traj.velocities
    np.savez_compressed(HERE / "track_grid.npz", **trk)

    # A5: config-2 style (clamp grid, continuous inlet on a lattice, mean flow +x)
    n = 10
    g = np.linspace(0, 1, n).astype(F32)
    nodes = grid_nodes(g, g, g)
    st = np.linspace(0, 2, 9).astype(F32)
    noise = np.random.default_rng(2).normal(0, 0.01, (len(st), len(nodes), 3))
    D = np.stack([abc(nodes, float(t)) + np.array([1.0, 0, 0]) for t in st]) + noise
    D = D.astype(F32)
    ts2 = TimeSeriesField(data=D, times=st, positions=nodes)

    def field2(p, t):
        V = np.asarray(ts2.sample_at_time(t)).reshape(n, n, n, 3)
        return StructuredGridSampler(V, g, g, g, bounds_handling="clamp").sample(p)

    from jaxtrace.tracking.seeding import uniform_grid_seeds
    x0 = uniform_grid_seeds((8, 6, 5), ((0, 0, 0), (1, 1, 1)))
    bc = bnd.continuous_inlet_boundary_factory(((0, 0, 0), (1, 1, 1)), "x", "positive", "grid",
                                               {"x": 16, "y": 16, "z": 16})
    tr = create_tracker("rk4", field2, bc, progress_style="none")
    traj = tr.track_particles(x0, (0.0, 0.6), 61, dt=0.01)
    np.savez_compressed(HERE / "track_inlet.npz", D=D, st=st, g=g, x0=x0, traj=traj.positions)

    # A6: nearest-node TimeSeriesField (cKDTree on the NumPy path)
    nodes = rng.random((400, 3)).astype(F32)
    Dn = rng.standard_normal((4, 400, 3)).astype(F32)
    stn = np.array([0, 1, 2, 3], dtype=F32)
    tsn = TimeSeriesField(data=Dn, times=stn, positions=nodes)
    q = rng.uniform(-0.2, 1.2, (500, 3)).astype(F32)
    outs = np.stack([np.asarray(tsn.sample_at_positions(q, t), dtype=F32) for t in (0.0, 0.7, 2.5, 3.5)])
    # test_quick.py scenario: 15x15x1 nodes, 2D vortex, 25 seeds, reflective, RK4, 100 steps, dt 0.02
    xs = np.linspace(-1, 1, 15)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    qn = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1).astype(F32)
    vt = np.linspace(0, 2, 5).astype(F32)
    vort = np.stack([np.stack([-qn[:, 1], qn[:, 0], np.zeros(len(qn))], 1) * (1 + 0.2 * t) for t in vt]).astype(F32)
    tsq = TimeSeriesField(data=vort, times=vt, positions=qn)
    s = np.linspace(-0.6, 0.6, 5)
    SX, SY = np.meshgrid(s, s, indexing="ij")
    seeds = np.stack([SX.ravel(), SY.ravel(), np.zeros(25)], 1).astype(F32)
    tr = create_tracker("rk4", tsq, bnd.reflective_boundary([[-1, -1, -1], [1, 1, 1]]), progress_style="none")
    traj = tr.track_particles(seeds, (0.0, 2.0), 101, dt=0.02)
    np.savez_compressed(HERE / "nearest.npz", nodes=nodes, D=Dn, st=stn, q=q, outs=outs, qn=qn, vort=vort, vt=vt,
                        seeds=seeds, quick_traj=traj.positions)
    # A7: density passes (KDE pure-NumPy formula with SciPy switched off; SPH brute force)
    from jaxtrace.density import kde as kde_mod
    from jaxtrace.density.kde import KDEEstimator
    from jaxtrace.density.sph import SPHDensityEstimator
    kde_mod.SCIPY_AVAILABLE = False
    drng = np.random.default_rng(99)
    Pd = np.concatenate([drng.normal(0.5, 0.12, (900, 3)), drng.random((600, 3))]).astype(F32)
    dens = {"P": Pd}
    k3 = KDEEstimator(Pd, bandwidth_rule="scott", resolution=12)
    X, Y, Z, D = k3.evaluate_3d()
    dens.update(kde_h=np.float64(k3.h), kde3_X=X, kde3_Y=Y, kde3_Z=Z, kde3_D=D)
    k2 = KDEEstimator(Pd, bandwidth_rule="silverman", resolution=20, plane="xz", slab_position=0.5, slab_thickness=0.3)
    X2, Y2, Z2 = k2.evaluate_2d()
    dens.update(kde2_h=np.float64(k2.h), kde2_X=X2, kde2_Y=Y2, kde2_Z=Z2)
    qk = drng.uniform(-0.1, 1.1, (300, 3)).astype(F32)
    dens.update(kde_q=qk, kde_pts=np.asarray(k3.evaluate(qk), dtype=F32))
    for kern in ("cubic_spline", "wendland", "gaussian"):
        s3 = SPHDensityEstimator(Pd, dimensions="3d", smoothing_length=0.08, kernel_type=kern)
        dens[f"sph3_{kern}"] = np.asarray(s3.evaluate(Pd), dtype=F32)
    s2 = SPHDensityEstimator(Pd, dimensions="2d", plane="xy", position=0.5, slab_thickness=0.4)
    dens["sph2_default_h"] = np.float64(s2._mean_h)
    dens["sph2_default"] = np.asarray(s2.evaluate(Pd), dtype=F32)
    sa = SPHDensityEstimator(Pd[:400], dimensions="3d", adaptive=True, n_neighbors=16)
    dens["sph3_adaptive_h"] = np.asarray(sa.smoothing_lengths, dtype=F32)
    dens["sph3_adaptive"] = np.asarray(sa.evaluate(Pd[:400]), dtype=F32)
    np.savez_compressed(HERE / "density.npz", **dens)
    print("phase numpy: done")


def phase_octree(ref: str):
    sys.path.insert(0, str(REPO / "oracle" / "jaxshim"))
    sys.path.insert(1, ref)
    import contextlib
    import io
    import warnings
    warnings.simplefilter("ignore")
    from jaxtrace.fields import octree_fem_interpolator_optimized as oc
    from jaxtrace.fields.octree_fem_time_series_optimized import OctreeFEMTimeSeriesFieldOptimized
    from jaxtrace.tracking import boundary as bnd
    from jaxtrace.tracking.tracker import create_tracker

    quiet = contextlib.redirect_stdout(io.StringIO())
    # B0: the module's own known answer (…optimized.py:413-433)
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1], [1, 0, 1], [1, 1, 0], [0, 1, 1]], F32)
    conn = np.array([[0, 1, 2, 3], [4, 5, 6, 7]], np.int32)
    with quiet:
        m = oc.build_octree_mesh_optimized(pts, conn, max_elements_per_leaf=1, max_depth=5)
        ka = np.asarray(oc.create_octree_fem_interpolator_optimized(m)(np.array([[0.25, 0.25, 0.25]], F32), pts))
    out = {"ka_pts": pts, "ka_conn": conn, "ka_out": ka}
    # B1-B3: jittered Kuhn mesh
    P, T4 = kuhn_mesh(6, 0.2, 1)
    st = np.linspace(0, 1, 5).astype(F32)
    D = np.stack([abc(P, float(t)) for t in st]).astype(F32)
    with quiet:
        f = OctreeFEMTimeSeriesFieldOptimized(D, st, P, T4, max_elements_per_leaf=32, max_depth=12)
    M = f.octree_mesh
    for k in ("nodes_min", "nodes_max", "nodes_elements", "nodes_elem_counts", "nodes_children", "nodes_is_leaf",
              "element_bounds", "element_centroids"):
        out[k] = np.asarray(getattr(M, k))
    rng = np.random.default_rng(7)
    q = np.concatenate([rng.random((400, 3)), rng.uniform(-0.1, 1.1, (60, 3))]).astype(F32)
    out.update(P=P, T4=T4, st=st, D=D, q=q)
    out["sample_t03"] = np.asarray(f.sample_at_positions(q, np.float32(0.3)), dtype=F32)
    out["sample_t10"] = np.asarray(f.sample_at_positions(q, np.float32(1.0)), dtype=F32)
    x0 = rng.random((60, 3)).astype(F32)
    bc = bnd.mixed_boundary(((0, 0, 0), (1, 1, 1)), {"x": "periodic", "y": "reflective", "z": "periodic"})
    tr = create_tracker("rk4", f, bc, use_jax_jit=False, progress_style="none")
    traj = tr.track_particles(x0, (0.0, 0.1), 11, dt=0.01)
    out.update(x0=x0, traj=traj.positions)
    np.savez_compressed(HERE / "octree.npz", **out)
    print("phase octree: done")


def phase_fem(ref: str):
    """Hash-grid FEM interpolation (fields/fem_interpolator.py,
    fields/fem_time_series.py) under the NumPy stand-in for jax."""
    sys.path.insert(0, str(REPO / "oracle" / "jaxshim"))
    sys.path.insert(1, ref)
    import contextlib
    import io
    import warnings
    warnings.simplefilter("ignore")
    from jaxtrace.fields import fem_interpolator as fi
    from jaxtrace.fields.fem_time_series import FEMTimeSeriesField
    from jaxtrace.tracking import boundary as bnd
    from jaxtrace.tracking.tracker import create_tracker

    quiet = contextlib.redirect_stdout(io.StringIO())
    # C0: the module's own example (fem_interpolator.py:385-413): two tets, a
    # query outside both, answered by the nearest node
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1], [1, 0, 1], [1, 1, 0], [0, 1, 1]], F32)
    conn = np.array([[0, 1, 2, 3], [4, 5, 6, 7]], np.int32)
    with quiet:
        m = fi.build_tetrahedral_mesh(pts, conn, grid_resolution=4)
        ka = np.asarray(fi.create_fem_interpolator(m)(np.array([[0.5, 0.5, 0.5], [0.1, 0.1, 0.1]], F32), pts))
    out = {"ka_pts": pts, "ka_conn": conn, "ka_out": ka}
    # C1-C3: jittered Kuhn mesh, squashed to half height in z so the hash
    # grid's aspect-ratio adjustment gives unequal cells per axis
    P, T4 = kuhn_mesh(6, 0.2, 1)
    P = (P * np.array([1.0, 1.0, 0.5], F32)).astype(F32)
    st = np.linspace(0, 1, 5).astype(F32)
    D = np.stack([abc(P, float(t)) for t in st]).astype(F32)
    with quiet:
        f = FEMTimeSeriesField(D, st, P, T4, fem_grid_resolution=8)
    M = f.fem_mesh
    out.update(grid_size=np.array(M.grid_size, np.int64), grid_min=np.asarray(M.grid_min),
               grid_cell_size=np.asarray(M.grid_cell_size), cell_to_elements=np.asarray(M.cell_to_elements),
               cell_elem_counts=np.asarray(M.cell_elem_counts), element_bounds=np.asarray(M.element_bounds))
    rng = np.random.default_rng(8)
    q = np.concatenate([rng.random((300, 3)) * np.array([1, 1, 0.5]), rng.uniform(-0.1, 1.1, (60, 3))]).astype(F32)
    out.update(P=P, T4=T4, st=st, D=D, q=q)
    out["sample_t03"] = np.asarray(f.sample_at_positions(q, np.float32(0.3)), dtype=F32)
    out["sample_t10"] = np.asarray(f.sample_at_positions(q, np.float32(1.0)), dtype=F32)
    x0 = (rng.random((40, 3)) * np.array([1, 1, 0.5])).astype(F32)
    bc = bnd.mixed_boundary(((0, 0, 0), (1, 1, 0.5)), {"x": "periodic", "y": "reflective", "z": "periodic"})
    tr = create_tracker("rk4", f, bc, use_jax_jit=False, progress_style="none")
    traj = tr.track_particles(x0, (0.0, 0.08), 9, dt=0.01)
    out.update(x0=x0, traj=traj.positions)
    np.savez_compressed(HERE / "fem.npz", **out)
    print("phase fem: done")


def phase_analytics(ref: str):
    """Trajectory statistics and mixing metrics of the reference on small
    random-walk trajectories (with and without stored velocities)."""
    sys.path.insert(0, ref)
    from jaxtrace.tracking.analysis import compute_mixing_metrics
    from jaxtrace.tracking.particles import Trajectory, compute_trajectory_statistics
    rng = np.random.default_rng(21)
    T, N = 40, 600
    steps = rng.normal(0.0, 0.01, (T, N, 3)).astype(F32)
    steps[0] = rng.random((N, 3)).astype(F32)
    pos = np.cumsum(steps, axis=0, dtype=F32)
    pos[T // 2:, : N // 10, 0] -= F32(1.0)                 # periodic-style jumps in x for a tenth
    times = np.linspace(0.0, 2.0, T).astype(F32)
    vel = rng.normal(0.0, 0.5, (T, N, 3)).astype(F32)
    out = {"positions": pos, "times": times, "velocities": vel}
    for tag, v in (("nov", None), ("vel", vel)):
        tr = Trajectory(positions=pos.copy(), times=times.copy(), velocities=None if v is None else v.copy())
        out[f"{tag}_displacement"] = tr.compute_displacement()
        out[f"{tag}_path_length"] = tr.compute_path_length()
        out[f"{tag}_speeds"] = tr.compute_speeds()
        stats = compute_trajectory_statistics(tr)
        for group, vals in stats.items():
            for k, val in vals.items():
                out[f"{tag}_stats_{group}_{k}"] = np.asarray(val, dtype=np.float64)
    mix = compute_mixing_metrics(Trajectory(positions=pos.copy(), times=times.copy()))
    for k, val in mix.items():
        out[f"mix_{k}"] = np.asarray(val, dtype=np.float64)
    np.savez_compressed(HERE / "analytics.npz", **out)
    print("phase analytics: done")


def phase_steps(ref: str):
    """The standalone step functions (integrators/rk4.py:62-129,
    rk2.py:117-180, euler.py:111-157) on the trilinear + linear-time field,
    with a scalar dt and with a per-particle dt (mean-dt stage times), at a
    float32 time, a Python float time and a time between snapshots."""
    sys.path.insert(0, ref)
    import warnings
    warnings.simplefilter("ignore")
    from jaxtrace.fields.structured import StructuredGridSampler
    from jaxtrace.fields.time_series import TimeSeriesField
    from jaxtrace.integrators.euler import euler_step
    from jaxtrace.integrators.rk2 import rk2_step
    from jaxtrace.integrators.rk4 import rk4_step
    from jaxtrace.utils.jax_utils import JAX_AVAILABLE
    assert not JAX_AVAILABLE, "phase steps must run without jax"
    n = 12
    g = (np.arange(n) / n).astype(F32)
    nodes = grid_nodes(g, g, g)
    st = np.linspace(0, 1, 8).astype(F32)
    D = np.stack([abc(nodes, float(t)) for t in st]).astype(F32)
    ts = TimeSeriesField(data=D, times=st, positions=nodes)

    def field(p, t):
        V = np.asarray(ts.sample_at_time(t)).reshape(n, n, n, 3)
        return StructuredGridSampler(V, g, g, g, bounds_handling="periodic").sample(p)

    rng = np.random.default_rng(77)
    # positions away from the periodic seam, so no stage lands in (-4e-8, 0)
    x = rng.uniform(0.05, 0.95, (256, 3)).astype(F32)
    dt_pp = rng.uniform(0.002, 0.02, 256).astype(F32)
    out = {"D": D, "st": st, "g": g, "x": x, "dt_pp": dt_pp, "times": np.array([0.13, 0.5, 0.71])}
    for name, fn in (("rk4", rk4_step), ("rk2", rk2_step), ("euler", euler_step)):
        for k, t in enumerate((0.13, 0.5, 0.71)):
            tf = np.float32(t) if k == 0 else t       # a float32 time and Python float times
            out[f"{name}_scalar_{k}"] = np.asarray(fn(x, tf, 0.01, field), dtype=F32)
            out[f"{name}_pp_{k}"] = np.asarray(fn(x, tf, dt_pp, field), dtype=F32)
    np.savez_compressed(HERE / "steps.npz", **out)



def phase_seeding(ref: str):
    """The NumPy branch of random_seeds and uniform_grid_seeds
    (tracking/seeding.py:140-247) over every accepted bounds form, with and
    without the boundaries, 3- and 2-tuple resolutions; a refusal is kept as
    its error type and message."""
    sys.path.insert(0, ref)
    import warnings
    warnings.simplefilter("ignore")
    from jaxtrace.tracking.seeding import random_seeds, uniform_grid_seeds
    from jaxtrace.utils.jax_utils import JAX_AVAILABLE
    assert not JAX_AVAILABLE, "phase seeding must run without jax"
    forms = {"b23": [[-1.0, 0.5, 2.0], [3.0, 1.5, 2.25]], "b6": [0.0, 2.0, -1.0, 1.0, 0.1, 0.3],
             "b32": [[0.0, 1.0], [0.0, 2.0], [0.0, 3.0]], "b4": [0.0, 1.0, -2.0, 2.0], "b22": [[0.0, 1.0], [2.0, 3.0]],
             "bad": [[1.0, 0.0, 0.0], [0.0, 1.0, 1.0]]}
    calls = {"rand": lambda b: random_seeds(1000, b, rng_seed=7),
             "rand0": lambda b: random_seeds(0, b),
             "grid": lambda b: uniform_grid_seeds((5, 4, 3), b, True),
             "grid_int": lambda b: uniform_grid_seeds(4, b, False),
             "grid2": lambda b: uniform_grid_seeds((6, 5), b, True),
             "grid2_int": lambda b: uniform_grid_seeds((6, 5), b, False)}
    out, errors = {}, {}
    for fname, b in forms.items():
        for cname, fn in calls.items():
            key = f"{cname}_{fname}"
            try:
                out[key] = np.asarray(fn(b))
            except Exception as e:  # noqa: BLE001 -- the reference's refusal is the fixture
                errors[key] = {"type": type(e).__name__, "message": str(e).split("\n")[0]}
    out["forms"] = np.array(json.dumps(forms))
    out["errors"] = np.array(json.dumps(errors))
    np.savez_compressed(HERE / "seeding.npz", **out)
    print(f"phase seeding: {len(out) - 2} arrays, {len(errors)} refusals")

def _vtk_scenarios():
    """The time-series directories of phase vtk: per scenario its files
    (name, points, point-data arrays, pieces of a .pvtu) and the reader's
    arguments.  Points and arrays are small seeded random sets."""
    rng = np.random.default_rng(31)

    def pts(n):
        return rng.uniform(-1.0, 2.0, (n, 3)).astype(F32)

    def vtu(name, p, arrays):
        return {"name": name, "kind": "vtu", "points": p, "arrays": arrays}

    sc = []
    # serial files in natural (not lexical) order, a scalar beside the velocity, a stray file
    p1 = pts(37)
    files = [vtu(f"flow_{k}.vtu", p1, [("p", rng.normal(size=37)), ("Velocity", rng.normal(size=(37, 3)).astype(F32))])
             for k in (10, 2, 0, 1)]
    files.append({"name": "notes.txt", "kind": "txt"})
    sc.append({"tag": "serial", "files": files, "pattern": "*", "kwargs": {}})
    # .pvtu files preferred over every .vtu, two pieces each, 2-component "U" padded to 3
    p2a, p2b = pts(11), pts(9)
    files = []
    for k in (0, 1):
        ua, ub = rng.normal(size=(11, 2)).astype(F32), rng.normal(size=(9, 2)).astype(F32)
        files.append(vtu(f"a_{k}_p0.vtu", p2a, [("U", ua)]))
        files.append(vtu(f"a_{k}_p1.vtu", p2b, [("U", ub)]))
        files.append({"name": f"a_{k}.pvtu", "kind": "pvtu", "pieces": [f"a_{k}_p0.vtu", f"a_{k}_p1.vtu"],
                      "points": np.concatenate([p2a, p2b]), "arrays": [("U", np.concatenate([ua, ub]))]})
    files.append(vtu("b_5.vtu", p2a, [("U", rng.normal(size=(11, 2)).astype(F32))]))
    sc.append({"tag": "parallel", "files": files, "pattern": "*", "kwargs": {}})
    # the last max_time_steps files, a named 4-component array cut to 3
    p3 = pts(23)
    files = [vtu(f"s_{k}.vtu", p3, [("velocity", rng.normal(size=(23, 3)).astype(F32)),
                                    ("w4", rng.normal(size=(23, 4)).astype(F32))]) for k in (1, 3, 2)]
    sc.append({"tag": "named_last2", "files": files, "pattern": "s_*.vtu",
               "kwargs": {"max_time_steps": 2, "velocity_field_name": "w4"}})
    # a scalar named as the velocity: VTK hands back a 1-D array, which the reader refuses
    sc.append({"tag": "scalar_named", "files": files, "pattern": "s_*.vtu", "kwargs": {"velocity_field_name": "p"}})
    # no array with a velocity name
    p5 = pts(8)
    files = [vtu(f"t_{k}.vtu", p5, [("pressure", rng.normal(size=8)), ("T", rng.normal(size=(8, 3)).astype(F32))])
             for k in (0, 1)]
    sc.append({"tag": "no_velocity", "files": files, "pattern": "*.vtu", "kwargs": {}})
    for s in sc:
        if s["tag"] == "scalar_named":
            s["files"] = [dict(f, arrays=f["arrays"] + [("p", rng.normal(size=23))]) for f in s["files"]]
    return sc


def write_vtk_scenario(root, scenario):
    """Write a scenario's files under root with this repository's writers."""
    sys.path.insert(0, str(REPO))
    from jaxtrace_gb300 import vtk_io as V
    os.makedirs(root, exist_ok=True)
    for f in scenario["files"]:
        path = os.path.join(root, f["name"])
        if f["kind"] == "txt":
            Path(path).write_text("not a VTK file\n")
        elif f["kind"] == "vtu":
            V.write_vtu(path, f["points"], None, dict(f["arrays"]), vertices=True)
        else:
            types = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64"}
            arrs = {n: (types[np.asarray(a).dtype], 1 if np.ndim(a) == 1 else np.shape(a)[1]) for n, a in f["arrays"]}
            V.write_pvtu(path, f["pieces"], arrs)


def phase_vtk(ref: str):
    """The reference's VTKUnstructuredTimeSeriesReader (io/vtk_reader.py:426-940)
    over series written by this repository's writers, with the VTK library
    replaced by the stand-in oracle/vtkshim: its file selection and order,
    velocity-name detection, component padding, bounds and time values."""
    import contextlib
    import io
    import tempfile
    import warnings
    warnings.simplefilter("ignore")
    sys.path.insert(0, str(REPO / "oracle" / "vtkshim"))
    sys.path.insert(1, ref)
    import vtk as fake
    from jaxtrace.io import vtk_reader as R
    assert R.VTK_AVAILABLE
    out, manifest = {}, []
    for s in _vtk_scenarios():
        with tempfile.TemporaryDirectory() as tmp:
            write_vtk_scenario(tmp, s)
            fake.REGISTRY.clear()
            for f in s["files"]:
                if f["kind"] != "txt":
                    fake.REGISTRY[os.path.abspath(os.path.join(tmp, f["name"]))] = {
                        "points": f["points"], "point_data": f["arrays"]}
            tag = s["tag"]
            rec = {"tag": tag, "pattern": s["pattern"], "kwargs": s["kwargs"], "files": []}
            for i, f in enumerate(s["files"]):
                entry = {"name": f["name"], "kind": f["kind"], "pieces": f.get("pieces", [])}
                if f["kind"] != "txt":
                    out[f"{tag}_f{i}_points"] = f["points"]
                    entry["arrays"] = [n for n, _ in f["arrays"]]
                    for n, a in f["arrays"]:
                        out[f"{tag}_f{i}_{n}"] = np.asarray(a)
                rec["files"].append(entry)
            try:
                with contextlib.redirect_stdout(io.StringIO()):
                    rd = R.VTKUnstructuredTimeSeriesReader(os.path.join(tmp, s["pattern"]), **s["kwargs"])
                    ts = rd.load_time_series()
                    bounds = rd.get_bounds()
                    info = rd.get_grid_info()
                rec["order"] = [os.path.basename(f) for f in rd.time_files]
                rec["velocity_field_name"] = ts["velocity_field_name"]
                rec["source"] = ts["source"]
                rec["info"] = {"n_points": int(info["n_points"]), "n_timesteps": int(info["n_timesteps"]),
                               "velocity_field_name": info["velocity_field_name"],
                               "time_files": [os.path.basename(f) for f in info["time_files"]],
                               "has_spatial_index": bool(info["has_spatial_index"]), "keys": sorted(info)}
                out[f"{tag}_velocity_data"] = ts["velocity_data"]
                out[f"{tag}_positions"] = ts["positions"]
                out[f"{tag}_times"] = ts["times"]
                out[f"{tag}_bounds"] = np.asarray(bounds, dtype=np.float64)
            except Exception as e:  # noqa: BLE001 -- the reference's refusal is the fixture
                rec["error"] = {"type": type(e).__name__, "message": str(e).split("\n")[0]}
            manifest.append(rec)
    out["manifest"] = np.array(json.dumps(manifest))
    np.savez_compressed(HERE / "vtk_reader.npz", **out)
    print("phase vtk: done")


PHASES = {"numpy": phase_numpy, "octree": phase_octree, "fem": phase_fem, "analytics": phase_analytics,
          "steps": phase_steps, "vtk": phase_vtk, "seeding": phase_seeding}

if __name__ == "__main__":
    if len(sys.argv) >= 3 and sys.argv[1] in PHASES:
        PHASES[sys.argv[1]](sys.argv[2])
        sys.exit(0)
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("JAXTRACE_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py /path/to/JAXTrace   (or set JAXTRACE_REFERENCE)")
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    for phase in PHASES:
        subprocess.run([sys.executable, __file__, phase, ref], check=True, env=env)
