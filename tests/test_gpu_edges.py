"""Edge cases of the public tracking API on the GPU: empty and ragged
particle counts, a run with no steps, a flat grid axis, non-finite starting
positions and particles far outside the grid, each against the float32
oracle (bit for bit on the exact path) or against the API's own contract."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle
from jaxtrace_gb300 import _lib as L
from jaxtrace_gb300 import workloads as W

pytestmark = pytest.mark.gpu
F32 = np.float32


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    L.load()
    yield


@pytest.fixture(scope="module")
def plain():
    c = W.plain_rk4(n_particles=1000, n=16, n_snap=6)
    g = c["grid"][0]
    f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "periodic")
    spec = oracle.GridSpec(c["data"], c["times"], g, g, g, "periodic")
    return c, f, spec


def _oracle(spec, kinds, x0, n_steps, dt):
    times = np.linspace(0.0, n_steps * dt, n_steps + 1, dtype=F32)
    ref, _, _ = oracle.track(spec, oracle.BoundarySpec(kinds=kinds), x0, times, dt)
    return ref


@pytest.mark.parametrize("n", [0, 1, 31, 33, 255, 257])
def test_ragged_and_empty_particle_counts(plain, n):
    """Counts below, at and above a warp and a block, and none at all."""
    c, f, spec = plain
    x0 = c["x0"][:n]
    tr = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT), record_final_only=True)
    traj = tr.track_particles(x0, (0.0, 0.2), 21, dt=0.01)
    assert traj.positions.shape == (2, n, 3)
    if n:
        assert same(traj.positions[-1], _oracle(spec, ("periodic",) * 3, x0, 20, 0.01))
        assert same(traj.positions[0], x0)


def test_a_run_without_steps_returns_the_input(plain):
    c, f, _ = plain
    tr = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT))
    traj = tr.track_particles(c["x0"][:100], (0.0, 0.0), 1, dt=0.01)
    assert traj.positions.shape == (1, 100, 3) and same(traj.positions[0], c["x0"][:100])


def test_a_flat_grid_axis_against_the_oracle():
    """One node along z (a planar field): the sampler's clamped successor is
    the node itself, and the z weight never matters."""
    rng = np.random.default_rng(4)
    gx, gy, gz = np.linspace(0, 1, 9, dtype=F32), np.linspace(0, 1, 7, dtype=F32), np.zeros(1, F32)
    times = np.array([0.0, 0.5, 1.0], F32)
    data = rng.normal(0, 0.5, (3, 9 * 7 * 1, 3)).astype(F32)
    data[..., 2] = 0.0
    f = jt.StructuredTimeSeriesField(data, times, gx, gy, gz, "clamp")
    x0 = rng.uniform(0, 1, (500, 3)).astype(F32)
    x0[:, 2] = 0.0
    tr = jt.create_tracker("rk4", f, jt.clamping_boundary(((0, 0, 0), (1, 1, 1))), record_final_only=True)
    out = tr.track_particles(x0, (0.0, 0.5), 51, dt=0.01).positions[-1]
    spec = oracle.GridSpec(data, times, gx, gy, gz, "clamp")
    b = oracle.BoundarySpec(kinds=("clamp",) * 3, bounds=((0, 0, 0), (1, 1, 1)))
    ref, _, _ = oracle.track(spec, b, x0, np.linspace(0.0, 0.5, 51, dtype=F32), 0.01)
    assert same(out, ref)


def test_non_finite_starts_are_reported_and_do_not_touch_the_others(plain):
    """NaN and infinite starting positions: the run completes, flags the
    non-finite result, and every finite particle still matches the oracle."""
    c, f, spec = plain
    x0 = c["x0"][:300].copy()
    x0[[3, 77]] = np.nan
    x0[150, 1] = np.inf
    tr = jt.create_tracker("rk4", f, jt.no_boundary(), record_final_only=True)
    out = tr.track_particles(x0, (0.0, 0.1), 11, dt=0.01).positions[-1]
    assert tr.last_status & L.JT_STATUS_NONFINITE
    ok = np.all(np.isfinite(x0), axis=1)
    ref = _oracle(spec, ("none",) * 3, x0[ok], 10, 0.01)
    assert same(out[ok], ref)
    assert not np.all(np.isfinite(out[~ok]))


@pytest.mark.parametrize("mode", ["clamp", "zero", "nan"])
def test_particles_far_outside_the_grid(mode):
    """Starts well outside the grid in every direction, with no boundary:
    clamp reads the nearest face, zero stops the particle, nan poisons it,
    each exactly as the oracle does."""
    rng = np.random.default_rng(8)
    g = np.linspace(0, 1, 10, dtype=F32)
    times = np.array([0.0, 1.0], F32)
    data = rng.normal(0, 1, (2, 1000, 3)).astype(F32)
    f = jt.StructuredTimeSeriesField(data, times, g, g, g, mode)
    x0 = np.concatenate([rng.uniform(-5, 6, (400, 3)), rng.uniform(0, 1, (100, 3))]).astype(F32)
    tr = jt.create_tracker("rk4", f, jt.no_boundary(), record_final_only=True)
    out = tr.track_particles(x0, (0.0, 0.3), 31, dt=0.01).positions[-1]
    spec = oracle.GridSpec(data, times, g, g, g, mode)
    ref = _oracle(spec, ("none",) * 3, x0, 30, 0.01)
    assert same(out, ref)


def test_device_inputs_and_device_results(plain):
    """A CUDA tensor as the initial positions gives the host input's
    trajectory bit for bit (the caller's tensor untouched), and
    return_device=True hands back the same final positions on the device."""
    import torch
    c, f, _ = plain
    x0 = c["x0"][:500]
    tr = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT), record_final_only=True)
    ref = tr.track_particles(x0, (0.0, 0.2), 21, dt=0.01)
    xd = torch.from_numpy(x0).cuda()
    keep = xd.clone()
    got = tr.track_particles(xd, (0.0, 0.2), 21, dt=0.01)
    assert same(got.positions, ref.positions) and torch.equal(xd, keep)
    fin = tr.track_particles(xd, (0.0, 0.2), 21, dt=0.01, return_device=True)
    assert fin.is_cuda and fin.shape == (500, 3) and same(fin.cpu().numpy(), ref.positions[-1])
    fin_host_in = tr.track_particles(x0, (0.0, 0.2), 21, dt=0.01, return_device=True)
    assert same(fin_host_in.cpu().numpy(), ref.positions[-1])
    # 2-D positions on the device get z = 0, as 2-D arrays do
    flat = np.ascontiguousarray(x0[:, :2])
    ref2 = tr.track_particles(flat, (0.0, 0.2), 21, dt=0.01)
    got2 = tr.track_particles(torch.from_numpy(flat).cuda(), (0.0, 0.2), 21, dt=0.01)
    assert same(got2.positions, ref2.positions)
    every = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT))
    with pytest.raises(ValueError, match="record_final_only"):
        every.track_particles(xd, (0.0, 0.2), 21, dt=0.01, return_device=True)


def test_octree_tracking_on_a_five_level_tree():
    """A 16^3-hexahedron Kuhn mesh (24,576 tetrahedra, 4,681 octree nodes over
    five levels, deeper than the other tests' trees): the breadth-first
    descent's trajectory is the oracle's bit for bit, inside the mesh and
    across its faces, with and without re-sorting."""
    P, tets = W.kuhn_mesh(16, 0.2, 3)
    st = np.linspace(0, 1, 4).astype(F32)
    data = W.abc_snapshots(P, st)
    f = jt.OctreeFEMTimeSeriesFieldOptimized(data, st, P, tets)
    m = f.octree_mesh
    assert len(m.nodes) > 585
    spec = oracle.MeshSpec(data, st, P, tets, m.element_bounds, m.nodes_min, m.nodes_max, m.nodes_elements,
                           m.nodes_children, m.nodes_is_leaf, max_depth=m.max_depth)
    rng = np.random.default_rng(12)
    x0 = rng.uniform(-0.05, 1.05, (3000, 3)).astype(F32)
    T, dt = 16, 0.01
    for sort_every in (0, 5):
        tr = jt.create_tracker("rk4", f, jt.no_boundary(), record_final_only=True, sort_every=sort_every)
        out = tr.track_particles(x0, (0.0, (T - 1) * dt), T, dt=dt).positions[-1]
        ref, _, _ = oracle.track(spec, oracle.BoundarySpec(kinds=("none",) * 3), x0,
                                 np.linspace(0.0, (T - 1) * dt, T, dtype=F32), dt)
        assert same(out, ref)
