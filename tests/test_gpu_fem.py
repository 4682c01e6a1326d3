"""Hash-grid FEM field (FEMTimeSeriesField) on the GPU against the float32
oracle (bit for bit) and against JAXTrace's own outputs (rtol 1e-5: the
reference's jnp.dot of the barycentrics runs through BLAS, whose summation
order is not the sequential one the kernel and the oracle share)."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle
from jaxtrace_gb300 import _lib as L
from jaxtrace_gb300 import workloads as W

pytestmark = pytest.mark.gpu
F32 = np.float32


def same(a, b):
    return np.array_equal(np.asarray(a, F32).view(np.uint32), np.asarray(b, F32).view(np.uint32))


def _field(g, **kw):
    return jt.FEMTimeSeriesField(g["D"], g["st"], g["P"], g["T4"], fem_grid_resolution=8, **kw)


def _spec(g):
    return oracle.FemSpec(g["D"], g["st"], g["P"], g["T4"], g["grid_size"], g["grid_min"], g["grid_cell_size"],
                          g["cell_to_elements"], g["element_bounds"])


def test_fem_sampling(golden):
    g = golden("fem")
    f = _field(g)
    spec = _spec(g)
    for key, t in (("sample_t03", 0.3), ("sample_t10", 1.0)):
        out = f.sample_at_positions(g["q"], F32(t))
        ref, fb = oracle.sample(spec, g["q"], float(F32(t)), t_is_f32=True)
        assert same(out, ref)
        assert np.allclose(out, g[key], rtol=1e-5, atol=1e-6)
        assert fb > 0


def test_fem_known_answer(golden):
    g = golden("fem")
    pts = g["ka_pts"]
    f = jt.FEMTimeSeriesField(np.stack([pts, pts]), np.array([0, 1], F32), pts, g["ka_conn"], fem_grid_resolution=4)
    out = f.sample_at_positions(np.array([[0.5, 0.5, 0.5], [0.1, 0.1, 0.1]], F32), 0.0)
    assert np.allclose(out, g["ka_out"])


def test_fem_tracking(golden):
    g = golden("fem")
    f = _field(g)
    bounds = ((0, 0, 0), (1, 1, 0.5))
    bc = jt.mixed_boundary(bounds, {"x": "periodic", "y": "reflective", "z": "periodic"})
    traj = jt.create_tracker("rk4", f, bc).track_particles(g["x0"], (0.0, 0.08), 9, dt=0.01)
    assert np.allclose(traj.positions, g["traj"], rtol=1e-5, atol=1e-6)
    obc = oracle.BoundarySpec(kinds=("periodic", "reflective", "periodic"), bounds=bounds)
    _, otraj, _ = oracle.track(_spec(g), obc, g["x0"], np.linspace(0, 0.08, 9, dtype=F32), 0.01, record=True)
    assert same(traj.positions, otraj)


def test_fem_larger_mesh_outside_and_nan_queries():
    P, T4 = W.kuhn_mesh(12, 0.2, 3)
    st = np.linspace(0, 1, 4).astype(F32)
    D = W.abc_snapshots(P, st)
    f = jt.FEMTimeSeriesField(D, st, P, T4, fem_grid_resolution=10)
    h = f.fem_mesh
    spec = oracle.FemSpec(D, st, P, T4, h.grid_size, h.grid_min, h.grid_cell_size, h.cell_to_elements(),
                          h.element_bounds)
    rng = np.random.default_rng(4)
    q = np.concatenate([rng.random((20000, 3)), rng.uniform(-0.5, 1.5, (2000, 3)),
                        P[:500],                                    # nodes: ties and faces
                        np.array([[np.nan, 0.5, 0.5], [0.5, np.inf, 0.5], [-1e30, 0.5, 0.5]])]).astype(F32)
    out = f.sample_at_positions(q, F32(0.45))
    ref, fb = oracle.sample(spec, q, float(F32(0.45)), t_is_f32=True)
    fin = np.all(np.isfinite(q), axis=1)
    assert same(out[fin], ref[fin])
    assert fb > 0
    # a non-finite query gives some node's value (the kernel's NaN-safe nearest search)
    assert np.all(np.isfinite(out[~fin]))


def test_fem_rk4_ensembles_and_16bit():
    P, T4 = W.kuhn_mesh(10, 0.2, 5)
    st = np.linspace(0, 1, 6).astype(F32)
    D = W.abc_snapshots(P, st)
    f = jt.FEMTimeSeriesField(D, st, P, T4, fem_grid_resolution=12)
    h = f.fem_mesh
    spec = oracle.FemSpec(D, st, P, T4, h.grid_size, h.grid_min, h.grid_cell_size, h.cell_to_elements(),
                          h.element_bounds)
    bc = jt.mixed_boundary(W.UNIT, {"x": "periodic", "y": "reflective", "z": "periodic"})
    obc = oracle.BoundarySpec(kinds=("periodic", "reflective", "periodic"))
    rng = np.random.default_rng(9)
    xs = [rng.random((n, 3)).astype(F32) for n in (700, 40, 1500)]
    rel = rng.uniform(0, 0.3, 3)
    tr = jt.create_tracker("rk4", f, bc, sort_every=6, sort_bits=3)
    outs = tr.track_ensembles(xs, rel, 25, dt=0.01)
    for x, t0, o in zip(xs, rel, outs):
        ref, _, _ = oracle.track(spec, obc, x, np.linspace(t0, t0 + 24 * 0.01, 25, dtype=F32), 0.01)
        assert same(o, ref)
    f16 = jt.FEMTimeSeriesField(D, st, P, T4, fem_grid_resolution=12, storage="f16")
    out16 = jt.create_tracker("rk4", f16, bc).track_particles(xs[0], (0.0, 0.24), 25, dt=0.01).positions[-1]
    ref64, _, _ = oracle.track(spec, obc, xs[0], np.linspace(0, 0.24, 25, dtype=F32), 0.01,
                               precision=oracle.ORC_F64)
    d = np.abs(out16 - ref64)
    d = np.minimum(d, 1.0 - d)
    # the nearest-node fallback is discontinuous: a few particles that take it
    # in one run and not the other end far apart, so bound the bulk
    assert np.median(d) < 1e-5 and np.quantile(d, 0.99) < 1e-3
    assert tr.last_status & ~(L.JT_STATUS_OCTREE_FALLBACK | L.JT_STATUS_INDEX_WRAPPED) == 0
