"""Known answers of the interpolants (the unit level of the reference's test
plan): trilinear cells and P1 tetrahedra reproduce an affine velocity field,
and the time blend of two snapshots is linear in time.  Each is checked on
the field samplers and through the tracking kernel (one Euler step), for
float32 pair gathers and pre-blended stage fields."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import workloads as W

pytestmark = pytest.mark.gpu
F32 = np.float32

A = np.array([[0.3, -0.2, 0.1], [0.05, 0.4, -0.3], [-0.1, 0.2, 0.25]])
B = np.array([0.5, -0.25, 0.125])


def affine(p, scale=1.0):
    return (scale * (p.astype(np.float64) @ A.T + B)).astype(F32)


def _grid_field(mode="clamp", storage="f32"):
    g = np.linspace(0.0, 1.0, 17).astype(F32)
    nodes = W.grid_nodes(g, g, g)
    st = np.array([0.0, 1.0], dtype=F32)
    data = np.stack([affine(nodes, 1.0), affine(nodes, 2.0)])        # v(x, t) = (1 + t)(A x + b)
    return jt.StructuredTimeSeriesField(data, st, g, g, g, mode, storage=storage)


def _queries(n=5000, seed=3):
    return np.random.default_rng(seed).uniform(0.02, 0.98, (n, 3)).astype(F32)


@pytest.mark.parametrize("t", [0.0, 0.25, 0.7, 1.0])
def test_trilinear_reproduces_an_affine_field_at_any_time(t):
    f = _grid_field()
    q = _queries()
    out = f.sample_at_positions(q, t)
    ref = affine(q, 1.0 + t)
    assert np.max(np.abs(out - ref)) < 2e-6


@pytest.mark.parametrize("stage", [False, True])
@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_euler_step_on_an_affine_field(stage, storage):
    """One Euler step x1 = x0 + dt v(x0, 0): the tracking kernel's gather
    (pair records or stage fields) of an affine field is exact up to float32
    rounding (float16 values: their rounding)."""
    f = _grid_field(storage=storage)
    x0 = _queries(4096, 5)
    dt = 0.01
    tr = jt.create_tracker("euler", f, jt.clamping_boundary(W.UNIT), stage_fields=stage, record_final_only=True)
    x1 = tr.track_particles(x0, (0.0, dt), 2, dt=dt).positions[-1]
    ref = (x0.astype(np.float64) + dt * affine(x0, 1.0).astype(np.float64))
    tol = 2e-7 if storage == "f32" else 3e-5
    assert np.max(np.abs(x1 - ref)) < tol


def _mesh():
    P, T4 = W.kuhn_mesh(8, 0.2, 2)
    st = np.array([0.0, 1.0], dtype=F32)
    D = np.stack([affine(P, 1.0), affine(P, 2.0)])
    return P, T4, st, D


@pytest.mark.parametrize("kind", ["octree", "hash"])
def test_p1_reproduces_an_affine_field(kind):
    P, T4, st, D = _mesh()
    if kind == "octree":
        f = jt.OctreeFEMTimeSeriesFieldOptimized(D, st, P, T4)
    else:
        f = jt.FEMTimeSeriesField(D, st, P, T4, fem_grid_resolution=8)
    # points well inside the mesh whose containing tetrahedron the location
    # finds (the reference's lookups fall back to a node value elsewhere)
    q = _queries(3000, 7)
    out = f.sample_at_positions(q, F32(0.5))
    ref = affine(q, 1.5)
    err = np.max(np.abs(out - ref), axis=1)
    # most points are located (fallbacks give a node's value, not the affine one)
    located = err < 5e-6
    assert located.mean() > 0.5
    # a located point is exact to float32 P1 rounding; the rest carry a
    # nearby node's value (within the field's variation over a cell)
    assert np.all(err[~located] < 0.3)
