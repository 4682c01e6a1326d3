"""The device octree build (jt_octree_build_device) against the host build,
which is pinned to the reference's arrays (build_octree_mesh_optimized,
fields/octree_fem_interpolator_optimized.py:41-215): every node record,
node bound, element list and per-tetrahedron record bit for bit."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import _lib as L
from jaxtrace_gb300 import workloads as W

pytestmark = pytest.mark.gpu
F32 = np.float32


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    L.load()
    yield


def _same_build(P, T4, mpl, depth):
    h = jt.OctreeMesh(P, T4, mpl, depth, build="host")
    d = jt.OctreeMesh(P, T4, mpl, depth, build="device")
    assert d.dev is not None
    for k in ("n_nodes", "n_elem_entries", "max_elems", "max_tree_depth", "n_leaves"):
        assert getattr(d.info, k) == getattr(h.info, k), k
    assert np.array_equal(d.nodes.view(np.int32), h.nodes.view(np.int32))
    assert np.array_equal(d.elems[:h.info.n_elem_entries], h.elems[:h.info.n_elem_entries])
    assert np.array_equal(d.tet_box.view(np.int32), h.tet_box.view(np.int32))
    assert np.array_equal(d.tet_geom.view(np.int32), h.tet_geom.view(np.int32))
    assert np.array_equal(d.nodes_min, h.nodes_min) and np.array_equal(d.nodes_max, h.nodes_max)
    return h, d


def test_device_octree_matches_reference_golden(golden):
    g = golden("octree")
    _, d = _same_build(g["P"], g["T4"], 32, 12)
    assert np.array_equal(d.nodes_children, g["nodes_children"])
    assert np.array_equal(d.nodes_elements, g["nodes_elements"])
    g2 = golden("octree")
    _same_build(g2["ka_pts"], g2["ka_conn"], 1, 5)


@pytest.mark.parametrize("mpl,depth", [(32, 12), (4, 3), (1, 20), (8, 0), (10 ** 6, 12)])
def test_device_octree_matches_host_build(mpl, depth):
    """Ordinary leaves, depth-limited leaves far above the leaf size, deep
    trees, and a root that is a leaf by depth or by count."""
    P, T4 = W.kuhn_mesh(12)[:2]
    _same_build(P, T4, mpl, depth)


def test_device_octree_on_a_shuffled_mesh():
    """Element order that is not spatially coherent: the leaf lists must
    still come out ascending, as the stable recursive split leaves them."""
    P, T4 = W.kuhn_mesh(10)[:2]
    perm = np.random.default_rng(4).permutation(len(T4))
    _same_build(P, T4[perm], 16, 12)


def test_device_octree_rejects_bad_connectivity():
    with pytest.raises(ValueError, match="outside"):
        jt.OctreeMesh(np.zeros((4, 3), F32), np.array([[0, 1, 2, 9]], np.int32), build="device")


def test_octree_field_runs_on_the_device_build(golden):
    """The field built on the device tracks like the host-built one."""
    c = W.fem_case(n=8, n_snap=4, n_particles=2000, n_steps=50)
    bc = jt.mixed_boundary(W.UNIT, c["conditions"])
    out = []
    for b in ("host", "device"):
        f = jt.OctreeFEMTimeSeriesFieldOptimized(c["data"], c["times"], c["points"], c["tets"], octree_build=b)
        tr = jt.create_tracker("rk4", f, bc, record_final_only=True)
        out.append(tr.track_particles(c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"]).positions)
    assert np.array_equal(out[0], out[1])


def test_device_builds_allocate_through_the_installed_allocator():
    """jt_set_allocator: the device builds take every scratch and handle
    array from the caller's allocator (here a counting wrapper around
    torch's caching allocator) and give all of it back."""
    import torch
    calls = {"alloc": 0, "free": 0, "live": set()}

    def alloc(n, stream, ctx):
        p = torch.cuda.caching_allocator_alloc(max(int(n), 1), stream=int(stream or 0))
        calls["alloc"] += 1
        calls["live"].add(p)
        return p

    def free(p, stream, ctx):
        calls["free"] += 1
        calls["live"].discard(int(p))
        torch.cuda.caching_allocator_delete(int(p))

    fa, ff = L.ALLOC_FN(alloc), L.FREE_FN(free)
    lib = L.load()
    L.check(lib.jt_set_allocator(fa, ff, None))
    try:
        P, T4 = W.kuhn_mesh(8, 0.2, 1)
        h, d = _same_build(P, T4, 32, 12)
        n_oct = calls["alloc"]
        g = jt.FemHashGrid(P, T4, 8, build="device")
        assert g.dev is not None and calls["alloc"] > n_oct
        del g, d
        torch.cuda.synchronize()
    finally:
        L.check(lib.jt_set_allocator(L._ALLOCATOR[0], L._ALLOCATOR[1], None))
    assert calls["alloc"] > 10
    assert calls["free"] == calls["alloc"] and not calls["live"]
