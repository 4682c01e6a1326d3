"""The device build of the FEM hash grid (jt_fem_grid_build_device) against
the host build, which is pinned to the reference's tables
(build_tetrahedral_mesh, fields/fem_interpolator.py:36-143): cell lists,
sub-cell lists and the per-tetrahedron records bit for bit."""
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


def _same(P, T4, res, sub_div):
    h = jt.FemHashGrid(P, T4, res, sub_div=sub_div, build="host")
    d = jt.FemHashGrid(P, T4, res, sub_div=sub_div, build="device")
    assert d.dev is not None
    assert d.sub_div == h.sub_div and d.max_elems_per_cell == h.max_elems_per_cell
    for k in ("cell_start", "cell_elems", "sub_start", "sub_elems", "cell_elem_counts"):
        assert np.array_equal(getattr(d, k), getattr(h, k)), k
    for k in ("tet_box", "tet_geom", "element_bounds"):
        assert np.array_equal(getattr(d, k).view(np.int32), getattr(h, k).view(np.int32)), k
    return h, d


def test_device_hash_grid_matches_reference_golden(golden):
    g = golden("fem")
    h, d = _same(g["P"], g["T4"], 8, 4)
    assert np.array_equal(d.cell_to_elements(), h.cell_to_elements())
    _same(g["ka_pts"], g["ka_conn"], 4, 4)


@pytest.mark.parametrize("res,sub_div", [(16, 0), (16, 2), (16, 4), (32, 4), (8, 16)])
def test_device_hash_grid_matches_host_build(res, sub_div):
    P, T4 = W.kuhn_mesh(12)[:2]
    _same(P, T4, res, sub_div)


def test_device_hash_grid_on_a_shuffled_mesh():
    P, T4 = W.kuhn_mesh(10)[:2]
    _same(P, T4[np.random.default_rng(9).permutation(len(T4))], 12, 4)


def test_grids_beyond_the_device_build_are_refused_before_allocating():
    """128^3 cells x 16^3 sub-cells (8.6e9 lists) exceed the device build's
    three-level scan: "device" says so before it allocates anything."""
    P, T4 = W.kuhn_mesh(4)[:2]
    with pytest.raises(NotImplementedError, match="exceeds"):
        jt.FemHashGrid(P, T4, 128, sub_div=16, build="device")


def test_device_build_with_more_lists_than_one_scan_level():
    """32^3 cells x 10^3 sub-cells: 32.8M sub-cell lists, beyond the
    two-level scan (2^22), built on the device identical to the host."""
    P, T4 = W.kuhn_mesh(10)[:2]
    _same(P, T4, 32, 10)


def test_fem_field_runs_on_the_device_build():
    c = W.fem_case(n=8, n_snap=4, n_particles=2000, n_steps=50)
    bc = jt.mixed_boundary(W.UNIT, c["conditions"])
    out = []
    for b in ("host", "device"):
        f = jt.FEMTimeSeriesField(c["data"], c["times"], c["points"], c["tets"], grid_build=b)
        tr = jt.create_tracker("rk4", f, bc, record_final_only=True)
        out.append(tr.track_particles(c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"]).positions)
    assert np.array_equal(out[0], out[1])
