"""The hash-grid FEM mesh build (host) against the arrays JAXTrace's own
build_tetrahedral_mesh produced for the golden fixture."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle

F32 = np.float32


def test_hash_grid_matches_reference_build(golden):
    g = golden("fem")
    h = jt.FemHashGrid(g["P"], g["T4"], grid_resolution=8)
    assert h.grid_size == tuple(int(v) for v in g["grid_size"])
    assert np.array_equal(h.grid_min.view(np.uint32), g["grid_min"].view(np.uint32))
    assert np.array_equal(h.grid_cell_size.view(np.uint32), g["grid_cell_size"].view(np.uint32))
    assert np.array_equal(h.cell_elem_counts, g["cell_elem_counts"])
    assert np.array_equal(h.cell_to_elements(), g["cell_to_elements"])
    assert np.array_equal(h.element_bounds, g["element_bounds"])


def test_hash_grid_known_answer_mesh(golden):
    g = golden("fem")
    h = jt.FemHashGrid(g["ka_pts"], g["ka_conn"], grid_resolution=4)
    assert h.grid_size == (4, 4, 4)
    # the oracle on our build reproduces the module's printed example
    D = np.stack([g["ka_pts"], g["ka_pts"]])
    spec = oracle.FemSpec(D, np.array([0, 1], F32), g["ka_pts"], g["ka_conn"], h.grid_size, h.grid_min,
                          h.grid_cell_size, h.cell_to_elements(), h.element_bounds)
    out, fb = oracle.sample(spec, np.array([[0.5, 0.5, 0.5], [0.1, 0.1, 0.1]], F32), 0.0)
    assert np.allclose(out, g["ka_out"]) and fb == 1


def test_hash_grid_anisotropic_and_degenerate_inputs():
    rng = np.random.default_rng(0)
    P = (rng.random((50, 3)) * np.array([4.0, 1.0, 0.25])).astype(F32)
    T4 = rng.integers(0, 50, (40, 4)).astype(np.int32)
    h = jt.FemHashGrid(P, T4, grid_resolution=16)
    assert h.grid_size[0] > h.grid_size[1] > h.grid_size[2] >= 1
    # every element is listed in the cell holding its box's lower corner
    for e in range(len(T4)):
        c = np.clip(np.floor((h.element_bounds[e, 0] - P.min(0)) / h.cell_size64).astype(int), 0,
                    np.array(h.grid_size) - 1)
        cid = (c[0] * h.grid_size[1] + c[1]) * h.grid_size[2] + c[2]
        assert e in h.cell_elems[h.cell_start[cid]:h.cell_start[cid + 1]]
    with pytest.raises(ValueError):
        jt.FemHashGrid(P, np.array([[0, 1, 2, 99]], np.int32))
    with pytest.raises(ValueError):
        jt.FemHashGrid(P[:, :2], T4)
