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


def test_sub_cell_lists_hold_every_candidate_the_cell_scan_can_pick():
    """Every element of the query's hash-cell list whose box holds the query
    is on the query's sub-cell list (sub-cell index computed with the
    kernel's float32 arithmetic), and sub lists stay ascending, so the first
    containing element found is the one the reference's cell scan finds."""
    from jaxtrace_gb300 import workloads as W
    P, T4 = W.kuhn_mesh(10, 0.2, 3)
    h = jt.FemHashGrid(P, T4, 12, sub_div=4)
    S = h.sub_div
    rng = np.random.default_rng(5)
    q = np.concatenate([rng.random((4000, 3)), rng.uniform(-0.2, 1.2, (500, 3)),
                        P[rng.integers(0, len(P), 500)]]).astype(F32)
    gmin, cs, gs = h.grid_min, h.grid_cell_size, np.array(h.grid_size)
    eb = h.element_bounds
    for p in q:
        c = np.clip(np.floor((p - gmin) / cs), 0, gs - 1).astype(int)        # float32 ops, as the kernel
        cell = (c[0] * gs[1] + c[1]) * gs[2] + c[2]
        lo = (c.astype(F32) * cs + gmin).astype(F32)
        f = np.floor((p - lo) * (F32(S) / cs))
        sc = np.clip(f, 0, S - 1).astype(int)
        sid = cell * S ** 3 + (sc[0] * S + sc[1]) * S + sc[2]
        sub = h.sub_elems[h.sub_start[sid]:h.sub_start[sid + 1]]
        assert np.all(np.diff(sub) > 0)
        cand = h.cell_elems[h.cell_start[cell]:h.cell_start[cell + 1]]
        holds = cand[np.all((eb[cand, 0] <= p) & (p <= eb[cand, 1]), axis=1)]
        assert np.isin(holds, sub).all()
