"""The hash-grid FEM mesh build (host) against the arrays JAXTrace's own
build_tetrahedral_mesh produced for the golden fixture."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle

F32 = np.float32


def test_hash_grid_matches_reference_build(golden):
    g = golden("fem")
    h = jt.FemHashGrid(g["P"], g["T4"], grid_resolution=8, build="host")
    assert h.grid_size == tuple(int(v) for v in g["grid_size"])
    assert np.array_equal(h.grid_min.view(np.uint32), g["grid_min"].view(np.uint32))
    assert np.array_equal(h.grid_cell_size.view(np.uint32), g["grid_cell_size"].view(np.uint32))
    assert np.array_equal(h.cell_elem_counts, g["cell_elem_counts"])
    assert np.array_equal(h.cell_to_elements(), g["cell_to_elements"])
    assert np.array_equal(h.element_bounds, g["element_bounds"])


def test_hash_grid_known_answer_mesh(golden):
    g = golden("fem")
    h = jt.FemHashGrid(g["ka_pts"], g["ka_conn"], grid_resolution=4, build="host")
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
    h = jt.FemHashGrid(P, T4, grid_resolution=16, build="host")
    assert h.grid_size[0] > h.grid_size[1] > h.grid_size[2] >= 1
    # every element is listed in the cell holding its box's lower corner
    for e in range(len(T4)):
        c = np.clip(np.floor((h.element_bounds[e, 0] - P.min(0)) / h.cell_size64).astype(int), 0,
                    np.array(h.grid_size) - 1)
        cid = (c[0] * h.grid_size[1] + c[1]) * h.grid_size[2] + c[2]
        assert e in h.cell_elems[h.cell_start[cid]:h.cell_start[cid + 1]]
    with pytest.raises(ValueError):
        jt.FemHashGrid(P, np.array([[0, 1, 2, 99]], np.int32), build="host")
    with pytest.raises(ValueError):
        jt.FemHashGrid(P[:, :2], T4, build="host")


def test_sub_cell_lists_hold_every_candidate_the_cell_scan_can_pick():
    """Every element of the query's hash-cell list whose box holds the query
    is on the query's sub-cell list (sub-cell index computed with the
    kernel's float32 arithmetic), and sub lists stay ascending, so the first
    containing element found is the one the reference's cell scan finds."""
    from jaxtrace_gb300 import workloads as W
    P, T4 = W.kuhn_mesh(10, 0.2, 3)
    h = jt.FemHashGrid(P, T4, 12, sub_div=4, build="host")
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


def _numpy_lists(P, T4, grid_size, bmin, cell64, S):
    """The hash-grid cell and sub-cell lists restated with NumPy array
    operations (the checker of the library's host builder)."""
    V = P[T4]
    emin, emax = V.min(axis=1), V.max(axis=1)
    hi = np.array(grid_size) - 1
    cmin = np.clip(np.floor((emin - bmin) / cell64).astype(int), 0, hi)
    cmax = np.clip(np.floor((emax - bmin) / cell64).astype(int), 0, hi)
    ext = cmax - cmin + 1
    count = ext.prod(axis=1)
    elem = np.repeat(np.arange(len(T4), dtype=np.int64), count)
    first = np.repeat(np.cumsum(count) - count, count)
    r = np.arange(len(elem), dtype=np.int64) - first
    ez, ey = np.repeat(ext[:, 2], count), np.repeat(ext[:, 1], count)
    k = np.repeat(cmin[:, 2], count) + r % ez
    j = np.repeat(cmin[:, 1], count) + (r // ez) % ey
    i = np.repeat(cmin[:, 0], count) + r // (ez * ey)
    cell = (i * grid_size[1] + j) * grid_size[2] + k
    n_cells = int(np.prod(grid_size))
    cell_start = np.concatenate([[0], np.cumsum(np.bincount(cell, minlength=n_cells))]).astype(np.int32)
    cell_elems = elem[np.argsort(cell, kind="stable")].astype(np.int32)
    sub = cell64 / S
    eps = 1e-3 * sub + 4e-7 * max(float(np.abs(P).max()), 1.0)
    cidx = np.stack([i, j, k], axis=1)
    lo = bmin.astype(np.float64) + cidx * cell64
    slo = np.clip(np.floor((emin[elem].astype(np.float64) - eps - lo) / sub), 0, S - 1).astype(np.int64)
    shi = np.clip(np.floor((emax[elem].astype(np.float64) + eps - lo) / sub), 0, S - 1).astype(np.int64)
    sext = shi - slo + 1
    scount = sext.prod(axis=1)
    el = np.repeat(elem, scount)
    first = np.repeat(np.cumsum(scount) - scount, scount)
    r = np.arange(len(el), dtype=np.int64) - first
    ez, ey = np.repeat(sext[:, 2], scount), np.repeat(sext[:, 1], scount)
    sz = np.repeat(slo[:, 2], scount) + r % ez
    sy = np.repeat(slo[:, 1], scount) + (r // ez) % ey
    sx = np.repeat(slo[:, 0], scount) + r // (ez * ey)
    sid = np.repeat(cell, scount) * S ** 3 + (sx * S + sy) * S + sz
    sub_start = np.concatenate([[0], np.cumsum(np.bincount(sid, minlength=n_cells * S ** 3))]).astype(np.int32)
    sub_elems = el[np.argsort(sid, kind="stable")].astype(np.int32)
    return cell_start, cell_elems, sub_start, sub_elems


@pytest.mark.parametrize("res,sub_div", [(6, 4), (10, 3), (7, 2)])
def test_host_builder_lists_equal_the_array_restatement(res, sub_div):
    from jaxtrace_gb300 import workloads as W
    P, T4 = W.kuhn_mesh(9, 0.2, res)
    P = (P * np.array([1.0, 0.6, 1.7], dtype=np.float32)).astype(np.float32)   # aspect-ratio cell counts
    h = jt.FemHashGrid(P, T4, res, sub_div=sub_div, build="host")
    bmin = P.min(axis=0)
    ref = _numpy_lists(P, T4, h.grid_size, bmin, h.cell_size64, sub_div)
    for ours, theirs in zip((h.cell_start, h.cell_elems, h.sub_start, h.sub_elems), ref):
        assert np.array_equal(ours, theirs)
    assert h.max_elems_per_cell == int(np.diff(h.cell_start).max())
