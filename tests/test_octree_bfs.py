"""The breadth-first copy of the octree that the mesh kernels descend
(fields.breadth_first_descent, jt_mesh_field.desc/dtab) makes the same moves
as the node records (…optimized.py:278-302): checked on the CPU by running
both descents over random points, in and around the mesh, for trees that
stop at leaves, at max_depth, and at internal nodes whose octant is empty."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import fields as F
from jaxtrace_gb300 import workloads as W


def _dfs(nodes, p, max_depth):
    node = 0
    for _ in range(max_depth):
        if nodes["is_leaf"][node]:
            break
        c = nodes["c"][node]
        o = int(p[0] >= c[0]) + 2 * int(p[1] >= c[1]) + 4 * int(p[2] >= c[2])
        ch = int(nodes["children"][node][o])
        if ch < 0:
            break
        node = ch
    return int(nodes["elem_offset"][node]), int(nodes["elem_count"][node])


def _bfs(desc, dtab, p, max_depth):
    node = 0
    for _ in range(max_depth):
        w = int(desc[node, 3].view(np.uint32))
        m = w & 0xFF
        if m == 0:
            break
        c = desc[node, :3].view(np.float32)
        o = int(p[0] >= c[0]) + 2 * int(p[1] >= c[1]) + 4 * int(p[2] >= c[2])
        if not (m >> o) & 1:
            break
        node = (w >> 8) + bin(m & ((1 << o) - 1)).count("1")
    return int(dtab[node, 0]), int(dtab[node, 1])


@pytest.mark.parametrize("n,mpl,depth", [(6, 32, 12), (10, 4, 12), (10, 1, 3), (8, 2, 5)])
def test_breadth_first_descent_makes_the_same_moves(n, mpl, depth):
    P, T4 = W.kuhn_mesh(n, 0.2, 1)
    m = jt.OctreeMesh(P, T4, mpl, depth, build="host")
    desc, dtab = F.breadth_first_descent(m.nodes)
    assert desc.shape == (len(m.nodes), 4) and dtab.shape == (len(m.nodes), 2)
    rng = np.random.default_rng(n * 100 + mpl)
    q = np.concatenate([rng.uniform(-0.2, 1.2, (3000, 3)),
                        m.nodes["c"][rng.integers(0, len(m.nodes), 1000)]]).astype(np.float32)
    for p in q:
        assert _dfs(m.nodes, p, depth) == _bfs(desc, dtab, p, depth)


def test_auto_sub_div_follows_the_element_size():
    """fields.auto_sub_div: sub-cells about a sixth of the median element box,
    1..16, lowered while the estimated list entries exceed the budget."""
    P, T4 = W.kuhn_mesh(64, 0.2, 1)
    size = P.max(axis=0) - P.min(axis=0)
    assert F.auto_sub_div(P, T4, size / 32) == 10            # the FEM configuration
    assert F.auto_sub_div(P, T4, size / 256) == 1            # cells already finer than elements
    assert F.auto_sub_div(P, T4, size / 4) == 16             # capped
    assert F.auto_sub_div(P, T4, size / 32, max_entries=10 ** 8) < 10
    assert F.auto_sub_div(P, T4[:0], size / 32) == 1
