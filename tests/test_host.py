"""Host-side logic of the GPU path: C-ABI surface, octree build, time-blend
schedules, boundary descriptors and tracker options.  No GPU needed."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import _lib as L
from jaxtrace_gb300 import schedule as S

ROOT = Path(__file__).resolve().parents[1]
F32 = np.float32


def header_functions():
    text = (ROOT / "include" / "jaxtrace_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void|size_t|const char\*)\s+(jt_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_header_symbol():
    lib = L.load()
    names = header_functions()
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n
    assert lib.jt_abi_version() == L.ABI_VERSION == 5
    # the scratch allocator hook: both functions or neither
    with pytest.raises(ValueError, match="alloc and free"):
        L.check(lib.jt_set_allocator(L.ALLOC_FN(lambda n, s, c: None), L.FREE_FN(), None))
    assert lib.jt_set_allocator(L.ALLOC_FN(), L.FREE_FN(), None) == 0
    L.use_torch_allocator(lib)


def test_struct_layouts_match():
    assert L.struct_sizes() == [C.sizeof(s) for s in L.STRUCTS]
    assert L.BLEND_DTYPE.itemsize == C.sizeof(L.Blend)
    assert L.OCTREE_NODE_DTYPE.itemsize == C.sizeof(L.OctreeNode)


def test_errors_are_mapped():
    lib = L.load()
    with pytest.raises(ValueError, match="field is NULL"):
        L.check(lib.jt_track(None, None, None, None))
    b = L.Boundary()
    b.axis_kind[0] = 9
    with pytest.raises(ValueError, match="unknown boundary kind"):
        L.check(lib.jt_boundary_apply(C.byref(b), None, 0, None))


def test_octree_build_matches_reference(golden):
    g = golden("octree")
    m = jt.OctreeMesh(g["P"], g["T4"], 32, 12, build="host")
    assert len(m.nodes) == g["nodes_min"].shape[0]
    assert np.array_equal(m.nodes_min, g["nodes_min"])
    assert np.array_equal(m.nodes_max, g["nodes_max"])
    assert np.array_equal(m.nodes_children, g["nodes_children"])
    assert np.array_equal(m.nodes_is_leaf, g["nodes_is_leaf"])
    assert np.array_equal(m.nodes_elem_counts, g["nodes_elem_counts"])
    assert np.array_equal(m.nodes_elements, g["nodes_elements"])
    assert np.array_equal(m.element_bounds, g["element_bounds"])
    # node centres used by the traversal
    assert np.array_equal(m.nodes["c"], (g["nodes_min"] + g["nodes_max"]) / F32(2.0))


def test_octree_build_known_answer_mesh(golden):
    g = golden("octree")
    m = jt.OctreeMesh(g["ka_pts"], g["ka_conn"], 1, 5, build="host")
    assert m.info.n_leaves >= 2


def test_octree_rejects_bad_connectivity():
    with pytest.raises(ValueError, match="outside"):
        jt.OctreeMesh(np.zeros((4, 3), F32), np.array([[0, 1, 2, 9]], np.int32), build="host")


@pytest.mark.parametrize("ex", ["constant", "linear", "zero", "nan"])
def test_schedule_blend_matches_reference(golden, ex):
    """The host schedule entries applied as the kernel applies them reproduce
    TimeSeriesField.sample_at_time bit for bit."""
    g = golden("time_blend")
    data, times = g["data"], g["times"]
    for i, t in enumerate(g["tq"]):
        e = S.blend_numpy(times, float(t), "linear", ex)
        e = np.array([e], dtype=L.BLEND_DTYPE)[0]
        p = int(e["pair"])
        A = data[p]
        B = data[p + 1] if len(times) > 1 else data[p]
        got = S.blend_nodes(e, A, B)
        ref = g[f"out_{ex}"][i]
        assert np.array_equal(got, ref, equal_nan=True), (ex, t)


def test_schedule_stage_times_rk4():
    times = np.linspace(0.0, 1.0, 11, dtype=F32)
    sch = S.build_schedule(times, 0.1, L.JT_RK4, np.linspace(0, 1, 4, dtype=F32))
    assert sch.shape == (40,)
    assert sch.dtype == L.BLEND_DTYPE
    # last stage of the final step sits at the last snapshot
    assert sch[4 * 9 + 2]["pair"] == 2


def test_bounds_forms():
    b = jt.boundary._ensure_bounds_shape([0, 1, 0, 2, 0, 3])
    assert b.tolist() == [[0, 0, 0], [1, 2, 3]]
    b = jt.boundary._ensure_bounds_shape([[0, 1], [0, 2], [0, 3]])
    assert b.tolist() == [[0, 0, 0], [1, 2, 3]]
    # 2-D forms put z = 0 on both sides, which the reference's own check
    # (boundary.py:83-84) rejects as min >= max
    with pytest.raises(ValueError):
        jt.boundary._ensure_bounds_shape([0, 1, 0, 2])
    with pytest.raises(ValueError):
        jt.boundary._ensure_bounds_shape([[1, 1, 1], [0, 0, 0]])


def test_inlet_descriptor():
    bc = jt.continuous_inlet_boundary_factory(((0, 0, 0), (1, 1, 1)), "x", "positive", "grid",
                                              {"x": 4, "y": 8, "z": 16})
    assert bc.__name__ == "_continuous_inlet_bc"
    assert [len(c) for c in bc.inlet["coords"]] == [8, 16]
    assert bc.inlet["nudge"] == F32(0) + F32(0.001) * (F32(1) - F32(0))
    with pytest.raises(NotImplementedError):
        jt.continuous_inlet_boundary_factory(((0, 0, 0), (1, 1, 1)))


def test_tracker_options_and_factory_errors():
    o = jt.TrackerOptions()
    assert o.estimate_batch_size(1_000_000, 1001) == 100_000 // 64 * 1 or o.estimate_batch_size(1_000_000, 1001) > 0
    assert jt.TrackerOptions(batch_size=5000).estimate_batch_size(10, 10) == 5000
    with pytest.raises(TypeError):
        jt.TrackerOptions(not_an_option=1)
    field = jt.StructuredGridSampler(np.zeros((2, 2, 2, 3), F32), [0, 1], [0, 1], [0, 1])
    with pytest.raises(ValueError, match="Unknown integrator"):
        jt.create_tracker("rk5", field, jt.no_boundary())
    with pytest.raises(TypeError):
        jt.create_tracker("rk4", lambda p, t: p, jt.no_boundary())
    with pytest.raises(TypeError):
        jt.create_tracker("rk4", field, lambda x: x)
    tr = jt.create_tracker("rk4", field, jt.periodic_boundary([[0, 0, 0], [1, 1, 1]]))
    assert tr._code == L.JT_RK4


def test_estimate_batch_size_matches_reference_rule():
    # tracker.py:142-153: halve from min(N, max_batch_size) until under max_memory_gb
    o = jt.TrackerOptions(max_memory_gb=1.0)
    bs = o.estimate_batch_size(1_000_000, 1001)
    from jaxtrace_gb300.tracker import _estimate_memory_usage
    assert _estimate_memory_usage(bs, 1001) <= 1.0
    assert _estimate_memory_usage(bs * 2, 1001) > 1.0 or bs * 2 > 100_000


def test_new_entry_points_validate_before_touching_the_device():
    """Argument checks of the entry points added beside the reference API
    return their error codes without a GPU."""
    lib = L.load()
    # stage fields need a regular-grid field and a known output storage
    with pytest.raises(ValueError, match="regular-grid"):
        L.check(lib.jt_stage_fields(None, None, None, 3, L.JT_STORE_STAGE_F32, None, None))
    g = L.GridField()
    g.nx = g.ny = g.nz = 4
    g.pair_stride = 64
    g.n_pairs = 1
    g.pairs = 256                    # never dereferenced: rejected first
    f = L.Field(kind=L.JT_FIELD_GRID, grid=C.pointer(g))
    with pytest.raises(ValueError, match="out_storage"):
        L.check(lib.jt_stage_fields(C.byref(f), C.c_void_p(256), None, 3, 7, C.c_void_p(256), None))
    with pytest.raises(ValueError, match="out_scales"):
        g.storage = L.JT_STORE_BF16
        L.check(lib.jt_stage_fields(C.byref(f), C.c_void_p(256), None, 3, L.JT_STORE_STAGE_F16, C.c_void_p(256), None))
    with pytest.raises(NotImplementedError, match="float32 stage fields"):
        L.check(lib.jt_stage_fields(C.byref(f), C.c_void_p(256), None, 3, L.JT_STORE_STAGE_F32, C.c_void_p(256), None))
    assert lib.jt_stage_fields(C.byref(f), None, None, 0, L.JT_STORE_STAGE_F32, None, None) == 0
    # grid shapes the kernels index safely: axes of at most 2^24 nodes, < 2^31 nodes in all
    g.storage = L.JT_STORE_F32
    for shape in ((1 << 24) + 1, 1, 1), (2048, 2048, 1024), (0, 4, 4):
        g.nx, g.ny, g.nz = shape
        g.pair_stride = max(1, shape[0] * shape[1] * shape[2])
        with pytest.raises(ValueError, match="grid"):
            L.check(lib.jt_stage_fields(C.byref(f), C.c_void_p(256), None, 3, L.JT_STORE_STAGE_F32, C.c_void_p(256),
                                        None))
    g.nx = g.ny = g.nz = 4
    g.pair_stride = 64
    # adjoint workspace: three float4 accumulators per step and node
    assert lib.jt_adjoint_workspace_bytes(1000, 50) == 3 * 50 * 1000 * 16
    assert lib.jt_adjoint_workspace_bytes(1000, 65) == 0
    # tracking launch parameters
    p = L.TrackParams()
    p.integrator, p.n_particles, p.step_end = L.JT_RK4, 10, 5
    p.schedule, p.pos = 16, 16
    p.block_size = 96
    bc = L.Boundary()
    g.storage = L.JT_STORE_F32
    with pytest.raises(ValueError, match="block_size"):
        L.check(lib.jt_track(C.byref(f), C.byref(bc), C.byref(p), None))
    # 256-bit records: pairs and stage outputs 32-byte aligned, float32-quad slots of an even stride
    with pytest.raises(ValueError, match="32-byte aligned"):
        L.check(lib.jt_stage_fields(C.byref(f), C.c_void_p(256), None, 3, L.JT_STORE_STAGE_F32Q, C.c_void_p(272),
                                    None))
    g.pairs = 272
    with pytest.raises(ValueError, match="32-byte aligned"):
        L.check(lib.jt_track(C.byref(f), C.byref(bc), C.byref(p), None))
    g.pairs, g.storage, g.pair_stride = 256, L.JT_STORE_STAGE_F32Q, 65
    with pytest.raises(ValueError, match="even pair_stride"):
        L.check(lib.jt_track(C.byref(f), C.byref(bc), C.byref(p), None))
    g.storage, g.pair_stride = L.JT_STORE_F32, 64
    # stage fields track without velocity recording (the host gathers pairs for it)
    p.block_size = 0
    p.traj, p.vel, p.record_every = 16, 16, 1
    for st in (L.JT_STORE_STAGE_F32, L.JT_STORE_STAGE_F32Q, L.JT_STORE_STAGE_F16):
        g.storage = st
        with pytest.raises(NotImplementedError, match="velocities"):
            L.check(lib.jt_track(C.byref(f), C.byref(bc), C.byref(p), None))
    p.traj, p.vel, p.record_every, p.block_size = None, None, 0, 96
    g.storage = L.JT_STORE_F32
    # FEM hash-grid descriptors
    h = L.FemField()
    ff = L.Field(kind=L.JT_FIELD_FEM, fem=C.pointer(h))
    with pytest.raises(ValueError, match="FEM field"):
        L.check(lib.jt_track(C.byref(ff), C.byref(bc), C.byref(p), None))


@pytest.mark.parametrize("n", [0, 1, 2, 5, 8])
def test_sph_pair_records_layout(n):
    """Particles 2k and 2k+1 share a row {x0, x1, y0, y1, z0, z1, m0, m1};
    an odd count pads the last row with zeros; unit masses by default."""
    import torch
    from jaxtrace_gb300.density import pair_records
    pos = torch.arange(3 * n, dtype=torch.float32).reshape(n, 3)
    m = torch.arange(n, dtype=torch.float32) + 100
    for masses, want_m in ((m, m), (None, torch.ones(n))):
        rec = pair_records(pos, masses)
        assert rec.shape == ((n + 1) // 2, 8) and rec.dtype == torch.float32 and rec.is_contiguous()
        for j in range(n):
            row, lane = rec[j // 2], j % 2
            assert [float(row[2 * c + lane]) for c in range(3)] == pos[j].tolist()
            assert float(row[6 + lane]) == float(want_m[j])
        if n % 2:
            assert rec[-1, 1::2].tolist() == [0.0] * 4


def test_sph_record_layouts_are_checked_before_launch():
    """jt_sph_density accepts record layouts 0, 1 and 2 only, and the packed
    ones only with a uniform smoothing length (their kernels read no h)."""
    lib = L.load()
    p = L.SphParams()
    p.dims, p.kernel = 3, L.JT_SPH_CUBIC
    p.n_particles, p.n_queries = 4, 4
    p.radius, p.h_const = 0.1, 0.05
    p.grid.bits = 3
    p.particles = p.cell_end = p.queries = p.out = 256      # never dereferenced: rejected first
    p.packed = 3
    with pytest.raises(ValueError, match="packed"):
        L.check(lib.jt_sph_density(C.byref(p), None))
    p.h = 256
    for packed in (1, 2):
        p.packed = packed
        with pytest.raises(NotImplementedError, match="uniform smoothing length"):
            L.check(lib.jt_sph_density(C.byref(p), None))


def test_tensor_positions_are_shaped_as_arrays_are():
    """Tensor inputs (kept on their device) get the checks and the 2-D
    padding of array inputs, with the same values and messages."""
    import torch
    from jaxtrace_gb300.fields import ensure_positions_shape, ensure_positions_tensor
    rng = np.random.default_rng(3)
    for a in (rng.uniform(0, 1, (7, 3)), rng.uniform(0, 1, (7, 2)), rng.uniform(0, 1, 3),
              rng.uniform(0, 1, (5, 3)).astype(np.float32)):
        got = ensure_positions_tensor(torch.from_numpy(a))
        assert got.dtype == torch.float32 and got.is_contiguous()
        assert np.array_equal(got.numpy(), ensure_positions_shape(a))
    for bad, msg in ((np.zeros((4, 4)), "2 or 3 columns"), (np.zeros((2, 2, 3)), "2D array")):
        with pytest.raises(ValueError, match=msg):
            ensure_positions_tensor(torch.from_numpy(bad))
