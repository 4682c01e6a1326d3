"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
vectors and the CPU oracle.  Float32 'exact' results are compared bit for
bit; the octree path, whose reference dot product order is not pinned, to
rtol 1e-5 (the spec float32 tolerance) with exact element choice."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle
from jaxtrace_gb300 import _lib as L

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


# ---------------------------------------------------------------- sampling
@pytest.mark.parametrize("mode", ["clamp", "zero", "nan", "periodic"])
def test_structured_sampler(golden, mode):
    g = golden("structured")
    s = jt.StructuredGridSampler(g[f"{mode}_V"], g[f"{mode}_gx"], g[f"{mode}_gy"], g[f"{mode}_gz"], mode)
    assert same(s.sample(g[f"{mode}_q"]), g[f"{mode}_out"])


@pytest.mark.parametrize("ex", ["constant", "linear", "zero", "nan"])
def test_time_blend_all_nodes(golden, ex):
    g = golden("time_blend")
    f = jt.TimeSeriesField(g["data"], g["times"], np.random.default_rng(0).random((7, 3)), extrapolation=ex)
    for i, t in enumerate(g["tq"]):
        assert same(f.sample_at_time(float(t)), g[f"out_{ex}"][i]), (ex, t)


def test_nearest_field(golden):
    g = golden("nearest")
    f = jt.TimeSeriesField(g["D"], g["st"], g["nodes"])
    spec = oracle.NearestSpec(g["D"], g["st"], g["nodes"])
    for i, t in enumerate((0.0, 0.7, 2.5, 3.5)):
        out = f.sample_at_positions(g["q"], t)
        ref, _ = oracle.sample(spec, g["q"], t, t_is_f32=False)
        assert same(out, ref)
        assert np.mean(np.all(out == g["outs"][i], axis=1)) > 0.99


def test_nearest_node_search_matches_brute_force_argmin_with_ties():
    """The cell-list search (row ranges, pruned first ring, ring stop) returns
    np.argmin of the float32 squared distances, lowest index on ties: lattice
    nodes make exact ties at cell centres, faces and edges; queries sit on
    nodes, on cell faces, far outside and at random."""
    g = np.arange(9, dtype=F32) / F32(8)
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(11)
    nodes = np.concatenate([lat, rng.random((300, 3)).astype(F32)]).astype(F32)
    n = len(nodes)
    data = np.zeros((2, n, 3), dtype=F32)
    data[:, :, 0] = np.arange(n, dtype=F32)
    f = jt.TimeSeriesField(data, np.array([0.0, 1.0], dtype=F32), nodes)
    half = (np.arange(8, dtype=F32) + F32(0.5)) / F32(8)
    mids = np.stack(np.meshgrid(half, half, half, indexing="ij"), -1).reshape(-1, 3)
    faces = mids.copy()
    faces[:, 0] = np.round(faces[:, 0] * 8) / 8
    q = np.concatenate([mids, faces, lat[::7], rng.random((4000, 3)), rng.uniform(-2, 3, (500, 3)),
                        lat[::11] + F32(1e-7)]).astype(F32)
    out = f.sample_at_positions(q, 0.0)[:, 0].astype(np.int64)
    d = np.zeros((len(q), n), dtype=F32)
    for a in range(3):
        diff = (q[:, None, a] - nodes[None, :, a]).astype(F32)
        d = (d + diff * diff).astype(F32) if a else (diff * diff).astype(F32)
    ref = np.argmin(d, axis=1)
    assert np.array_equal(out, ref)


# ---------------------------------------------------------------- boundaries
def _bc(name, B):
    conc = {"x": 9, "y": 17, "z": 5}
    return {
        "periodic": lambda: jt.periodic_boundary(B),
        "reflective": lambda: jt.reflective_boundary(B),
        "clamping": lambda: jt.clamping_boundary(B),
        "absorbing": lambda: jt.absorbing_boundary_factory(B),
        "absorbing_m7": lambda: jt.absorbing_boundary_factory(B, outside_value=-7.0),
        "mixed_prc": lambda: jt.mixed_boundary(B, {"x": "periodic", "y": "reflective", "z": "clamping"}),
        "mixed_ab": lambda: jt.mixed_boundary(B, {"x": "absorbing", "z": "reflective"}),
        "inlet_xpos": lambda: jt.continuous_inlet_boundary_factory(B, "x", "positive", "grid", conc),
        "inlet_yneg": lambda: jt.continuous_inlet_boundary_factory(B, "y", "negative", "grid", conc),
        "inlet_zpos": lambda: jt.continuous_inlet_boundary_factory(B, "z", "positive", "grid", conc),
    }[name]()


@pytest.mark.parametrize("name", ["periodic", "reflective", "clamping", "absorbing", "absorbing_m7", "mixed_prc",
                                  "mixed_ab", "inlet_xpos", "inlet_yneg", "inlet_zpos"])
def test_boundaries(golden, name):
    g = golden("boundary")
    P = g["Pin"] if name.startswith("inlet") else g["P"]
    assert same(_bc(name, g["B"])(P), g[name])


# ---------------------------------------------------------------- tracking
@pytest.mark.parametrize("integ", ["rk4", "rk2", "euler"])
def test_track_grid_matches_reference(golden, integ):
    g = golden("track_grid")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    tr = jt.create_tracker(integ, f, jt.periodic_boundary(((0, 0, 0), (1, 1, 1))))
    ref = g[f"{integ}_traj"]
    traj = tr.track_particles(g["x0"], (0.0, 0.3 if integ == "rk4" else 0.2), ref.shape[0], dt=0.01)
    assert same(traj.positions, ref)
    assert traj.metadata["device_status"] == 0


def test_recording_interval_and_velocities(golden):
    g = golden("track_grid")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    tr = jt.create_tracker("rk4", f, jt.periodic_boundary(((0, 0, 0), (1, 1, 1))), record_velocities=True,
                           recording_interval=3)
    traj = tr.track_particles(g["x0"][:50], (0.0, 0.1), 11, dt=0.01)
    assert same(traj.positions, g["rec_pos"])
    assert same(traj.velocities, g["rec_vel"])


def test_track_inlet_matches_reference(golden):
    g = golden("track_inlet")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "clamp")
    bc = jt.continuous_inlet_boundary_factory(((0, 0, 0), (1, 1, 1)), "x", "positive", "grid",
                                              {"x": 16, "y": 16, "z": 16})
    traj = jt.create_tracker("rk4", f, bc).track_particles(g["x0"], (0.0, 0.6), 61, dt=0.01)
    assert same(traj.positions, g["traj"])


def test_quick_scenario(golden):
    g = golden("nearest")
    f = jt.TimeSeriesField(g["vort"], g["vt"], g["qn"])
    tr = jt.create_tracker("rk4", f, jt.reflective_boundary([[-1, -1, -1], [1, 1, 1]]))
    traj = tr.track_particles(g["seeds"], (0.0, 2.0), 101, dt=0.02)
    assert np.allclose(traj.positions, g["quick_traj"], atol=1e-6)


def test_time_chunks_and_compact_recording(golden):
    g = golden("track_grid")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    bc = jt.periodic_boundary(((0, 0, 0), (1, 1, 1)))
    ref = g["rk4_traj"]
    t1 = jt.create_tracker("rk4", f, bc, time_chunk=7).track_particles(g["x0"], (0.0, 0.3), 31, dt=0.01)
    assert same(t1.positions, ref) and t1.metadata["time_chunks"] == 5
    t2 = jt.create_tracker("rk4", f, bc, record_every=4).track_particles(g["x0"], (0.0, 0.3), 31, dt=0.01)
    assert same(t2.positions, ref[::4]) and same(t2.times, np.linspace(0, 0.3, 31, dtype=F32)[::4])
    t3 = jt.create_tracker("rk4", f, bc, record_final_only=True).track_particles(g["x0"], (0.0, 0.3), 31, dt=0.01)
    assert same(t3.positions, ref[[0, -1]])


# ---------------------------------------------------------------- octree
@pytest.mark.parametrize("opts", [dict(time_chunk=7), dict(time_chunk=5, record_every=3),
                                  dict(record_final_only=True),
                                  dict(time_chunk=4, record_velocities=True, recording_interval=2)])
def test_row_sink_streams_every_row_once_in_order(golden, opts):
    """Slabs copied on the side stream land in the same rows as the
    reference trajectory, and the sink sees every row once, in order."""
    g = golden("track_grid")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    bc = jt.periodic_boundary(((0, 0, 0), (1, 1, 1)))
    got = []

    def sink(r0, pos, vel, t):
        got.append((r0, pos.copy(), None if vel is None else vel.copy(), t.copy()))

    traj = jt.create_tracker("rk4", f, bc, row_sink=sink, **opts).track_particles(g["x0"][:64], (0.0, 0.3), 31,
                                                                                   dt=0.01)
    plain = jt.create_tracker("rk4", f, bc, **{k: v for k, v in opts.items() if k != "time_chunk"}) \
        .track_particles(g["x0"][:64], (0.0, 0.3), 31, dt=0.01)
    assert same(traj.positions, plain.positions)
    starts = np.cumsum([0] + [len(p) for _, p, _, _ in got])[:-1]
    assert [r for r, _, _, _ in got] == list(starts)
    assert same(np.concatenate([p for _, p, _, _ in got]), traj.positions)
    assert same(np.concatenate([t for _, _, _, t in got]), traj.times)
    if traj.velocities is not None:
        assert same(np.concatenate([v for _, _, v, _ in got]), traj.velocities)


def test_vtk_series_sink_writes_the_trajectory(golden, tmp_path):
    import xml.etree.ElementTree as ET
    from jaxtrace_gb300 import vtk_io
    g = golden("track_grid")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    bc = jt.periodic_boundary(((0, 0, 0), (1, 1, 1)))
    series = vtk_io.VTKTrajectorySeries(tmp_path, compress=True)
    traj = jt.create_tracker("rk4", f, bc, row_sink=series, time_chunk=10, record_every=2) \
        .track_particles(g["x0"], (0.0, 0.3), 31, dt=0.01)
    pvd = series.close()
    sets = ET.parse(pvd).getroot().findall("Collection/DataSet")
    assert len(sets) == traj.T
    for r, ds in enumerate(sets):
        d = vtk_io.read_vtk_xml(str(tmp_path / ds.get("file")))
        assert same(d["points"], traj.positions[r])
        assert np.all(d["point_data"]["Time"] == traj.times[r])
        assert float(ds.get("timestep")) == pytest.approx(float(traj.times[r]), abs=1e-6)


def _octree_field(g):
    return jt.OctreeFEMTimeSeriesFieldOptimized(g["D"], g["st"], g["P"], g["T4"], max_elements_per_leaf=32,
                                                max_depth=12)


def test_octree_sampling(golden):
    g = golden("octree")
    f = _octree_field(g)
    spec = oracle.MeshSpec(g["D"], g["st"], g["P"], g["T4"], g["element_bounds"], g["nodes_min"], g["nodes_max"],
                           g["nodes_elements"], g["nodes_children"], g["nodes_is_leaf"])
    for key, t in (("sample_t03", 0.3), ("sample_t10", 1.0)):
        out = f.sample_at_positions(g["q"], F32(t))
        ref_o, _ = oracle.sample(spec, g["q"], float(F32(t)), t_is_f32=True)
        assert same(out, ref_o)  # same float32 arithmetic as the oracle
        assert np.allclose(out, g[key], rtol=1e-5, atol=1e-6)


def test_octree_known_answer(golden):
    g = golden("octree")
    pts = g["ka_pts"]
    f = jt.OctreeFEMTimeSeriesFieldOptimized(np.stack([pts, pts]), np.array([0, 1], F32), pts, g["ka_conn"],
                                             max_elements_per_leaf=1, max_depth=5)
    out = f.sample_at_positions(np.array([[0.25, 0.25, 0.25]], F32), 0.0)
    assert np.allclose(out, g["ka_out"])


def test_octree_tracking(golden):
    g = golden("octree")
    f = _octree_field(g)
    bc = jt.mixed_boundary(((0, 0, 0), (1, 1, 1)), {"x": "periodic", "y": "reflective", "z": "periodic"})
    traj = jt.create_tracker("rk4", f, bc).track_particles(g["x0"], (0.0, 0.1), 11, dt=0.01)
    assert np.allclose(traj.positions, g["traj"], rtol=1e-5, atol=1e-6)


# ---------------------------------------------------------------- scale
def test_plain_config_bit_exact_vs_oracle():
    """The plain RK4 configuration at full size (10k particles, 32^3, 16
    snapshots, 100 steps) against the float32 oracle, bit for bit."""
    from jaxtrace_gb300 import workloads as W
    c = W.plain_rk4()
    g = c["grid"][0]
    f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "periodic")
    tr = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT), record_final_only=True)
    traj = tr.track_particles(c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"])
    spec = oracle.GridSpec(c["data"], c["times"], g, g, g, "periodic")
    times = np.linspace(0.0, 1.0, 101, dtype=F32)
    ref, _, info = oracle.track(spec, oracle.BoundarySpec(kinds=("periodic",) * 3), c["x0"], times, 0.01)
    gpu = traj.positions[-1]
    if info["wrapped_count"] == 0:
        assert same(gpu, ref)
    else:  # the oracle wraps exactly like the kernel, the reference would have raised
        assert same(gpu, ref)
        assert tr.last_status & L.JT_STATUS_INDEX_WRAPPED


def test_periodic_wrap_is_flagged():
    g = (np.arange(12) / 12).astype(F32)
    V = np.random.default_rng(0).standard_normal((12, 12, 12, 3)).astype(F32)
    s = jt.StructuredGridSampler(V, g, g, g, "periodic")
    out = s.sample(np.array([[0.5, 0.5, -6.05359673500061e-09]], F32))
    spec = oracle.GridSpec(V[None], np.zeros(1, F32), g, g, g, "periodic")
    ref, _ = oracle.sample(spec, np.array([[0.5, 0.5, -6.05359673500061e-09]], F32), 0.0)
    assert same(out, ref)


# ---------------------------------------------------------------- 16-bit storage
def _quantize(data, storage):
    """The values 16-bit storage holds, as float32: round(v/s) * s per snapshot."""
    import torch
    from jaxtrace_gb300.fields import snapshot_scales
    code = L.STORAGE_CODES[storage]
    s = snapshot_scales(data, code)
    dt = torch.bfloat16 if storage == "bf16" else torch.float16
    q = np.stack([(torch.from_numpy(data[t]) / float(s[t])).to(dt).float().numpy() * s[t] for t in range(len(data))])
    return q.astype(F32)


@pytest.mark.parametrize("storage", ["bf16", "f16"])
@pytest.mark.parametrize("mode", ["clamp", "periodic", "nan"])
def test_16bit_sampler_matches_oracle_on_quantized_values(golden, storage, mode):
    """BF16/FP16 snapshots (z-pair records) give the float32 result of the
    quantized values up to the fast path's rounding: FMA contraction and the
    cell coordinate taken as (x - x_min) * (1/dx), whose error grows with |fx|
    (queries here reach several periods outside the box).  Tolerance: 1e-5
    of the field's largest magnitude."""
    g = golden("structured")
    V, gx, gy, gz, q = (g[f"{mode}_{k}"] for k in ("V", "gx", "gy", "gz", "q"))
    s = jt.StructuredGridSampler(V, gx, gy, gz, mode, storage=storage, encoding="snapshot")
    out = s.sample(q)
    Vq = _quantize(V[None], storage)
    ref, _ = oracle.sample(oracle.GridSpec(Vq, np.zeros(1, F32), gx, gy, gz, mode), q, 0.0)
    assert np.allclose(out, ref, rtol=0, atol=1e-5 * float(np.abs(Vq).max()), equal_nan=True)


@pytest.mark.parametrize("stage", [False, True])
@pytest.mark.parametrize("storage", ["bf16", "f16"])
def test_16bit_tracking_matches_oracle_on_quantized_values(storage, stage):
    """Pair gathers (stage False) and float16 stage fields (stage True) on
    BF16/FP16 snapshots (the per-snapshot-scale encoding) against the float32
    oracle on the quantized values.  Stage fields round the blended values'
    residuals from their quad's offset to float16 and interpolate them in
    float16, so they get 3e-4 absolute."""
    from jaxtrace_gb300 import workloads as W
    c = W.precision_case(n=20, n_snap=6, seeds=(16, 16, 16), lattice=16, n_steps=25, dt=0.01)
    g = c["grid"][0]
    f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "clamp", storage=storage, encoding="snapshot")
    bc = jt.continuous_inlet_boundary_factory(W.UNIT, "x", "positive", "grid", c["concentrations"])
    traj = jt.create_tracker("rk4", f, bc, record_final_only=True, stage_fields=stage).track_particles(
        c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"])
    spec = oracle.GridSpec(_quantize(c["data"], storage), c["times"], g, g, g, "clamp")
    lat = np.linspace(F32(0), F32(1), 16, dtype=F32)
    times = np.linspace(0.0, 0.25, 26, dtype=F32)
    ref, _, _ = oracle.track(spec, oracle.BoundarySpec(inlet_axis=0, inlet_positive=True, lattices=[lat, lat]),
                             c["x0"], times, 0.01)
    atol = 3e-4 if stage else 1e-5
    close = np.all(np.isclose(traj.positions[-1], ref, rtol=1e-4, atol=atol), axis=1)
    assert close.mean() > 0.995  # an inlet snap can flip on a last-bit difference


@pytest.mark.parametrize("sort_every", [0, 7])
@pytest.mark.parametrize("mode", ["periodic", "clamp", "zero"])
def test_stage_fields_float32_bit_identical_to_pair_gathers(mode, sort_every):
    """Blending every node once per stage time (the reference's order) gives
    the same bits as blending the gathered corners, through launches that
    wrap the stage-slot ring (stage_chunk 5, 23 steps)."""
    from jaxtrace_gb300 import workloads as W
    n = 12
    g = (np.arange(n) / n).astype(F32) if mode == "periodic" else np.linspace(0, 1, n).astype(F32)
    st = np.linspace(0, 0.2, 5).astype(F32)
    data = W.abc_snapshots(W.grid_nodes(g, g, g), st)
    f = jt.StructuredTimeSeriesField(data, st, g, g, g, mode)
    bc = jt.periodic_boundary(W.UNIT) if mode == "periodic" else jt.reflective_boundary(W.UNIT)
    x0 = np.random.default_rng(2).random((3000, 3)).astype(F32)
    outs = []
    for stage in (False, True):
        tr = jt.create_tracker("rk4", f, bc, stage_fields=stage, stage_chunk=5, sort_every=sort_every)
        outs.append(tr.track_particles(x0, (0.0, 0.23), 24, dt=0.01).positions)
    assert same(outs[0], outs[1])
    spec = oracle.GridSpec(data, st, g, g, g, mode)
    obc = oracle.BoundarySpec(kinds=(("periodic",) if mode == "periodic" else ("reflective",)) * 3)
    ref, _, _ = oracle.track(spec, obc, x0, np.linspace(0.0, 0.23, 24, dtype=F32), 0.01)
    assert same(outs[1][-1], ref)


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_stage_field_overlap_and_ring_depth_give_the_same_bits(storage):
    """Blending the next chunk on the side stream (a ring twice as deep) gives
    the same trajectory as blending each chunk before its launch, for chunk
    sizes that make launches wrap the ring and cut at re-sorts."""
    from jaxtrace_gb300 import workloads as W
    c = W.precision_case(n=20, n_snap=6, seeds=(16, 16, 16), lattice=16, n_steps=41, dt=0.01)
    g = c["grid"][0]
    f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "clamp", storage=storage)
    bc = jt.continuous_inlet_boundary_factory(W.UNIT, "x", "positive", "grid", c["concentrations"])
    outs = []
    for overlap, chunk in ((False, 5), (True, 5), (True, 3), (False, 32)):
        tr = jt.create_tracker("rk4", f, bc, stage_overlap=overlap, stage_chunk=chunk, sort_every=7)
        outs.append(tr.track_particles(c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"]).positions)
    for o in outs[1:]:
        assert same(outs[0], o)


def test_stage_fields_with_velocity_recording_fall_back_to_pairs():
    from jaxtrace_gb300 import workloads as W
    g = (np.arange(10) / 10).astype(F32)
    st = np.linspace(0, 1, 3).astype(F32)
    f = jt.StructuredTimeSeriesField(W.abc_snapshots(W.grid_nodes(g, g, g), st), st, g, g, g, "periodic")
    x0 = np.random.default_rng(1).random((500, 3)).astype(F32)
    a = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT), record_velocities=True).track_particles(
        x0, (0.0, 0.1), 11, dt=0.01)
    b = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT), record_velocities=True,
                          stage_fields=False).track_particles(x0, (0.0, 0.1), 11, dt=0.01)
    assert same(a.positions, b.positions) and same(a.velocities, b.velocities)


# ---------------------------------------------------------------- locality sort
def test_cell_sort_is_a_permutation_in_morton_order():
    import ctypes as C
    import torch
    n = 100_003
    x = torch.rand((n, 3), device="cuda")
    g = L.SortGrid()
    g.origin[:] = [0.0, 0.0, 0.0]
    g.inv_cell[:] = [16.0, 16.0, 16.0]
    g.bits = 4
    lib = L.load()
    ws = torch.empty(int(lib.jt_cell_sort_workspace_bytes(n, 4)), dtype=torch.uint8, device="cuda")
    out = torch.empty_like(x)
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    L.check(lib.jt_cell_sort(C.byref(g), n, L.ptr(x), None, None, L.ptr(out), None, L.ptr(ids), L.ptr(ws),
                             ws.numel(), L.stream_ptr()))
    ids_h = ids.cpu().numpy()
    assert np.array_equal(np.sort(ids_h), np.arange(n))
    assert torch.equal(out, x[ids.long()])
    c = np.clip(np.floor(out.cpu().numpy() * 16), 0, 15).astype(np.int64)

    def spread(v):
        r = np.zeros_like(v)
        for b in range(4):
            r |= ((v >> b) & 1) << (3 * b)
        return r
    key = spread(c[:, 0]) | (spread(c[:, 1]) << 1) | (spread(c[:, 2]) << 2)
    assert np.all(np.diff(key) >= 0)
    back = torch.empty_like(x)
    L.check(lib.jt_unpermute(n, L.ptr(out), L.ptr(ids), L.ptr(back), L.stream_ptr()))
    assert torch.equal(back, x)


def test_sorted_tracking_is_bit_identical(golden):
    g = golden("track_grid")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    bc = jt.periodic_boundary(((0, 0, 0), (1, 1, 1)))
    ref = g["rk4_traj"]
    tr = jt.create_tracker("rk4", f, bc, sort_every=4, record_velocities=True)
    traj = tr.track_particles(g["x0"], (0.0, 0.3), 31, dt=0.01)
    assert same(traj.positions, ref)
    assert traj.metadata["time_chunks"] == 8
    plain = jt.create_tracker("rk4", f, bc, sort_every=0, record_velocities=True).track_particles(
        g["x0"], (0.0, 0.3), 31, dt=0.01)
    assert same(traj.velocities, plain.velocities)


def test_sorted_compensated_precision_matches_unsorted():
    from jaxtrace_gb300 import workloads as W
    c = W.precision_case(n=24, n_snap=8, seeds=(24, 24, 24), lattice=24, n_steps=200, dt=0.005)
    g = c["grid"][0]
    bc = jt.continuous_inlet_boundary_factory(W.UNIT, "x", "positive", "grid", c["concentrations"])
    outs = []
    for se in (0, 16):
        f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "clamp", storage="bf16")
        tr = jt.create_tracker("rk4", f, bc, record_final_only=True, sort_every=se)
        outs.append(tr.track_particles(c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"]).positions[-1])
    # FMA contraction is the same per particle whatever its slot
    assert same(outs[0], outs[1])

