"""Affine-tile 16-bit snapshots on the GPU: the stage blend of
jt_stage_tile_fields against a host restatement, field values through the
tracking kernel against the float64 oracle, and tracked positions against
the float64 oracle next to the per-snapshot-scale encoding."""
import ctypes as C

import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle
from jaxtrace_gb300 import _lib as L
from jaxtrace_gb300 import fields as F
from jaxtrace_gb300 import workloads as W
from jaxtrace_gb300.schedule import BLEND_DTYPE

pytestmark = pytest.mark.gpu
F32 = np.float32
K = L.JT_TILE + 1


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    L.load()
    yield


def _entries(rows):
    e = np.zeros(len(rows), dtype=BLEND_DTYPE)
    for i, (pair, form, wa, wb) in enumerate(rows):
        e[i]["pair"], e[i]["form"], e[i]["wa"], e[i]["wb"], e[i]["sa"], e[i]["sb"] = pair, form, wa, wb, 1.0, 1.0
    return e


def decode_offset_quads(buf, scales, n, N):
    """Host decode of JT_STORE_STAGE_F16 offset quads: (n, N, 4, 3) values of
    the nodes (j,k), (j,k1), (j1,k), (j1,k1) of every node's quad."""
    w = buf.view(np.uint32).reshape(n, N, 8)
    h = buf.view(np.float16).reshape(n, N, 16).astype(np.float64)
    ox = w[..., 6].view(np.float32).astype(np.float64)
    oy = w[..., 7].view(np.float32).astype(np.float64)
    oz = (w[..., 7] & 0xFFFF).astype(np.uint16).view(np.float16).astype(np.float64)
    v = np.empty((n, N, 4, 3))
    for c in range(4):
        v[..., c, 0] = ox + h[..., 2 * c]
        v[..., c, 1] = oy + h[..., 2 * c + 1]
    v[..., 0, 2], v[..., 1, 2] = oz + h[..., 8], oz + h[..., 9]
    v[..., 2, 2], v[..., 3, 2] = oz + h[..., 10], oz + h[..., 11]
    return v * np.asarray(scales, np.float64)[:, None, None, None]


def _quad_nodes(dims, periodic):
    """Grid node ids of (j,k), (j,k1), (j1,k), (j1,k1) of every node's quad."""
    nx, ny, nz = dims
    nxt = lambda n: (np.arange(n) + 1) % n if periodic else np.minimum(np.arange(n) + 1, n - 1)  # noqa: E731
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    j1, k1 = nxt(ny)[j], nxt(nz)[k]
    ids = [(i * ny + a) * nz + b for a, b in ((j, k), (j, k1), (j1, k), (j1, k1))]
    return np.stack([x.reshape(-1) for x in ids], axis=1)


@pytest.mark.parametrize("storage", ["bf16", "f16"])
@pytest.mark.parametrize("mode", ["clamp", "periodic"])
def test_stage_tile_fields_match_host_blend(storage, mode):
    """jt_stage_tile_fields rebuilds each node's quad values from the tile
    that holds its cell (base plus residual), blends them per entry form and
    writes offset quads: decoded, they equal the blended snapshot values to
    the storage's and the stage's 16-bit rounding of the residuals."""
    import torch
    rng = np.random.default_rng(5)
    dims = (10, 7, 13)
    N = int(np.prod(dims))
    gs = [np.linspace(0, 1, n, dtype=F32) for n in dims]
    data = rng.normal(size=(4, N, 3)).astype(F32)
    f = jt.StructuredTimeSeriesField(data, np.linspace(0, 1, 4, dtype=F32), *gs, mode, storage=storage,
                                     encoding="tile")
    src = f.tile_field()
    res = f._tiles["res"].float().cpu().numpy()[..., :3]
    ent = _entries([(0, L.JT_BLEND_WEIGHTED, 0.75, 0.25), (2, L.JT_BLEND_WEIGHTED, 0.125, 0.875),
                    (1, L.JT_BLEND_LERP_FWD, 0.0, -0.5), (2, L.JT_BLEND_SAME_B, 0.5, 0.5),
                    (0, L.JT_BLEND_WEIGHTED, 1.0, 0.0)])
    n = len(ent)
    scales = np.array([4.0, 4.0, 8.0, 4.0, 4.0], F32)
    ent_d = torch.from_numpy(ent.view(np.int32).reshape(-1, 8).copy()).cuda()
    sc_d = torch.from_numpy(scales).cuda()
    out = torch.zeros(n * N * 16, dtype=torch.float16, device="cuda")
    L.check(L.load().jt_stage_tile_fields(C.byref(src), L.ptr(ent_d), L.ptr(sc_d), n, L.ptr(out), L.stream_ptr()))
    got = decode_offset_quads(out.cpu().numpy(), scales, n, N)
    ids = _quad_nodes(dims, mode == "periodic")
    D = data.astype(np.float64)
    ulp = 2.0 ** -8 if storage == "bf16" else 2.0 ** -11
    for j, e in enumerate(ent):
        p, form, wa, wb = int(e["pair"]), int(e["form"]), float(e["wa"]), float(e["wb"])
        A, B = D[p][ids], D[p + 1][ids]
        if form == L.JT_BLEND_WEIGHTED:
            want = wa * A + wb * B
        elif form == L.JT_BLEND_LERP_FWD:
            want = A + wb * (B - A)
        else:
            want = wa * B + wb * B
        spread = np.abs(want - want.mean(axis=1, keepdims=True)).max()
        tol = 3 * ulp * np.abs(res).max() + 2.0 ** -10 * (spread + 0.02 * np.abs(want).max()) + 1e-6
        assert np.abs(got[j] - want).max() <= tol, (j, np.abs(got[j] - want).max(), tol)


def _velocity_through_euler(field, x0, t0):
    """v(x0, t0) read back from one Euler step of dt = 1 with no boundary:
    x1 = x0 + v, so v = x1 - x0 up to one float32 rounding of x1."""
    tr = jt.create_tracker("euler", field, jt.no_boundary(), record_final_only=True)
    traj = tr.track_particles(x0, (t0, t0 + 1.0), 2, dt=1.0)
    return traj.positions[-1].astype(np.float64) - x0.astype(np.float64)


@pytest.mark.parametrize("mode", ["clamp", "periodic"])
def test_tile_field_values_against_float64(mode):
    """Velocities the tracking kernel gathers from affine-tile stage fields,
    against the float64 oracle's trilinear time-blended field: the error is
    the 16-bit rounding of residuals (noise-sized), 10 times below the
    per-snapshot-scale encoding's rounding of the values."""
    c = W.precision_case(n=48, n_snap=8, seeds=(2, 2, 2), lattice=2)
    g = c["grid"][0]
    rng = np.random.default_rng(3)
    x0 = rng.uniform(0.0, 1.0, (20000, 3)).astype(F32)
    t0 = 0.37
    spec = oracle.GridSpec(c["data"], c["times"], g, g, g, mode)
    ref, _ = oracle.sample(spec, x0, np.float32(t0), precision=oracle.ORC_F64)
    errs = {}
    for storage in ("bf16", "f16"):
        for enc in ("tile", "snapshot"):
            f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, mode, storage=storage, encoding=enc)
            v = _velocity_through_euler(f, x0, t0)
            errs[(storage, enc)] = np.abs(v - ref).max()
    vmax = np.abs(ref).max()
    assert errs[("bf16", "tile")] < 4e-4 * vmax
    assert errs[("f16", "tile")] < 1e-4 * vmax
    assert errs[("bf16", "tile")] * 5 < errs[("bf16", "snapshot")]
    assert errs[("f16", "tile")] * 2 < errs[("f16", "snapshot")]


def test_tile_tracking_against_float64():
    """RK4 with the continuous inlet on a reduced precision configuration:
    tile-encoded 16-bit storage stays closer to the float64 oracle than the
    per-snapshot scale, with a median error near float32's."""
    c = W.precision_case(n=64, n_snap=16, seeds=(24, 24, 24), lattice=24, n_steps=300, dt=0.002)
    g = c["grid"][0]
    bc = jt.continuous_inlet_boundary_factory(W.UNIT, "x", "positive", "grid", c["concentrations"])
    spec = oracle.GridSpec(c["data"], c["times"], g, g, g, "clamp")
    lat = np.linspace(F32(0), F32(1), 24, dtype=F32)
    obc = oracle.BoundarySpec(inlet_axis=0, inlet_positive=True, lattices=[lat, lat])
    times = np.linspace(c["time_span"][0], c["time_span"][1], c["n_timesteps"], dtype=F32)
    ref, _, _ = oracle.track(spec, obc, c["x0"], times, c["dt"], precision=oracle.ORC_F64)
    med = {}
    for enc in ("tile", "snapshot"):
        f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "clamp", storage="bf16", encoding=enc)
        tr = jt.create_tracker("rk4", f, bc, record_final_only=True, stage_chunk=8)
        fin = tr.track_particles(c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"]).positions[-1]
        rel = np.linalg.norm(fin - ref, axis=1) / np.linalg.norm(ref, axis=1)
        med[enc] = float(np.median(rel))
    assert med["tile"] < 1e-5
    assert med["tile"] * 5 < med["snapshot"]


def test_tile_chunking_and_overlap_give_identical_bits():
    c = W.precision_case(n=32, n_snap=8, seeds=(16, 16, 16), lattice=16, n_steps=60, dt=0.002)
    g = c["grid"][0]
    bc = jt.continuous_inlet_boundary_factory(W.UNIT, "x", "positive", "grid", c["concentrations"])
    f = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "clamp", storage="f16", encoding="tile")
    outs = []
    for kw in (dict(stage_chunk=32), dict(stage_chunk=5, stage_overlap=False), dict(stage_chunk=7, sort_every=13)):
        tr = jt.create_tracker("rk4", f, bc, record_final_only=True, **kw)
        outs.append(tr.track_particles(c["x0"], c["time_span"], c["n_timesteps"], dt=c["dt"]).positions[-1])
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_tile_field_gathering_paths_read_float32_pairs():
    """Paths that gather snapshot pairs (here: velocity recording) read the
    tile field's float32 pairs, so they match a float32 field run in the
    same compensated arithmetic bit for bit."""
    c = W.plain_rk4(n_particles=512, n=16, n_snap=6)
    g = c["grid"][0]
    bc = jt.periodic_boundary(W.UNIT)
    ft = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "periodic", storage="bf16", encoding="tile")
    f32 = jt.StructuredTimeSeriesField(c["data"], c["times"], g, g, g, "periodic")
    a = jt.create_tracker("rk4", ft, bc, record_velocities=True).track_particles(c["x0"], (0.0, 0.1), 11, dt=0.01)
    b = jt.create_tracker("rk4", f32, bc, record_velocities=True, precision="compensated").track_particles(
        c["x0"], (0.0, 0.1), 11, dt=0.01)
    assert np.array_equal(a.positions, b.positions)
    assert np.array_equal(a.velocities, b.velocities)
