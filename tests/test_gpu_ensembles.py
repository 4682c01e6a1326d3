"""Batched ensembles of uneven size and release time (one launch per time
chunk, per-ensemble schedules), with and without the locality sort, replayed
from a CUDA graph, and after autotuning.  Every ensemble must equal, bit for
bit, what track_particles gives for it alone (exact float32 path), and the
oracle's float32 run of the same ensemble."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle
from jaxtrace_gb300 import workloads as W

pytestmark = pytest.mark.gpu
F32 = np.float32


def same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def _grid_case():
    g = (np.arange(16) / 16).astype(F32)
    st = np.linspace(0, 1, 9).astype(F32)
    data = W.abc_snapshots(W.grid_nodes(g, g, g), st)
    f = jt.StructuredTimeSeriesField(data, st, g, g, g, "periodic")
    spec = oracle.GridSpec(data, st, g, g, g, "periodic")
    return f, spec, jt.periodic_boundary(W.UNIT), oracle.BoundarySpec(kinds=("periodic",) * 3)


def _ensembles(sizes, seed=5):
    rng = np.random.default_rng(seed)
    xs = [rng.uniform(size=(s, 3)).astype(F32) for s in sizes]
    rel = rng.uniform(0, 0.5, len(sizes))
    return xs, rel


SIZES = [1000, 0, 1, 33, 4000, 257, 3, 2048]


@pytest.mark.parametrize("sort_every", [0, 10])
def test_ensembles_match_single_runs(sort_every):
    f, spec, bc, obc = _grid_case()
    xs, rel = _ensembles(SIZES)
    T, dt = 41, 0.01
    tr = jt.create_tracker("rk4", f, bc, record_final_only=True, sort_every=sort_every, sort_bits=4)
    outs = tr.track_ensembles(xs, rel, T, dt=dt)
    single = jt.create_tracker("rk4", f, bc, record_final_only=True, sort_every=0)
    for x, t0, out in zip(xs, rel, outs):
        assert out.shape == x.shape
        if len(x) == 0:
            continue
        ref = single.track_particles(x, (t0, t0 + (T - 1) * dt), T, dt=dt).positions[-1]
        assert same(out, ref)
        times = np.linspace(t0, t0 + (T - 1) * dt, T, dtype=F32)
        o, _, _ = oracle.track(spec, obc, x, times, dt)
        assert same(out, o)


def test_ensembles_cuda_graph_replay():
    import torch
    f, spec, bc, obc = _grid_case()
    xs, rel = _ensembles(SIZES, seed=9)
    tr = jt.create_tracker("rk4", f, bc, sort_every=8, sort_bits=4)
    eager = tr.ensemble_batch(xs, rel, 33, dt=0.01).run().finals()
    b = tr.ensemble_batch(xs, rel, 33, dt=0.01).capture()
    for _ in range(3):              # replays start again from x0
        b.pos.fill_(float("nan"))
        got = b.run().finals()
        for a, c in zip(eager, got):
            assert same(a, c)
    assert b.launches >= 4
    assert b.check_status() & ~jt._lib.JT_STATUS_INDEX_WRAPPED == 0
    torch.cuda.synchronize()


def test_ensembles_on_octree_mesh_and_mixed_boundary():
    P, tets = W.kuhn_mesh(8, 0.2, 1)
    st = np.linspace(0, 1, 5).astype(F32)
    data = W.abc_snapshots(P, st)
    f = jt.OctreeFEMTimeSeriesFieldOptimized(data, st, P, tets)
    m = f.octree_mesh
    spec = oracle.MeshSpec(data, st, P, tets, m.element_bounds, m.nodes_min, m.nodes_max, m.nodes_elements,
                           m.nodes_children, m.nodes_is_leaf, max_depth=m.max_depth)
    cond = {"x": "periodic", "y": "reflective", "z": "periodic"}
    bc = jt.mixed_boundary(W.UNIT, cond)
    obc = oracle.BoundarySpec(kinds=("periodic", "reflective", "periodic"))
    xs, rel = _ensembles([300, 17, 900, 5], seed=2)
    T, dt = 21, 0.005
    outs = jt.create_tracker("rk4", f, bc, sort_every=5, sort_bits=3).track_ensembles(xs, rel, T, dt=dt)
    for x, t0, out in zip(xs, rel, outs):
        times = np.linspace(t0, t0 + (T - 1) * dt, T, dtype=F32)
        o, _, _ = oracle.track(spec, obc, x, times, dt)
        assert same(out, o)


def test_ensembles_16bit_storage_close_to_oracle():
    f, spec, bc, obc = _grid_case()
    g = (np.arange(16) / 16).astype(F32)
    st = f.times
    f16 = jt.StructuredTimeSeriesField(f.data, st, g, g, g, "periodic", storage="bf16", encoding="snapshot")
    xs, rel = _ensembles([500, 1500], seed=4)
    outs = jt.create_tracker("rk4", f16, bc, sort_every=0).track_ensembles(xs, rel, 21, dt=0.01)
    for x, t0, out in zip(xs, rel, outs):
        times = np.linspace(t0, t0 + 0.2, 21, dtype=F32)
        o, _, _ = oracle.track(spec, obc, x, times, 0.01, precision=oracle.ORC_F64)
        d = np.abs(out.astype(np.float64) - o)
        d = np.minimum(d, 1.0 - d)          # periodic distance
        assert d.max() < 5e-3               # bf16 snapshots: ~3 significant digits of velocity


def test_autotuned_batch_stays_exact(tmp_path):
    f, spec, bc, obc = _grid_case()
    xs, rel = _ensembles([20000, 3000, 70000], seed=6)
    tuner = jt.Autotuner(cache_path=str(tmp_path / "tune.json"), sample_particles=8192, sample_steps=12)
    tr = jt.create_tracker("rk4", f, bc, record_final_only=True)
    b = tr.ensemble_batch(xs, rel, 25, dt=0.01)
    res = tuner.tune_batch(b)
    assert res.block_size in (64, 128, 256) and res.sort_bits in (5, 6, 7)
    assert len(res.trials) >= 7 and (tmp_path / "tune.json").exists()
    outs = b.run().finals()
    single = jt.create_tracker("rk4", f, bc, record_final_only=True, sort_every=0)
    for x, t0, out in zip(xs, rel, outs):
        assert same(out, single.track_particles(x, (t0, t0 + 24 * 0.01), 25, dt=0.01).positions[-1])
    # a second tuner on the same cache file answers from it
    again = jt.Autotuner(cache_path=str(tmp_path / "tune.json")).tune_batch(b)
    assert (again.block_size, again.sort_every, again.sort_bits) == (res.block_size, res.sort_every, res.sort_bits)
    assert again.trials == []
