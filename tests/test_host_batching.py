"""Host logic of ensemble batching and of the autotuner (no GPU)."""
import json

import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import autotune as A
from jaxtrace_gb300 import workloads as W

F32 = np.float32


def _tracker():
    g = (np.arange(8) / 8).astype(F32)
    st = np.linspace(0, 1, 3).astype(F32)
    f = jt.StructuredTimeSeriesField(W.abc_snapshots(W.grid_nodes(g, g, g), st), st, g, g, g, "periodic")
    return jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT))


def test_ensemble_batch_validates_before_touching_the_device():
    tr = _tracker()
    x = np.zeros((4, 3), F32)
    with pytest.raises(ValueError):
        tr.ensemble_batch([x, x], [0.0], 11, dt=0.01)          # one release time short
    with pytest.raises(ValueError):
        tr.ensemble_batch([], [], 11, dt=0.01)
    with pytest.raises(ValueError):
        tr.ensemble_batch([x], [0.0], 1, dt=0.01)              # no step
    with pytest.raises(ValueError):
        tr.ensemble_batch([x], [0.0], 11)                      # neither dt nor duration
    with pytest.raises(ValueError):
        tr.ensemble_batch([np.zeros((4, 4), F32)], [0.0], 11, dt=0.01)
    # dt=None needs one float32 step shared by all ensembles' grids
    with pytest.raises(ValueError):
        tr.ensemble_batch([x, x], [0.0, 0.3], 11, duration=0.1)


def test_ensemble_schedules_follow_each_release_time():
    from jaxtrace_gb300 import _lib as L
    from jaxtrace_gb300.schedule import build_schedule, single_blend
    st = np.linspace(0, 1, 32).astype(F32)
    rel = np.random.default_rng(7).uniform(0, 0.5, 4)
    rows = []
    for t0 in rel:
        times = np.linspace(t0, t0 + 400 * 0.005, 401, dtype=F32)
        s = build_schedule(times, 0.005, L.JT_RK4, st, semantics="jax")
        assert s.shape[0] == 4 * 400
        # stage 1 of step 0 blends the snapshots bracketing the ensemble's own t0
        b = single_blend(st, F32(times[0]), semantics="jax")[0]
        assert s[0]["pair"] == b["pair"] and s[0]["wa"] == b["wa"] and s[0]["wb"] == b["wb"]
        rows.append(s)
    assert not np.array_equal(rows[0], rows[1])


class _Opts:
    block_size, sort_every, sort_bits = 0, None, None


class _FakeTracker:
    options = _Opts()


def test_autotuner_coordinate_descent_picks_fastest():
    cost = {128: 3.0, 256: 2.0, 64: 4.0}
    every = {0: 5.0, 20: 1.5, 50: 1.0, 100: 1.2}
    bits = {7: 1.0, 6: 0.5, 5: 0.8}
    tr = _FakeTracker()

    def sample():
        o = tr.options
        return cost[o.block_size] * every[o.sort_every] * (bits[o.sort_bits] if o.sort_every else 1.0)

    res = A.Autotuner(cache_path="").search(tr, sample)
    assert (res.block_size, res.sort_every, res.sort_bits) == (256, 50, 6)
    assert res.ms == pytest.approx(2.0 * 1.0 * 0.5)
    assert len(res.trials) == len(A.BLOCK_SIZES) + len(A.SORT_EVERY) + len(A.SORT_BITS)
    # the tracker's own options are restored after the search
    assert (tr.options.block_size, tr.options.sort_every, tr.options.sort_bits) == (0, None, None)


def test_autotuner_skips_cell_size_without_sorting(tmp_path):
    tr = _FakeTracker()
    res = A.Autotuner(cache_path="").search(tr, lambda: 1.0 + 0.1 * (tr.options.sort_every or 0))
    assert res.sort_every == 0
    assert len(res.trials) == len(A.BLOCK_SIZES) + len(A.SORT_EVERY)


def test_autotuner_cache_file_roundtrip(tmp_path):
    p = tmp_path / "t.json"
    t = A.Autotuner(cache_path=str(p))
    t.cache["k"] = {"block_size": 128, "sort_every": 50, "sort_bits": 6, "ms": 1.0}
    t._save()
    assert json.loads(p.read_text())["k"]["sort_bits"] == 6
    assert A.Autotuner(cache_path=str(p)).cache["k"]["block_size"] == 128


def test_stage_field_numbers_share_equal_consecutive_entries():
    from jaxtrace_gb300 import _lib as L
    from jaxtrace_gb300.schedule import build_schedule
    from jaxtrace_gb300.tracker import _stage_numbers
    times = np.linspace(0, 2, 1001, dtype=F32)
    sched = build_schedule(times[:-1], F32(0.002), L.JT_RK4, np.linspace(0, 2, 64).astype(F32))
    every = sched.reshape(-1, 4)[:, :3].reshape(-1)
    uid = _stage_numbers(every)
    assert uid[0] == 0 and np.all(np.diff(uid) >= 0) and np.all(np.diff(uid) <= 1)
    # equal numbers <=> equal bytes, and only between neighbours
    same = np.diff(uid) == 0
    raw = every.view(np.uint8).reshape(len(every), -1)
    assert np.array_equal(same, np.all(raw[1:] == raw[:-1], axis=1))
    # t + h of a step and t of the next coincide on most steps of this float32 time grid
    assert 0.6 < same.mean() * 3 < 0.9
    # t and t + h/2 never coincide here (they bracket different times)
    assert not np.any(same[0::3])


@pytest.mark.parametrize("overlap", [False, True])
@pytest.mark.parametrize("chunk", [1, 2, 5, 32])
def test_stage_field_ring_holds_every_field_of_each_launch(chunk, overlap):
    """Simulate the slot ring: before each tracking launch, every stage field
    of its steps sits in its slot, for launches cut by chunks and sort
    intervals, with coincident and constant-extrapolation entries.  With
    overlap, the next launch's fields are written while the current launch
    runs: none of those writes may land in a slot the current launch reads."""
    from jaxtrace_gb300.tracker import _stage_numbers, _stage_plan
    from jaxtrace_gb300.schedule import BLEND_DTYPE
    rng = np.random.default_rng(5)
    n_steps = 97
    ent = np.zeros(3 * n_steps, dtype=BLEND_DTYPE)
    ent["wa"] = rng.uniform(size=len(ent)).astype(F32)
    for i in range(1, len(ent)):                      # coincidences of both kinds, and long constant runs
        if (i % 3 == 0 and rng.uniform() < 0.7) or i > 250:
            ent[i] = ent[i - 1]
    uid = _stage_numbers(ent)
    slots = (6 if overlap else 3) * chunk
    ring = np.full(slots, -1)

    def stop_of(s, sort_every):
        stop = n_steps
        if sort_every:
            stop = min(stop, (s // sort_every + 1) * sort_every)
        return min(stop, s + chunk)

    def write(runs):
        for lo, run in runs:
            assert (lo % slots) + run <= slots
            ring[np.arange(lo, lo + run) % slots] = np.arange(lo, lo + run)

    for sort_every in (0, 7, 10):
        s = 0
        ring[:] = -1
        ready = -1
        while s < n_steps:
            stop = stop_of(s, sort_every)
            runs, ready = _stage_plan(uid, s, stop, ready, slots)
            write(runs)
            need = uid[3 * s:3 * stop]
            assert np.array_equal(ring[need % slots], need)
            if overlap and stop < n_steps:        # prefetch while [s, stop) is tracked
                runs, ready = _stage_plan(uid, stop, stop_of(stop, sort_every), ready, slots)
                write(runs)
                assert np.array_equal(ring[need % slots], need)
            s = stop
    with pytest.raises(ValueError):
        _stage_plan(np.arange(30), 0, 10, -1, 9)   # 30 numbers cannot fit 9 slots


def test_stage_chunk_fits_a_quarter_of_free_memory():
    from jaxtrace_gb300.tracker import _stage_chunk
    nodes = 128 ** 3
    # 128^3 float16 quads: 3 x 67 MB per step; 100 GB free holds the full 32-step ring
    assert _stage_chunk(32, 1000, nodes, 32, 100 << 30) == 32
    # 8 GB free: 2 GB for the ring -> 10 steps
    assert _stage_chunk(32, 1000, nodes, 32, 8 << 30) == 10
    # too little room for 4 steps: gather snapshot pairs instead
    assert _stage_chunk(32, 1000, nodes, 32, 2 << 30) == 0
    # short runs keep a chunk of their own length, and a requested short chunk is kept
    assert _stage_chunk(32, 3, nodes, 16, 100 << 30) == 3
    assert _stage_chunk(32, 1, 8, 16, 1 << 20) == 1
    assert _stage_chunk(3, 1000, nodes, 32, 100 << 30) == 3
