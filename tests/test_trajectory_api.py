"""Trajectory container API (tracking/particles.py): indexing, accessors,
2-D slices, convergence summary and the module-level constructors, merge and
validation, checked against the reference's documented behaviour."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt

F32 = np.float32


def _traj(T=12, N=5, vel=True, seed=0):
    rng = np.random.default_rng(seed)
    pos = rng.random((T, N, 3)).astype(F32)
    v = rng.random((T, N, 3)).astype(F32) if vel else None
    return jt.Trajectory(positions=pos, times=np.linspace(0, 1, T).astype(F32), velocities=v)


def test_indexing_and_accessors():
    tr = _traj()
    one = tr[3]
    assert one.positions.shape == (1, 5, 3) and np.array_equal(one.positions[0], tr.positions[3])
    sl = tr[2:8:2]
    assert sl.T == 3 and np.array_equal(sl.times, tr.times[2:8:2]) and np.array_equal(sl.velocities,
                                                                                    tr.velocities[2:8:2])
    sub = tr[1:4, [0, 2]]
    assert sub.positions.shape == (3, 2, 3) and np.array_equal(sub.positions, tr.positions[1:4][:, [0, 2]])
    with pytest.raises(TypeError):
        tr["x"]
    p = tr.get_positions_at_time(4)
    assert np.array_equal(p, tr.positions[4]) and p is not tr.positions[4]
    with pytest.raises(IndexError):
        tr.get_positions_at_time(12)
    pp, tt = tr.get_particle_trajectory(2)
    assert np.array_equal(pp, tr.positions[:, 2]) and np.array_equal(tt, tr.times)
    with pytest.raises(IndexError):
        tr.get_particle_trajectory(-1)
    assert repr(tr).startswith("Trajectory(T=12, N=5, duration=1.000")


@pytest.mark.parametrize("plane,axis", [("xy", 2), ("XZ", 1), ("yz", 0)])
def test_extract_2d_slice(plane, axis):
    tr = _traj()
    s = tr.extract_2d_slice(plane)
    assert np.all(s.positions[:, :, axis] == 0) and np.all(s.velocities[:, :, axis] == 0)
    keep = [a for a in range(3) if a != axis]
    assert np.array_equal(s.positions[:, :, keep], tr.positions[:, :, keep])
    assert s.metadata["extracted_plane"] == plane.lower()
    with pytest.raises(ValueError):
        tr.extract_2d_slice("xx")


def test_convergence_and_copies():
    tr = _traj()
    c = tr.analyze_convergence()
    disp = np.linalg.norm(tr.positions - tr.positions[0][None], axis=2)
    assert c["status"] == "success" and c["mean_final_displacement"] == float(np.mean(disp[-1]))
    assert c["mean_max_displacement"] == float(np.mean(np.max(disp, axis=0)))
    assert _traj(T=5).analyze_convergence() == {"status": "insufficient_data", "num_timesteps": 5}
    n = tr.to_numpy()
    assert np.array_equal(n.positions, tr.positions) and n.positions is not tr.positions
    with pytest.warns(UserWarning):
        assert np.array_equal(tr.to_jax().positions, tr.positions)


def test_constructors_merge_and_validation():
    rng = np.random.default_rng(3)
    t = jt.create_trajectory_from_positions(rng.random((4, 6, 2)), tag="a")
    assert t.positions.shape == (4, 6, 3) and np.array_equal(t.times, np.arange(4, dtype=F32))
    assert np.all(t.positions[:, :, 2] == 0) and t.metadata["tag"] == "a"
    with pytest.raises(ValueError):
        jt.create_trajectory_from_positions(rng.random((4, 6, 3)), times=np.zeros(3))
    s = jt.create_single_particle_trajectory(rng.random((7, 2)), velocities=rng.random((7, 2)))
    assert s.positions.shape == (7, 1, 3) and s.velocities.shape == (7, 1, 3)
    assert s.metadata["particle_type"] == "single"
    e = jt.create_empty_trajectory(3, 4)
    assert e.positions.shape == (4, 3, 3) and e.metadata["status"] == "empty"
    a, b = _traj(T=4, N=5, seed=1), _traj(T=6, N=5, seed=2)
    m = jt.merge_trajectories([a, b], axis="time")
    assert m.T == 10 and np.array_equal(m.positions[4:], b.positions) and m.metadata["merged_count"] == 2
    c = _traj(T=4, N=2, seed=3)
    mp = jt.merge_trajectories([a, c], axis="particles")
    assert mp.N == 7 and np.array_equal(mp.positions[:, 5:], c.positions)
    with pytest.raises(ValueError):
        jt.merge_trajectories([a, b], axis="particles")
    with pytest.raises(ValueError):
        jt.merge_trajectories([a], axis="bogus") if False else jt.merge_trajectories([a, c], axis="bogus")
    ok = jt.validate_trajectory_data(a)
    assert ok["valid"] and ok["errors"] == []
    bad = _traj(T=4)
    bad.positions[1, 0, 0] = np.nan
    bad.times[:] = [0, 0.5, 0.4, 1.0]
    r = jt.validate_trajectory_data(bad)
    assert not r["valid"] and any("non-finite" in x for x in r["errors"]) and any("monoton" in x for x in r["errors"])


def test_analyze_trajectory_results():
    tr = _traj()
    stats, val = jt.analyze_trajectory_results(tr, verbose=False)
    assert val["valid"] and stats["displacement"]["mean"] == float(np.mean(tr.compute_displacement()))
    s0, s1 = np.std(tr.positions[0], axis=0), np.std(tr.positions[-1], axis=0)
    assert np.array_equal(stats["spatial"]["spread_change_percent"], (s1 / s0 - 1) * 100)
    assert stats["spatial"]["mixing_efficiency"] == 0.0


def test_open_dataset(tmp_path):
    from jaxtrace_gb300 import vtk_io as V
    rng = np.random.default_rng(1)
    P = rng.random((8, 3)).astype(F32)
    for k in range(3):
        V.write_vtu(str(tmp_path / f"s_{k}.vtu"), P, None, {"velocity": rng.random((8, 3)).astype(F32)})
    r = jt.open_dataset(str(tmp_path / "s_*.vtu"))
    assert len(r) == 3 and r.load_time_series()["velocity_data"].shape == (3, 8, 3)
    r2 = jt.open_dataset([str(tmp_path / "s_2.vtu"), str(tmp_path / "s_0.vtu")])
    assert len(r2) == 2
    (tmp_path / "a.h5").write_bytes(b"")
    with pytest.raises(ImportError, match="HDF5"):
        jt.open_dataset(str(tmp_path / "a.h5"))
    (tmp_path / "a.xyz").write_bytes(b"")
    with pytest.raises(ValueError, match="Unknown file format"):
        jt.open_dataset(str(tmp_path / "a.xyz"))
    with pytest.raises(FileNotFoundError):
        jt.open_dataset(str(tmp_path / "none_*.vtu"))
