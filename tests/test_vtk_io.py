"""VTK XML unstructured-grid ingest (no VTK library): every DataArray
encoding the writer produces reads back bit for bit, parallel files append
their pieces, and time series follow the reference reader's file rules
(io/vtk_reader.py:496-545, :558-604, :697-765)."""
import numpy as np
import pytest

from jaxtrace_gb300 import vtk_io as V
from jaxtrace_gb300 import workloads as W

F32 = np.float32


def _mesh():
    P, T4 = W.kuhn_mesh(3, 0.2, 4)
    return P.astype(F32), T4.astype(np.int32)


@pytest.mark.parametrize("encoding,compress,header", [("appended", False, "UInt64"), ("appended", True, "UInt32"),
                                                      ("binary", False, "UInt32"), ("binary", True, "UInt64"),
                                                      ("ascii", False, "UInt64")])
def test_vtu_round_trip(tmp_path, encoding, compress, header):
    P, T4 = _mesh()
    rng = np.random.default_rng(1)
    vel = rng.normal(size=(len(P), 3)).astype(F32)
    pres = rng.normal(size=len(P)).astype(np.float64)
    f = tmp_path / "a.vtu"
    V.write_vtu(str(f), P, T4, {"velocity": vel, "p": pres}, encoding=encoding, compress=compress, header=header)
    d = V.read_vtk_xml(str(f))
    assert np.array_equal(d["points"], P)
    assert np.array_equal(d["point_data"]["velocity"], vel)
    assert np.array_equal(d["point_data"]["p"], pres)
    assert np.array_equal(d["cells"]["connectivity"].reshape(-1, 4), T4)
    assert np.all(d["cells"]["types"] == V.VTK_TETRA)


def test_pvtu_appends_pieces(tmp_path):
    P, T4 = _mesh()
    half = len(P) // 2
    v = np.arange(len(P) * 3, dtype=F32).reshape(-1, 3)
    V.write_vtu(str(tmp_path / "p0.vtu"), P[:half], None, {"U": v[:half]})
    V.write_vtu(str(tmp_path / "p1.vtu"), P[half:], None, {"U": v[half:]})
    V.write_pvtu(str(tmp_path / "s.pvtu"), ["p0.vtu", "p1.vtu"], {"U": ("Float32", 3)})
    d = V.read_vtk_xml(str(tmp_path / "s.pvtu"))
    assert np.array_equal(d["points"], P) and np.array_equal(d["point_data"]["U"], v)


def test_time_series_order_field_detection_and_tetrahedra(tmp_path):
    P, T4 = _mesh()
    rng = np.random.default_rng(2)
    frames = [rng.normal(size=(len(P), 2)).astype(F32) for _ in range(12)]
    for k, fr in enumerate(frames):                  # written out of order; 2-D velocities
        V.write_vtu(str(tmp_path / f"case_{k}.vtu"), P, T4, {"Velocity": fr, "T": fr[:, 0]})
    (tmp_path / "notes.txt").write_text("x")
    r = V.VTKUnstructuredTimeSeriesReader(str(tmp_path / "case_*.vtu"), max_time_steps=10)
    assert [p.split("/")[-1] for p in r.time_files] == [f"case_{k}.vtu" for k in range(2, 12)]
    d = r.load_time_series()
    assert d["velocity_data"].shape == (10, len(P), 3) and d["velocity_data"].dtype == F32
    assert np.array_equal(d["velocity_data"][:, :, :2], np.stack(frames[2:]))
    assert np.all(d["velocity_data"][:, :, 2] == 0)
    assert np.array_equal(d["times"], np.arange(10, dtype=F32))
    assert d["velocity_field_name"] == "Velocity" and np.array_equal(d["positions"], P)
    assert np.array_equal(r.tetrahedra(), T4)
    with pytest.raises(ValueError, match="Velocity field not found"):
        V.VTKUnstructuredTimeSeriesReader(str(tmp_path / "case_1.vtu"))._field_name({"T": None})
    # .pvtu files shadow the .vtu of the same series
    V.write_pvtu(str(tmp_path / "case_0.pvtu"), ["case_0.vtu"], {"Velocity": ("Float32", 2)})
    r2 = V.VTKUnstructuredTimeSeriesReader(str(tmp_path / "case_*"))
    assert len(r2) == 1 and r2.time_files[0].endswith(".pvtu")


def test_missing_files_raise(tmp_path):
    with pytest.raises(ValueError, match="No VTK files"):
        V.VTKUnstructuredTimeSeriesReader(str(tmp_path / "*.vtu"))


def test_trajectory_export_matches_the_reference_layout(tmp_path):
    """export_to_vtk writes the reference's arrays (particles.py:448-539),
    restated here as its per-point loop."""
    import jaxtrace_gb300 as jt
    rng = np.random.default_rng(6)
    T, N = 5, 7
    pos = rng.random((T, N, 3)).astype(F32)
    times = np.array([0.0, 0.1, 0.25, 0.3, 0.7], dtype=F32)
    tr = jt.Trajectory(positions=pos, times=times)
    f = tmp_path / "traj.vtu"
    tr.export_to_vtk(str(f), time_indices=[0, 2, 4])
    d = V.read_vtk_xml(str(f))
    vel, tm, pid = [], [], []
    for t in (0, 2, 4):
        for p in range(N):
            if t > 0:
                dt = times[t] - times[t - 1]
                vel.append((pos[t, p] - pos[t - 1, p]) / dt)
            else:
                vel.append(np.zeros(3, F32))
            tm.append(times[t])
            pid.append(p)
    vel = np.array(vel, dtype=F32)
    assert np.array_equal(d["points"], pos[[0, 2, 4]].reshape(-1, 3))
    assert np.array_equal(d["point_data"]["Velocity"], vel)
    assert np.array_equal(d["point_data"]["Time"], np.array(tm, F32))
    assert np.array_equal(d["point_data"]["ParticleID"], np.array(pid, np.int32))
    assert np.array_equal(d["point_data"]["Speed"], np.linalg.norm(vel, axis=1).astype(F32))
    assert np.all(d["cells"]["types"] == V.VTK_VERTEX) and len(d["cells"]["types"]) == 3 * N


def test_trajectory_writer_points_and_lines(tmp_path):
    """VTKTrajectoryWriter's .vtp files hold the reference's arrays
    (io/vtk_writer.py:84-300), restated here as its loops."""
    rng = np.random.default_rng(8)
    T, N = 40, 9            # T > 8 rows: the path-length sums are pairwise
    pos = rng.random((T, N, 3)).astype(F32)
    times = np.linspace(0.0, 1.0, T).astype(F32)
    w = V.VTKTrajectoryWriter(tmp_path / "out")
    speed = rng.random((T, N)).astype(F32)
    tag = rng.random(N).astype(F32)
    with pytest.warns(UserWarning, match="bad"):
        f = w.write_trajectory_points(pos, times, particle_data={"speed": speed, "tag": tag,
                                                                 "bad": np.zeros(3)}, time_subset=slice(2, 30, 3))
    d = V.read_vtk_xml(f)
    rows = np.arange(T)[2:30:3]
    assert np.array_equal(d["points"], pos[rows].reshape(-1, 3))
    pd = d["point_data"]
    assert np.array_equal(pd["Time"], np.repeat(times[rows], N))
    assert np.array_equal(pd["ParticleID"], np.tile(np.arange(N, dtype=F32), len(rows)))
    assert np.array_equal(pd["TimeStep"], np.repeat(np.arange(len(rows), dtype=F32), N))
    assert np.array_equal(pd["speed"], speed[rows].ravel()) and np.array_equal(pd["tag"], np.tile(tag, len(rows)))
    assert "bad" not in pd
    v = d["cells"]["verts"]
    assert np.array_equal(v["connectivity"], np.arange(len(rows) * N))
    assert np.array_equal(v["offsets"], np.arange(1, len(rows) * N + 1))

    f = w.write_trajectory_lines(pos, times, max_particles=4)
    d = V.read_vtk_xml(f)
    idx = np.linspace(0, N - 1, 4, dtype=int)
    sel = pos[:, idx, :]
    ref_len = np.zeros(4, dtype=F32)
    conn = []
    for i in range(4):
        ref_len[i] = np.sum(np.linalg.norm(np.diff(sel[:, i, :], axis=0), axis=1))
        conn += [t * 4 + i for t in range(T)]
    assert np.array_equal(d["points"], sel.reshape(-1, 3))
    assert np.array_equal(d["cells"]["lines"]["connectivity"], np.array(conn))
    assert np.array_equal(d["cells"]["lines"]["offsets"], T * np.arange(1, 5))
    assert np.array_equal(d["cell_data"]["PathLength"], ref_len)
    assert np.array_equal(d["point_data"]["ParticleID"], np.tile(idx.astype(F32), T))
    assert np.array_equal(d["point_data"]["Time"], np.repeat(times, 4))


@pytest.mark.parametrize("binary", [True, False])
@pytest.mark.parametrize("layout", ["classic", "5.1"])
def test_legacy_vtk_round_trip(tmp_path, binary, layout):
    """Legacy .vtk (vtkUnstructuredGridReader's format, io/vtk_reader.py:633)
    in ASCII and big-endian binary, both cell layouts, SCALARS, VECTORS and
    FIELD arrays."""
    rng = np.random.default_rng(2)
    P = rng.random((30, 3)).astype(F32)
    T4 = rng.integers(0, 30, size=(12, 4))
    vel = rng.normal(size=(30, 3)).astype(F32)
    p = rng.random(30).astype(F32)
    six = rng.random((30, 6)).astype(F32)
    ids = np.arange(30, dtype=np.int32)
    f = tmp_path / "mesh.vtk"
    V.write_vtk_legacy(str(f), P, T4, {"velocity": vel, "p": p, "tensor": six, "id": ids}, binary=binary,
                       layout=layout)
    d = V.read_vtk_xml(str(f))
    assert np.array_equal(d["points"], P)
    assert np.array_equal(d["cells"]["connectivity"], T4.reshape(-1))
    assert np.array_equal(d["cells"]["offsets"], 4 * np.arange(1, 13))
    assert np.all(d["cells"]["types"] == V.VTK_TETRA)
    pd = d["point_data"]
    assert np.array_equal(pd["velocity"], vel) and np.array_equal(pd["p"], p)
    assert np.array_equal(pd["tensor"], six) and np.array_equal(pd["id"], ids)


def test_legacy_vtk_skips_metadata_blocks(tmp_path):
    f = tmp_path / "m.vtk"
    f.write_text("# vtk DataFile Version 5.1\nt\nASCII\nDATASET UNSTRUCTURED_GRID\n"
                 "POINTS 2 float\n0 0 0 1 1 1\nMETADATA\nINFORMATION 0\n\n"
                 "CELLS 2 1\nOFFSETS vtktypeint64\n0 1\nCONNECTIVITY vtktypeint64\n0\n"
                 "CELL_TYPES 1\n1\nPOINT_DATA 2\nVECTORS U float\n1 2 3 4 5 6\nMETADATA\nINFORMATION 0\n\n")
    d = V.read_vtk_xml(str(f))
    assert np.array_equal(d["point_data"]["U"], np.array([[1, 2, 3], [4, 5, 6]], F32))
    assert np.array_equal(d["cells"]["offsets"], [1]) and np.array_equal(d["cells"]["types"], [1])


def test_fields_from_vtk_files(tmp_path):
    """create_field_from_vtk / create_time_series_from_vtk_files
    (fields/__init__.py:114-207, fields/time_series.py:606-628)."""
    import jaxtrace_gb300 as jt
    rng = np.random.default_rng(4)
    P = rng.random((20, 3)).astype(F32)
    U = rng.normal(size=(3, 20, 3)).astype(F32)
    for k in range(3):
        V.write_vtu(str(tmp_path / f"flow_{k}.vtu"), P, None, {"velocity": U[k]})
    f = jt.create_field_from_vtk(str(tmp_path / "flow_*.vtu"))
    assert isinstance(f, jt.TimeSeriesField) and np.array_equal(f.data, U)
    assert np.array_equal(f.times, np.arange(3, dtype=F32)) and np.array_equal(f.positions, P)
    d = jt.create_field_from_vtk(str(tmp_path))
    assert np.array_equal(d.data, U)
    one = jt.create_field_from_vtk(str(tmp_path / "flow_1.vtu"))
    assert one.data.shape == (1, 20, 3) and np.array_equal(one.data[0], U[1])
    g = jt.create_time_series_from_vtk_files(str(tmp_path / "flow_*.vtu"), velocity_field_name="U",
                                             max_time_steps=2)
    assert np.array_equal(g.data, U[1:])
    assert jt.TimeVaryingField is jt.TimeSeriesField
    with pytest.raises(FileNotFoundError):
        jt.create_field_from_vtk(str(tmp_path / "nothing_*.vtu"))


def test_legacy_vtk_time_series(tmp_path):
    """A directory or a pattern of legacy .vtk files reads as a time series
    (the reader falls back to .vtk when there is no .pvtu/.vtu file)."""
    import jaxtrace_gb300 as jt
    rng = np.random.default_rng(8)
    P = rng.random((15, 3)).astype(F32)
    T4 = rng.integers(0, 15, size=(6, 4))
    U = rng.normal(size=(3, 15, 3)).astype(F32)
    d = tmp_path / "legacy"
    d.mkdir()
    for k in range(3):
        V.write_vtk_legacy(str(d / f"step_{k}.vtk"), P, T4, {"velocity": U[k]}, binary=bool(k % 2))
    for spec in (str(d), str(d / "step_*.vtk")):
        f = jt.create_field_from_vtk(spec)
        assert isinstance(f, jt.TimeSeriesField) and np.array_equal(f.data, U)
        assert np.array_equal(f.positions, P)
