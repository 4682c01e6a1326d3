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
