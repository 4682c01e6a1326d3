"""The VTK time-series reader against the reference reader's own logic.

tests/golden/vtk_reader.npz holds, per scenario, the files of a series
(points and point-data arrays) and what the reference's
VTKUnstructuredTimeSeriesReader (io/vtk_reader.py:426-940) returned for them
when it ran with the VTK library replaced by the stand-in oracle/vtkshim:
the files it picked and their order, the velocity array it took, the
padded (T, N, 3) velocities, positions, times, bounds and grid info, or the
error it raised.  Here the same files are written with this repository's
writers and read back by jaxtrace_gb300.vtk_io, which parses the files
itself.
"""
import importlib.util
import json
import os
from pathlib import Path

import numpy as np
import pytest

from jaxtrace_gb300 import vtk_io as V

GOLDEN = Path(__file__).parent / "golden"
Z = np.load(GOLDEN / "vtk_reader.npz")
MANIFEST = json.loads(str(Z["manifest"]))


def _writer():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.write_vtk_scenario


def _scenario(rec):
    """The scenario's files rebuilt from the fixture arrays."""
    tag, files = rec["tag"], []
    for i, f in enumerate(rec["files"]):
        g = {"name": f["name"], "kind": f["kind"], "pieces": f["pieces"]}
        if f["kind"] != "txt":
            g["points"] = Z[f"{tag}_f{i}_points"]
            g["arrays"] = [(n, Z[f"{tag}_f{i}_{n}"]) for n in f["arrays"]]
        files.append(g)
    return {"tag": tag, "files": files}


@pytest.mark.parametrize("rec", MANIFEST, ids=[r["tag"] for r in MANIFEST])
def test_reader_matches_reference(tmp_path, rec):
    _writer()(str(tmp_path), _scenario(rec))
    pattern = os.path.join(str(tmp_path), rec["pattern"])
    tag = rec["tag"]
    if "error" in rec:
        err = {"ValueError": ValueError}[rec["error"]["type"]]
        with pytest.raises(err) as ei:
            V.VTKUnstructuredTimeSeriesReader(pattern, **rec["kwargs"]).load_time_series()
        assert str(ei.value).split("\n")[0] == rec["error"]["message"]
        return
    rd = V.VTKUnstructuredTimeSeriesReader(pattern, **rec["kwargs"])
    ts = rd.load_time_series()
    assert [os.path.basename(f) for f in rd.time_files] == rec["order"]
    assert ts["velocity_field_name"] == rec["velocity_field_name"]
    assert ts["source"] == rec["source"]
    for k in ("velocity_data", "positions", "times"):
        want = Z[f"{tag}_{k}"]
        assert ts[k].dtype == want.dtype and ts[k].shape == want.shape, k
        assert np.array_equal(ts[k], want), k
    assert np.array_equal(np.asarray(rd.get_bounds(), np.float64), Z[f"{tag}_bounds"])
    info = rd.get_grid_info()
    ref = rec["info"]
    assert sorted(info) == ref["keys"]
    assert info["n_points"] == ref["n_points"] and info["n_timesteps"] == ref["n_timesteps"]
    assert [os.path.basename(f) for f in info["time_files"]] == ref["time_files"]
    assert info["velocity_field_name"] == ref["velocity_field_name"]
    assert np.array_equal(info["grid_points"], Z[f"{tag}_positions"])
