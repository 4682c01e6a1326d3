"""Host side of trajectory streaming: the row hand-off to a sink (order,
readiness, error propagation) and the .pvd collection, without a GPU."""
import threading
import time
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from jaxtrace_gb300 import tracker as TR
from jaxtrace_gb300 import vtk_io as V

F32 = np.float32


class _Ready:
    """Stands in for a copy-done CUDA event: fills its rows when waited on."""

    def __init__(self, arr, r0, nr, value):
        self.arr, self.r0, self.nr, self.value = arr, r0, nr, value

    def synchronize(self):
        time.sleep(0.01)
        self.arr[self.r0:self.r0 + self.nr] = self.value


def test_row_stream_waits_for_each_slab_and_keeps_order():
    pos = np.zeros((7, 3, 3), F32)
    seen = []
    rs = TR._RowStream(lambda r0, p, v, t: seen.append((r0, p.copy(), v, t.copy())), pos, None,
                       np.arange(7, dtype=F32) * 0.5)
    t0 = threading.Thread(target=lambda: pos.__setitem__(0, 9.0))
    t0.start()
    rs.put(0, 1, t0)
    rs.put(1, 3, _Ready(pos, 1, 3, 1.0))
    rs.put(4, 3, _Ready(pos, 4, 3, 2.0))
    rs.close()
    assert [r for r, _, _, _ in seen] == [0, 1, 4]
    assert np.all(seen[0][1] == 9.0) and np.all(seen[1][1] == 1.0) and np.all(seen[2][1] == 2.0)
    assert np.array_equal(np.concatenate([t for _, _, _, t in seen]), np.arange(7, dtype=F32) * 0.5)


def test_row_stream_reraises_the_sink_error_and_stops_calling_it():
    calls = []

    def sink(r0, p, v, t):
        calls.append(r0)
        raise OSError("disk full")

    rs = TR._RowStream(sink, np.zeros((4, 2, 3), F32), None, np.zeros(4, F32))
    for r in range(4):
        rs.put(r, 1)
    with pytest.raises(OSError, match="disk full"):
        rs.close()
    assert calls == [0]


def test_vtk_series_sink_and_collection(tmp_path):
    rng = np.random.default_rng(3)
    pos = rng.random((5, 6, 3)).astype(F32)
    vel = rng.random((5, 6, 3)).astype(F32)
    times = np.linspace(0, 1, 5).astype(F32)
    s = V.VTKTrajectorySeries(tmp_path / "series", prefix="p")
    s(0, pos[:2], vel[:2], times[:2])
    s(2, pos[2:], vel[2:], times[2:])
    root = ET.parse(s.close()).getroot()
    assert root.get("type") == "Collection"
    sets = root.findall("Collection/DataSet")
    assert [d.get("file") for d in sets] == [f"p_{r:04d}.vtu" for r in range(5)]
    assert [d.get("timestep") for d in sets] == [f"{t:.6f}" for t in times]
    for r, d in enumerate(sets):
        got = V.read_vtk_xml(str(tmp_path / "series" / d.get("file")))
        assert np.array_equal(got["points"], pos[r])
        assert np.array_equal(got["point_data"]["Velocity"], vel[r])
        assert np.array_equal(got["point_data"]["Speed"], np.linalg.norm(vel[r], axis=1).astype(F32))
        assert np.array_equal(got["point_data"]["ParticleID"], np.arange(6, dtype=np.int32))
        assert np.all(got["cells"]["types"] == V.VTK_VERTEX)
