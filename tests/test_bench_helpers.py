"""The benchmark's host-side helpers, on the CPU: inlet-replacement events of
a recorded trajectory, the error statistics against float64 and the budget
test, the ncu csv reader and the capture summary it feeds, the roofline
arithmetic of the bench line, and the reference-timing record both arms
attach."""
import json
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402

F32 = np.float32


def test_reseed_events_find_the_last_replacement():
    """A replacement puts x exactly on the inlet plane and y, z on lattice
    points; the last one counts, and off-lattice coordinates are marked -2."""
    lat = np.linspace(F32(0), F32(1), 5, dtype=F32)
    T, n = 10, 3
    traj = np.full((T, n, 3), 0.5, F32)
    traj[:, :, 0] = np.linspace(0.1, 0.9, T, dtype=F32)[:, None]
    traj[4, 0] = (0.0, lat[1], lat[3])          # particle 0: step 3
    traj[2, 2] = (0.0, lat[0], lat[4])          # particle 2: steps 1 and 7, the last off-lattice in z
    traj[8, 2] = (0.0, lat[2], F32(0.3))
    ev = bench.reseed_events(traj, lat)
    assert ev[0].tolist() == [3, 1, 3]
    assert ev[1].tolist() == [-1, -1, -1]
    assert ev[2].tolist() == [7, 2, -2]


def test_error_stats_split_by_replacement_and_budget():
    rng = np.random.default_rng(1)
    ref = rng.uniform(0.5, 1.0, (1000, 3))
    fin = (ref * (1 + 1e-6)).astype(F32)
    flipped = np.zeros(1000, bool)
    flipped[:5] = True
    fin[:5] += F32(0.1)                          # the flipped ones are far off
    st = bench.error_stats(fin, ref, flipped)
    assert st["reseed_differs"] == 5
    assert st["max"] > 0.05 and st["not_reseed_differs"]["max"] < 2e-6
    assert st["budget_met"] is True
    fin2 = fin.copy()
    fin2[5:100] += F32(0.01)                     # 9.5 % of the kept particles above the budget
    assert bench.error_stats(fin2, ref, flipped)["budget_met"] is False


def _ncu_csv(path, rows):
    hdr = ["ID", "Process ID", "Kernel Name", "Metric Name", "Metric Unit", "Metric Value"]
    lines = ['"==PROF== Connected to process"', ",".join(f'"{h}"' for h in hdr)]
    for r in rows:
        lines.append(",".join(f'"{v}"' for v in r))
    Path(path).write_text("\n".join(lines) + "\n")


def test_ncu_csv_reader_scales_units_and_keeps_k_track(tmp_path):
    f = tmp_path / "a.csv"
    _ncu_csv(f, [
        ("0", "1", "void jt::k_track<0>(x)", "gpu__time_duration.sum", "ms", "8.5"),
        ("0", "1", "void jt::k_track<0>(x)", "dram__bytes_read.sum", "Gbyte", "6.4"),
        ("1", "1", "void jt::k_stage_tile<5>(x)", "gpu__time_duration.sum", "us", "630"),
        ("2", "1", "void jt::k_track<0>(x)", "gpu__time_duration.sum", "ns", "8,400,000"),
        ("2", "1", "void jt::k_track<0>(x)", "launch__grid_size", "", "65536"),
    ])
    got = bench._ncu_launches(f)
    assert set(got) == {"0", "2"}
    assert got["0"]["gpu__time_duration.sum"] == pytest.approx(8.5e-3)
    assert got["0"]["dram__bytes_read.sum"] == pytest.approx(6.4e9)
    assert got["2"]["gpu__time_duration.sum"] == pytest.approx(8.4e-3)
    assert got["2"]["launch__grid_size"] == 65536


def test_capture_summary_feeds_the_roofline(tmp_path, monkeypatch):
    """--ncu-summary turns the captures into per-particle-step figures, and
    roofline_of turns those and a live launch time into the line's figures."""
    dram, inst = tmp_path / "dram.csv", tmp_path / "inst.csv"
    _ncu_csv(dram, [("0", "1", "k_track", m, u, v) for m, u, v in (
        ("dram__bytes_read.sum", "Gbyte", "6.0"), ("dram__bytes_write.sum", "Gbyte", "0.4"),
        ("gpu__time_duration.sum", "ms", "8.0"), ("launch__grid_size", "", "65536"),
        ("launch__block_size", "", "256"))])
    _ncu_csv(inst, [("0", "1", "k_track", m, u, v) for m, u, v in (
        ("smsp__inst_executed.sum", "inst", str(437 * 884736 // 32 * 32)), ("gpu__time_duration.sum", "ms", "5"),
        ("launch__grid_size", "", "3456"), ("launch__block_size", "", "256"))])
    out = tmp_path / "cap.json"
    monkeypatch.setattr(bench, "CAPTURE_JSON", out)
    a = SimpleNamespace(ncu_steps=32, ncu_command=["cmd"], ncu_dram=[f"16bit={dram}"], ncu_inst=[f"16bit={inst}"])
    bench.ncu_summary(a)
    cap = json.loads(out.read_text())
    v = cap["variants"]["16bit"]
    assert v["dram_bytes_per_particle_step"] == pytest.approx(6.4e9 / (65536 * 256 * 32))
    assert v["warp_inst_per_warp_step"] == pytest.approx(437 * 884736 // 32 * 32 / (3456 * 256 / 32 * 32))
    n = 65536 * 256
    r = {"track_launches": 2, "particle_steps_per_launch": n * 32, "launch_ms": 8.0, "stage_fields": 10,
         "stage_field_bytes": 67_108_864}
    roof = bench.roofline_of("bf16", r, n, 6800.0, {"hbm_gbs": 6800.0}, cap)
    alg = 5 * 67_108_864 + n * 48
    assert roof["achieved"] == pytest.approx(alg / 8e-3 / 1e9)
    assert roof["frac"] == pytest.approx(roof["achieved"] / 6800.0)
    assert roof["traffic"] == pytest.approx(v["dram_bytes_per_particle_step"] * n * 32)
    assert roof["dram_frac"] == pytest.approx(roof["traffic"] / 8e-3 / 1e9 / 6800.0)
    assert roof["issue"]["achieved"] == pytest.approx(n * 32 / 32 * v["warp_inst_per_warp_step"] / 8e-3)


def test_reference_timing_record_is_attached_whole():
    rec = bench.reference_numpy_record()
    assert rec is not None and rec["kind"] == "reference"
    for leg in ("precision", "plain", "fem_octree", "density_sph"):
        rows = rec["legs"][leg]
        assert [r["processes"] for r in rows] == [1, rec["host_cores"]]
        assert all(r["value"] > 0 for r in rows)
