"""Device trajectory analytics: the path length fused into the tracking
kernel against Trajectory.compute_path_length on an every-step recording (bit
for bit, through locality sorts, stage fields and periodic wraps), and the
pair term of the mixing metrics against the reference's own output."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import workloads as W

pytestmark = pytest.mark.gpu
F32 = np.float32


def _grid_case(mode="periodic", storage="f32"):
    n = 16
    g = (np.arange(n) / n).astype(F32) if mode == "periodic" else np.linspace(0, 1, n).astype(F32)
    st = np.linspace(0, 0.5, 6).astype(F32)
    f = jt.StructuredTimeSeriesField(W.abc_snapshots(W.grid_nodes(g, g, g), st), st, g, g, g, mode, storage=storage)
    bc = jt.periodic_boundary(W.UNIT) if mode == "periodic" else jt.reflective_boundary(W.UNIT)
    x0 = np.random.default_rng(8).random((6000, 3)).astype(F32)
    return f, bc, x0


@pytest.mark.parametrize("storage", ["f32", "f16"])
@pytest.mark.parametrize("mode", ["periodic", "clamp"])
def test_fused_path_length_equals_the_every_step_recording(storage, mode):
    f, bc, x0 = _grid_case(mode, storage)
    tr = jt.create_tracker("rk4", f, bc, record_path_length=True, sort_every=7, stage_chunk=5)
    traj = tr.track_particles(x0, (0.0, 0.4), 41, dt=0.01)
    assert traj.path_length is not None and traj.path_length.dtype == np.float32
    ref = traj.compute_path_length()
    assert np.array_equal(traj.path_length.view(np.uint32), ref.view(np.uint32))
    # a final-only run of the same steps carries the same path length
    tr2 = jt.create_tracker("rk4", f, bc, record_path_length=True, record_final_only=True, sort_every=7)
    t2 = tr2.track_particles(x0, (0.0, 0.4), 41, dt=0.01)
    assert t2.positions.shape[0] == 2
    assert np.array_equal(t2.path_length.view(np.uint32), ref.view(np.uint32))
    # without the option nothing is attached
    assert jt.create_tracker("rk4", f, bc).track_particles(x0[:10], (0.0, 0.1), 11, dt=0.01).path_length is None


def test_mixing_metrics_match_the_reference(golden):
    g = golden("analytics")
    tr = jt.Trajectory(positions=g["positions"].copy(), times=g["times"].copy())
    out = jt.compute_mixing_metrics(tr)
    for k in ("variance_growth_rate", "final_variance", "poincare_return_ratio"):
        assert np.float64(out[k]) == g[f"mix_{k}"], k
    # float64 sum of logf terms against the reference's float32 mean of np.log
    assert out["lyapunov_approximation"] == pytest.approx(float(g["mix_lyapunov_approximation"]), rel=1e-5)
    assert out["mixing_efficiency"] == pytest.approx(float(g["mix_mixing_efficiency"]), rel=1e-6)


def test_pair_term_counts_ordered_pairs_within_the_cutoff():
    from jaxtrace_gb300.analysis import pair_log_ratio
    rng = np.random.default_rng(3)
    x0 = rng.random((700, 3)).astype(F32)
    x0[5] = x0[4]                                   # a zero distance: excluded
    x1 = (x0 * F32(1.5)).astype(F32)                # every ratio 1.5 up to rounding
    s, n = pair_log_ratio(x0, x1, 0.1)
    d0 = np.linalg.norm(x0[:, None, :] - x0[None, :, :], axis=2)
    mask = (d0 > 0) & (d0 < F32(0.1))
    assert n == int(mask.sum())
    assert s / n == pytest.approx(np.log(1.5), rel=1e-5)
    assert pair_log_ratio(x0[:0], x1[:0]) == (0.0, 0)


def test_tracker_diagnostics(golden):
    """benchmark_performance, analyze_field_sampling, get_memory_info and
    compare_integrators (tracking/tracker.py:590-805, :882-951)."""
    g = golden("track_grid")
    f = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    tr = jt.create_tracker("rk4", f, jt.periodic_boundary(((0, 0, 0), (1, 1, 1))))
    b = tr.benchmark_performance((64, 256, 2048), n_timesteps=11)   # the slope needs unequal size ratios
    assert all(b["throughput"][n] > 0 for n in (64, 256, 2048)) and "scaling_exponent" in b["scalability"]
    q = np.random.default_rng(0).random((100, 3)).astype(np.float32)
    a = tr.analyze_field_sampling(q, [0.0, 0.05])
    assert a["performance"]["total_samples"] == 200 and a["field_properties"]["finite_values"] == 200
    ref = np.concatenate([f.sample_at_positions(q, 0.0), f.sample_at_positions(q, 0.05)])
    assert a["field_properties"]["velocity_magnitude"]["max"] == float(np.linalg.norm(ref, axis=1).max())
    m = tr.get_memory_info()
    assert m["device_total_mb"] > 0
    c = jt.compare_integrators(g["x0"][:50], f, (0.0, 0.1), 11, dt=0.01)
    assert set(c["timing"]) == {"euler", "rk2", "rk4"} and "rk2_vs_euler" in c["comparison"]
    assert c["comparison"]["rk4_vs_euler"]["max_difference"] > 0


def test_reflect_and_clamp_helpers_match_the_reference(golden):
    """reflect_boundary / clamp_to_bounds (tracking/boundary.py:127-172)
    against the reference's outputs."""
    g = golden("boundary")
    assert np.array_equal(np.asarray(jt.reflect_boundary(g["P"], g["B"])), g["reflective"])
    assert np.array_equal(np.asarray(jt.clamp_to_bounds(g["P"], g["B"])), g["clamping"])
