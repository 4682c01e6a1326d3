"""Trajectory statistics against the reference's own outputs
(tests/golden/analytics.npz, made by running tracking/particles.py and
tracking/analysis.py of the reference): displacement, path length, speeds,
the statistics summary and the row reductions of the mixing metrics, bit
for bit (same float32 NumPy arithmetic)."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300.analysis import mixing_host_terms

F32 = np.float32


@pytest.fixture(scope="module")
def g(golden):
    return golden("analytics")


def _traj(g, vel):
    return jt.Trajectory(positions=g["positions"].copy(), times=g["times"].copy(),
                         velocities=g["velocities"].copy() if vel else None)


@pytest.mark.parametrize("tag", ["nov", "vel"])
def test_per_particle_statistics_match_the_reference(g, tag):
    tr = _traj(g, tag == "vel")
    for name in ("displacement", "path_length", "speeds"):
        ours = getattr(tr, "compute_" + name)()
        ref = g[f"{tag}_{name}"]
        assert ours.dtype == np.float32 and ours.shape == ref.shape
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), name


@pytest.mark.parametrize("tag", ["nov", "vel"])
def test_trajectory_statistics_match_the_reference(g, tag):
    stats = jt.compute_trajectory_statistics(_traj(g, tag == "vel"))
    seen = 0
    for group, vals in stats.items():
        for k, v in vals.items():
            assert np.array_equal(np.asarray(v, dtype=np.float64), g[f"{tag}_stats_{group}_{k}"]), (group, k)
            seen += 1
    assert seen == sum(1 for f in g.files if f.startswith(f"{tag}_stats_"))


def test_mixing_row_reductions_match_the_reference(g):
    out = mixing_host_terms(_traj(g, False))
    for k in ("variance_growth_rate", "final_variance", "poincare_return_ratio"):
        assert np.float64(out[k]) == g[f"mix_{k}"], k


def test_short_trajectories():
    one = jt.Trajectory(positions=np.zeros((1, 5, 3), F32), times=np.zeros(1, F32))
    assert one.compute_path_length().shape == (5,) and one.compute_speeds().shape == (0, 5)
    assert one.dt_mean == 0.0 and one.duration == 0.0
    assert jt.compute_trajectory_statistics(one)["basic"]["num_timesteps"] == 1
