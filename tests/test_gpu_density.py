"""GPU density passes against the reference's golden vectors and the float64
oracle.  Tolerances: rtol 2e-5 (the reference computes in float32; the GPU
sums float32 cell/chunk partials in float64, uses the fast exponential and
skips KDE terms beyond 5 bandwidths along an axis, each below 4e-6)."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300.density import KDEEstimator, SPHDensityEstimator
from oracle import density as OD

pytestmark = pytest.mark.gpu
F32 = np.float32


def test_kde_3d_grid(golden):
    g = golden("density")
    k = KDEEstimator(g["P"], bandwidth_rule="scott", resolution=12)
    assert abs(k.h - float(g["kde_h"])) < 1e-6 * k.h
    X, Y, Z, D = k.evaluate_3d()
    assert np.array_equal(X, g["kde3_X"]) and np.array_equal(Y, g["kde3_Y"]) and np.array_equal(Z, g["kde3_Z"])
    assert np.allclose(D, g["kde3_D"], rtol=2e-5, atol=1e-7)


def test_kde_2d_slab_grid(golden):
    g = golden("density")
    k = KDEEstimator(g["P"], bandwidth_rule="silverman", resolution=20, plane="xz", slab_position=0.5,
                     slab_thickness=0.3)
    X, Y, Z = k.evaluate_2d()
    assert np.array_equal(X, g["kde2_X"]) and np.array_equal(Y, g["kde2_Y"])
    assert np.allclose(Z, g["kde2_Z"], rtol=2e-5, atol=1e-7)


def test_kde_points(golden):
    g = golden("density")
    k = KDEEstimator(g["P"], bandwidth_rule="scott")
    assert np.allclose(k.evaluate(g["kde_q"]), g["kde_pts"], rtol=2e-5, atol=1e-9)


@pytest.mark.parametrize("kind", ["cubic_spline", "wendland", "gaussian"])
def test_sph_3d(golden, kind):
    g = golden("density")
    s = SPHDensityEstimator(g["P"], dimensions="3d", smoothing_length=0.08, kernel_type=kind)
    assert np.allclose(s.evaluate(g["P"]), g[f"sph3_{kind}"], rtol=2e-5, atol=1e-6)


def test_sph_2d_default_h(golden):
    g = golden("density")
    s = SPHDensityEstimator(g["P"], dimensions="2d", plane="xy", position=0.5, slab_thickness=0.4)
    assert abs(s._mean_h - float(g["sph2_default_h"])) < 1e-6
    assert np.allclose(s.evaluate(g["P"]), g["sph2_default"], rtol=2e-5, atol=1e-6)


def test_sph_adaptive(golden):
    g = golden("density")
    s = SPHDensityEstimator(g["P"][:400], dimensions="3d", adaptive=True, n_neighbors=16)
    assert np.allclose(s.smoothing_lengths.cpu().numpy(), g["sph3_adaptive_h"], rtol=1e-6)
    assert np.allclose(s.evaluate(g["P"][:400]), g["sph3_adaptive"], rtol=2e-5, atol=1e-6)


def test_sph_and_kde_at_scale_vs_oracle():
    """200k uniform particles: every 97th query against the float64 brute force."""
    rng = np.random.default_rng(5)
    P = rng.random((200_000, 3)).astype(F32)
    s = SPHDensityEstimator(P, dimensions="3d", smoothing_length=0.02, normalize=False)
    rho = s.evaluate(P)
    sub = np.arange(0, len(P), 97)
    ref = OD.sph_sum(P[sub], P, np.float32(0.02))
    assert np.allclose(rho[sub], ref, rtol=2e-5)
    k = KDEEstimator(P, bandwidth=0.03)
    q = rng.random((500, 3)).astype(F32)
    assert np.allclose(k.evaluate(q), OD.kde_mean(q, P, 0.03), rtol=2e-5)
