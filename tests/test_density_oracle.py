"""The float64 density restatement (oracle/density.py) against golden
vectors produced by the reference's NumPy path (tests/golden/make_golden.py).
The reference computes in float32, so the comparison is to rtol 2e-5."""
import numpy as np
import pytest

from oracle import density as OD

F32 = np.float32


def test_kde_3d_grid(golden):
    g = golden("density")
    P = g["P"].astype(np.float64)
    h = float(g["kde_h"])
    assert abs(OD.scott(g["P"]) - h) < 1e-6 * h
    X, Y, Z = g["kde3_X"], g["kde3_Y"], g["kde3_Z"]
    Q = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    D = OD.kde_mean(Q, P, h).reshape(X.shape)
    D = OD.kde_normalise(D, [X, Y, Z], [1, 0, 2], len(P))
    assert np.allclose(D, g["kde3_D"], rtol=2e-5, atol=1e-7)


def test_kde_2d_slab_grid(golden):
    g = golden("density")
    P = g["P"]
    mask = np.abs(P[:, 1] - 0.5) <= 0.15          # plane 'xz': normal axis y
    pts = P[mask][:, [0, 2]]
    h = float(g["kde2_h"])
    assert abs(OD.silverman(P) - h) < 1e-6 * h
    X, Y = g["kde2_X"], g["kde2_Y"]
    Q = np.stack([X.ravel(), Y.ravel()], 1)
    Z = OD.kde_mean(Q, pts, h).reshape(X.shape)
    Z = OD.kde_normalise(Z, [X, Y], [1, 0], len(P))
    assert np.allclose(Z, g["kde2_Z"], rtol=2e-5, atol=1e-7)


def test_kde_points(golden):
    g = golden("density")
    out = OD.kde_mean(g["kde_q"], g["P"], float(g["kde_h"]))
    assert np.allclose(out, g["kde_pts"], rtol=2e-5, atol=1e-9)


@pytest.mark.parametrize("kind", ["cubic_spline", "wendland", "gaussian"])
def test_sph_3d(golden, kind):
    g = golden("density")
    P = g["P"]
    rho = OD.sph_normalise(OD.sph_sum(P, P, np.float32(0.08), kind=kind), P, len(P))
    assert np.allclose(rho, g[f"sph3_{kind}"], rtol=2e-5, atol=1e-6)


def test_sph_2d_default_h(golden):
    g = golden("density")
    P = g["P"]
    mask = np.abs(P[:, 2] - 0.5) <= 0.2
    P2 = P[mask][:, [0, 1]]
    n = len(P2)
    h = float(np.clip(np.mean(P2.max(0) - P2.min(0)) / n ** 0.5 * 2.0, 0.01, np.mean(P2.max(0) - P2.min(0)) * 0.1))
    assert abs(h - float(g["sph2_default_h"])) < 1e-6
    Q = P[:, [0, 1]]
    rho = OD.sph_normalise(OD.sph_sum(Q, P2, np.float32(h)), Q, n)
    assert np.allclose(rho, g["sph2_default"], rtol=2e-5, atol=1e-6)


def test_sph_adaptive(golden):
    g = golden("density")
    P = g["P"][:400].astype(np.float64)
    d = np.sqrt(((P[:, None, :] - P[None, :, :]) ** 2).sum(-1))
    h = 1.2 * np.sort(d, axis=1)[:, 16]
    assert np.allclose(h, g["sph3_adaptive_h"], rtol=1e-6)
    rho = OD.sph_normalise(OD.sph_sum(P, P, g["sph3_adaptive_h"]), P, len(P))
    assert np.allclose(rho, g["sph3_adaptive"], rtol=2e-5, atol=1e-6)
