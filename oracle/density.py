"""Brute-force float64 restatement of the reference density passes -- TEST
INFRASTRUCTURE ONLY (checked against tests/golden/density.npz).

* KDE: density/kde.py:244-282 (JAX / pure-NumPy formula) and the grid
  normalisation of kde.py:205-240.
* SPH: density/sph.py:227-292 (kernels; brute-force sum within 3*mean(h))
  and the normalisation of sph.py:365-378.
"""
from __future__ import annotations

import math

import numpy as np


def scott(P):
    n, d = P.shape
    return float(np.std(P, axis=0, ddof=1).mean() * n ** (-1.0 / (d + 4.0)))


def silverman(P):
    n, d = P.shape
    return float(((4.0 / (d + 2.0)) ** (1.0 / (d + 4.0))) * np.std(P, axis=0, ddof=1).mean() * n ** (-1.0 / (d + 4.0)))


def kde_mean(Q, P, h, chunk=2048):
    """mean_j (2 pi)^(-d/2) exp(-|q - p_j|^2 / 2h^2) in float64."""
    Q = np.asarray(Q, np.float64)
    P = np.asarray(P, np.float64)
    d = Q.shape[1]
    out = np.empty(len(Q))
    for s in range(0, len(Q), chunk):
        diff = Q[s:s + chunk, None, :] - P[None, :, :]
        r2 = np.sum(diff * diff, axis=-1) / (h * h)
        out[s:s + chunk] = np.mean(np.exp(-0.5 * r2), axis=1)
    return out * (2.0 * math.pi) ** (-0.5 * d)


def kde_normalise(D, grids, axis_of, n):
    cell, dom = 1.0, 1.0
    for k, G in enumerate(grids):
        span = float(G.max() - G.min())
        cell *= span / max(G.shape[axis_of[k]] - 1, 1)
        dom *= span
    total = float((D * cell).sum())
    if total > 0:
        D = D * (n / total)
    return D / max(n / max(dom, 1e-12), 1e-12)


def sph_kernel(r, h, dim, kind):
    h = np.maximum(h, 1e-12)
    q = r / h
    if kind == "cubic_spline":
        sigma = 10.0 / (7.0 * np.pi * h ** 2) if dim == 2 else 1.0 / (np.pi * h ** 3)
        w1 = sigma * (1.0 - 1.5 * q ** 2 + 0.75 * q ** 3)
        w2 = sigma * 0.25 * (2.0 - q) ** 3
        return np.where(q <= 1.0, w1, np.where(q <= 2.0, w2, 0.0))
    if kind == "wendland":
        sigma = 7.0 / (np.pi * h ** 2) if dim == 2 else 21.0 / (2.0 * np.pi * h ** 3)
        t = np.maximum(1.0 - q, 0.0)
        return sigma * t ** 4 * (1.0 + 4.0 * q)
    sigma = 1.0 / (np.pi * h ** 2) if dim == 2 else 1.0 / ((np.pi * h ** 2) ** 1.5)
    return sigma * np.exp(-q ** 2)


def sph_sum(Q, P, h, masses=None, kind="cubic_spline", chunk=1024):
    """sum_j m_j W(|q - p_j|, h_j) over |q - p_j| <= 3*mean(h), float64."""
    Q = np.asarray(Q, np.float64)
    P = np.asarray(P, np.float64)
    h = np.broadcast_to(np.asarray(h, np.float64), (len(P),))
    m = np.ones(len(P)) if masses is None else np.asarray(masses, np.float64)
    cutoff = 3.0 * float(np.mean(h))
    dim = Q.shape[1]
    out = np.empty(len(Q))
    for s in range(0, len(Q), chunk):
        d = np.sqrt(np.sum((Q[s:s + chunk, None, :] - P[None, :, :]) ** 2, axis=-1))
        w = np.where(d <= cutoff, m[None, :] * sph_kernel(d, h[None, :], dim, kind), 0.0)
        out[s:s + chunk] = w.sum(axis=1)
    return out


def sph_normalise(rho, Q, n):
    Q = np.asarray(Q, np.float64)
    vol = max(float(np.prod(Q.max(axis=0) - Q.min(axis=0))), 1e-12)
    return rho / (n / vol)
