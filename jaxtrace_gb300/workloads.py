"""Seeded synthetic inputs of the benchmark configurations.

No public dataset is involved: every input is generated here from fixed
seeds with the shapes, sizes and value distributions the configurations
name (ABC flow on regular grids or a jittered Kuhn-split tetrahedral mesh,
uniform or lattice seeds).

* plain RK4 (CPU-runnable): 10,000 particles, 32^3 periodic grid, 16
  snapshots over [0,1], dt 0.01, 100 steps
* unstructured FEM: 64^3 hexes x 6 tets (1,572,864 tets), interior nodes
  jittered +-0.2 cell, 32 snapshots, 1M particles, mixed BC, dt 0.005, 1000 steps
* precision: 128^3 grid, 64 snapshots over [0,2] of ABC + (1,0,0) + N(0,0.01^2),
  16,777,216 lattice seeds, continuous inlet on a 256x256 lattice, dt 0.002,
  1000 steps
* differentiation: plain field at 64^3, 256x256x64 seeds, dt 0.01, 500 steps
* batching: 256 ensembles of log-uniform size in [1e3,1e6] on the FEM mesh
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
UNIT = ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))


def abc_velocity(points01: np.ndarray, t: float, A: float = 1.0, B: float = 0.7, C: float = 0.43) -> np.ndarray:
    """ABC flow u = (A sin z + C cos y, B sin x + A cos z, C sin y + B cos x)(1 + 0.1 sin 2 pi t)
    at points of the unit cube (coordinates scaled to [0, 2 pi]); float64."""
    p = np.asarray(points01, dtype=np.float64)
    x, y, z = 2 * np.pi * p[..., 0], 2 * np.pi * p[..., 1], 2 * np.pi * p[..., 2]
    s = 1.0 + 0.1 * np.sin(2 * np.pi * t)
    out = np.empty(p.shape[:-1] + (3,), dtype=np.float64)
    out[..., 0] = (A * np.sin(z) + C * np.cos(y)) * s
    out[..., 1] = (B * np.sin(x) + A * np.cos(z)) * s
    out[..., 2] = (C * np.sin(y) + B * np.cos(x)) * s
    return out


def grid_nodes(gx, gy, gz) -> np.ndarray:
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(F32)


def abc_snapshots(nodes: np.ndarray, times: np.ndarray, offset=(0.0, 0.0, 0.0), noise_sigma: float = 0.0,
                  noise_seed: int | None = None) -> np.ndarray:
    """(T, N, 3) float32 snapshots of the ABC flow (+ offset + Gaussian noise)."""
    rng = np.random.default_rng(noise_seed) if noise_sigma > 0 else None
    out = np.empty((len(times), len(nodes), 3), dtype=F32)
    off = np.asarray(offset, dtype=np.float64)
    for k, t in enumerate(times):
        v = abc_velocity(nodes, float(t)) + off
        if rng is not None:
            v += rng.normal(0.0, noise_sigma, v.shape)
        out[k] = v
    return out


def kuhn_mesh(n: int, jitter: float = 0.2, seed: int = 1):
    """(n+1)^3 nodes of [0,1]^3 in ij order, interior nodes jittered by
    U(-jitter, jitter)/n (default_rng(seed), node order); every hex split into
    the 6 Kuhn tets (0,1,3,7),(0,1,5,7),(0,2,3,7),(0,2,6,7),(0,4,5,7),(0,4,6,7)
    of its corners v[a+2b+4c]."""
    g = np.linspace(0.0, 1.0, n + 1)
    P = grid_nodes(g, g, g).astype(np.float64)
    interior = np.all((P > 0) & (P < 1), axis=1)
    rng = np.random.default_rng(seed)
    P[interior] += rng.uniform(-jitter, jitter, (int(interior.sum()), 3)) / n
    idx = np.arange((n + 1) ** 3, dtype=np.int64).reshape(n + 1, n + 1, n + 1)
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    corners = np.stack([idx[i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1)] for c in range(8)], axis=1)
    local = np.array([(0, 1, 3, 7), (0, 1, 5, 7), (0, 2, 3, 7), (0, 2, 6, 7), (0, 4, 5, 7), (0, 4, 6, 7)])
    tets = corners[:, local].reshape(-1, 4).astype(np.int32)
    return P.astype(F32), tets


def plain_rk4(n_particles: int = 10_000, n: int = 32, n_snap: int = 16):
    """The CPU-runnable plain case (and, at n=64, the differentiation field)."""
    g = (np.arange(n) / n).astype(F32)
    times = np.linspace(0.0, 1.0, n_snap).astype(F32)
    data = abc_snapshots(grid_nodes(g, g, g), times)
    np.random.seed(42)
    x0 = np.random.uniform(0, 1, (n_particles, 3)).astype(F32)
    return dict(data=data, times=times, grid=(g, g, g), bounds_handling="periodic", x0=x0,
                time_span=(0.0, 1.0), n_timesteps=101, dt=0.01)


def precision_case(n: int = 128, n_snap: int = 64, seeds=(256, 256, 256), lattice: int = 256,
                   n_steps: int = 1000, dt: float = 0.002):
    """The precision configuration: clamp grid, noisy ABC + mean flow, inlet lattice."""
    from .seeding import uniform_grid_seeds
    g = np.linspace(0.0, 1.0, n).astype(F32)
    times = np.linspace(0.0, 2.0, n_snap).astype(F32)
    data = abc_snapshots(grid_nodes(g, g, g), times, offset=(1.0, 0.0, 0.0), noise_sigma=0.01, noise_seed=2)
    x0 = uniform_grid_seeds(tuple(seeds), UNIT)
    return dict(data=data, times=times, grid=(g, g, g), bounds_handling="clamp", x0=x0,
                concentrations={"x": lattice, "y": lattice, "z": lattice},
                time_span=(0.0, n_steps * dt), n_timesteps=n_steps + 1, dt=dt)


def fem_case(n: int = 64, n_snap: int = 32, n_particles: int = 1_000_000, n_steps: int = 1000, dt: float = 0.005):
    """The unstructured FEM configuration."""
    P, tets = kuhn_mesh(n, 0.2, 1)
    times = np.linspace(0.0, 1.0, n_snap).astype(F32)
    data = abc_snapshots(P, times)
    x0 = np.random.default_rng(42).uniform(size=(n_particles, 3)).astype(F32)
    return dict(points=P, tets=tets, data=data, times=times, x0=x0,
                conditions={"x": "periodic", "y": "reflective", "z": "periodic"},
                time_span=(0.0, n_steps * dt), n_timesteps=n_steps + 1, dt=dt)


def ensembles(n_ens: int = 256, seed: int = 7):
    """Sizes round(10**U(3,6)), release times U(0,0.5), positions U[0,1)^3 per ensemble."""
    rng = np.random.default_rng(seed)
    sizes = np.round(10 ** rng.uniform(3, 6, n_ens)).astype(np.int64)
    release = rng.uniform(0, 0.5, n_ens)
    pos = [rng.uniform(size=(int(s), 3)).astype(F32) for s in sizes]
    return sizes, release, pos
