"""Affine-tile 16-bit encoding of regular-grid snapshots, checked on the CPU.

The encoder (fields.build_tile_snapshots) runs here on torch's CPU device.
A host restatement of the stage quads and of the tracking kernel's
evaluation (tile of the cell, quad index, base b(f) plus the trilinear
interpolant of the residuals) must reproduce trilinear interpolation of the
snapshot values, which pins the layout the CUDA kernels index.
"""
import numpy as np
import pytest

from jaxtrace_gb300 import _lib as L
from jaxtrace_gb300 import fields as F
from jaxtrace_gb300 import workloads as W

K = L.JT_TILE + 1


def decode_base(rec):
    """(o, Gx, Gy, Gz) of a 16-float base record, each (3,)."""
    o = np.array([rec[0], rec[1], rec[8]], np.float64)
    g = [np.array([rec[2 + 2 * a], rec[3 + 2 * a], rec[9 + a]], np.float64) for a in range(3)]
    return o, g


def encode(data, dims, periodic, storage):
    res, base, tiles = F.build_tile_snapshots(data, dims, periodic, storage, device="cpu")
    return res.float().numpy()[..., :3].astype(np.float64), base.numpy(), tiles


def axis_index(f, n, periodic):
    """Cell index and weight as the tracking kernel computes them."""
    if periodic:
        f = np.mod(f, n)
        i = np.floor(f).astype(np.int64)
        return np.minimum(i, n - 1), f - np.floor(f), f
    f = np.clip(f, 0, n - 1)
    i = np.floor(f).astype(np.int64)
    return i, f - i, f


def tile_eval(res, base, tiles, dims, periodic, t, f):
    """Host restatement of StageTileField: tile and quad of the cell, the
    quads' residuals at planes lx and lx+1, lerp x -> y -> z, plus b(f)."""
    TX, TY, TZ = tiles
    i0, wx, fx = axis_index(f[:, 0], dims[0], periodic)
    j0, wy, fy = axis_index(f[:, 1], dims[1], periodic)
    k0, wz, fz = axis_index(f[:, 2], dims[2], periodic)
    tile = ((i0 >> 2) * TY + (j0 >> 2)) * TZ + (k0 >> 2)
    lx, ly, lz = i0 & 3, j0 & 3, k0 & 3
    r = res[t].reshape(-1, K, K, K, 3)

    def node(a, b, c):
        return r[tile, a, b, c]

    lerp = lambda w, a, b: a + w[:, None] * (b - a)  # noqa: E731
    c00 = lerp(wx, node(lx, ly, lz), node(lx + 1, ly, lz))
    c01 = lerp(wx, node(lx, ly, lz + 1), node(lx + 1, ly, lz + 1))
    c10 = lerp(wx, node(lx, ly + 1, lz), node(lx + 1, ly + 1, lz))
    c11 = lerp(wx, node(lx, ly + 1, lz + 1), node(lx + 1, ly + 1, lz + 1))
    rv = lerp(wz, lerp(wy, c00, c10), lerp(wy, c01, c11))
    out = np.empty_like(rv)
    for m in range(len(f)):
        o, g = decode_base(base[t, tile[m]])
        out[m] = o + g[0] * fx[m] + g[1] * fy[m] + g[2] * fz[m] + rv[m]
    return out


def trilinear_ref(V, dims, periodic, f):
    """Trilinear interpolation of node values V (nx,ny,nz,3) at continuous
    index coordinates f (structured.py:284-349 in index space)."""
    idx, w = [], []
    for a in range(3):
        i, wa, _ = axis_index(f[:, a], dims[a], periodic)
        i1 = (i + 1) % dims[a] if periodic else np.minimum(i + 1, dims[a] - 1)
        idx.append((i, i1))
        w.append(wa)
    out = 0.0
    for bx in range(2):
        for by in range(2):
            for bz in range(2):
                wgt = ((w[0] if bx else 1 - w[0]) * (w[1] if by else 1 - w[1]) * (w[2] if bz else 1 - w[2]))
                out = out + wgt[:, None] * V[idx[0][bx], idx[1][by], idx[2][bz]]
    return out


@pytest.mark.parametrize("dims", [(8, 8, 8), (10, 7, 13), (1, 6, 5)])
@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("storage", [L.JT_STORE_TILE_BF16, L.JT_STORE_TILE_F16])
def test_tile_evaluation_reproduces_trilinear(dims, periodic, storage):
    rng = np.random.default_rng(11)
    T = 2
    data = rng.normal(size=(T, int(np.prod(dims)), 3)).astype(np.float32)
    res, base, tiles = encode(data, dims, periodic, storage)
    assert tiles == tuple((n + 3) // 4 for n in dims)
    assert res.shape == (T, np.prod(tiles), K ** 3, 3) and base.shape == (T, np.prod(tiles), 16)
    hi = [n if periodic else n - 1 for n in dims]
    f = rng.uniform(0, 1, size=(2000, 3)) * np.array([max(h, 0) for h in hi], np.float64)
    f[:7] = np.array([h for h in hi], np.float64) * np.array([[0, 0, 0], [1, 1, 1], [1, 0, 1], [0.5, 1, 0],
                                                            [0.25, 0.75, 1], [1, 1, 0], [0, 1, 1]])
    ulp = 2.0 ** -8 if storage == L.JT_STORE_TILE_BF16 else 2.0 ** -11
    for t in range(T):
        V = data[t].reshape(*dims, 3).astype(np.float64)
        got = tile_eval(res, base, tiles, dims, periodic, t, f)
        want = trilinear_ref(V, dims, periodic, f)
        # each corner residual is rounded once to 16 bits (relative ulp/2) and
        # the float32 base coefficients carry their own rounding
        rmax = np.abs(res[t]).max()
        assert np.abs(got - want).max() <= ulp * rmax + 1e-5 * np.abs(V).max() * max(dims)


def test_affine_field_has_zero_residuals():
    dims = (9, 6, 11)
    i, j, k = np.meshgrid(*(np.arange(n, dtype=np.float64) for n in dims), indexing="ij")
    v = np.stack([0.5 + 0.25 * i - 0.125 * j + 0.0625 * k, -1.0 + 0.5 * j, 2.0 - 0.25 * k + 0.5 * i], -1)
    data = v.reshape(1, -1, 3).astype(np.float32)
    for periodic in (False,):
        res, base, _ = encode(data, dims, periodic, L.JT_STORE_TILE_BF16)
        # every tile fits the affine field exactly (the float32 coefficients
        # are exact binary fractions here): residuals are float64 rounding
        assert np.abs(res).max() < 1e-12
        o, g = decode_base(base[0, 0])
        assert np.allclose(o, [0.5, -1.0, 2.0]) and np.allclose(g[0], [0.25, 0.0, 0.5])


def test_residuals_are_the_noise_on_the_precision_field():
    """On the precision configuration's grid (ABC flow + mean flow + 0.01
    noise at 128^3) the residual of the affine tiles is the noise: its rms is
    about 0.01 against about 0.95 for the values, so a 16-bit residual rounds
    about 95 times finer than the 16-bit value would."""
    c = W.precision_case(n=128, n_snap=64, seeds=(2, 2, 2), lattice=2)
    data = c["data"][:1]
    res, base, _ = encode(data, (128, 128, 128), False, L.JT_STORE_TILE_BF16)
    rms = np.sqrt(np.mean(res[0] ** 2))
    assert 0.008 < rms < 0.012
    assert np.abs(res[0]).max() < 0.1


def test_stage_ring_sizes():
    from jaxtrace_gb300.tracker import _stage_node_bytes
    g = np.linspace(0, 1, 128, dtype=np.float32)
    data = np.zeros((2, 128 ** 3, 3), np.float32)
    f = F.StructuredTimeSeriesField(data, np.array([0, 1], np.float32), g, g, g, storage="bf16", encoding="tile")
    assert _stage_node_bytes(f) == 32          # one offset quad per node, as the per-snapshot scale
    f2 = F.StructuredTimeSeriesField(data, np.array([0, 1], np.float32), g, g, g, storage="bf16")
    assert _stage_node_bytes(f2) == 32
    with pytest.raises(ValueError, match="16-bit"):
        F.StructuredTimeSeriesField(data, np.array([0, 1], np.float32), g, g, g, encoding="tile")
    with pytest.raises(ValueError, match="encoding"):
        F.StructuredTimeSeriesField(data, np.array([0, 1], np.float32), g, g, g, storage="f16", encoding="x")
