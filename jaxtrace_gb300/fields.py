"""Velocity fields of the GPU path.

Each class keeps the constructor and sampling signatures of its JAXTrace
counterpart and owns device-resident snapshot PAIRS (record n of pair p holds
snapshot p and p+1 of node n side by side, so one load returns both
bracketing snapshots).  Calling ``sample_at_positions`` runs a CUDA kernel;
``create_tracker`` fuses the same field into the persistent tracking kernel.

* ``TimeSeriesField``        -- fields/time_series.py:82 (nearest-node space)
* ``StructuredGridSampler``  -- fields/structured.py:65 (static trilinear)
* ``StructuredTimeSeriesField`` -- trilinear space + linear time; the
  reference has no single class for it and composes
  ``TimeSeriesField.sample_at_time`` with ``StructuredGridSampler``.
* ``OctreeFEMTimeSeriesFieldOptimized`` --
  fields/octree_fem_time_series_optimized.py:17 (octree + P1).
"""
from __future__ import annotations

import ctypes as C
import warnings
from typing import Optional, Tuple

import numpy as np

from . import _lib as L
from .schedule import single_blend

F32 = np.float32


def _torch_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("jaxtrace_gb300 runs on a CUDA GPU; no CUDA device is visible (there is no CPU fallback)")
    return torch


def _mark_near_degenerate(tet_box, tet_geom) -> int:
    """Flag the near-degenerate tetrahedra of a field's device box records
    (jt_mark_near_degenerate); returns how many there are."""
    n = C.c_int32(0)
    L.check(L.load().jt_mark_near_degenerate(tet_box.data_ptr(), tet_geom.data_ptr(), tet_box.shape[0],
                                             C.byref(n), L.stream_ptr()))
    return int(n.value)


def _as_f32(a) -> np.ndarray:
    return np.asarray(a, dtype=F32)


def ensure_positions_shape(positions) -> np.ndarray:
    """(N,2|3) -> (N,3) float32, as tracker.py:72-87 / base.py _ensure_positions_shape."""
    pos = _as_f32(positions)
    if pos.ndim == 1:
        pos = pos.reshape(1, -1)
    if pos.ndim != 2:
        raise ValueError(f"Positions must be 2D array, got shape {pos.shape}")
    if pos.shape[1] == 2:
        pos = np.concatenate([pos, np.zeros((pos.shape[0], 1), dtype=F32)], axis=1)
    elif pos.shape[1] != 3:
        raise ValueError(f"Positions must have 2 or 3 columns, got {pos.shape[1]}")
    return np.ascontiguousarray(pos)


def ensure_positions_tensor(positions):
    """ensure_positions_shape for a torch tensor, on the tensor's own device:
    (N,2|3) -> contiguous float32 (N,3), a 1-D tensor as one row, 2-D
    positions given z = 0; the same errors."""
    import torch
    pos = positions.to(torch.float32)
    if pos.ndim == 1:
        pos = pos.reshape(1, -1)
    if pos.ndim != 2:
        raise ValueError(f"Positions must be 2D array, got shape {tuple(pos.shape)}")
    if pos.shape[1] == 2:
        pos = torch.cat([pos, pos.new_zeros((pos.shape[0], 1))], dim=1)
    elif pos.shape[1] != 3:
        raise ValueError(f"Positions must have 2 or 3 columns, got {pos.shape[1]}")
    return pos.contiguous()


def storage_code(storage: str) -> int:
    try:
        return L.STORAGE_CODES[str(storage).lower()]
    except KeyError:
        raise ValueError(f"storage must be one of f32/bf16/f16, got {storage!r}") from None


def snapshot_scales(data: np.ndarray, storage: int) -> np.ndarray:
    """Per-snapshot power-of-two decode scales for 16-bit storage.

    Each snapshot is divided by 2**ceil(log2(max|v|)) before rounding, so its
    largest magnitude lands in [0.5, 1]; decoding multiplies back exactly.
    """
    T = data.shape[0]
    if storage == L.JT_STORE_F32:
        return np.ones(T, dtype=F32)
    amax = np.abs(data.reshape(T, -1)).max(axis=1).astype(np.float64)
    amax = np.where(np.isfinite(amax) & (amax > 0), amax, 1.0)
    return np.exp2(np.ceil(np.log2(amax))).astype(F32)


A_SLOTS, B_SLOTS = [0, 1, 4], [2, 3, 5]   # record {Ax,Ay,Bx,By,Az,Bz,0,0}


def build_pairs_device(data: np.ndarray, storage: int, device="cuda", quad: tuple | None = None):
    """Upload (T,N,3) snapshots as (max(T-1,1), N, 8) pair records
    {Ax,Ay,Bx,By,Az,Bz,0,0} (A = snapshot p, B = snapshot p+1).

    With ``quad`` = (z_succ, y_succ) (16-bit grid fields) each node n gets a
    48-byte yz-quad record of the nodes n, z_succ[n], y_succ[n] and
    y_succ[z_succ[n]], six halves each in node order, split into a 32-byte
    part A (halves 0-15, all part-A records first) and a 16-byte part B
    (halves 16-23, after every part-A record) so both parts stay aligned for
    one 256-bit and one 128-bit load.  Returns the flat buffer and scales."""
    torch = _torch_cuda()
    T, N, _ = data.shape
    P = max(T - 1, 1)
    scales = snapshot_scales(data, storage)
    qd = quad is not None and storage != L.JT_STORE_F32
    if storage == L.JT_STORE_F32:
        dt = torch.float32
    else:
        dt = torch.bfloat16 if storage == L.JT_STORE_BF16 else torch.float16
    if qd:
        buf = torch.zeros(P * N * 24, dtype=dt, device=device)
        part_a = buf[: P * N * 16].view(P, N, 16)
        part_b = buf[P * N * 16:].view(P, N, 8)
        zs = torch.from_numpy(np.asarray(quad[0], dtype=np.int64)).to(device)
        ys = torch.from_numpy(np.asarray(quad[1], dtype=np.int64)).to(device)
        yzs = ys[zs]
    else:
        buf = torch.zeros((P, N, 8), dtype=dt, device=device)
    ix = lambda v: torch.tensor(v, device=device)  # noqa: E731
    # part-A slots of the A and B snapshots of quad nodes 0 (n) and 1 (z_succ)
    quad_slots = [([0, 1, 4], [2, 3, 5]), ([6, 7, 10], [8, 9, 11])]
    for t in range(T):
        snap = torch.from_numpy(np.ascontiguousarray(data[t])).to(device)
        if storage != L.JT_STORE_F32:
            snap = (snap / float(scales[t])).to(dt)
        targets = []
        if t < P:
            targets.append((t, 0))      # this snapshot is A of pair t
        if t >= 1:
            targets.append((t - 1, 1))  # and B of pair t-1
        if T == 1:
            targets.append((0, 1))
        for pr, side in targets:
            if not qd:
                buf[pr].index_copy_(1, ix(A_SLOTS if side == 0 else B_SLOTS), snap)
                continue
            vals = (snap, snap[zs], snap[ys], snap[yzs])
            for node in range(2):
                part_a[pr].index_copy_(1, ix(quad_slots[node][side]), vals[node])
            # node y_succ: x, y in part A (A: 12,13 / B: 14,15), z in part B (A: 0 / B: 1)
            part_a[pr].index_copy_(1, ix([12, 13] if side == 0 else [14, 15]), vals[2][:, :2].contiguous())
            part_b[pr][:, 0 if side == 0 else 1] = vals[2][:, 2]
            # node y_succ(z_succ): part B (A: 2,3,6 / B: 4,5,7)
            part_b[pr].index_copy_(1, ix([2, 3, 6] if side == 0 else [4, 5, 7]), vals[3])
    return buf, scales


def tile_axis_maps(n: int, periodic: bool):
    """Grid node and continuous index coordinate of every tile's local nodes
    along one axis of n nodes: two (tiles, JT_TILE + 1) arrays.  Local node l
    of tile t is grid node JT_TILE*t + l, clipped to n - 1 (the sampler's
    clamp, zero and nan modes) or wrapped mod n (periodic, where the
    coordinate keeps counting past n so that the tile stays one affine piece)."""
    T = (n + L.JT_TILE - 1) // L.JT_TILE
    loc = L.JT_TILE * np.arange(T)[:, None] + np.arange(L.JT_TILE + 1)[None, :]
    if periodic:
        return loc % max(n, 1), loc.astype(np.float64)
    c = np.minimum(loc, max(n - 1, 0))
    return c, c.astype(np.float64)


def build_tile_snapshots(data: np.ndarray, dims, periodic: bool, storage: int, device="cuda"):
    """Affine-tile snapshots (JT_STORE_TILE_BF16 / _F16) of (T, nx*ny*nz, 3)
    float32 data on a regular grid.

    Each tile of JT_TILE^3 cells gets, per snapshot and component, the least-
    squares affine function b(f) = o + Gx fx + Gy fy + Gz fz of the continuous
    index coordinates over its (JT_TILE+1)^3 nodes (a tensor-product design,
    so the centred columns are orthogonal and the fit is three projections),
    rounded to float32; each node then stores the 16-bit rounding of the
    residual v - b(f_node), computed in float64 from the float32 coefficients.
    Returns (residuals (S, tiles, JT_TILE_NODES, 4) 16-bit with {x, y, z, 0}
    per node, bases (S, tiles, 16) float32 records) for S = max(T, 2)
    snapshots (a single snapshot is stored twice, the pair it forms with
    itself).  ``device`` is where the arithmetic runs (CUDA for a field;
    the host suite checks the encoding on the CPU)."""
    import torch
    if str(device).startswith("cuda"):
        _torch_cuda()
    T = data.shape[0]
    nx, ny, nz = (int(v) for v in dims)
    maps = [tile_axis_maps(n, periodic) for n in (nx, ny, nz)]
    TX, TY, TZ = (m[0].shape[0] for m in maps)
    tiles = TX * TY * TZ
    K = L.JT_TILE + 1
    S = max(T, 2)
    dt16 = torch.bfloat16 if storage in (L.JT_STORE_BF16, L.JT_STORE_TILE_BF16) else torch.float16
    res = torch.zeros((S, tiles, K ** 3, 4), dtype=dt16, device=device)
    base = torch.zeros((S, tiles, 16), dtype=torch.float32, device=device)
    t64 = lambda a: torch.as_tensor(a, dtype=torch.float64, device=device)  # noqa: E731
    IX, IY, IZ = (torch.as_tensor(m[0], dtype=torch.int64, device=device) for m in maps)
    node = ((IX[:, None, None, :, None, None] * ny + IY[None, :, None, None, :, None]) * nz
            + IZ[None, None, :, None, None, :])                                   # (TX,TY,TZ,K,K,K)
    CX, CY, CZ = (t64(m[1]) for m in maps)                                        # (T_a, K)
    means = [c.mean(dim=1) for c in (CX, CY, CZ)]
    dev = [c - m[:, None] for c, m in zip((CX, CY, CZ), means)]
    # sum over the tile's K^3 nodes of the centred coordinate squared
    ss = [K * K * (d * d).sum(dim=1) for d in dev]
    shape = [(TX, 1, 1, K, 1, 1), (1, TY, 1, 1, K, 1), (1, 1, TZ, 1, 1, K)]
    tshape = [(TX, 1, 1), (1, TY, 1), (1, 1, TZ)]
    for t in range(S):
        V = torch.from_numpy(np.ascontiguousarray(data[min(t, T - 1)])).to(device=device, dtype=torch.float64)
        Vt = V[node]                                                               # (TX,TY,TZ,K,K,K,3)
        o = Vt.mean(dim=(3, 4, 5))                                                 # (TX,TY,TZ,3)
        G = []
        for a in range(3):
            num = (Vt * dev[a].reshape(shape[a] + (1,))).sum(dim=(3, 4, 5))
            den = ss[a].reshape(tshape[a] + (1,))
            G.append(torch.where(den > 0, num / torch.where(den > 0, den, 1.0), 0.0))
        off = o - sum(G[a] * means[a].reshape(tshape[a] + (1,)) for a in range(3))
        off32 = off.float().double()
        G32 = [g.float().double() for g in G]
        b = off32[:, :, :, None, None, None, :] + sum(
            G32[a][:, :, :, None, None, None, :] * (CX, CY, CZ)[a].reshape(shape[a] + (1,)) for a in range(3))
        r = (Vt - b).reshape(tiles, K ** 3, 3)
        res[t, :, :, :3] = r.float().to(dt16)
        rec = base[t]
        off32f, Gf = off32.reshape(tiles, 3).float(), [g.reshape(tiles, 3).float() for g in G32]
        rec[:, 0], rec[:, 1] = off32f[:, 0], off32f[:, 1]
        for a in range(3):
            rec[:, 2 + 2 * a], rec[:, 3 + 2 * a] = Gf[a][:, 0], Gf[a][:, 1]
            rec[:, 9 + a] = Gf[a][:, 2]
        rec[:, 8] = off32f[:, 2]
    return res, base, (TX, TY, TZ)


class _DeviceField:
    """Shared plumbing: snapshot times, blend semantics and the jt_field struct."""

    _semantics = "numpy"

    def _init_time(self, times, interpolation, extrapolation, storage, semantics):
        self.times = _as_f32(times)
        self.interpolation = interpolation
        self.extrapolation = extrapolation
        if interpolation.lower() not in ("nearest", "linear", "cubic"):
            raise ValueError(f"Unsupported interpolation: {interpolation}")
        if extrapolation.lower() not in ("constant", "linear", "nan", "zero"):
            raise ValueError(f"Unsupported extrapolation: {extrapolation}")
        if semantics not in ("numpy", "jax"):
            raise ValueError("time_semantics must be 'numpy' or 'jax'")
        self._semantics = semantics
        self.storage = str(storage).lower()
        self._storage = storage_code(storage)
        self.t_min, self.t_max = float(self.times[0]), float(self.times[-1])
        if not np.all(np.diff(self.times) >= 0):
            warnings.warn("Times are not monotonically non-decreasing; interpolation may be unreliable")
        self._dev = None

    # -- schedule hooks used by the tracker --
    def _blend_args(self):
        return dict(semantics=self._semantics, interpolation=self.interpolation,
                    extrapolation=self.extrapolation, scales=self._scales_or_none())

    def _scales_or_none(self):
        if getattr(self, "encoding", "snapshot") == "tile":
            # affine tiles are unscaled; their gathering pairs are float32
            return None
        self._device()
        return None if self._storage == L.JT_STORE_F32 else self._scales

    def _default_arith(self):
        return L.JT_ARITH_EXACT if self._storage == L.JT_STORE_F32 else L.JT_ARITH_COMPENSATED

    def blend_at(self, t) -> np.ndarray:
        return single_blend(self.times, t, **self._blend_args())

    def sort_grid(self, bits: int = 7):
        """Morton cell grid (2^bits per axis over the field's bounding box)
        used to reorder particles for gather locality."""
        lo, hi = (np.asarray(v, dtype=np.float64) for v in self.get_spatial_bounds())
        ext = hi - lo
        g = L.SortGrid()
        g.origin[:] = [float(v) for v in lo]
        g.inv_cell[:] = [float((1 << bits) / e) if e > 0 else 0.0 for e in ext]
        g.bits = bits
        return g

    def get_time_bounds(self) -> Tuple[float, float]:
        return float(self.t_min), float(self.t_max)

    def validate_time(self, t: float) -> bool:
        return self.t_min <= float(t) <= self.t_max

    # -- device sampling --
    def jt_field(self):
        """The ctypes ``jt_field`` of this field (device buffers built on first use)."""
        self._device()
        return self._cfield

    def sample_at_positions(self, query_positions, t, *, arith=None):
        """Velocities at (M,3) positions and time t (fields/base.py:106-122).

        Accepts numpy (returns numpy) or CUDA torch tensors (returns a tensor).
        ``arith`` (JT_ARITH_*): the arithmetic of a tracker that records
        velocities, so that its row 0 matches the rows its kernel records;
        the field's own default otherwise.
        """
        torch = _torch_cuda()
        self._device()
        is_tensor = isinstance(query_positions, torch.Tensor)
        if is_tensor:
            q = query_positions.to(device="cuda", dtype=torch.float32)
            if q.ndim == 1:
                q = q.reshape(1, -1)
            if q.shape[1] == 2:
                q = torch.cat([q, torch.zeros_like(q[:, :1])], dim=1)
            q = q.contiguous()
        else:
            q = torch.from_numpy(ensure_positions_shape(query_positions)).cuda()
        out = torch.empty_like(q)
        e = self.blend_at(t)
        blend = L.Blend.from_buffer_copy(e.tobytes())
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        L.check(L.load().jt_field_sample(C.byref(self._cfield), C.byref(blend),
                                         self._default_arith() if arith is None else int(arith),
                                         L.ptr(q), L.ptr(out), q.shape[0], L.ptr(status), L.stream_ptr()))
        return out if is_tensor else out.cpu().numpy()

    def __call__(self, a, b):
        t, positions = _parse_time_and_positions(a, b)
        return self.sample_at_positions(positions, t)

    def evaluate(self, a, b):
        return self(a, b)

    def sample_at_time(self, t):
        """All node values at time t (time_series.py:306), blended on the device."""
        torch = _torch_cuda()
        pairs = self._device_pairs()
        e = self.blend_at(t)[0]
        A = pairs[int(e["pair"])][:, A_SLOTS].float()
        B = pairs[int(e["pair"])][:, B_SLOTS].float()
        form = int(e["form"])
        if form == L.JT_BLEND_WEIGHTED:
            v = A * float(e["wa"]) + B * float(e["wb"])
        elif form == L.JT_BLEND_SAME_A:
            v = A * float(e["wa"]) + A * float(e["wb"])
        elif form == L.JT_BLEND_SAME_B:
            v = B * float(e["wa"]) + B * float(e["wb"])
        else:
            A = A * float(e["sa"])
            B = B * float(e["sb"])
            base = A if form == L.JT_BLEND_LERP_FWD else B
            v = base + float(e["wb"]) * (B - A)
        return v.cpu().numpy().astype(F32, copy=False)

    def memory_usage_mb(self) -> float:
        if self._dev is None:
            return 0.0
        return sum(t.numel() * t.element_size() for t in self._dev.values()) / 1024 ** 2


def _parse_time_and_positions(a, b):
    """time_series.py:285-294: accept field(t, positions) or field(positions, t)."""
    def pos_like(x):
        try:
            arr = np.asarray(x) if not hasattr(x, "shape") else x
        except Exception:
            return False
        nd = len(arr.shape)
        return (nd == 2 and arr.shape[1] in (2, 3)) or (nd == 1 and arr.shape[0] in (2, 3))

    def scalar_like(x):
        return len(getattr(x, "shape", np.shape(x))) == 0

    if pos_like(a) and scalar_like(b):
        return float(b), a
    if pos_like(b) and scalar_like(a):
        return float(a), b
    if scalar_like(a) and not scalar_like(b):
        return float(a), b
    if scalar_like(b) and not scalar_like(a):
        return float(b), a
    raise TypeError("Cannot determine (t, positions) from arguments")


# ---------------------------------------------------------------------------
class StructuredTimeSeriesField(_DeviceField):
    """Trilinear-in-space, linear-in-time field on a regular grid.

    data: (T, Nx, Ny, Nz, 3) or (T, Nx*Ny*Nz, 3) in ij order; grid_x/y/z the
    axis coordinates.  Semantics: StructuredGridSampler.sample (structured.py:
    284-349) of TimeSeriesField.sample_at_time (time_series.py:326-367).
    """

    def __init__(self, data, times, grid_x, grid_y, grid_z, bounds_handling: str = "clamp",
                 interpolation: str = "linear", extrapolation: str = "constant", *,
                 storage: str = "f32", time_semantics: str = "numpy", encoding: str = "auto"):
        gx, gy, gz = _as_f32(grid_x), _as_f32(grid_y), _as_f32(grid_z)
        if gx.ndim != 1 or gy.ndim != 1 or gz.ndim != 1:
            raise ValueError("grid axes must be 1-D")
        nx, ny, nz = len(gx), len(gy), len(gz)
        data = _as_f32(data)
        if data.ndim == 5:
            if data.shape[1:] != (nx, ny, nz, 3):
                raise ValueError(f"data shape {data.shape} does not match grid ({nx},{ny},{nz})")
            data = data.reshape(data.shape[0], nx * ny * nz, 3)
        if data.ndim != 3 or data.shape[1:] != (nx * ny * nz, 3):
            raise ValueError(f"data must be (T,Nx,Ny,Nz,3) or (T,Nx*Ny*Nz,3), got {data.shape}")
        mode = bounds_handling.lower()
        codes = {"clamp": L.JT_GRID_CLAMP, "zero": L.JT_GRID_ZERO, "nan": L.JT_GRID_NAN,
                 "periodic": L.JT_GRID_PERIODIC}
        if mode not in codes:
            raise ValueError(f"Unsupported bounds_handling: {bounds_handling}")
        self._init_time(times, interpolation, extrapolation, storage, time_semantics)
        if self.times.shape != (data.shape[0],):
            raise ValueError(f"times shape {self.times.shape} != (T,) with T={data.shape[0]}")
        self.data = data
        self.grid_x, self.grid_y, self.grid_z = gx, gy, gz
        self.bounds_handling = bounds_handling
        self.Nx, self.Ny, self.Nz = nx, ny, nz
        self.T, self.N = data.shape[0], data.shape[1]
        # structured.py:125-132
        self.dx = float(gx[1] - gx[0]) if nx > 1 else 1.0
        self.dy = float(gy[1] - gy[0]) if ny > 1 else 1.0
        self.dz = float(gz[1] - gz[0]) if nz > 1 else 1.0
        self.x_min, self.x_max = float(gx[0]), float(gx[-1])
        self.y_min, self.y_max = float(gy[0]), float(gy[-1])
        self.z_min, self.z_max = float(gz[0]), float(gz[-1])
        self._mode = codes[mode]
        # 16-bit encodings of the snapshots: "tile" (the default for 16-bit
        # storage) -- per tile of JT_TILE^3 cells a float32 affine base and
        # 16-bit residuals, read by the pre-blended stage fields of
        # track_particles (the paths that gather snapshot pairs read float32
        # pairs then); "snapshot" -- every value over a per-snapshot
        # power-of-two scale, read by every path
        enc = str(encoding).lower()
        if enc == "auto":
            enc = "snapshot" if self._storage == L.JT_STORE_F32 else "tile"
        if enc not in ("snapshot", "tile"):
            raise ValueError(f"encoding must be 'auto', 'snapshot' or 'tile', got {encoding!r}")
        if enc == "tile" and self._storage == L.JT_STORE_F32:
            raise ValueError("the tile encoding is a 16-bit storage (storage='bf16' or 'f16')")
        self.encoding = enc
        self._tiles = None

    def _successors(self):
        """Node indices of (i, j, k1) and (i, j1, k) for every node (i, j, k),
        j1 and k1 as the sampler computes them (structured.py:311-318)."""
        nx, ny, nz = self.Nx, self.Ny, self.Nz
        per = self._mode == L.JT_GRID_PERIODIC

        def nxt(n):
            a = np.arange(n)
            return (a + 1) % max(n, 1) if per else np.minimum(a + 1, max(n - 1, 0))

        i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        zs = (i * ny + j) * nz + nxt(nz)[k]
        ys = (i * ny + nxt(ny)[j]) * nz + k
        return zs.reshape(-1).astype(np.int64), ys.reshape(-1).astype(np.int64)

    def _pair_storage(self) -> int:
        """Storage of the snapshot pairs the gathering paths read."""
        return L.JT_STORE_F32 if self.encoding == "tile" else self._storage

    def _grid_desc(self) -> "L.GridField":
        g = L.GridField()
        g.nx, g.ny, g.nz = self.Nx, self.Ny, self.Nz
        g.bounds_mode = self._mode
        g.origin[:] = [F32(self.x_min), F32(self.y_min), F32(self.z_min)]
        g.spacing[:] = [F32(self.dx), F32(self.dy), F32(self.dz)]
        g.inv_spacing[:] = [float(F32(1.0) / F32(v)) for v in (self.dx, self.dy, self.dz)]
        # structured.py:299-301: x <= x_min + (Nx-1)*dx, the Python float rounded to float32
        g.valid_hi[:] = [F32(self.x_min + (self.Nx - 1) * self.dx), F32(self.y_min + (self.Ny - 1) * self.dy),
                         F32(self.z_min + (self.Nz - 1) * self.dz)]
        return g

    def tile_field(self):
        """The ctypes ``jt_field`` of the affine-tile snapshots (storage
        JT_STORE_TILE_*), built on first use; the input of
        jt_stage_tile_fields."""
        if self.encoding != "tile":
            raise ValueError("tile_field() needs encoding='tile'")
        if self._tiles is None:
            res, base, tiles = build_tile_snapshots(self.data, (self.Nx, self.Ny, self.Nz),
                                                    self._mode == L.JT_GRID_PERIODIC, self._storage)
            g = self._grid_desc()
            g.storage = L.JT_STORE_TILE_BF16 if self._storage == L.JT_STORE_BF16 else L.JT_STORE_TILE_F16
            g.n_pairs = res.shape[0] - 1
            g.pair_stride = res.shape[1] * res.shape[2]
            g.pairs = res.data_ptr()
            g.tile_base = base.data_ptr()
            g.tiles[:] = list(tiles)
            # per-snapshot max |v|: the bound the stage fields' scales come from
            amax = np.abs(self.data.reshape(self.data.shape[0], -1)).max(axis=1).astype(np.float64)
            if len(amax) == 1:
                amax = np.repeat(amax, 2)
            self._tiles = {"res": res, "base": base, "tiles": tiles, "grid": g, "amax": amax,
                           "field": L.Field(kind=L.JT_FIELD_GRID, grid=C.pointer(g))}
        return self._tiles["field"]

    def _device(self):
        if self._dev is not None:
            return
        ps = self._pair_storage()
        pairs, scales = build_pairs_device(self.data, ps, quad=self._successors())
        self._scales = scales
        P = max(self.data.shape[0] - 1, 1)
        # node n's own six values sit in slots 0-5 of both record layouts
        view = pairs if ps == L.JT_STORE_F32 else pairs[: P * self.N * 16].view(P, self.N, 16)
        self._dev = {"pairs": view, "buffer": pairs}
        g = self._grid_desc()
        g.storage = ps
        g.n_pairs = P
        g.pair_stride = self.N
        g.pairs = pairs.data_ptr()
        self._cgrid = g
        self._cfield = L.Field(kind=L.JT_FIELD_GRID, grid=C.pointer(g))

    def _device_pairs(self):
        self._device()
        return self._dev["pairs"]

    def get_spatial_bounds(self):
        return (np.array([self.x_min, self.y_min, self.z_min], dtype=F32),
                np.array([self.x_max, self.y_max, self.z_max], dtype=F32))


class StructuredGridSampler(StructuredTimeSeriesField):
    """Static trilinear sampler, structured.py:65 (velocity_data (Nx,Ny,Nz,3))."""

    def __init__(self, velocity_data, grid_x, grid_y, grid_z, bounds_handling: str = "clamp",
                 grid_meta=None, *, storage: str = "f32", encoding: str = "auto"):
        v = _as_f32(velocity_data)
        if v.ndim != 4:
            raise ValueError(f"velocity_data must be 4D (Nx,Ny,Nz,3), got {v.shape}")
        if v.shape[3] != 3:
            raise ValueError(f"velocity_data must have 3 components, got {v.shape[3]}")
        for name, g, n in (("grid_x", grid_x, v.shape[0]), ("grid_y", grid_y, v.shape[1]), ("grid_z", grid_z, v.shape[2])):
            if _as_f32(g).shape != (n,):
                raise ValueError(f"{name} shape {_as_f32(g).shape} doesn't match velocity_data")
        super().__init__(v[None], np.zeros(1, dtype=F32), grid_x, grid_y, grid_z, bounds_handling,
                         storage=storage, encoding=encoding)
        self.velocity_data = v
        self.grid_meta = grid_meta

    def sample(self, positions):
        return self.sample_at_positions(positions, 0.0)


# ---------------------------------------------------------------------------
class TimeSeriesField(_DeviceField):
    """time_series.py:82 -- snapshots at scattered nodes, nearest-node in space.

    The reference samples space by the nearest node (argmin of the float32
    squared distance, lowest index on ties); here a uniform cell list
    limits the search (exact, not approximate).
    """

    def __init__(self, data, times, positions, interpolation: str = "linear",
                 extrapolation: str = "constant", _source_info: Optional[dict] = None, *,
                 storage: str = "f32", time_semantics: str = "numpy"):
        data = _as_f32(data)
        positions = ensure_positions_shape(positions)
        if data.ndim != 3:
            raise ValueError(f"data must have 3 dims (T,N,3), got {data.shape}")
        T, N, D = data.shape
        if D != 3:
            raise ValueError(f"data last dimension must be 3, got {D}")
        self._init_time(times, interpolation, extrapolation, storage, time_semantics)
        if self.times.shape != (T,):
            raise ValueError(f"times shape {self.times.shape} != (T,) with T={T}")
        if positions.shape != (N, 3):
            raise ValueError(f"positions shape {positions.shape} != (N,3) with N={N}")
        self.data, self.positions = data, positions
        self.T, self.N = T, N
        self._source_info = _source_info or {}

    def _cell_list(self):
        P = self.positions.astype(np.float64)
        lo, hi = P.min(axis=0), P.max(axis=0)
        ext = hi - lo
        live = ext > 0
        n = self.N
        vol = np.prod(ext[live]) if live.any() else 1.0
        dim = max(int(live.sum()), 1)
        h = (vol / max(n / 2.0, 1.0)) ** (1.0 / dim) if live.any() else 1.0
        cells = np.where(live, np.clip(np.ceil(ext / h), 1, 1024), 1).astype(np.int64)
        while np.prod(cells) > 8 * n + 64:
            cells = np.maximum(cells // 2, 1)
        inv = np.where(live, cells / np.where(live, ext, 1.0), 0.0)
        # cell of each node, computed exactly as the kernel does (float32)
        o32, inv32 = lo.astype(F32), inv.astype(F32)
        c = np.floor((self.positions - o32) * inv32)
        c = np.clip(np.nan_to_num(c), 0, cells - 1).astype(np.int64)
        cid = (c[:, 2] * cells[1] + c[:, 1]) * cells[0] + c[:, 0]
        order = np.argsort(cid, kind="stable")
        counts = np.bincount(cid, minlength=int(np.prod(cells)))
        start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        return o32, inv32, cells.astype(np.int32), order.astype(np.int32), start

    def _device(self):
        if self._dev is not None:
            return
        torch = _torch_cuda()
        pairs, scales = build_pairs_device(self.data, self._storage)
        self._scales = scales
        o32, inv32, cells, order, start = self._cell_list()
        pts = np.zeros((self.N, 4), dtype=F32)
        pts[:, :3] = self.positions[order]
        self._dev = {"pairs": pairs, "points": torch.from_numpy(pts).cuda(),
                     "ids": torch.from_numpy(order).cuda(), "start": torch.from_numpy(start).cuda()}
        q = L.NearestField()
        q.n_points = self.N
        q.cells[:] = [int(v) for v in cells]
        q.origin[:] = [float(v) for v in o32]
        q.inv_cell[:] = [float(v) for v in inv32]
        q.storage = self._storage
        q.n_pairs = pairs.shape[0]
        q.pair_stride = self.N
        q.points = self._dev["points"].data_ptr()
        q.point_ids = self._dev["ids"].data_ptr()
        q.cell_start = self._dev["start"].data_ptr()
        q.pairs = pairs.data_ptr()
        self._cnear = q
        self._cfield = L.Field(kind=L.JT_FIELD_NEAREST, nearest=C.pointer(q))

    def _device_pairs(self):
        self._device()
        return self._dev["pairs"]

    def get_spatial_bounds(self):
        return self.positions.min(axis=0).astype(F32), self.positions.max(axis=0).astype(F32)

    def validate_data(self) -> bool:
        if not np.all(np.isfinite(self.data)):
            raise ValueError("Velocity data contains non-finite values")
        if not np.all(np.isfinite(self.times)):
            raise ValueError("Time data contains non-finite values")
        if not np.all(np.isfinite(self.positions)):
            raise ValueError("Position data contains non-finite values")
        if not np.all(np.diff(self.times) >= 0):
            raise ValueError("Times must be monotonically non-decreasing")
        return True


# ---------------------------------------------------------------------------
def auto_sub_div(P, T4, cell64, sample: int = 4096, max_entries: int = 1 << 30) -> int:
    """Sub-cells per hash-cell axis such that a sub-cell edge is about a sixth
    of the median element box edge (measured on an even sample of elements),
    in 1..16, lowered while the estimated list entries (elements x sub-cells
    their boxes meet) exceed ``max_entries``.  On the FEM configuration
    (64^3 x 6 jittered tetrahedra, 32^3 cells) it gives 10: 1.60e9
    particle-steps/s against 1.30e9 with 4 and 1.49e9 with 8."""
    M = len(T4)
    if M == 0:
        return 1
    idx = np.linspace(0, M - 1, min(M, sample)).astype(np.int64)
    V = np.asarray(P, dtype=np.float64)[np.asarray(T4)[idx]]
    edge = float(np.median((V.max(axis=1) - V.min(axis=1)).max(axis=1)))
    cell = float(np.min(cell64))
    if not edge > 0 or not cell > 0:
        return 1
    S = int(min(16, max(1, round(6.0 * cell / edge))))
    while S > 1 and M * (edge / (cell / S) + 1.0) ** 3 > max_entries:
        S -= 1
    return S


class FemHashGrid:
    """Spatial hash grid of build_tetrahedral_mesh (fem_interpolator.py:36-143),
    built with array operations instead of the per-element loop but with the
    same arithmetic: float32 node bounding box; cells per axis
    ``max(1, ceil(aspect * R))`` with float32 aspect ratios and R the cube
    root of grid_resolution^3 as a Python float; float64 cell edges for the
    element-to-cell assignment (float32 box offsets divided by them, floored,
    clipped) and their float32 copy for lookups; an element is listed in
    every cell its box overlaps, in ascending element order.

    Stored as CSR (``cell_start``, ``cell_elems``) plus the per-tet box and
    geometry records the device kernels read; ``cell_to_elements()`` gives
    the reference's -1-padded table.
    """

    _HOST = ("cell_start", "cell_elems", "sub_start", "sub_elems", "cell_elem_counts", "tet_box", "tet_geom",
             "element_bounds")

    def __init__(self, points, connectivity, grid_resolution: int = 32, sub_div: Optional[int] = None,
                 build: str = "auto"):
        """``build``: "host" (jt_fem_grid_build and NumPy element records),
        "device" (jt_fem_grid_build_device: the same arrays, kept on the GPU
        in ``dev``, host copies made on first use) or "auto" (device when
        CUDA is visible and the grid is within the device build's limits).
        ``sub_div``: sub-cells per cell axis (any value gives the same first
        hits); None picks sub-cells about a sixth of a typical element box
        (``auto_sub_div``)."""
        if build not in ("auto", "host", "device"):
            raise ValueError(f"build must be 'auto', 'host' or 'device', got {build!r}")
        P = np.asarray(points, dtype=F32)
        T4 = np.asarray(connectivity, dtype=np.int32)
        if P.ndim != 2 or P.shape[1] != 3:
            raise ValueError("points must be (N,3)")
        if T4.ndim != 2 or T4.shape[1] != 4:
            raise ValueError("connectivity must be (M,4)")
        if T4.size and (T4.min() < 0 or T4.max() >= len(P)):
            raise ValueError("connectivity indexes outside the points array")
        self.points, self.connectivity = P, T4
        bmin, bmax = P.min(axis=0), P.max(axis=0)
        size = bmax - bmin
        aspect = size / size.max()
        gsf = aspect * (int(grid_resolution) ** 3) ** (1 / 3)
        gs = np.maximum(1, np.ceil(gsf).astype(int))
        self.grid_size = tuple(int(v) for v in gs)
        cell64 = size / np.array(self.grid_size)
        self.grid_min = bmin.astype(F32)
        self.cell_size64 = cell64
        self.grid_cell_size = cell64.astype(F32)
        if sub_div is None:
            sub_div = auto_sub_div(P, T4, cell64)
        self.dev = None
        use_device = build == "device"
        if build == "auto":
            import torch
            use_device = torch.cuda.is_available() and len(T4) > 0
        if use_device:
            try:
                self._build_device(int(sub_div), bmin, cell64)
                return
            except NotImplementedError:
                if build == "device":
                    raise          # auto: beyond the device build's limits, build on the host
        V = P[T4]                                           # (M,4,3)
        emin, emax = V.min(axis=1), V.max(axis=1)
        self.element_bounds = np.stack([emin, emax], axis=1)
        self._build_lists(int(sub_div), bmin, cell64)
        # device records: box (min xyz,0,max xyz,0) and geometry (v0, v1-v0, v2-v0, v3-v0, ids)
        M = len(T4)
        self.tet_box = np.zeros((M, 8), dtype=F32)
        self.tet_box[:, 0:3], self.tet_box[:, 4:7] = emin, emax
        self.tet_geom = np.zeros((M, 16), dtype=F32)
        v0 = V[:, 0]
        self.tet_geom[:, 0:3] = v0
        self.tet_geom[:, 3:6] = V[:, 1] - v0
        self.tet_geom[:, 6:9] = V[:, 2] - v0
        self.tet_geom[:, 9:12] = V[:, 3] - v0
        self.tet_geom[:, 12:16] = T4.view(F32)

    def _eps(self, S, cell64):
        """Per-axis margin of the sub-cell lists: covers the float32 rounding
        of the device's sub-cell index."""
        sub = cell64 / max(S, 1)
        scale = float(np.abs(self.points).max()) if len(self.points) else 1.0
        return np.ascontiguousarray(1e-3 * sub + 4e-7 * max(scale, 1.0), dtype=np.float64)

    def _build_device(self, S, bmin, cell64):
        torch = _torch_cuda()
        lib = L.load()
        M = len(self.connectivity)
        eps = self._eps(S, cell64)
        gs = np.ascontiguousarray(self.grid_size, dtype=np.int32)
        gmin = np.ascontiguousarray(bmin, dtype=F32)
        edge = np.ascontiguousarray(cell64, dtype=np.float64)
        pts = torch.from_numpy(np.ascontiguousarray(self.points)).cuda()
        conn = torch.from_numpy(np.ascontiguousarray(self.connectivity)).cuda()
        d = {"tet_box": torch.empty((M, 8), dtype=torch.float32, device="cuda"),
             "tet_geom": torch.empty((M, 16), dtype=torch.float32, device="cuda")}
        handle = C.c_void_p()
        info = L.FemGridInfo()
        stream = L.stream_ptr()
        L.check(lib.jt_fem_grid_build_device(pts.data_ptr(), len(self.points), conn.data_ptr(), M, gs.ctypes.data,
                                             gmin.ctypes.data, edge.ctypes.data, max(int(S), 0), eps.ctypes.data,
                                             d["tet_box"].data_ptr(), d["tet_geom"].data_ptr(), stream,
                                             C.byref(handle), C.byref(info)))
        try:
            i32 = dict(dtype=torch.int32, device="cuda")
            d["cell_start"] = torch.empty(info.n_cells + 1, **i32)
            d["cell_elems"] = torch.zeros(max(info.n_entries, 1), **i32)
            d["sub_start"] = torch.zeros(max(info.n_sub_cells + 1, 1), **i32)
            d["sub_elems"] = torch.zeros(max(info.n_sub_entries, 1), **i32)
            L.check(lib.jt_fem_grid_fetch_device(handle, d["cell_start"].data_ptr(), d["cell_elems"].data_ptr(),
                                                 d["sub_start"].data_ptr(), d["sub_elems"].data_ptr(), stream))
        finally:
            lib.jt_fem_grid_free_device(handle, stream)
        self.dev = d
        self._n_entries, self._n_sub_entries = int(info.n_entries), int(info.n_sub_entries)
        self.max_elems_per_cell = int(info.max_per_cell)
        self.sub_div = int(S) if (S > 0 and info.n_sub_cells > 0) else 0

    def __getattr__(self, name):
        # host arrays of a device build, copied down on first use
        if name in FemHashGrid._HOST and self.__dict__.get("dev") is not None:
            d = self.dev
            self.cell_start = d["cell_start"].cpu().numpy()
            self.cell_elems = d["cell_elems"][:self._n_entries].cpu().numpy()
            if self.sub_div:
                self.sub_start = d["sub_start"].cpu().numpy()
                self.sub_elems = d["sub_elems"][:self._n_sub_entries].cpu().numpy()
            else:
                self.sub_start = np.zeros(1, np.int32)
                self.sub_elems = np.zeros(1, np.int32)
            self.cell_elem_counts = np.diff(self.cell_start).astype(np.int32)
            self.tet_box = d["tet_box"].cpu().numpy()
            self.tet_geom = d["tet_geom"].cpu().numpy()
            self.element_bounds = np.stack([self.tet_box[:, 0:3], self.tet_box[:, 4:7]], axis=1)
            return self.__dict__[name]
        raise AttributeError(name)

    def _build_lists(self, S, bmin, cell64):
        """Cell lists and sub-cell lists (S^3 per hash cell) through the
        library's host builder (jt_fem_grid_build): the reference's float64
        element-to-cell assignment, elements ascending per list; sub-cells
        take each (element, cell) entry where its box, widened by a margin
        that covers the float32 rounding of the device's sub-cell index,
        meets them."""
        eps = self._eps(S, cell64)
        gs = np.ascontiguousarray(self.grid_size, dtype=np.int32)
        gmin = np.ascontiguousarray(bmin, dtype=F32)
        edge = np.ascontiguousarray(cell64, dtype=np.float64)
        P = np.ascontiguousarray(self.points, dtype=F32)
        T4 = np.ascontiguousarray(self.connectivity, dtype=np.int32)
        lib = L.load()
        handle = C.c_void_p()
        info = L.FemGridInfo()
        L.check(lib.jt_fem_grid_build(P.ctypes.data, len(P), T4.ctypes.data, len(T4), gs.ctypes.data,
                                      gmin.ctypes.data, edge.ctypes.data, max(int(S), 0), eps.ctypes.data,
                                      C.byref(handle), C.byref(info)))
        try:
            self.cell_start = np.zeros(info.n_cells + 1, np.int32)
            self.cell_elems = np.zeros(info.n_entries, np.int32)
            self.sub_start = np.zeros(max(info.n_sub_cells + 1, 1), np.int32)
            self.sub_elems = np.zeros(info.n_sub_entries, np.int32)
            L.check(lib.jt_fem_grid_fetch(handle, self.cell_start.ctypes.data, self.cell_elems.ctypes.data,
                                          self.sub_start.ctypes.data, self.sub_elems.ctypes.data))
        finally:
            lib.jt_fem_grid_free(handle)
        self.cell_elem_counts = np.diff(self.cell_start).astype(np.int32)
        self.max_elems_per_cell = int(info.max_per_cell)
        self.sub_div = int(S) if (S > 0 and info.n_sub_cells > 0) else 0
        if self.sub_div == 0:
            self.sub_start = np.zeros(1, np.int32)
            self.sub_elems = np.zeros(1, np.int32)

    def cell_to_elements(self) -> np.ndarray:
        """The reference's (cells, max_per_cell) table, -1 padded."""
        n = len(self.cell_elem_counts)
        out = np.full((n, max(self.max_elems_per_cell, 1)), -1, dtype=np.int32)
        slot = np.arange(len(self.cell_elems)) - np.repeat(self.cell_start[:-1], self.cell_elem_counts)
        out[np.repeat(np.arange(n), self.cell_elem_counts), slot] = self.cell_elems
        return out


class FEMTimeSeriesField(TimeSeriesField):
    """fem_time_series.py:16-110: TimeSeriesField whose spatial sampling is
    hash-grid point location + P1 over a tetrahedral mesh, the nearest node
    of the whole mesh where no tetrahedron holds the query; float32 (JAX)
    time blend."""

    def __init__(self, data, times, positions, connectivity, interpolation: str = "linear",
                 extrapolation: str = "constant", _source_info: Optional[dict] = None,
                 fem_grid_resolution: int = 32, *, storage: str = "f32", sub_div: Optional[int] = None,
                 grid_build: str = "auto"):
        super().__init__(data, times, positions, interpolation, extrapolation, _source_info, storage=storage,
                         time_semantics="jax")
        self.fem_mesh = FemHashGrid(self.positions, connectivity, fem_grid_resolution, sub_div=sub_div,
                                    build=grid_build)

    def _device(self):
        if self._dev is not None:
            return
        torch = _torch_cuda()
        super()._device()
        h = self.fem_mesh
        d = self._dev
        if h.dev is not None:       # built on the device: no upload (the box records get their own copy)
            d.update({k: h.dev[k] for k in ("tet_geom", "cell_start", "cell_elems", "sub_start", "sub_elems")})
            d["tet_box"] = h.dev["tet_box"].clone()
        else:
            d["tet_box"] = torch.from_numpy(h.tet_box).cuda()
            d["tet_geom"] = torch.from_numpy(h.tet_geom).cuda()
            d["cell_start"] = torch.from_numpy(h.cell_start).cuda()
            d["cell_elems"] = torch.from_numpy(h.cell_elems if len(h.cell_elems) else np.zeros(1, np.int32)).cuda()
            d["sub_start"] = torch.from_numpy(h.sub_start).cuda()
            d["sub_elems"] = torch.from_numpy(h.sub_elems if len(h.sub_elems) else np.zeros(1, np.int32)).cuda()
        self.n_near_degenerate = _mark_near_degenerate(d["tet_box"], d["tet_geom"])
        f = L.FemField()
        f.nearest = self._cnear
        f.n_tets = len(h.connectivity)
        f.grid_size[:] = list(h.grid_size)
        f.grid_min[:] = [float(v) for v in h.grid_min]
        f.cell_size[:] = [float(v) for v in h.grid_cell_size]
        f.tet_box, f.tet_geom = d["tet_box"].data_ptr(), d["tet_geom"].data_ptr()
        f.cell_start, f.cell_elems = d["cell_start"].data_ptr(), d["cell_elems"].data_ptr()
        f.sub_div = h.sub_div
        f.sub_start, f.sub_elems = d["sub_start"].data_ptr(), d["sub_elems"].data_ptr()
        f.near_degenerate = int(self.n_near_degenerate > 0)
        self._cfem = f
        self._cfield = L.Field(kind=L.JT_FIELD_FEM, fem=C.pointer(f))

    def __repr__(self) -> str:
        return (f"FEMTimeSeriesField(data={self.data.shape}, times={self.times.shape}, "
                f"positions={self.positions.shape}, elements={self.fem_mesh.connectivity.shape[0]}, "
                f"interpolation='{self.interpolation}', extrapolation='{self.extrapolation}')")


def breadth_first_descent(nodes: np.ndarray):
    """The compact descent arrays of jt_mesh_field (desc, dtab) from the
    octree's node records: nodes renumbered breadth-first from the root, the
    present children of a node consecutive in octant order, so that a child's
    index is the node's first child plus the present octants below it.
    Returns (desc (K,4) int32: centre bits and mask | first << 8, dtab (K,2)
    int32: elem_offset, elem_count), or None when a first-child index would
    not fit 24 bits."""
    K = len(nodes)
    children = np.asarray(nodes["children"], dtype=np.int64)
    order, level = [], np.array([0], dtype=np.int64)
    while len(level):
        order.append(level)
        ch = children[level]
        level = ch[ch >= 0]                    # node order, then octant order
    order = np.concatenate(order)
    if len(order) != K or K >= (1 << 24):
        return None
    ch = children[order]                        # (K, 8) DFS ids, -1 absent
    present = ch >= 0
    mask = (present * (1 << np.arange(8))).sum(axis=1)
    count = present.sum(axis=1)
    first = 1 + np.concatenate([[0], np.cumsum(count)[:-1]])   # children follow in BFS order
    first = np.where(count > 0, first, 0)
    desc = np.empty((K, 4), dtype=np.int32)
    desc[:, :3] = np.asarray(nodes["c"], dtype=np.float32)[order].view(np.int32)
    desc[:, 3] = (mask | (first << 8)).astype(np.uint32).view(np.int32)
    dtab = np.stack([nodes["elem_offset"][order], nodes["elem_count"][order]], axis=1).astype(np.int32)
    return desc, dtab


class OctreeMesh:
    """The octree in the reference's array layout (OctreeMeshOptimized,
    octree_fem_interpolator_optimized.py:18-38).

    ``build``: "host" (jt_octree_build), "device" (jt_octree_build_device:
    the same arrays, built on the GPU and kept there in ``dev``; the host
    arrays are copied down on first use) or "auto" (device when CUDA is
    visible)."""

    _HOST = ("nodes", "elems", "tet_box", "tet_geom", "nodes_min", "nodes_max", "nodes_children", "nodes_is_leaf",
             "nodes_elem_counts", "node_depth")

    def __init__(self, points, connectivity, max_elements_per_leaf=32, max_depth=12, build: str = "auto"):
        points = np.ascontiguousarray(_as_f32(points))
        conn = np.ascontiguousarray(np.asarray(connectivity, dtype=np.int32))
        if points.ndim != 2 or points.shape[1] != 3:
            raise ValueError(f"points must be (N,3), got {points.shape}")
        if conn.ndim != 2 or conn.shape[1] != 4:
            raise ValueError(f"connectivity must be (M,4), got {conn.shape}")
        if build not in ("auto", "host", "device"):
            raise ValueError(f"build must be 'auto', 'host' or 'device', got {build!r}")
        self.dev = None
        if build == "auto":
            import torch
            build = "device" if torch.cuda.is_available() else "host"
        self.points, self.connectivity = points, conn
        self.max_elements_per_leaf, self.max_depth = int(max_elements_per_leaf), int(max_depth)
        if build == "device":
            self._build_device()
            return
        lib = L.load()
        handle = C.c_void_p()
        info = L.OctreeInfo()
        L.check(lib.jt_octree_build(points.ctypes.data, points.shape[0], conn.ctypes.data, conn.shape[0],
                                    int(max_elements_per_leaf), int(max_depth), C.byref(handle), C.byref(info)))
        try:
            K, M = info.n_nodes, conn.shape[0]
            self.nodes = np.zeros(K, dtype=L.OCTREE_NODE_DTYPE)
            self.elems = np.zeros(max(info.n_elem_entries, 1), dtype=np.int32)
            self.tet_box = np.zeros((M, 8), dtype=F32)
            self.tet_geom = np.zeros((M, 16), dtype=F32)
            bounds = np.zeros((K, 6), dtype=F32)
            L.check(lib.jt_octree_fetch(handle, self.nodes.ctypes.data, self.elems.ctypes.data,
                                        self.tet_box.ctypes.data, self.tet_geom.ctypes.data, bounds.ctypes.data))
        finally:
            lib.jt_octree_free(handle)
        self.info = info
        self._host_views(bounds)

    def _host_views(self, bounds):
        self.nodes_min, self.nodes_max = bounds[:, :3].copy(), bounds[:, 3:].copy()
        self.nodes_children = self.nodes["children"].copy()
        self.nodes_is_leaf = self.nodes["is_leaf"].astype(bool)
        self.nodes_elem_counts = self.nodes["elem_count"].copy()
        self.node_depth = self.nodes["pad"][:, 0].copy()

    def _build_device(self):
        torch = _torch_cuda()
        lib = L.load()
        M = self.connectivity.shape[0]
        pts = torch.from_numpy(self.points).cuda()
        conn = torch.from_numpy(self.connectivity).cuda()
        d = {"elems": torch.empty(max(M, 1), dtype=torch.int32, device="cuda"),
             "tet_box": torch.empty((M, 8), dtype=torch.float32, device="cuda"),
             "tet_geom": torch.empty((M, 16), dtype=torch.float32, device="cuda")}
        handle = C.c_void_p()
        info = L.OctreeInfo()
        stream = L.stream_ptr()
        L.check(lib.jt_octree_build_device(pts.data_ptr(), self.points.shape[0], conn.data_ptr(), M,
                                           self.max_elements_per_leaf, self.max_depth, d["elems"].data_ptr(),
                                           d["tet_box"].data_ptr(), d["tet_geom"].data_ptr(), stream,
                                           C.byref(handle), C.byref(info)))
        try:
            d["nodes"] = torch.empty((info.n_nodes, 16), dtype=torch.int32, device="cuda")
            d["bounds"] = torch.empty((info.n_nodes, 6), dtype=torch.float32, device="cuda")
            L.check(lib.jt_octree_fetch_device(handle, d["nodes"].data_ptr(), d["bounds"].data_ptr(), stream))
        finally:
            lib.jt_octree_free_device(handle, stream)
        self.info, self.dev = info, d

    def __getattr__(self, name):
        # host arrays of a device build, copied down on first use
        if name in OctreeMesh._HOST and self.__dict__.get("dev") is not None:
            d = self.dev
            self.nodes = np.ascontiguousarray(d["nodes"].cpu().numpy()).view(L.OCTREE_NODE_DTYPE).reshape(-1)
            self.elems = d["elems"].cpu().numpy()
            self.tet_box = d["tet_box"].cpu().numpy()
            self.tet_geom = d["tet_geom"].cpu().numpy()
            self._host_views(d["bounds"].cpu().numpy())
            return self.__dict__[name]
        raise AttributeError(name)

    @property
    def nodes_elements(self) -> np.ndarray:
        """(K, max_elems) int32 padded with -1 (…optimized.py:183)."""
        K = len(self.nodes)
        W = max(int(self.info.max_elems), 0)
        out = np.full((K, W), -1, dtype=np.int32)
        for k in np.nonzero(self.nodes_elem_counts)[0]:
            o, c = self.nodes["elem_offset"][k], self.nodes_elem_counts[k]
            out[k, :c] = self.elems[o:o + c]
        return out

    @property
    def element_bounds(self) -> np.ndarray:
        return np.stack([self.tet_box[:, :3], self.tet_box[:, 4:7]], axis=1)


class OctreeFEMTimeSeriesFieldOptimized(_DeviceField):
    """Octree point location + P1 interpolation over a tetrahedral mesh with
    the JAX float32 time blend (octree_fem_time_series_optimized.py:17-113)."""

    def __init__(self, data, times, positions, connectivity, interpolation: str = "linear",
                 extrapolation: str = "constant", _source_info: Optional[dict] = None,
                 max_elements_per_leaf: int = 32, max_depth: int = 12, *, storage: str = "f32",
                 octree_build: str = "auto"):
        data = _as_f32(data)
        positions = ensure_positions_shape(positions)
        if data.ndim != 3 or data.shape[2] != 3:
            raise ValueError(f"data must have 3 dims (T,N,3), got {data.shape}")
        T, N, _ = data.shape
        self._init_time(times, interpolation, extrapolation, storage, "jax")
        if self.times.shape != (T,):
            raise ValueError(f"times shape {self.times.shape} != (T,) with T={T}")
        if positions.shape != (N, 3):
            raise ValueError(f"positions shape {positions.shape} != (N,3) with N={N}")
        self.data, self.positions = data, positions
        self.T, self.N = T, N
        self._source_info = _source_info or {}
        self.octree_mesh = OctreeMesh(positions, connectivity, max_elements_per_leaf, max_depth, octree_build)

    def _device(self):
        if self._dev is not None:
            return
        torch = _torch_cuda()
        m = self.octree_mesh
        pairs, scales = build_pairs_device(self.data, self._storage)
        self._scales = scales
        pts = np.zeros((self.N, 4), dtype=F32)
        pts[:, :3] = self.positions
        d = {"pairs": pairs, "points": torch.from_numpy(pts).cuda()}
        if m.dev is not None:       # built on the device: no upload (the box records get their own copy)
            d.update({k: m.dev[k] for k in ("tet_geom", "nodes", "elems")})
            d["tet_box"] = m.dev["tet_box"].clone()
        else:
            d.update({"tet_box": torch.from_numpy(m.tet_box).cuda(), "tet_geom": torch.from_numpy(m.tet_geom).cuda(),
                      "nodes": torch.from_numpy(m.nodes.view(np.int32).reshape(len(m.nodes), 16)).cuda(),
                      "elems": torch.from_numpy(m.elems).cuda()})
        self._dev = d
        self.n_near_degenerate = _mark_near_degenerate(d["tet_box"], d["tet_geom"])
        f = L.MeshField()
        f.n_points, f.n_tets = self.N, m.connectivity.shape[0]
        f.n_nodes, f.max_depth = int(m.info.n_nodes), m.max_depth
        f.storage, f.n_pairs, f.pair_stride = self._storage, pairs.shape[0], self.N
        f.points, f.tet_box, f.tet_geom = d["points"].data_ptr(), d["tet_box"].data_ptr(), d["tet_geom"].data_ptr()
        f.nodes, f.elems, f.pairs = d["nodes"].data_ptr(), d["elems"].data_ptr(), pairs.data_ptr()
        f.near_degenerate = int(self.n_near_degenerate > 0)
        bfs = breadth_first_descent(m.nodes)
        if bfs is not None:
            d["desc"], d["dtab"] = (torch.from_numpy(a).cuda() for a in bfs)
            f.desc, f.dtab = d["desc"].data_ptr(), d["dtab"].data_ptr()
        self._cmesh = f
        self._cfield = L.Field(kind=L.JT_FIELD_MESH, mesh=C.pointer(f))

    def _device_pairs(self):
        self._device()
        return self._dev["pairs"]

    def get_spatial_bounds(self):
        return self.positions.min(axis=0).astype(F32), self.positions.max(axis=0).astype(F32)

    def __repr__(self) -> str:
        m = self.octree_mesh
        return (f"OctreeFEMTimeSeriesFieldOptimized(data={self.data.shape}, times={self.times.shape}, "
                f"positions={self.positions.shape}, elements={m.connectivity.shape[0]}, "
                f"octree_nodes={len(m.nodes)}, octree_leaves={int(m.nodes_is_leaf.sum())}, "
                f"interpolation='{self.interpolation}', extrapolation='{self.extrapolation}')")


# names the reference keeps for TimeSeriesField (fields/time_series.py:631-633)
TimeDependentVelocityField = TimeSeriesField
TimeVaryingField = TimeSeriesField
