"""Density passes of the GPU path: ``KDEEstimator`` (density/kde.py:43-282)
and ``SPHDensityEstimator`` (density/sph.py:42-380), same constructor fields.

Semantics (exact, not truncated):

* KDE: ``mean_j (2 pi)^{-d/2} exp(-|q - p_j|^2 / 2h^2)``, the formula of the
  JAX and pure-NumPy paths (kde.py:249-282), with Scott/Silverman bandwidths
  (kernels.py:30-68) and the grid normalisation of kde.py:205-240 done in
  float64.  Terms farther than ``cutoff_sigmas * h`` along an axis are
  skipped (each is below exp(-cutoff_sigmas^2/2); 5 sigma by default).
  SciPy's ``gaussian_kde(bw_method=h)`` (the reference's fallback when SciPy
  is present, kde.py:273-275) scales the kernel by the data covariance and is
  a different estimator; it is not reproduced.
* SPH: ``sum_j m_j W(|q - p_j|, h_j)`` over every particle within
  ``3 * mean(h)`` -- the NumPy brute-force path (sph.py:282-292).  The JAX
  hash grid's cap of 64 particles per cell and 512 nearest neighbours
  (neighbors.py:145-159) truncates the sum at high densities and is not
  reproduced.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Optional, Tuple, Union

import numpy as np

from . import _lib as L

F32 = np.float32


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("jaxtrace_gb300 density passes run on a CUDA GPU; none is visible")
    return torch


# ---------------------------------------------------------------------------
def scott_bandwidth(data) -> float:
    """kernels.py:30-47: mean of per-axis std (ddof=1) times n^(-1/(d+4))."""
    x = np.asarray(data)
    n, d = x.shape
    sigma = np.std(x, axis=0, ddof=1).mean()
    return sigma * n ** (-1.0 / (d + 4.0))


def silverman_bandwidth(data) -> float:
    """kernels.py:50-68."""
    x = np.asarray(data)
    n, d = x.shape
    sigma = np.std(x, axis=0, ddof=1).mean()
    factor = (4.0 / (d + 2.0)) ** (1.0 / (d + 4.0))
    return factor * sigma * n ** (-1.0 / (d + 4.0))


def gaussian_kernel(r2_over_h2, d: int):
    """kernels.py:73-95: (2 pi)^(-d/2) exp(-r^2/2h^2)."""
    norm = (2.0 * math.pi) ** (-0.5 * d)
    return norm * np.exp(-0.5 * np.asarray(r2_over_h2))


def _device_bandwidth(P_dev, rule: str) -> float:
    """The same rules on device data (float64 statistics)."""
    torch = _torch()
    x = P_dev.double()
    n, d = x.shape
    sigma = float(torch.std(x, dim=0, unbiased=True).mean())
    h = sigma * n ** (-1.0 / (d + 4.0))
    if rule == "silverman":
        h *= (4.0 / (d + 2.0)) ** (1.0 / (d + 4.0))
    return h


# ---------------------------------------------------------------------------
def _sph_cell(search: float, lo, hi, dims: int, n: int, per_cell: float = 8.0) -> float:
    """Cell edge of the SPH candidate search: about ``per_cell`` particles per
    cell on average, between search/8 and search/2.  Finer cells hug the
    support sphere (the trimmed rows of a coarse grid scan about 3x the
    sphere's particles) at the price of more rows per query, so the edge
    follows the particle density."""
    ext = [max(float(hi[a]) - float(lo[a]), 0.0) for a in range(dims)]
    live = [e for e in ext if e > 0]
    if not live or n <= 0:
        return max(search / 2.0, 1e-6)
    vol = float(np.prod(live))
    edge = (vol * per_cell / n) ** (1.0 / len(live))
    return max(min(edge, search / 2.0), search / 8.0, 1e-6)


class CellList:
    """Particles sorted by row-major cells of a uniform grid (device)."""

    def __init__(self, pos, lo, hi, cell: float, dims: int):
        torch = _torch()
        lib = L.load()
        lo = np.asarray(lo, dtype=np.float64)
        hi = np.asarray(hi, dtype=np.float64)
        ext = np.maximum(hi - lo, 0.0)
        live = [a < dims and ext[a] > 0 for a in range(3)]
        want = max(ext[a] / max(cell, 1e-30) for a in range(3) if live[a]) if any(live) else 1.0
        bits = int(np.clip(math.ceil(math.log2(max(want, 2.0))), 1, 7))
        g = L.SortGrid()
        g.origin[:] = [float(v) for v in lo]
        g.inv_cell[:] = [float((1 << bits) / ext[a]) if live[a] else 0.0 for a in range(3)]
        g.bits = bits
        g.order = L.JT_ORDER_LINEAR
        self.grid = g
        self.cell = [float(ext[a] / (1 << bits)) if live[a] else float("inf") for a in range(3)]
        n = int(pos.shape[0])
        self.n = n
        self.sorted = torch.empty_like(pos)
        self.ids = torch.empty(n, dtype=torch.int32, device=pos.device)
        self.cell_end = torch.empty(1 << (3 * bits), dtype=torch.int32, device=pos.device)
        ws = torch.empty(max(int(lib.jt_cell_sort_workspace_bytes(n, bits)), 1), dtype=torch.uint8, device=pos.device)
        L.check(lib.jt_cell_list(C.byref(g), n, L.ptr(pos), L.ptr(self.sorted), L.ptr(self.ids), L.ptr(self.cell_end),
                                 L.ptr(ws), ws.numel(), L.stream_ptr()))

    def reach(self, radius: float):
        return [int(math.ceil(radius / c)) if math.isfinite(c) and c > 0 else 0 for c in self.cell]


# The device the estimators keep their arrays on (the kernels read them
# there); the host suite substitutes the CPU to drive the multi-rank
# exchange with host stand-ins for the kernels.
_DEV = "cuda"


def _as_device_f32(positions):
    torch = _torch()
    if isinstance(positions, torch.Tensor):
        return positions.to(device=_DEV, dtype=torch.float32).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(positions, dtype=F32))).to(_DEV)


def _pad3(P2):
    torch = _torch()
    if P2.shape[1] == 3:
        return P2.contiguous()
    return torch.cat([P2, torch.zeros((P2.shape[0], 3 - P2.shape[1]), device=P2.device, dtype=P2.dtype)],
                     dim=1).contiguous()


# ---------------------------------------------------------------------------
@dataclass
class KDEEstimator:
    """kde.py:43-282 on the GPU (same fields; ``cutoff_sigmas`` is new)."""
    positions: np.ndarray
    bandwidth: Optional[float] = None
    bandwidth_rule: str = "scott"
    normalize: bool = True
    plane: str = "xy"
    slab_position: float = 0.0
    slab_thickness: float = 0.1
    resolution: Union[int, Tuple[int, int, int]] = 100
    bounds: Optional[Tuple[Tuple[float, float], ...]] = None
    cutoff_sigmas: float = 5.0
    # a torch.distributed group whose ranks each hold a share of the
    # particles: the bandwidth and the grid bounds come from all of them, each
    # rank sums its share on the grid and one float64 all-reduce adds the
    # shares (the density is a sum over particles, kde.py:249-270)
    process_group: Optional[object] = None

    def __post_init__(self):
        torch = _torch()
        P = _as_device_f32(self.positions)
        if P.ndim != 2 or P.shape[1] not in (2, 3):
            raise ValueError("positions must be (N,2) or (N,3)")
        self.N, self.D = int(P.shape[0]), int(P.shape[1])
        self.P = P
        self._lohi = None
        self.N_total = self.N
        if self.process_group is not None:
            from .distributed import global_stats
            n, _, var, lo, hi = global_stats(P, self.process_group)
            self.N_total, self._lohi = n, (lo, hi)
        if self.bandwidth is None:
            if self.bandwidth_rule not in ("scott", "silverman"):
                raise ValueError("bandwidth_rule must be 'scott' or 'silverman' if bandwidth is None")
            if self.process_group is not None:
                # the rules of kernels.py:46-68 on the moments of all ranks' particles
                d = self.D
                self.h = float(np.mean(np.sqrt(var))) * self.N_total ** (-1.0 / (d + 4.0))
                if self.bandwidth_rule == "silverman":
                    self.h *= (4.0 / (d + 2.0)) ** (1.0 / (d + 4.0))
            elif isinstance(self.positions, torch.Tensor):
                self.h = _device_bandwidth(P, self.bandwidth_rule)
            else:
                rule = scott_bandwidth if self.bandwidth_rule == "scott" else silverman_bandwidth
                self.h = float(rule(np.asarray(self.positions, dtype=F32)))
        else:
            self.h = float(self.bandwidth)

    def _reduce(self, a):
        """Sum of every rank's array (identity without a process group)."""
        if self.process_group is None:
            return a
        from .distributed import allreduce_array
        return allreduce_array(a, self.process_group)

    def _count(self, n: int) -> int:
        if self.process_group is None:
            return int(n)
        return int(round(float(self._reduce(np.array([float(n)]))[0])))

    # -- helpers (kde.py:101-119) --
    def _axes_for_plane(self):
        m = {"xy": (0, 1, 2), "xz": (0, 2, 1), "yz": (1, 2, 0)}
        if self.plane.lower() not in m:
            raise ValueError("plane must be one of 'xy','xz','yz'")
        return m[self.plane.lower()]

    def _slice_2d_points(self):
        if self.D == 2:
            return self.P
        i, j, k = self._axes_for_plane()
        mask = (self.P[:, k] - float(self.slab_position)).abs() <= float(self.slab_thickness) * 0.5
        pts2 = self.P[mask][:, [i, j]]
        if pts2.numel() == 0:
            pts2 = self.P[:, [i, j]]
        return pts2.contiguous()

    def _params(self, pts, dims, extent_lo, extent_hi):
        radius = float(self.cutoff_sigmas * self.h)
        cl = CellList(_pad3(pts), extent_lo, extent_hi, max(radius / 2.0, 1e-6), dims)
        p = L.KdeParams()
        p.dims = dims
        p.n_particles = cl.n
        p.half_inv_h2 = float(0.5 / (self.h * self.h))
        p.radius = radius
        p.grid = cl.grid
        p.particles = cl.sorted.data_ptr()
        p.cell_end = cl.cell_end.data_ptr()
        return p, cl

    def _grid_sum(self, pts, axes):
        """sum_j exp(-|g-p_j|^2/2h^2) on the tensor grid of `axes` (x, y[, z])."""
        torch = _torch()
        dims = len(axes)
        ax = [torch.from_numpy(np.ascontiguousarray(a, dtype=F32)).cuda() for a in axes]
        lo = [min(float(pts[:, a].min()), float(axes[a][0])) for a in range(dims)] + [0.0] * (3 - dims)
        hi = [max(float(pts[:, a].max()), float(axes[a][-1])) for a in range(dims)] + [0.0] * (3 - dims)
        p, cl = self._params(pts, dims, lo, hi)
        res = [len(a) for a in axes] + [1] * (3 - dims)
        out = torch.empty(int(np.prod(res)), dtype=torch.float64, device="cuda")
        p.res[:] = res
        for a in range(dims):
            p.axis[a] = ax[a].data_ptr()
        # work counters for measurement (a device int64 pair), when asked for
        counters = getattr(self, "count_into", None)
        if counters is not None and dims == 3:
            p.counters = counters.data_ptr()
        p.out = out.data_ptr()
        L.check(L.load().jt_kde_grid(C.byref(p), L.stream_ptr()))
        return out.reshape(res[:dims]).cpu().numpy()

    def _evaluate_points(self, Q, pts):
        torch = _torch()
        d = int(Q.shape[1])
        Q3 = _pad3(_as_device_f32(Q))
        lo = [min(float(pts[:, a].min()), float(Q3[:, a].min())) for a in range(d)] + [0.0] * (3 - d)
        hi = [max(float(pts[:, a].max()), float(Q3[:, a].max())) for a in range(d)] + [0.0] * (3 - d)
        p, cl = self._params(pts, d, lo, hi)
        out = torch.empty(Q3.shape[0], dtype=torch.float64, device="cuda")
        L.check(L.load().jt_kde_points(C.byref(p), L.ptr(Q3), Q3.shape[0], L.ptr(out), L.stream_ptr()))
        return out.cpu().numpy()                       # sum_j exp(-|q - p_j|^2 / 2h^2)

    # -- public API --
    def evaluate(self, points) -> np.ndarray:
        """kde.py:123-169."""
        Q = np.asarray(points, dtype=F32) if not hasattr(points, "device") else points
        if Q.ndim != 2:
            raise ValueError(f"points must be 2D, got {tuple(Q.shape)}")
        if self.D == 2:
            if Q.shape[1] == 3:
                i, j, _ = self._axes_for_plane()
                Q = Q[:, [i, j]]
            elif Q.shape[1] != 2:
                raise ValueError(f"Expected points with 2 or 3 columns, got {Q.shape[1]}")
            pts = self.P
        else:
            if Q.shape[1] == 3:
                pts = self.P
            elif Q.shape[1] == 2:
                pts = self._slice_2d_points()
                Q = Q[:, [0, 1]]
            else:
                raise ValueError(f"Expected points with 2 or 3 columns, got {Q.shape[1]}")
        d = int(Q.shape[1])
        s = self._reduce(self._evaluate_points(Q, pts))
        norm = (2.0 * math.pi) ** (-0.5 * d)
        return (s * (norm / max(self._count(int(pts.shape[0])), 1))).astype(F32)

    def _bounds_lohi(self, pts, k):
        if self.bounds is None:
            if self._lohi is not None and pts is self.P:
                return self._lohi[0][:k], self._lohi[1][:k]
            return pts.min(dim=0).values.cpu().numpy(), pts.max(dim=0).values.cpu().numpy()
        lo = np.array([b[0] for b in self.bounds[:k]], dtype=float)
        hi = np.array([b[1] for b in self.bounds[:k]], dtype=float)
        return lo, hi

    def evaluate_3d(self):
        """kde.py:188-201 grid, :223-240 normalisation; returns X, Y, Z, D of shape (ny, nx, nz)."""
        lo, hi = self._bounds_lohi(self.P, 3)
        res = self.resolution if not isinstance(self.resolution, int) else (self.resolution,) * 3
        nx, ny, nz = map(int, res)
        x = np.linspace(lo[0], hi[0], nx, dtype=np.float32)
        y = np.linspace(lo[1], hi[1], ny, dtype=np.float32)
        z = np.linspace(lo[2], hi[2], nz, dtype=np.float32)
        X, Y, Z = np.meshgrid(x, y, z, indexing="xy")
        s = self._reduce(self._grid_sum(self.P, (x, y, z)))   # (nx, ny, nz), all ranks' particles
        D = s.transpose(1, 0, 2) * ((2.0 * math.pi) ** -1.5 / self.N_total)
        if self.normalize:
            D = self._normalise(D, [X, Y, Z], [1, 0, 2])
        return X, Y, Z, D.astype(F32)

    def evaluate_2d(self):
        """kde.py:173-186 grid, :205-221 normalisation; returns X, Y, Z of shape (ny, nx)."""
        pts = self.P[:, :2].contiguous() if self.D == 2 else self._slice_2d_points()
        if self.bounds is None:
            lo, hi = pts.min(dim=0).values.cpu().numpy(), pts.max(dim=0).values.cpu().numpy()
            if self.process_group is not None:
                from .distributed import global_stats
                _, _, _, lo, hi = global_stats(pts, self.process_group)
        else:
            lo = np.array([self.bounds[0][0], self.bounds[1][0]], dtype=float)
            hi = np.array([self.bounds[0][1], self.bounds[1][1]], dtype=float)
        res = self.resolution if isinstance(self.resolution, int) else self.resolution[:2]
        nx = ny = int(res) if isinstance(res, int) else int(res[0])
        x = np.linspace(lo[0], hi[0], nx, dtype=np.float32)
        y = np.linspace(lo[1], hi[1], ny, dtype=np.float32)
        X, Y = np.meshgrid(x, y, indexing="xy")
        s = self._reduce(self._grid_sum(pts, (x, y)))         # (nx, ny), all ranks' particles
        Z = s.T * ((2.0 * math.pi) ** -1.0 / max(self._count(int(pts.shape[0])), 1))
        if self.normalize:
            Z = self._normalise(Z, [X, Y], [1, 0])
        return X, Y, Z.astype(F32)

    def _normalise(self, D, grids, axis_of):
        """Rescale so sum(D)*cell = N, then divide by N/domain (float64)."""
        cell = 1.0
        dom = 1.0
        for k, G in enumerate(grids):
            span = float(G.max() - G.min())
            cell *= span / max(G.shape[axis_of[k]] - 1, 1)
            dom *= span
        total = float((D * cell).sum())
        if total > 0:
            D = D * (self.N / total)
        avg = self.N / max(dom, 1e-12)
        return D / max(avg, 1e-12)


# ---------------------------------------------------------------------------
_SPH_KERNELS = {"cubic_spline": L.JT_SPH_CUBIC, "wendland": L.JT_SPH_WENDLAND, "gaussian": L.JT_SPH_GAUSSIAN}


def pair_records(positions, masses=None):
    """The paired particle records of jt_sph_params (packed = 2): (ceil(N/2), 8)
    float32 rows {x0, x1, y0, y1, z0, z1, m0, m1} for particles 2k and 2k+1
    of ``positions`` (N,3), unit masses when ``masses`` is None; an odd N
    pads the last row with zeros.  On the positions' device."""
    import torch
    n = int(positions.shape[0])
    m = masses[:, None] if masses is not None else torch.ones((n, 1), dtype=torch.float32, device=positions.device)
    rec = torch.cat([positions, m], dim=1)
    n_pairs = (n + 1) // 2
    if 2 * n_pairs != n:
        rec = torch.cat([rec, rec.new_zeros((1, 4))])
    return rec.reshape(n_pairs, 2, 4).transpose(1, 2).reshape(n_pairs, 8).contiguous()


@dataclass
class SPHDensityEstimator:
    """sph.py:42-380 on the GPU (same fields)."""
    positions: np.ndarray
    dimensions: str = "2d"
    plane: str = "xy"
    position: float = 0.0
    slab_thickness: float = 0.1
    smoothing_length: Optional[float] = None
    kernel_type: str = "cubic_spline"
    adaptive: bool = False
    n_neighbors: int = 32
    masses: Optional[np.ndarray] = None
    max_particles_for_adaptive: int = 5000
    neighbor_search: str = "hashgrid"
    per_cell_cap: int = 64
    max_neighbors: int = 512
    normalize: bool = True
    resolution: Union[int, Tuple[int, int, int]] = 100
    bounds: Optional[Tuple[Tuple[float, float], ...]] = None
    # a torch.distributed group whose ranks each hold a share of the
    # particles: every query needs every particle within reach, so the shares
    # (and masses) are all-gathered first and each rank then evaluates its
    # own queries against all particles
    process_group: Optional[object] = None

    def __post_init__(self):
        torch = _torch()
        if self.kernel_type not in _SPH_KERNELS:
            raise ValueError(f"Unknown kernel type: {self.kernel_type}")
        P3 = _as_device_f32(self.positions)
        if self.process_group is not None:
            from .distributed import gather_all
            P3 = gather_all(P3, self.process_group).contiguous()
            if self.masses is not None:
                self.masses = gather_all(_as_device_f32(np.asarray(self.masses, dtype=F32).reshape(-1)),
                                         self.process_group).cpu().numpy()
        if self.dimensions.lower() == "2d":
            if P3.shape[1] != 3:
                raise ValueError("2D SPH requires (N,3) positions for slicing")
            self.P = self._extract_2d(P3)
            self.D = 2
        else:
            if P3.shape[1] != 3:
                raise ValueError("3D SPH requires (N,3) positions")
            self.P = P3
            self.D = 3
        self.N = int(self.P.shape[0])
        if self.N < 2:
            raise ValueError("At least two particles are required")
        if self.masses is None:
            self.masses_dev = None
        else:
            m = _as_device_f32(np.asarray(self.masses, dtype=F32).reshape(-1))
            if m.shape[0] != self.N:
                raise ValueError("masses must be length N")
            self.masses_dev = m
        if self.smoothing_length is not None:
            self.smoothing_lengths = torch.full((self.N,), float(self.smoothing_length), dtype=torch.float32,
                                                device=_DEV)
            self._uniform_h = float(F32(self.smoothing_length))
        else:
            self.smoothing_lengths = self._calculate_smoothing_lengths()
        self._mean_h = float(self.smoothing_lengths.mean())

    # sph.py:164-177
    def _extract_2d(self, P3):
        m = {"xy": (0, 1, 2), "xz": (0, 2, 1), "yz": (1, 2, 0)}
        if self.plane.lower() not in m:
            raise ValueError("plane must be one of 'xy','xz','yz'")
        i, j, k = m[self.plane.lower()]
        mask = (P3[:, k] - float(self.position)).abs() <= float(self.slab_thickness) * 0.5
        pts2 = P3[mask][:, [i, j]]
        if pts2.numel() == 0:
            pts2 = P3[:, [i, j]]
        return pts2.contiguous()

    # sph.py:181-223
    def _calculate_smoothing_lengths(self):
        torch = _torch()
        self._uniform_h = None
        if self.adaptive and self.N <= int(self.max_particles_for_adaptive):
            k = int(min(self.n_neighbors, max(self.N - 1, 1)))
            d = torch.cdist(self.P.double(), self.P.double())
            kth = torch.kthvalue(d, k + 1, dim=1).values          # argpartition(d, k)[k]
            return (1.2 * kth).float()
        n_per_dim = self.N ** (1.0 / self.D)
        pmin = self.P.min(dim=0).values.cpu().numpy()
        pmax = self.P.max(dim=0).values.cpu().numpy()
        domain_size = np.mean(pmax - pmin)
        h = domain_size / n_per_dim * 2.0
        h = np.clip(h, 0.01, domain_size * 0.1)
        self._uniform_h = float(F32(h))
        return torch.full((self.N,), float(h), dtype=torch.float32, device=_DEV)

    def _density_sum(self, Q):
        torch = _torch()
        Q3 = _pad3(Q)
        M = int(Q3.shape[0])
        radius = float(F32(3.0) * F32(self._mean_h))           # sph.py:284-285
        hmax = float(self.smoothing_lengths.max())
        kern = _SPH_KERNELS[self.kernel_type]
        support = {L.JT_SPH_CUBIC: 2.0 * hmax, L.JT_SPH_WENDLAND: hmax, L.JT_SPH_GAUSSIAN: radius}[kern]
        search = min(radius, support * 1.0001)
        P3 = _pad3(self.P)
        d = self.D
        lo = [min(float(P3[:, a].min()), float(Q3[:, a].min())) for a in range(d)] + [0.0] * (3 - d)
        hi = [max(float(P3[:, a].max()), float(Q3[:, a].max())) for a in range(d)] + [0.0] * (3 - d)
        cell = _sph_cell(search, lo, hi, d, int(P3.shape[0]))
        cl = CellList(P3, lo, hi, cell, d)
        # queries in the same cell order, so a warp's queries walk the same
        # candidate cells together (broadcast loads); results scattered back
        qcl = CellList(Q3, lo, hi, cell, d)
        idx = cl.ids.long()
        h_sorted = None if self._uniform_h is not None else self.smoothing_lengths[idx].contiguous()
        m_sorted = None if self.masses_dev is None else self.masses_dev[idx].contiguous()
        out = torch.empty(M, dtype=torch.float64, device="cuda")
        p = L.SphParams()
        p.dims, p.kernel = d, kern
        p.n_particles, p.n_queries = cl.n, M
        p.radius = radius
        p.h_const = self._uniform_h if self._uniform_h is not None else 0.0
        p.grid = cl.grid
        p.reach[:] = cl.reach(search)
        p.masses = None
        if h_sorted is None:
            # uniform h: two 16-byte loads per two candidates
            P4 = pair_records(cl.sorted, m_sorted)
            p.packed = 2
            p.particles = P4.data_ptr()
        else:
            p.packed = 0
            p.particles = cl.sorted.data_ptr()
            p.masses = m_sorted.data_ptr() if m_sorted is not None else None
        p.h = h_sorted.data_ptr() if h_sorted is not None else None
        p.cell_end = cl.cell_end.data_ptr()
        p.queries = qcl.sorted.data_ptr()
        out_sorted = torch.empty(M, dtype=torch.float64, device="cuda")
        p.out = out_sorted.data_ptr()
        # work counters for measurement (a device int64 pair), when asked for
        counters = getattr(self, "count_into", None)
        if counters is not None:
            p.counters = counters.data_ptr()
        L.check(L.load().jt_sph_density(C.byref(p), L.stream_ptr()))
        out.index_copy_(0, qcl.ids.long(), out_sorted)
        return out

    def evaluate(self, eval_points) -> np.ndarray:
        """sph.py:333-380."""
        Q = _as_device_f32(eval_points)
        if Q.ndim != 2:
            raise ValueError(f"eval_points must be 2D, got {tuple(Q.shape)}")
        if self.D == 2:
            if Q.shape[1] == 3:
                m = {"xy": (0, 1, 2), "xz": (0, 2, 1), "yz": (1, 2, 0)}
                i, j, _ = m[self.plane.lower()]
                Q = Q[:, [i, j]].contiguous()
            elif Q.shape[1] != 2:
                raise ValueError(f"2D SPH expects (M,2) or (M,3) points, got {tuple(Q.shape)}")
        elif Q.shape[1] != 3:
            raise ValueError(f"3D SPH expects (M,3) points, got {tuple(Q.shape)}")
        rho = self._density_sum(Q)
        if self.normalize:
            mins = Q.min(dim=0).values.cpu().numpy().astype(np.float64)
            maxs = Q.max(dim=0).values.cpu().numpy().astype(np.float64)
            vol = float(np.prod(maxs[: self.D] - mins[: self.D]))
            vol = max(vol, 1e-12)
            rho = rho / (self.N / vol)
        return rho.float().cpu().numpy()


__all__ = ["KDEEstimator", "SPHDensityEstimator", "scott_bandwidth", "silverman_bandwidth", "gaussian_kernel",
           "CellList"]
