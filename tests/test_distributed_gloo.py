"""The multi-GPU sharding logic on CPU ranks (gloo, world size 2): particle
slices, ensemble assignment, row gathering and the KDE grid reduction.  The
tracking itself is replaced by a host function of the positions; what is
checked is that every particle is advanced exactly once and comes back in
its original place."""
import os
import socket

import numpy as np
import pytest

from jaxtrace_gb300 import distributed as D


def test_shard_bounds_cover_every_particle_once():
    for n in (0, 1, 5, 1001, 16_777_216):
        for world in (1, 2, 3, 8):
            spans = [D.shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        D.shard_bounds(10, 2, 2)


def test_shard_ensembles_balanced_and_complete():
    rng = np.random.default_rng(7)
    sizes = np.round(10 ** rng.uniform(3, 6, 256)).astype(np.int64)
    for world in (2, 4, 8):
        parts = D.shard_ensembles(sizes, world)
        flat = sorted(e for p in parts for e in p)
        assert flat == list(range(256))
        loads = [int(sizes[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= sizes.max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(1)
        x0 = rng.random((1001, 3)).astype(np.float32)
        seen = []

        def run(x):
            seen.append(len(x))
            return x * 2.0 + 1.0                     # stands in for the tracking kernel

        out = D.track_sharded(run, x0)
        out_all = D.track_sharded(run, x0, to_all=True)
        grid = torch.full((4, 5), float(rank + 1), dtype=torch.float32)
        D.allreduce_sum(grid)
        res = {"rank": rank, "local": seen, "grid": grid.numpy().copy(),
               "all_ok": bool(np.array_equal(out_all, x0 * 2.0 + 1.0))}
        if rank == 0:
            res["ok"] = bool(np.array_equal(out, x0 * 2.0 + 1.0))
        else:
            res["none"] = out is None
        q.put(res)
    finally:
        dist.destroy_process_group()


def test_sharded_tracking_and_grid_reduction_on_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda r: r["rank"])
    assert res[0]["ok"] and res[1]["none"]
    assert res[0]["all_ok"] and res[1]["all_ok"]
    assert res[0]["local"] == [501, 501] and res[1]["local"] == [500, 500]
    for r in res:
        assert np.all(r["grid"] == 3.0)


def test_nccl_collectives_take_device_tensors(monkeypatch):
    """Under NCCL the helpers hand the collectives tensors on the rank's
    CUDA device (NCCL rejects host tensors); the backend, the device and the
    collective are stand-ins here, so this runs without a GPU."""
    import torch
    import torch.distributed as dist
    monkeypatch.setattr(dist, "is_initialized", lambda: True)
    monkeypatch.setattr(dist, "get_world_size", lambda *a: 2)
    monkeypatch.setattr(dist, "get_rank", lambda *a: 0)
    monkeypatch.setattr(dist, "get_backend", lambda *a: "nccl")
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 3)
    assert D.collective_device() == torch.device("cuda", 3)
    # route "the device" to the meta device to watch what the collectives get
    monkeypatch.setattr(D, "collective_device", lambda: torch.device("meta"))
    seen = []

    def fake_all_gather(parts, t):
        seen.append(t.device.type)
        for p in parts:
            p.copy_(t)

    def fake_all_reduce(t, op=None):
        seen.append(t.device.type)

    monkeypatch.setattr(dist, "all_gather", fake_all_gather)
    monkeypatch.setattr(dist, "all_reduce", fake_all_reduce)
    out = D.gather_rows(torch.zeros((3, 3)), 5)
    assert out.device.type == "meta" and out.shape == (5, 3)
    with pytest.raises(ValueError, match="slice of 5 is 3"):   # rank 0 of 2 owns rows [0, 3)
        D.gather_rows(torch.zeros((4, 3)), 5)
    D.allreduce_sum(torch.ones((2, 2), device="meta"))
    assert seen == ["meta", "meta"]
    monkeypatch.undo()
    assert D.collective_device() == torch.device("cpu")


def _host_stand_ins():
    """Run the density estimators on the CPU: the device is the host and the
    two kernels are brute-force float64 sums (the exchange is what these
    tests check, not the kernels)."""
    import math

    import torch
    import jaxtrace_gb300.density as Dn

    Dn._torch = lambda: torch
    Dn._DEV = "cpu"

    def grid_sum(self, pts, axes):
        P = pts.double().numpy()
        g = np.meshgrid(*[np.asarray(a, np.float64) for a in axes], indexing="ij")
        G = np.stack([x.reshape(-1) for x in g], axis=1)
        d2 = ((G[:, None, :] - P[None, :, : G.shape[1]]) ** 2).sum(-1)
        return np.exp(-d2 / (2 * self.h * self.h)).sum(1).reshape([len(a) for a in axes])

    def points_sum(self, Q, pts):
        q = np.asarray(Q, np.float64)
        P = pts.double().numpy()[:, : q.shape[1]]
        d2 = ((q[:, None, :] - P[None]) ** 2).sum(-1)
        return np.exp(-d2 / (2 * self.h * self.h)).sum(1)

    def density_sum(self, Q):
        q, P = Q.double(), self.P.double()
        h = float(self._mean_h)
        r = torch.cdist(q, P) / h
        w = torch.where(r <= 1, 1 - 1.5 * r ** 2 + 0.75 * r ** 3, torch.where(r <= 2, 0.25 * (2 - r) ** 3,
                                                                              torch.zeros_like(r)))
        return w.sum(1) / (math.pi * h ** 3)

    Dn.KDEEstimator._grid_sum = grid_sum
    Dn.KDEEstimator._evaluate_points = points_sum
    Dn.SPHDensityEstimator._density_sum = density_sum
    return Dn


def _density_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        Dn = _host_stand_ins()
        rng = np.random.default_rng(9)
        P = rng.normal(0.5, 0.15, (301, 3)).astype(np.float32)
        lo, hi = D.shard_bounds(len(P), rank, world)
        mine = P[lo:hi]
        g = dist.group.WORLD
        kde_all = Dn.KDEEstimator(P, resolution=6)
        kde = Dn.KDEEstimator(mine, resolution=6, process_group=g)
        _, _, _, d_all = kde_all.evaluate_3d()
        _, _, _, d_sh = kde.evaluate_3d()
        Q = rng.random((40, 3)).astype(np.float32)
        e_all, e_sh = kde_all.evaluate(Q), kde.evaluate(Q)
        sph_all = Dn.SPHDensityEstimator(P, dimensions="3d", smoothing_length=0.1)
        sph = Dn.SPHDensityEstimator(mine, dimensions="3d", smoothing_length=0.1, process_group=g)
        q.put({"rank": rank, "h": (kde_all.h, kde.h), "n": (kde_all.N_total, kde.N_total, kde.N),
               "grid": (d_all, d_sh), "points": (e_all, e_sh),
               "sph": (sph_all.evaluate(Q), sph.evaluate(Q)), "sph_n": sph.N})
    finally:
        dist.destroy_process_group()


def test_density_estimators_shard_particles_on_two_gloo_ranks():
    """KDE: bandwidth and bounds from all ranks' moments, one grid sum per
    share, a float64 all-reduce; SPH: the shares all-gathered so every query
    sees every particle.  Each rank's result equals the single-process
    estimator on all particles."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_density_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in res:
        h_all, h_sh = r["h"]
        assert abs(h_all - h_sh) <= 1e-6 * h_all
        assert r["n"][0] == r["n"][1] == 301 and r["n"][2] in (150, 151)
        a, b = r["grid"]
        assert np.allclose(a, b, rtol=1e-5, atol=1e-7 * np.abs(a).max())
        a, b = r["points"]
        assert np.allclose(a, b, rtol=1e-5, atol=1e-7 * np.abs(a).max())
        a, b = r["sph"]
        assert r["sph_n"] == 301 and np.allclose(a, b, rtol=1e-6)
